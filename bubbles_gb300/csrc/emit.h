// emit.h -- particle seeding on the device: VolumeParticleEmitter3's BCC lattice in a box
// or sphere (emit.cu).
#pragma once

#include "bbg_kernels.h"

namespace bbg {

// The lattice of BccLatticePointGenerator::ForEach (src/generator/bcclattice.cpp:6-36)
// over [lo, lo + extent]: layer k at z = k * half + lo.z, rows and columns at
// j * spacing + offset, offset = half on odd layers.  Even layers hold j0 x i0 points, odd
// layers j1 x i1; points are numbered in the reference's loop order (k, j, i).
struct Lattice {
    float lo[3];
    float spacing, half;
    int layers;
    int i0, j0, i1, j1;
    long long total;
};

struct EmitBufs {
    size_t cap = 0;
    float *target = nullptr;     // 3 per lattice point
    float *offset = nullptr;     // 3 per lattice point (jitter), host-made
    unsigned *flag = nullptr, *flag_copy = nullptr, *index = nullptr, *part = nullptr;
};

// Each lattice point (plus its jitter offset, when given) tested against the shape
// (Shape::SignedDistance <= 0); returns how many are inside (synchronises).
cudaError_t emit_test(const Lattice &L, const ShapeDev &shape, float iz, float iz6, bool jitter, EmitBufs &E,
                      unsigned *inside, unsigned *h_scratch, cudaStream_t s);
// The first n inside points, in lattice order, to pos (xyz); vel = v.
void launch_emit_scatter(const Lattice &L, int n, const EmitBufs &E, float3 v, float *pos, float *vel,
                         cudaStream_t s);
// Appends n particles (xyz arrays) after the first `first` sorted slots of the state
// buffers, with ids first .. first + n - 1 and zero forces, density and pressure.
void launch_append(DevBufs &B, int state, int pid_cur, const float *pos, const float *vel, int first, int n,
                   cudaStream_t s);

}  // namespace bbg
