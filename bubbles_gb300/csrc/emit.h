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

// ---- continuous emission (ContinuousParticleSetBuilder3, src/core/grid.h:1246-1450) ----
constexpr int kMaxPerCell = 100;   // MaximumParticlesPerBucket (src/core/particle.h:10)

// MapGrid: the particles of every occupied cell, positions in chain (sorted) order.
struct MapBufs {
    int count = 0, cap = 0;
    float4 *pos = nullptr;       // mapped positions
    unsigned *cell = nullptr;    // their cells
    uint2 *rank = nullptr;       // (index within the cell, the cell's mapped count)
    unsigned *flag = nullptr, *flag_copy = nullptr, *index = nullptr, *part = nullptr;
};

// Cell lists of the particles in sorted slots [first, n) (those not in the last grid
// distribution's ranges): count, start (cells + 1), list of slots grouped by cell.
struct BucketBufs {
    size_t cells = 0, cap = 0;
    unsigned *count = nullptr, *start = nullptr, *part = nullptr;
    unsigned *cell = nullptr, *sub = nullptr, *list = nullptr;
};

// MapGrid from the last grid distribution: n sorted slots with their cells and cell starts.
void launch_map(int n, const float4 *pos, const unsigned *cell, const unsigned *start, MapBufs &M,
                cudaStream_t s);
// Cell lists of slots [first, n) of pos.
void launch_buckets(const Params &P, const float4 *pos, int first, int n, BucketBufs &K, cudaStream_t s);
// MapGridEmit's test of each mapped position against the particles of its cell now (the
// sorted ranges of the last distribution when `sorted`, plus the bucketed slots when
// `bucketed`); returns how many pass (synchronises).
cudaError_t map_emit_test(const MapBufs &M, bool sorted, const unsigned *start, bool bucketed,
                          const BucketBufs &K, const float4 *pos, float d, unsigned *passed,
                          unsigned *h_scratch, cudaStream_t s);
// The first n passing positions, in map order, to pos (xyz); vel = v.
void launch_map_scatter(const MapBufs &M, int n, float3 v, float *pos, float *vel, cudaStream_t s);

}  // namespace bbg
