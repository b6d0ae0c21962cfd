// emit.cu -- VolumeParticleEmitter3 (src/core/emitter.cpp:241-330) on the device.
//
// The reference walks the BCC lattice of the emitter's bounds point by point, moves each
// point by a random jitter, keeps it when the shape's signed distance is <= 0 and appends
// it to a host vector.  Here one thread takes one lattice point (its coordinates from its
// index, in the reference's float operations), the jitter offsets come from the host
// (they are the C library's rand() sequence, which is sequential), a scan of the inside
// flags numbers the kept points in lattice order, and they are written straight into the
// solver's buffers.
#include "bbg_internal.cuh"
#include "emit.h"

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ v3 lattice_point(const Lattice &L, long long t) {
    const long long s0 = (long long)L.j0 * L.i0, s1 = (long long)L.j1 * L.i1;
    const long long pair = t / (s0 + s1), rem = t - pair * (s0 + s1);
    int k, cols;
    long long local;
    float off;
    if (rem < s0) {
        k = (int)(2 * pair);
        local = rem;
        cols = L.i0;
        off = 0.f;
    } else {
        k = (int)(2 * pair + 1);
        local = rem - s0;
        cols = L.i1;
        off = L.half;
    }
    const int j = (int)(local / cols), i = (int)(local - (long long)j * cols);
    // pos = (i * spacing + offset) + pMin, unfused as the reference's host loops
    return V(__fadd_rn(__fadd_rn(__fmul_rn((float)i, L.spacing), off), L.lo[0]),
             __fadd_rn(__fadd_rn(__fmul_rn((float)j, L.spacing), off), L.lo[1]),
             __fadd_rn(__fmul_rn((float)k, L.half), L.lo[2]));
}

__global__ void k_emit_test(Lattice L, const float *__restrict__ offset, ShapeDev shape, float iz, float iz6,
                            float *__restrict__ target, unsigned *__restrict__ flag) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.total) return;
    v3 p = lattice_point(L, t);
    if (offset) {
        p.x = __fadd_rn(p.x, offset[3 * t]);
        p.y = __fadd_rn(p.y, offset[3 * t + 1]);
        p.z = __fadd_rn(p.z, offset[3 * t + 2]);
    }
    // Shape::SignedDistance (shape.cpp:284-288) <= 0: inside, or on the surface
    const Cpq q = shape_closest_point(shape, p, iz, iz6);
    const bool inside = (shape.reverse != 0) == !(q.sd < 0.f);
    const float sd = inside ? -fabsf(q.sd) : fabsf(q.sd);
    flag[t] = sd <= 0.f ? 1u : 0u;
    target[3 * t] = p.x;
    target[3 * t + 1] = p.y;
    target[3 * t + 2] = p.z;
}

__global__ void k_emit_scatter(long long total, int n, const unsigned *__restrict__ flag,
                               const unsigned *__restrict__ index, const float *__restrict__ target, float3 v,
                               float *__restrict__ pos, float *__restrict__ vel) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total || !flag[t]) return;
    const unsigned q = index[t];
    if ((int)q >= n) return;
    for (int k = 0; k < 3; k++) pos[3 * (size_t)q + k] = target[3 * t + k];
    vel[3 * (size_t)q] = v.x;
    vel[3 * (size_t)q + 1] = v.y;
    vel[3 * (size_t)q + 2] = v.z;
}

__global__ void k_append(int first, int n, const float *__restrict__ p, const float *__restrict__ v, float4 *pos,
                         float4 *vel, int *pid, int *slot, float4 *force, float4 *pforce, float *rho,
                         float *press) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = first + j;
    pos[i] = make_float4(p[3 * j], p[3 * j + 1], p[3 * j + 2], 0.f);
    vel[i] = make_float4(v[3 * j], v[3 * j + 1], v[3 * j + 2], 0.f);
    pid[i] = i;
    slot[i] = i;
    force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    pforce[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    rho[i] = 0.f;
    press[i] = 0.f;
}

cudaError_t emit_test(const Lattice &L, const ShapeDev &shape, float iz, float iz6, bool jitter, EmitBufs &E,
                      unsigned *inside, unsigned *h_scratch, cudaStream_t s) {
    k_emit_test<<<blocks_for(L.total, 256), 256, 0, s>>>(L, jitter ? E.offset : nullptr, shape, iz, iz6, E.target,
                                                         E.flag);
    // the scan zeroes its input: number the kept points from a copy of the flags
    cudaMemcpyAsync(E.flag_copy, E.flag, sizeof(unsigned) * (size_t)L.total, cudaMemcpyDeviceToDevice, s);
    launch_cell_scan(E.flag_copy, (unsigned)L.total, E.part, E.index, s);
    cudaMemcpyAsync(h_scratch, E.index + L.total, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    *inside = *h_scratch;
    return e;
}

void launch_emit_scatter(const Lattice &L, int n, const EmitBufs &E, float3 v, float *pos, float *vel,
                         cudaStream_t s) {
    k_emit_scatter<<<blocks_for(L.total, 256), 256, 0, s>>>(L.total, n, E.flag, E.index, E.target, v, pos, vel);
}

void launch_append(DevBufs &B, int state, int pid_cur, const float *pos, const float *vel, int first, int n,
                   cudaStream_t s) {
    k_append<<<blocks_for(n, 256), 256, 0, s>>>(first, n, pos, vel, B.pos[state], B.vel[state], B.pid[pid_cur],
                                                B.slot, B.force, B.pforce, B.rho, B.press);
}

}  // namespace bbg
