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

// ----------------------------------------------------------------------------
// continuous emission: MapGrid / MapGridEmit (src/core/grid.h:1289-1402)
// ----------------------------------------------------------------------------
__global__ void k_map(int n, const float4 *__restrict__ pos, const unsigned *__restrict__ cell,
                      const unsigned *__restrict__ start, float4 *__restrict__ mpos, unsigned *__restrict__ mcell,
                      uint2 *__restrict__ mrank) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const unsigned c = cell[q];
    mpos[q] = pos[q];
    mcell[q] = c;
    mrank[q] = make_uint2((unsigned)q - start[c], start[c + 1] - start[c]);
}

__global__ void k_bucket_count(Params P, const float4 *__restrict__ pos, int first, int n,
                               unsigned *__restrict__ cellof, unsigned *__restrict__ sub,
                               unsigned *__restrict__ count) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (first + k >= n) return;
    unsigned bad = 0;
    const unsigned c = grid_hash(P.g, pos[first + k], P.iz, &bad);
    cellof[k] = c;
    sub[k] = atomicAdd(&count[c], 1u);
}

__global__ void k_bucket_place(int first, int n, const unsigned *__restrict__ cellof,
                               const unsigned *__restrict__ sub, const unsigned *__restrict__ start,
                               unsigned *__restrict__ list) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (first + k >= n) return;
    list[start[cellof[k]] + sub[k]] = (unsigned)(first + k);
}

// Distance(pj, pi) < d (geometry.h:798-800): sqrt of x*x + y*y + z*z, unfused
__device__ __forceinline__ bool closer_than(float4 a, float4 b, float d) {
    const float x = __fsub_rn(a.x, b.x), y = __fsub_rn(a.y, b.y), z = __fsub_rn(a.z, b.z);
    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
    return __fsqrt_rn(l2) < d;
}

// One mapped position: skipped when its cell holds kMaxPerCell particles or more, or when
// it is past the first (kMaxPerCell - size) positions of its cell, or when a particle of the
// cell is closer than d.
__global__ void k_map_emit(int count, const float4 *__restrict__ mpos, const unsigned *__restrict__ mcell,
                           const uint2 *__restrict__ mrank, bool sorted, const unsigned *__restrict__ start,
                           bool bucketed, const unsigned *__restrict__ bstart, const unsigned *__restrict__ blist,
                           const float4 *__restrict__ pos, float d, unsigned *__restrict__ flag) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const unsigned c = mcell[q];
    const uint2 r = mrank[q];
    const unsigned a0 = sorted ? start[c] : 0u, a1 = sorted ? start[c + 1] : 0u;
    const unsigned b0 = bucketed ? bstart[c] : 0u, b1 = bucketed ? bstart[c + 1] : 0u;
    const unsigned size = (a1 - a0) + (b1 - b0);
    bool ok = size < (unsigned)kMaxPerCell;
    if (ok) {
        const unsigned room = (unsigned)kMaxPerCell - size;
        ok = r.x < (room < r.y ? room : r.y);
    }
    if (ok) {
        const float4 p = mpos[q];
        for (unsigned j = a0; j < a1 && ok; j++) ok = !closer_than(pos[j], p, d);
        for (unsigned j = b0; j < b1 && ok; j++) ok = !closer_than(pos[blist[j]], p, d);
    }
    flag[q] = ok ? 1u : 0u;
}

__global__ void k_map_scatter(int count, int n, const unsigned *__restrict__ flag, const unsigned *__restrict__ index,
                              const float4 *__restrict__ mpos, float3 v, float *__restrict__ pos,
                              float *__restrict__ vel) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count || !flag[q]) return;
    const unsigned k = index[q];
    if ((int)k >= n) return;
    const float4 p = mpos[q];
    pos[3 * (size_t)k] = p.x;
    pos[3 * (size_t)k + 1] = p.y;
    pos[3 * (size_t)k + 2] = p.z;
    vel[3 * (size_t)k] = v.x;
    vel[3 * (size_t)k + 1] = v.y;
    vel[3 * (size_t)k + 2] = v.z;
}

void launch_map(int n, const float4 *pos, const unsigned *cell, const unsigned *start, MapBufs &M,
                cudaStream_t s) {
    k_map<<<blocks_for(n, 256), 256, 0, s>>>(n, pos, cell, start, M.pos, M.cell, M.rank);
    M.count = n;
}

void launch_buckets(const Params &P, const float4 *pos, int first, int n, BucketBufs &K, cudaStream_t s) {
    const int m = n - first;
    if (m > 0) k_bucket_count<<<blocks_for(m, 256), 256, 0, s>>>(P, pos, first, n, K.cell, K.sub, K.count);
    launch_cell_scan(K.count, (unsigned)K.cells, K.part, K.start, s);   // leaves count zeroed
    if (m > 0) k_bucket_place<<<blocks_for(m, 256), 256, 0, s>>>(first, n, K.cell, K.sub, K.start, K.list);
}

cudaError_t map_emit_test(const MapBufs &M, bool sorted, const unsigned *start, bool bucketed,
                          const BucketBufs &K, const float4 *pos, float d, unsigned *passed,
                          unsigned *h_scratch, cudaStream_t s) {
    k_map_emit<<<blocks_for(M.count, 128), 128, 0, s>>>(M.count, M.pos, M.cell, M.rank, sorted, start, bucketed,
                                                        K.start, K.list, pos, d, M.flag);
    cudaMemcpyAsync(M.flag_copy, M.flag, sizeof(unsigned) * (size_t)M.count, cudaMemcpyDeviceToDevice, s);
    launch_cell_scan(M.flag_copy, (unsigned)M.count, M.part, M.index, s);
    cudaMemcpyAsync(h_scratch, M.index + M.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    *passed = *h_scratch;
    return e;
}

void launch_map_scatter(const MapBufs &M, int n, float3 v, float *pos, float *vel, cudaStream_t s) {
    k_map_scatter<<<blocks_for(M.count, 256), 256, 0, s>>>(M.count, n, M.flag, M.index, M.pos, v, pos, vel);
}

}  // namespace bbg
