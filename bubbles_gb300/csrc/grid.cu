// grid.cu -- neighbour-grid rebuild and particle layout kernels.
//
// Replaces the reference's per-cell double-buffered chains and per-particle buckets
// (src/core/grid.h:391-494, src/equations/sph_equations3.cpp:487-539) with a full
// counting sort every substep:
//   1. hash + count:  cell id of every particle (exact reference hash) and its arrival
//                     index inside the cell, one atomic per distinct cell per warp
//                     (__match_any_sync aggregation);
//   2. scan:          exclusive scan of the per-cell counts -> cell start offsets (tile
//                     totals, then each tile's scan plus the sum of the tiles before it);
//   3. place:         (original id, old slot) written into its cell's range;
//   4. rank + gather: each particle's final slot is its cell start plus its rank by
//                     original id inside the cell, which makes the permutation the
//                     stable sort by (cell id, particle index) -- the reference's chain
//                     order right after DistributeByParticle (grid.h:391-407) --
//                     independent of atomic arrival order; position, velocity and id
//                     are gathered into the other ping-pong buffer.
// The reference's incremental update (DistributeToCellOpt) yields the same cell
// contents; only the chain order differs, which changes FP32 sum order, not sets.
#include "bbg_kernels.h"

namespace bbg {

constexpr int kThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__global__ void __launch_bounds__(kThreads)
k_hash_count(Params P, const float4 *__restrict__ pos, int n, unsigned *__restrict__ cell_old,
             unsigned *__restrict__ sub, unsigned *__restrict__ count, StepState *st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    unsigned bad = 0, c = 0xffffffffu;
    if (valid) c = grid_hash(P.g, pos[i], P.iz, &bad);
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    const unsigned peers = __match_any_sync(mask, c);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    const unsigned rank = __popc(peers & ((1u << lane) - 1u));
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&count[c], (unsigned)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    sub[i] = base + rank;
    cell_old[i] = c;
    if (bad) atomicAdd(&st->out_of_grid, 1u);
}

// Block-wide exclusive scan of one value per thread (kScanThreads threads).
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned *total) {
    __shared__ unsigned warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const unsigned warp_prefix = wid > 0 ? warp_sums[wid - 1] : 0u;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const unsigned *__restrict__ count, unsigned cells, unsigned *__restrict__ partials) {
    const unsigned base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    unsigned s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        unsigned idx = base + k;
        if (idx < cells) s += count[idx];
    }
    unsigned total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

// Each block scans its tile of counts and adds the sum of the tiles before it, which it
// reduces itself from the per-tile totals of k_scan_reduce (a few hundred to a few thousand
// values), so the scan takes two launches.
__global__ void __launch_bounds__(kScanThreads)
k_scan_apply(unsigned *__restrict__ count, unsigned cells, const unsigned *__restrict__ partials,
             unsigned *__restrict__ start) {
    unsigned before = 0;
    for (int t = threadIdx.x; t < (int)blockIdx.x; t += kScanThreads) before += partials[t];
    unsigned carry;
    block_excl_scan(before, &carry);
    const unsigned base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    unsigned v[kScanItems];
    unsigned s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        unsigned idx = base + k;
        v[k] = idx < cells ? count[idx] : 0u;
        s += v[k];
    }
    unsigned total;
    unsigned run = block_excl_scan(s, &total) + carry;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        unsigned idx = base + k;
        if (idx < cells) {
            start[idx] = run;
            count[idx] = 0u;   // leave the histogram zeroed for the next update
            if (idx == cells - 1) start[cells] = run + v[k];
        }
        run += v[k];
    }
}

__global__ void __launch_bounds__(kThreads)
k_place(int n, const unsigned *__restrict__ cell_old, const unsigned *__restrict__ sub,
        const unsigned *__restrict__ start, const int *__restrict__ pid, uint2 *__restrict__ tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned c = cell_old[i];
    tmp[start[c] + sub[i]] = make_uint2((unsigned)pid[i], (unsigned)i);
}

__global__ void __launch_bounds__(kThreads)
k_rank_gather(int n, const uint2 *__restrict__ tmp, const unsigned *__restrict__ cell_old,
              const unsigned *__restrict__ start, const float4 *__restrict__ pos_in,
              const float4 *__restrict__ vel_in, float4 *__restrict__ pos_out,
              float4 *__restrict__ vel_out, int *__restrict__ pid_out, int *__restrict__ slot,
              unsigned *__restrict__ cell, const float *__restrict__ press_in,
              float *__restrict__ pprev, StepState *st, const float *__restrict__ carry_in,
              float *__restrict__ carry_out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint2 e = tmp[t];
    const unsigned c = cell_old[e.y];
    const unsigned a = start[c], b = start[c + 1];
    unsigned dst = (unsigned)t;   // arrival order: only for cells past the cap
    if (b - a <= kRankCap) {
        unsigned rank = 0;
        for (unsigned q = a; q < b; ++q) rank += (tmp[q].x < e.x) ? 1u : 0u;
        dst = a + rank;
    } else if ((unsigned)t == a) {
        atomicAdd(&st->crowded, 1u);
    }
    pos_out[dst] = pos_in[e.y];
    vel_out[dst] = vel_in[e.y];
    pid_out[dst] = (int)e.x;
    slot[e.x] = (int)dst;
    cell[dst] = c;
    pprev[dst] = press_in[e.y];   // carried for a warm-started corrector
    if (carry_out) carry_out[dst] = carry_in[e.y];
}

size_t scan_partials_needed(unsigned cells) { return (size_t)blocks_for(cells, kScanTile) + 1; }

void launch_cell_scan(unsigned *count, unsigned cells, unsigned *partials, unsigned *start,
                      cudaStream_t s) {
    const int nb = blocks_for(cells, kScanTile);
    k_scan_reduce<<<nb, kScanThreads, 0, s>>>(count, cells, partials);
    k_scan_apply<<<nb, kScanThreads, 0, s>>>(count, cells, partials, start);
}

void launch_grid_update(const Params &P, const DevBufs &B, int src, int pid_src, cudaStream_t s,
                        const float *carry_in, float *carry_out) {
    const int n = P.n;
    const unsigned cells = P.g.total;
    const int nb = blocks_for(cells, kScanTile);
    BBG_PBEGIN(B, KID_HASH_COUNT, s, -1);
    k_hash_count<<<blocks_for(n, kThreads), kThreads, 0, s>>>(P, B.pos[src], n, B.cell_old, B.sub,
                                                              B.count, B.st);
    BBG_PEND(B, s);
    BBG_PBEGIN(B, KID_SCAN, s, -1);
    k_scan_reduce<<<nb, kScanThreads, 0, s>>>(B.count, cells, B.partials);
    k_scan_apply<<<nb, kScanThreads, 0, s>>>(B.count, cells, B.partials, B.start);
    BBG_PEND(B, s);
    if (B.prof && B.prof->on) B.prof->launches += 1;   // two scan kernels in one record
    BBG_PBEGIN(B, KID_PLACE, s, -1);
    k_place<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, B.cell_old, B.sub, B.start,
                                                         B.pid[pid_src], B.tmp);
    BBG_PEND(B, s);
    BBG_PBEGIN(B, KID_RANK_GATHER, s, -1);
    k_rank_gather<<<blocks_for(n, kThreads), kThreads, 0, s>>>(
        n, B.tmp, B.cell_old, B.start, B.pos[src], B.vel[src], B.pos[1 - src], B.vel[1 - src],
        B.pid[1 - pid_src], B.slot, B.cell, B.press, B.pprev, B.st, carry_in, carry_out);
    BBG_PEND(B, s);
}

// ----------------------------------------------------------------------------
// layout kernels
// ----------------------------------------------------------------------------
__global__ void k_upload(int n, const float *__restrict__ p, const float *__restrict__ v,
                         float4 *pos, float4 *vel, int *pid, int *slot, float4 *force,
                         float4 *pforce, float *rho, float *press) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(p[3 * i], p[3 * i + 1], p[3 * i + 2], 0.f);
    vel[i] = v ? make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    pid[i] = i;
    slot[i] = i;
    force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    pforce[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    rho[i] = 0.f;
    press[i] = 0.f;
}

__global__ void k_download(int n, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                           const int *__restrict__ pid, float *p, float *v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int id = pid[i];
    const float4 a = pos[i];
    if (p) { p[3 * id] = a.x; p[3 * id + 1] = a.y; p[3 * id + 2] = a.z; }
    if (v) {
        const float4 b = vel[i];
        v[3 * id] = b.x; v[3 * id + 1] = b.y; v[3 * id + 2] = b.z;
    }
}

__global__ void k_get_vec(const float4 *__restrict__ src, const int *__restrict__ slot, float *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = src[slot[i]];
    out[3 * i] = a.x; out[3 * i + 1] = a.y; out[3 * i + 2] = a.z;
}
__global__ void k_set_vec(float4 *dst, const int *__restrict__ slot, const float *__restrict__ in, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[slot[i]] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.f);
}
__global__ void k_get_scalar(const float *__restrict__ src, const int *__restrict__ slot, float *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = src[slot[i]];
}
__global__ void k_set_scalar(float *dst, const int *__restrict__ slot, const float *__restrict__ in, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[slot[i]] = in[i];
}
__global__ void k_get_uint(const unsigned *__restrict__ src, const int *__restrict__ slot, unsigned *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = src[slot[i]];
}
__global__ void k_get_int(const int *__restrict__ src, const int *__restrict__ slot, int *out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = src[slot[i]];
}
__global__ void k_fill_vec(float4 *dst, float x, float y, float z, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float4(x, y, z, 0.f);
}

// max_i |F_i| with the reference's Length() (sqrt of x*x + y*y + z*z, no contraction)
__global__ void __launch_bounds__(kThreads)
k_max_force(const float4 *__restrict__ f, int n, unsigned *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned bits = 0;
    if (i < n) bits = __float_as_uint(vlen(V(f[i])));
    bits = warp_max_u(bits);
    if ((threadIdx.x & 31) == 0 && bits) atomicMax(out, bits);
}

void launch_upload(const DevBufs &B, int buf, int pid_buf, const float *d_pos, const float *d_vel,
                   int n, cudaStream_t s) {
    BBG_PBEGIN(B, KID_LAYOUT, s, -1);
    k_upload<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, d_pos, d_vel, B.pos[buf], B.vel[buf],
                                                          B.pid[pid_buf], B.slot, B.force, B.pforce,
                                                          B.rho, B.press);
    BBG_PEND(B, s);
}
void launch_download(const DevBufs &B, int buf, int pid_buf, float *d_pos, float *d_vel, int n,
                     cudaStream_t s) {
    BBG_PBEGIN(B, KID_LAYOUT, s, -1);
    k_download<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, B.pos[buf], B.vel[buf], B.pid[pid_buf],
                                                            d_pos, d_vel);
    BBG_PEND(B, s);
}
void launch_get_vec(const float4 *src, const int *slot, float *out, int n, cudaStream_t s) {
    k_get_vec<<<blocks_for(n, kThreads), kThreads, 0, s>>>(src, slot, out, n);
}
void launch_set_vec(float4 *dst, const int *slot, const float *in, int n, cudaStream_t s) {
    k_set_vec<<<blocks_for(n, kThreads), kThreads, 0, s>>>(dst, slot, in, n);
}
void launch_get_scalar(const float *src, const int *slot, float *out, int n, cudaStream_t s) {
    k_get_scalar<<<blocks_for(n, kThreads), kThreads, 0, s>>>(src, slot, out, n);
}
void launch_set_scalar(float *dst, const int *slot, const float *in, int n, cudaStream_t s) {
    k_set_scalar<<<blocks_for(n, kThreads), kThreads, 0, s>>>(dst, slot, in, n);
}
void launch_get_uint(const unsigned *src, const int *slot, unsigned *out, int n, cudaStream_t s) {
    k_get_uint<<<blocks_for(n, kThreads), kThreads, 0, s>>>(src, slot, out, n);
}
void launch_get_int(const int *src, const int *slot, int *out, int n, cudaStream_t s) {
    k_get_int<<<blocks_for(n, kThreads), kThreads, 0, s>>>(src, slot, out, n);
}
void launch_fill_vec(float4 *dst, float x, float y, float z, int n, cudaStream_t s) {
    k_fill_vec<<<blocks_for(n, kThreads), kThreads, 0, s>>>(dst, x, y, z, n);
}
void launch_max_force(const float4 *force, int n, unsigned *out_bits, cudaStream_t s) {
    cudaMemsetAsync(out_bits, 0, sizeof(unsigned), s);
    k_max_force<<<blocks_for(n, kThreads), kThreads, 0, s>>>(force, n, out_bits);
}

}  // namespace bbg
