// boundary.cu -- boundary classification of the particles on the sorted grid:
// src/boundaries/lnm.h (LNMBoundary with its fast, Xiaowei and Dilts L2 filters,
// LNMBoundarySingle, LNMBoundaryExtended), xiaowei.h and dilts.h.
//
// The reference walks its cells' chains; here a cell's particles are the slot range of the
// last grid distribution (the chain order).  Cell passes run one thread per cell and only
// write their own cell's level, reading levels that no pass of the same launch changes,
// so they equal the reference's sequential sweeps.  Particle passes run one thread per
// slot and write in the caller's order.  Every float operation of the two geometric tests
// is explicitly rounded in the reference's order, the kernel weights' double steps included.
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

namespace {

__device__ __forceinline__ unsigned held(const unsigned *start, unsigned c) { return start[c + 1] - start[c]; }

__global__ void k_lnm_l1(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    level[c] = -1;
    if (held(start, c) < 1) return;
    const int x = (int)(c % (unsigned)g.nx), y = (int)((c / (unsigned)g.nx) % (unsigned)g.ny);
    const int z = (int)(c / ((unsigned)g.nx * (unsigned)g.ny));
    const int x0 = x > 0 ? x - 1 : 0, x1 = x + 1 < g.nx ? x + 1 : g.nx - 1;
    const int y0 = y > 0 ? y - 1 : 0, y1 = y + 1 < g.ny ? y + 1 : g.ny - 1;
    const int z0 = z > 0 ? z - 1 : 0, z1 = z + 1 < g.nz ? z + 1 : g.nz - 1;
    if ((x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1) != 27) {   // GetNeighborsOf count
        level[c] = 1;
        return;
    }
    for (int k = z0; k <= z1; k++)
        for (int j = y0; j <= y1; j++)
            for (int i = x0; i <= x1; i++)
                if (held(start, (unsigned)i + (unsigned)j * g.nx + (unsigned)k * g.nx * g.ny) == 0) {
                    level[c] = 1;
                    return;
                }
}

__global__ void k_lnm_l2(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level, int delta) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    if (held(start, c) < 1 || level[c] == 1) return;
    const int x = (int)(c % (unsigned)g.nx), y = (int)((c / (unsigned)g.nx) % (unsigned)g.ny);
    const int z = (int)(c / ((unsigned)g.nx * (unsigned)g.ny));
    for (int k = z > 0 ? z - 1 : 0; k <= (z + 1 < g.nz ? z + 1 : g.nz - 1); k++)
        for (int j = y > 0 ? y - 1 : 0; j <= (y + 1 < g.ny ? y + 1 : g.ny - 1); j++)
            for (int i = x > 0 ? x - 1 : 0; i <= (x + 1 < g.nx ? x + 1 : g.nx - 1); i++) {
                const unsigned nb = (unsigned)i + (unsigned)j * g.nx + (unsigned)k * g.nx * g.ny;
                // an L2 write never turns a cell into or out of L1, so the reads are stable
                if (level[nb] == 1 && held(start, nb) <= (unsigned)delta) {
                    level[c] = 2;
                    return;
                }
            }
}

__global__ void k_lnm_particles(int n, const unsigned *__restrict__ cell, const int *__restrict__ pid,
                                const int *__restrict__ level, int *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int L = level[cell[q] & ~kWide];
    out[pid[q]] = (L == 1 || L == 2) ? L : 0;
}

__device__ __forceinline__ void coords(const GridDev &g, unsigned c, int u[3]) {
    u[0] = (int)(c % (unsigned)g.nx);
    u[1] = (int)((c / (unsigned)g.nx) % (unsigned)g.ny);
    u[2] = (int)(c / ((unsigned)g.nx * (unsigned)g.ny));
}

__device__ __forceinline__ unsigned linear(const GridDev &g, int x, int y, int z) {
    return (unsigned)x + (unsigned)y * (unsigned)g.nx + (unsigned)z * (unsigned)g.nx * (unsigned)g.ny;
}

__device__ __forceinline__ bool on_border(const GridDev &g, const int u[3]) {
    return u[0] == 0 || u[1] == 0 || u[2] == 0 || u[0] == g.nx - 1 || u[1] == g.ny - 1 || u[2] == g.nz - 1 ||
           g.nx < 3 || g.ny < 3 || g.nz < 3;
}

// LNMBoundaryAreCoords1x1: distinct cells at most one step apart on every axis
__device__ __forceinline__ bool adjacent(const int a[3], const int b[3]) {
    const int dx = abs(a[0] - b[0]), dy = abs(a[1] - b[1]), dz = abs(a[2] - b[2]);
    return dx < 2 && dy < 2 && dz < 2 && dx + dy + dz > 0;
}

// LNMBoundarySingleKernel (lnm.h:167-238).  The 5x5x5 walk (y, then x, then z) stops at the
// first empty adjacent cell (L1) or the first adjacent cell holding at most delta particles
// that lies on the border (L2).  Without a stop every empty cell of the walk is a source and
// every adjacent cell holding 1..delta particles a candidate, and the cell is L2 when a
// candidate touches a source: with no empty cell adjacent to this one, the sources a
// candidate touches are exactly the empty cells adjacent to the candidate, all inside the walk.
__global__ void k_lnm_single(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level, int delta) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    level[c] = -1;
    if (held(start, c) == 0) return;
    int u[3];
    coords(g, c, u);
    if (on_border(g, u)) {
        level[c] = 1;
        return;
    }
    for (int j = u[1] - 2; j <= u[1] + 2; j++) {
        if (j < 0 || j >= g.ny) continue;
        for (int i = u[0] - 2; i <= u[0] + 2; i++) {
            if (i < 0 || i >= g.nx) continue;
            for (int k = u[2] - 2; k <= u[2] + 2; k++) {
                if (k < 0 || k >= g.nz) continue;
                const int f[3] = {i, j, k};
                const unsigned fid = linear(g, i, j, k);
                if (fid == c || !adjacent(f, u)) continue;
                const unsigned n = held(start, fid);
                if (n == 0) {
                    level[c] = 1;
                    return;
                }
                if (n <= (unsigned)delta && on_border(g, f)) {
                    level[c] = 2;
                    return;
                }
            }
        }
    }
    for (int j = u[1] - 1; j <= u[1] + 1; j++)
        for (int i = u[0] - 1; i <= u[0] + 1; i++)
            for (int k = u[2] - 1; k <= u[2] + 1; k++) {
                const unsigned fid = linear(g, i, j, k);
                if (fid == c || held(start, fid) > (unsigned)delta) continue;
                for (int b = j - 1; b <= j + 1; b++) {
                    if (b < 0 || b >= g.ny) continue;
                    for (int a = i - 1; a <= i + 1; a++) {
                        if (a < 0 || a >= g.nx) continue;
                        for (int e = k - 1; e <= k + 1; e++) {
                            if (e < 0 || e >= g.nz) continue;
                            if (held(start, linear(g, a, b, e)) == 0) {
                                level[c] = 2;
                                return;
                            }
                        }
                    }
                }
            }
}

// LNMOnceKernel / LNMComputeOnce (lnm.h:332-378) at reference level L
__global__ void k_lnm_once(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level, int L,
                           int *__restrict__ changed) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    if (L == 0) level[c] = -1;   // LNMInvalidateCells
    if (level[c] > -1) return;
    int u[3];
    coords(g, c, u);
    int v = -1;
    if (held(start, c) == 0) v = 0;
    else if (on_border(g, u)) v = 1;
    else if (L > 0) {
        for (int k = u[2] - 1; k <= u[2] + 1 && v < 0; k++)
            for (int j = u[1] - 1; j <= u[1] + 1 && v < 0; j++)
                for (int i = u[0] - 1; i <= u[0] + 1; i++) {
                    const unsigned nb = linear(g, i, j, k);
                    if (nb != c && level[nb] == L - 1) {
                        v = L;
                        break;
                    }
                }
    }
    if (v >= 0) {
        level[c] = v;
        *changed = 1;
    }
}

// LNMParticleAttributesKernel (lnm.h:418-432): the level of the cell of each particle's
// hashed position (positive levels only)
__global__ void k_lnm_attributes(int n, GridDev g, float iz, const float4 *__restrict__ pos,
                                 const int *__restrict__ level, int *__restrict__ val) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    unsigned bad = 0;
    const int L = level[grid_hash(g, pos[q], iz, &bad)];
    val[q] = L > 0 ? L : 0;
}

// LNMBoundaryLKKernel (lnm.h:304-330): a non-L1 cell with particles next to an L1 cell holding
// at most delta particles becomes -2 (its particles L2)
__global__ void k_lnm_lk(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level, int delta) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    if (held(start, c) == 0 || level[c] == 1) return;
    int u[3];
    coords(g, c, u);
    for (int k = max(u[2] - 1, 0); k <= min(u[2] + 1, g.nz - 1); k++)
        for (int j = max(u[1] - 1, 0); j <= min(u[1] + 1, g.ny - 1); j++)
            for (int i = max(u[0] - 1, 0); i <= min(u[0] + 1, g.nx - 1); i++) {
                const unsigned nb = linear(g, i, j, k);
                if (level[nb] == 1 && held(start, nb) <= (unsigned)delta) {
                    level[c] = -2;
                    return;
                }
            }
}

// the extended variant's particle levels: L1 cells 1, filtered cells 2, unfiltered level-2
// cells 3 (LNMBoundaryExtendL2Kernel), else the attribute of the hashed position
__global__ void k_lnm_extended_out(int n, const unsigned *__restrict__ cell, const int *__restrict__ pid,
                                   const int *__restrict__ level, const int *__restrict__ val, int *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int L = level[cell[q] & ~kWide];
    out[pid[q]] = L == 1 ? 1 : L == -2 ? 2 : L == 2 ? 3 : val[q];
}

// per slot: the L1 cells' particles 1, the rest 0; the particles of L2 cells queued
__global__ void k_lnm_queue(int n, const unsigned *__restrict__ cell, const int *__restrict__ pid,
                            const int *__restrict__ level, int *__restrict__ queue, int *__restrict__ counts,
                            int *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int L = level[cell[q] & ~kWide];
    out[pid[q]] = L == 1 ? 1 : 0;
    if (L == 2) queue[atomicAdd(&counts[0], 1)] = q;
}

__device__ __forceinline__ float exact_distance(float4 a, float4 b) {
    const float ex = fs(a.x, b.x), ey = fs(a.y, b.y), ez = fs(a.z, b.z);
    return __fsqrt_rn(fa(fa(fm(ex, ex), fm(ey, ey)), fm(ez, ez)));
}

// the 27 cells around the cell of p (GetNeighborsOf order: y, then x, then z), each cell's
// slots in chain order; fn(slot) returns true to stop
template <typename Fn>
__device__ __forceinline__ void around(const BoundaryArgs &A, float4 p, Fn fn) {
    unsigned bad = 0;
    int u[3];
    coords(A.g, grid_hash(A.g, p, A.iz, &bad), u);
    for (int j = max(u[1] - 1, 0); j <= min(u[1] + 1, A.g.ny - 1); j++)
        for (int i = max(u[0] - 1, 0); i <= min(u[0] + 1, A.g.nx - 1); i++)
            for (int k = max(u[2] - 1, 0); k <= min(u[2] + 1, A.g.nz - 1); k++) {
                const unsigned nb = linear(A.g, i, j, k);
                for (unsigned s = A.start[nb]; s < A.start[nb + 1]; s++)
                    if (fn(s)) return;
            }
}

// XiaoweiParticleIsBoundary (xiaowei.h:21-78)
__device__ int xiaowei(const BoundaryArgs &A, unsigned q) {
    if (A.rho[q] < A.x_rhot) return 1;
    const float4 pi = A.pos[q];
    float sx = 0.f, sy = 0.f, sz = 0.f, wsum = 0.f;
    around(A, pi, [&](unsigned s) {
        const float4 pj = A.pos[s];
        const float d = exact_distance(pi, pj);
        // SphStdKernel3::W at radius 6h (kernel.cpp:123-132)
        const float d2 = fm(d, d);
        const float of = fs(d2, A.x_h2);
        float w = 0.f;
        if (!(fabsf(of) < A.iz || of > 0.f)) {
            const double x = (double)fs(1.f, fdv(d2, A.x_h2));
            w = __double2float_rn(__dmul_rn(__dmul_rn(__dmul_rn(A.x_wc, x), x), x));
        }
        sx = fa(sx, fm(pj.x, w));
        sy = fa(sy, fm(pj.y, w));
        sz = fa(sz, fm(pj.z, w));
        wsum = fa(wsum, w);
        return false;
    });
    const float inv = fdv(1.f, wsum);
    const float4 m = make_float4(fm(sx, inv), fm(sy, inv), fm(sz, inv), 0.f);
    return (double)exact_distance(pi, m) > A.x_limit ? 1 : 0;
}

// DiltsSpokeParticleIsBoundary (dilts.h:110-153).  The overlapping neighbours (at most 1024,
// in walk order) are kept in a per-thread array up to kDiltsLocal; past that the spoke test
// walks the cells again for the rest.
constexpr int kDiltsLocal = 48;

__device__ int dilts(const BoundaryArgs &A, unsigned q) {
    const float4 pi = A.pos[q];
    const float rad = A.d_rad, lim = A.d_lim;
    float4 loc[kDiltsLocal];
    int n = 0;
    around(A, pi, [&](unsigned s) {
        if (s != q) {
            const float4 pj = A.pos[s];
            if (!(exact_distance(pi, pj) > lim)) {
                if (n < kDiltsLocal) loc[n] = pj;
                n++;
                if (n == 1024) return true;
            }
        }
        return false;
    });
    const int nl = n < kDiltsLocal ? n : kDiltsLocal;
    for (int i = 0; i <= 64; i++) {
        const float su = A.spoke[i], cu = A.spoke[65 + i];
        for (int j = 0; j <= 64; j++) {
            const float sv = A.spoke[130 + j], cv = A.spoke[195 + j];
            const float4 pt = make_float4(fa(fm(fm(su, cv), rad), pi.x), fa(fm(fm(su, sv), rad), pi.y),
                                          fa(fm(cu, rad), pi.z), 0.f);
            bool inside = false;
            for (int t = 0; t < nl; t++)
                if (exact_distance(loc[t], pt) <= rad) {
                    inside = true;
                    break;
                }
            if (!inside && n > kDiltsLocal) {
                int seen = 0;
                around(A, pi, [&](unsigned s) {
                    if (s == q) return false;
                    const float4 pj = A.pos[s];
                    if (exact_distance(pi, pj) > lim) return false;
                    if (seen++ < kDiltsLocal) return false;
                    if (exact_distance(pj, pt) <= rad) inside = true;
                    return inside || seen >= 1024;
                });
            }
            if (!inside) return 1;
        }
    }
    return 0;
}

// LNMBoundaryL2GeomKernel (lnm.h:57-79): each queued particle marked 2 when the test says so
__global__ void k_lnm_geometric(BoundaryArgs A, int algorithm, const int *__restrict__ queue, int *__restrict__ counts,
                                int *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= counts[0]) return;
    const unsigned q = (unsigned)queue[t];
    const int b = algorithm == 1 ? xiaowei(A, q) : dilts(A, q);
    if (b > 0) {
        out[A.pid[q]] = 2;
        atomicAdd(&counts[1], 1);
    }
}

// XiaoweiBoundary / DiltsSpokeBoundary over every particle
__global__ void k_boundary_test(BoundaryArgs A, int algorithm, int n, int *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    out[A.pid[q]] = algorithm == 1 ? xiaowei(A, (unsigned)q) : dilts(A, (unsigned)q);
}

}  // namespace

void launch_lnm_single(const GridDev &g, const unsigned *start, const unsigned *cell, const int *pid, int n,
                       int delta, int *level, int *out, cudaStream_t s) {
    k_lnm_single<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level, delta);
    k_lnm_particles<<<blocks_for(n, 256), 256, 0, s>>>(n, cell, pid, level, out);
}

void launch_lnm_once(const GridDev &g, const unsigned *start, int *level, int L, int *changed, cudaStream_t s) {
    k_lnm_once<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level, L, changed);
}

void launch_lnm_extended_finish(const GridDev &g, float iz, const float4 *pos, const unsigned *start,
                                const unsigned *cell, const int *pid, int n, int delta, int *level, int *val,
                                int *out, cudaStream_t s) {
    k_lnm_attributes<<<blocks_for(n, 256), 256, 0, s>>>(n, g, iz, pos, level, val);
    k_lnm_lk<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level, delta);
    k_lnm_extended_out<<<blocks_for(n, 256), 256, 0, s>>>(n, cell, pid, level, val, out);
}

void launch_lnm_geometric(const BoundaryArgs &A, const unsigned *cell, int n, int delta, int algorithm,
                          int *level, int *queue, int *counts, int *out, cudaStream_t s) {
    k_lnm_l1<<<blocks_for(A.g.total, 256), 256, 0, s>>>(A.g, A.start, level);
    k_lnm_l2<<<blocks_for(A.g.total, 256), 256, 0, s>>>(A.g, A.start, level, delta);
    cudaMemsetAsync(counts, 0, 2 * sizeof(int), s);
    k_lnm_queue<<<blocks_for(n, 256), 256, 0, s>>>(n, cell, A.pid, level, queue, counts, out);
    k_lnm_geometric<<<blocks_for(n, 128), 128, 0, s>>>(A, algorithm, queue, counts, out);
}

void launch_boundary_test(const BoundaryArgs &A, int algorithm, int n, int *out, cudaStream_t s) {
    k_boundary_test<<<blocks_for(n, 128), 128, 0, s>>>(A, algorithm, n, out);
}

void launch_lnm(const GridDev &g, const unsigned *start, const unsigned *cell, const int *pid, int n, int delta,
                int *level, int *out, cudaStream_t s) {
    k_lnm_l1<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level);
    k_lnm_l2<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level, delta);
    k_lnm_particles<<<blocks_for(n, 256), 256, 0, s>>>(n, cell, pid, level, out);
}

}  // namespace bbg
