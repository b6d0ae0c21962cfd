// sph.cu -- neighbour-sum passes of the 3D SPH / PCISPH step (FP32, one thread per
// particle over the cell-sorted arrays).
//
// Neighbour sets follow the reference buckets: j is a neighbour of i when
// IsWithinStd(|x_i - x_j|, h) holds at the positions of the last grid update
// (src/core/grid.h:423-447).  The density pass tests every candidate of the 27 cells
// (9 contiguous slot ranges) once per substep with the exact FP32 membership test and
// records the members in a compact list (tile.cuh); later passes walk that list.  The
// predicted-density pass uses the step-start membership with values at predicted
// positions, which is what the reference does with its stale bucket
// (src/equations/pcisph_equations3.cpp:58-89).
//
// Fusions (per PCISPH substep: density, non-pressure, 2 per corrector iteration):
//   - non-pressure force + the k = 0 prediction (PredictVelocityAndPositionFor);
//   - pressure force of iteration k + either the prediction of iteration k+1 or, once
//     the density error of iteration k is below tolerance (or k is the last allowed
//     iteration), AccumulateForcesFor + TimeIntegrationFor into the other buffer.
// The iteration decision is read from device memory (max error of each iteration), so
// the host launches max_iterations x 2 kernels without synchronising; kernels of
// iterations after convergence return immediately.
#include <climits>

#include "bbg_kernels.h"
#include "tile.cuh"

namespace bbg {

constexpr int kThreads = kTile;

#ifndef BBG_NBR_MIN_BLOCKS
#define BBG_NBR_MIN_BLOCKS 8
#endif
#ifndef BBG_PF_MIN_BLOCKS
#define BBG_PF_MIN_BLOCKS 12
#endif
// resident 128-thread blocks per SM the member-walking passes are compiled for (register
// budget; build-time tuning knobs, measured: 12 for the pressure-force pass, which trades
// a few spilled registers for occupancy, 8 for the others).  Kernels are compiled for
// blocks of up to kMaxTile threads with the same register budget.
constexpr int kNbrMinBlocks = BBG_NBR_MIN_BLOCKS * kTile / kMaxTile;
#ifndef BBG_PD_MIN_BLOCKS
#define BBG_PD_MIN_BLOCKS 16
#endif
// the predicted-density pass fits 32 registers without spilling (gather batch 4): full
// occupancy for its latency-bound gathers
constexpr int kPdMinBlocks = BBG_PD_MIN_BLOCKS * kTile / kMaxTile;
constexpr int kPfMinBlocks = BBG_PF_MIN_BLOCKS * kTile / kMaxTile;
#ifndef BBG_PDWL_MIN_BLOCKS
#define BBG_PDWL_MIN_BLOCKS 16
#endif
#ifndef BBG_PFWL_MIN_BLOCKS
#define BBG_PFWL_MIN_BLOCKS 12
#endif
// register budgets of the persistent batch passes, as the per-tile passes' (measured on
// config 4: 8 blocks per SM, 48 and 64 registers without spills, lost 6 % to these, which
// spill a little)
constexpr int kPdWlMinBlocks = BBG_PDWL_MIN_BLOCKS * kTile / kMaxTile;
constexpr int kPfWlMinBlocks = BBG_PFWL_MIN_BLOCKS * kTile / kMaxTile;
constexpr int kDensityMinBlocks = 12 * kTile / kMaxTile;
#ifndef BBG_DENSITY_MASK
#define BBG_DENSITY_MASK 1
#endif
// density pass: branch-free candidate loop with membership bit masks (build-time choice;
// measured 4 % faster than the branchy loop on GB300)
constexpr bool kDensityMask = BBG_DENSITY_MASK != 0;
#ifndef BBG_DENSITY_X2
#define BBG_DENSITY_X2 1
#endif
// density pass on packed pairs of candidates (f32x2 arithmetic on structure-of-arrays
// positions; build-time choice)
constexpr bool kDensityX2 = BBG_DENSITY_X2 != 0;

// Two floats in one 64-bit register pair, for the packed f32x2 instructions of sm_100+.
typedef unsigned long long f2;
__device__ __forceinline__ f2 f2_pack(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// a neighbour's position and velocity records
struct PosVel {
    float4 p, v;
};

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ bool finite_state(v3 x, v3 v) {
    return isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
}

// warp-aggregated count of the lanes with a non-finite integrated state (all lanes call it)
__device__ __forceinline__ void count_nonfinite(bool bad, StepState *st) {
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(&st->nonfinite, (unsigned)__popc(m));
}

// True when some corrector iteration before k already met the tolerance
// (ComputePressureForceAndIntegrate's break, pcisph_equations3.cpp:243-246).
__device__ __forceinline__ bool converged_before(const Params &P, const StepState *st, int k) {
    for (int q = 0; q < k; q++) {
        float e = __uint_as_float(st->err_bits[q]);
        if (fdv(e, P.target_density) < P.max_err_ratio) return true;
    }
    return false;
}

// Batch: true when scene s met the tolerance at an iteration before k (its particles
// are integrated and skip the rest of the corrector).
__device__ __forceinline__ bool scene_converged_before(const Params &P, int s, int k) {
    const SceneState &ss = P.scene_st[s];
    for (int q = 0; q < k; q++) {
        float e = __uint_as_float(ss.err_bits[q]);
        if (fdv(e, P.target_density) < P.max_err_ratio) return true;
    }
    return false;
}

// ComputeDensityFor + ComputePressureValue, src/equations/sph_equations3.cpp:7-58.
// Tests every candidate of the 27 cells exactly once per substep and records the
// neighbour set (the reference bucket, grid.h:423-447) as a compact member list.
__global__ void __launch_bounds__(kMaxTile, kDensityMinBlocks)
k_density(Params P, float4 *__restrict__ pos, float4 *__restrict__ vel, unsigned *__restrict__ cell,
          const unsigned *__restrict__ start, float *__restrict__ rho, float *__restrict__ inv_rho,
          float *__restrict__ press, int *__restrict__ nbr, ListEntry *__restrict__ list,
          int compute_pressure, StepState *st) {
    __shared__ TileMap T;
    tile_setup(P.g, cell, start, P.n, T);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float4 pi = pos[i];
    const unsigned cw = cell[i];
    const size_t n = (size_t)P.n;
    float sum = 0.f;
    int cnt = 0;      // bucket members, i included
    int listed = 0;   // members other than i
    bool fits = true;
    const bool crowded = candidate_count(P.g, start, cw & ~kWide) > kMaxCandidates;
    if (crowded) {
        // past the work cap: the particle itself only (counted, see kMaxCandidates)
        sum = 1.f;
        cnt = 1;
        atomicAdd(&st->crowded, 1u);
    } else if (kDensityMask) {
        // branch-free candidate loop: membership of up to 32 consecutive candidates as a bit
        // mask, the list entries of the members written afterwards
        tile_rows(P.g, start, cw & ~kWide, [&](int r, unsigned b, unsigned e) {
            const unsigned base = kListRelative ? ((unsigned)r << kOffBits) - (unsigned)T.lo[r] : 0u;
            if (kListRelative && e - (unsigned)T.lo[r] > (unsigned)kOffLimit) fits = false;
            for (unsigned cb = b; cb < e; cb += 32u) {
                const unsigned ce = min(e, cb + 32u);
                unsigned m = 0u;
                for (unsigned j = cb; j < ce; ++j) {
                    const float4 pj = __ldg(&pos[j]);
                    const float r2 = dist2(pi, pj);
                    const bool mem = r2 < P.nb_lo || (r2 <= P.nb_hi && std_member_exact(P, pi, pj));
                    const float x = 1.f - r2 * P.inv_h2;
                    sum += mem ? x * x * x : 0.f;
                    m |= (unsigned)mem << (j - cb);
                }
                cnt += __popc(m);
                if ((unsigned)i - cb < ce - cb) m &= ~(1u << ((unsigned)i - cb));   // the particle itself
                while (m) {
                    const unsigned j = cb + (unsigned)(__ffs((int)m) - 1);
                    m &= m - 1u;
                    if (listed < kMaxList) list[(size_t)listed * n + (size_t)i] = list_code(j, base);
                    listed++;
                }
            }
        });
    } else tile_candidates_coded(P.g, start, T, cw & ~kWide, &fits, [&](unsigned j, unsigned base) {
        const float4 pj = __ldg(&pos[j]);
        const float r2 = dist2(pi, pj);
        if (std_member(P, pi, pj, r2)) {
            const float x = 1.f - r2 * P.inv_h2;
            sum += x * x * x;
            cnt++;
            if (j != (unsigned)i) {
                if (listed < kMaxList) list[(size_t)listed * n + (size_t)i] = list_code(j, base);
                listed++;
            }
        }
    });
    const float di = sum * P.std_c * P.mass;
    if (compute_pressure) {
        float p = P.eos_scale_over_exp * (powf(di / P.target_density, P.eos_exp) - 1.f);
        if (p < 0.f) p *= P.neg_scale;
        press[i] = p;
        reinterpret_cast<float *>(&pos[i])[3] = p / (di * di);   // pos.w = p / rho^2
    }
    rho[i] = di;
    const float ir = 1.f / di;
    inv_rho[i] = ir;
    reinterpret_cast<float *>(&vel[i])[3] = ir;                   // vel.w = 1 / rho
    nbr[i] = cnt;
    if (P.nscenes > 0) P.scene[i] = (unsigned short)scene_of(P, pi.z);
    if (listed > kMaxList || !fits) cell[i] = cw | kWide;
    if (cnt > kBucketCap) atomicAdd(&st->nbr_overflow, 1u);
}

// Positions regrouped for the packed density pass: slots 2k and 2k + 1 share a record of six
// floats (x of both, y of both, z of both), so a pair's coordinates are three float2 loads
// from one address.
__global__ void __launch_bounds__(kThreads)
k_soa(int n, const float4 *__restrict__ pos, float *__restrict__ rec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    float *r = rec + 6 * (size_t)(i >> 1) + (i & 1);
    r[0] = p.x;
    r[2] = p.y;
    r[4] = p.z;
}

// k_density with candidates taken two at a time: the even-aligned pairs of each 32-candidate
// chunk load x, y, z as float2 from the structure-of-arrays copy and compute both squared
// distances and kernel terms with f32x2 instructions; the membership test, the running sum
// in candidate order and the member list are those of k_density.
__global__ void __launch_bounds__(kMaxTile, kDensityMinBlocks)
k_density_x2(Params P, float4 *__restrict__ pos, float4 *__restrict__ vel, unsigned *__restrict__ cell,
             const unsigned *__restrict__ start, const float *__restrict__ rec, float *__restrict__ rho,
             float *__restrict__ inv_rho,
             float *__restrict__ press, int *__restrict__ nbr, ListEntry *__restrict__ list, int compute_pressure,
             StepState *st, int prune) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float4 pi = pos[i];
    const unsigned cw = cell[i];
    const size_t n = (size_t)P.n;
    float s0 = 0.f;
    int cnt = 0;      // bucket members, i included
    int listed = 0;   // members other than i
    // past kMaxCandidates in its 27 cells a particle is crowded: its rows stop being walked
    // as soon as the running candidate count passes the cap (the work stays bounded), and
    // it keeps only itself, as in k_density
    bool crowded = false;
    unsigned seen = 0;
    {
        const f2 X = f2_pack(pi.x, pi.x), Y = f2_pack(pi.y, pi.y), Z = f2_pack(pi.z, pi.z);
        const f2 NIH = f2_pack(-P.inv_h2, -P.inv_h2), ONE = f2_pack(1.f, 1.f);
        const float lo = P.nb_lo, hi = P.nb_hi, ih2 = P.inv_h2;
        tile_rows_pruned(P, start, pi, cw & ~kWide, prune != 0, [&](int, unsigned b, unsigned e, unsigned whole) {
            if (crowded) return;
            seen += whole;   // the work cap counts the 27 cells' candidates, walked or not
            if (seen > kMaxCandidates) {
                crowded = true;
                return;
            }
            for (unsigned cb = b; cb < e; cb += 32u) {
                const unsigned ce = min(e, cb + 32u);
                unsigned m = 0u;
                unsigned j = cb;
                auto single = [&](unsigned q) {
                    const float *r = rec + 6 * (size_t)(q >> 1) + (q & 1u);
                    const float4 pj = make_float4(__ldg(&r[0]), __ldg(&r[2]), __ldg(&r[4]), 0.f);
                    const float r2 = dist2(pi, pj);
                    const bool mem = r2 < lo || (r2 <= hi && std_member_exact(P, pi, pj));
                    const float x = 1.f - r2 * ih2;
                    s0 += mem ? x * x * x : 0.f;
                    m |= (unsigned)mem << (q - cb);
                };
                if (j & 1u) single(j++);
                for (; j + 1u < ce; j += 2u) {
                    const float2 *r = reinterpret_cast<const float2 *>(rec + 3 * (size_t)j);   // j even
                    const float2 ax = __ldg(&r[0]), ay = __ldg(&r[1]), az = __ldg(&r[2]);
                    const f2 dx = f2_sub(f2_pack(ax.x, ax.y), X);
                    const f2 dy = f2_sub(f2_pack(ay.x, ay.y), Y);
                    const f2 dz = f2_sub(f2_pack(az.x, az.y), Z);
                    const f2 r2 = f2_fma(dz, dz, f2_fma(dx, dx, f2_mul(dy, dy)));
                    const f2 x = f2_fma(r2, NIH, ONE);
                    const f2 x3 = f2_mul(f2_mul(x, x), x);
                    float r0, r1, c0, c1;
                    f2_unpack(r2, r0, r1);
                    f2_unpack(x3, c0, c1);
                    bool m0 = r0 < lo, m1 = r1 < lo;
                    if ((!m0 && r0 <= hi) || (!m1 && r1 <= hi)) {   // rare: the exact test's band
                        if (!m0 && r0 <= hi) m0 = std_member_exact(P, pi, make_float4(ax.x, ay.x, az.x, 0.f));
                        if (!m1 && r1 <= hi) m1 = std_member_exact(P, pi, make_float4(ax.y, ay.y, az.y, 0.f));
                    }
                    s0 += m0 ? c0 : 0.f;   // one running sum in candidate order
                    s0 += m1 ? c1 : 0.f;
                    m |= ((unsigned)m0 | ((unsigned)m1 << 1)) << (j - cb);
                }
                if (j < ce) single(j);
                cnt += __popc(m);
                if ((unsigned)i - cb < ce - cb) m &= ~(1u << ((unsigned)i - cb));   // the particle itself
                while (m) {
                    const unsigned q = cb + (unsigned)(__ffs((int)m) - 1);
                    m &= m - 1u;
                    if (listed < kMaxList) list[(size_t)listed * n + (size_t)i] = list_code(q, 0u);
                    listed++;
                }
            }
        });
    }
    if (crowded) {
        s0 = 1.f;
        cnt = 1;
        listed = 0;
        atomicAdd(&st->crowded, 1u);
    }
    const float di = s0 * P.std_c * P.mass;
    if (compute_pressure) {
        float p = P.eos_scale_over_exp * (powf(di / P.target_density, P.eos_exp) - 1.f);
        if (p < 0.f) p *= P.neg_scale;
        press[i] = p;
        reinterpret_cast<float *>(&pos[i])[3] = p / (di * di);   // pos.w = p / rho^2
    }
    rho[i] = di;
    const float ir = 1.f / di;
    inv_rho[i] = ir;
    reinterpret_cast<float *>(&vel[i])[3] = ir;                   // vel.w = 1 / rho
    nbr[i] = cnt;
    if (P.nscenes > 0) P.scene[i] = (unsigned short)scene_of(P, pi.z);
    if (listed > kMaxList) cell[i] = cw | kWide;
    if (cnt > kBucketCap) atomicAdd(&st->nbr_overflow, 1u);
}

// ComputeNonPressureForceFor (sph_equations3.cpp:80-110), optionally followed by the
// k = 0 PredictVelocityAndPositionFor (pcisph_equations3.cpp:3-28).
//   predict 0: forces only; 1: the reference's k = 0 prediction (p = 0, Fp = 0, x* from F);
//   WARM: the corrector's warm start has set p and pos.w = p / rho^2 for every particle,
//   so the same member walk also sums the pressure force of that start
//   (PredictPressureForceFor, pcisph_equations3.cpp:114-155) and x* comes from F + Fp.
// With DIV it also accumulates sum_j (1/rho_j) (1 - d/h)^2 / d (v_j - v_i).(x_j - x_i),
// the velocity divergence up to m * 45 / (pi h^4), a feature of the learned warm start.
template <bool DIV, bool WARM, int NB>
__global__ void __launch_bounds__(kMaxTile, kNbrMinBlocks)
k_non_pressure(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
               const unsigned *__restrict__ cell,
               const unsigned *__restrict__ start, const ListEntry *__restrict__ list, const int *__restrict__ nbr,
               float4 *__restrict__ force, float4 *__restrict__ xstar, float4 *__restrict__ pforce,
               float *__restrict__ press, float *__restrict__ divsum, int predict, float dt, float dt_over_m) {
    const int s0 = tile_of_block(P, blockIdx.x, (P.n + (int)blockDim.x - 1) / (int)blockDim.x) * blockDim.x;
    if (s0 >= P.n) return;
    __shared__ TileMap T;
    tile_setup_at(P.g, cell, start, s0, T);
    const int i = s0 + threadIdx.x;
    if (i >= P.n) return;
    const float4 pi = pos[i];
    const float4 vi = vel[i];
    const float ai = pi.w;   // WARM: p_i / rho_i^2
    float fx = P.mass * P.gx - P.drag * vi.x;
    float fy = P.mass * P.gy - P.drag * vi.y;
    float fz = P.mass * P.gz - P.drag * vi.z;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    float dv = 0.f;
    const float kv = P.visc_m2 * P.spiky_d2w_c;
    const float kg = P.m2 * P.spiky_dw_c;
    tile_members<NB>(
        P, start, T, list, nbr, pos, cell[i], i,
        [&](unsigned j) { return PosVel{__ldg(&pos[j]), __ldg(&vel[j])}; },
        [&](const PosVel &nb) {
            const float4 pj = nb.p, vj = nb.v;   // vj.w = 1 / rho_j
            const float r2 = dist2(pi, pj);
            const float inv_d = rsqrtf(r2);
            const float d = r2 > 0.f ? r2 * inv_d : 0.f;   // coincident particles: distance 0
            const float x = 1.f - d * P.inv_h;
            const float w = kv * x * vj.w;
            fx += (vj.x - vi.x) * w;
            fy += (vj.y - vi.y) * w;
            fz += (vj.z - vi.z) * w;
            if (WARM) {
                // as k_pressure_force: IsWithinSpiky(d, h) and d > 0 && !IsZero(d)
                if (d - P.h <= -P.iz && d >= P.iz) {
                    const float c = kg * (ai + pj.w) * x * x * inv_d;
                    tx += (pj.x - pi.x) * c;
                    ty += (pj.y - pi.y) * c;
                    tz += (pj.z - pi.z) * c;
                }
            }
            if (DIV && r2 > 0.f) {
                const float dot = (vj.x - vi.x) * (pj.x - pi.x) + (vj.y - vi.y) * (pj.y - pi.y) +
                                  (vj.z - vi.z) * (pj.z - pi.z);
                dv += vj.w * x * x * inv_d * dot;
            }
        });
    force[i] = make_float4(fx, fy, fz, 0.f);
    if (DIV) divsum[i] = dv;
    if (WARM) {
        const v3 fp = V(-tx, -ty, -tz);
        pforce[i] = F4(fp);
        v3 xs;
        predict_particle(P, dt, dt_over_m, V(fx, fy, fz), fp, V(pi), V(vi), &xs);
        xstar[i] = F4(xs);
    } else if (predict) {
        press[i] = 0.f;
        pforce[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        v3 xs;
        predict_particle(P, dt, dt_over_m, V(fx, fy, fz), V(0.f, 0.f, 0.f), V(pi), V(vi), &xs);
        xstar[i] = F4(xs);
    }
}

// PredictVelocityAndPositionFor (pcisph_equations3.cpp:3-28) on the forces already in
// `force`; with is_first: p = 0, Fp = 0, rho* = rho, so x* comes from F alone.
__global__ void __launch_bounds__(kThreads)
k_predict_first(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                const float4 *__restrict__ force, float4 *__restrict__ xstar,
                float4 *__restrict__ pforce, float *__restrict__ press,
                float *__restrict__ rhostar, const float *__restrict__ rho, float *__restrict__ derr,
                int is_first, float dt, float dt_over_m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (is_first) {
        rhostar[i] = rho[i];
        pforce[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        derr[i] = 0.f;
        press[i] = 0.f;
    }
    v3 xs;
    predict_particle(P, dt, dt_over_m, V(force[i]), V(pforce[i]), V(pos[i]), V(vel[i]), &xs);
    xstar[i] = F4(xs);
}

// Warm start of the corrector: p = scale * the start estimate (the previous substep's
// pressure), rho* = rho, and pos.w = p / rho^2 for the pressure-force pass that predicts
// x* from F + Fp(p).
__global__ void k_warm_start(int n, float4 *pos, const float *__restrict__ rho,
                             const float *__restrict__ pinit, float *__restrict__ press,
                             float *__restrict__ rhostar, float *__restrict__ derr, float scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = rho[i];
    const float p = scale * pinit[i];
    press[i] = p;
    rhostar[i] = d;
    derr[i] = 0.f;
    reinterpret_cast<float *>(&pos[i])[3] = p / (d * d);
}

// pos.w = p / rho*^2 from the pressure and predicted-density fields (used when those
// fields were set from outside rather than by the predicted-density pass).
__global__ void k_pack_acoef(int n, float4 *pos, const float *__restrict__ press,
                             const float *__restrict__ rhostar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = rhostar[i];
    reinterpret_cast<float *>(&pos[i])[3] = press[i] / (d * d);
}

// PredictPressureFor (pcisph_equations3.cpp:60-90) of particle i over the step-start
// neighbour set at predicted positions, with the density error stored (tolerance mode);
// also p / rho*^2 for the pressure force.  Returns |err| (0 for a particle not updated)
// and, in a batch, its scene (-2 once that scene met the tolerance before iteration k).
template <int NB>
__device__ __forceinline__ float pred_density_one(const Params &P, float4 *pos, const float4 *__restrict__ xstar,
                                                  const unsigned *__restrict__ cell,
                                                  const unsigned *__restrict__ start, const TileMap &T,
                                                  const ListEntry *__restrict__ list,
                                                  const int *__restrict__ nbr, float *__restrict__ press,
                                                  float *__restrict__ rhostar, float *__restrict__ derr, int k,
                                                  float delta, int clamp_total, int i, int &sc) {
    float aerr = 0.f;
    sc = -1;   // batch: scene of particle i while its corrector still runs
    if (i < P.n && P.nscenes > 0) {
        sc = P.scene[i];
        if (scene_converged_before(P, sc, k)) sc = -2;
    }
    if (i < P.n && sc != -2) {
        const float4 xi = xstar[i];
        float sum = 1.f;   // the particle itself: W_std(0) / (315 / (64 pi h^3))
        tile_members<NB, true>(
            P, start, T, list, nbr, pos, cell[i], i, [&](unsigned j) { return __ldg(&xstar[j]); },
            [&](const float4 xj) {
                const float r2 = dist2(xi, xj);
                if (r2 < P.h2mz) {
                    const float x = 1.f - r2 * P.inv_h2;
                    sum += x * x * x;
                }
            });
        const float density = sum * P.std_c * P.mass;
        float err = density - P.target_density;
        float pr = delta * err;
        float p;
        if (clamp_total) {
            // warm-started corrector: the increment may be negative, the total is scaled
            // like a negative pressure, so an overestimated start can be corrected
            if (err < 0.f) err *= P.neg_scale;
            p = press[i] + pr;
            if (p < 0.f) p *= P.neg_scale;
        } else {
            if (pr < 0.f) {
                pr *= P.neg_scale;
                err *= P.neg_scale;
            }
            p = press[i] + pr;
        }
        press[i] = p;
        rhostar[i] = density;
        derr[i] = err;
        reinterpret_cast<float *>(&pos[i])[3] = p / (density * density);   // pos.w = p / rho*^2
        aerr = fabsf(err);
    }
    return aerr;
}

// Per-scene maximum and sum of |err| of one warp's particles (lanes grouped by scene: one
// group per warp except at the boundaries between scenes).  All lanes call it.  Sums: FP32
// over the 32 lanes, FP64 from there on.
__device__ __forceinline__ void scene_error_reduce(const Params &P, int sc, float aerr, int k) {
    const int lane = threadIdx.x & 31;
    const double s = (double)warp_sum_f(aerr);
    const unsigned grp = __match_any_sync(0xffffffffu, sc);
    const unsigned gm = __reduce_max_sync(grp, __float_as_uint(aerr));
    if (sc >= 0) {
        if ((__ffs(grp) - 1) == lane && gm) atomicMax(&P.scene_st[sc].err_bits[k], gm);
        if (grp == 0xffffffffu) {
            if (lane == 0) atomicAdd(&P.scene_st[sc].err_sum[k], s);
        } else {
            atomicAdd(&P.scene_st[sc].err_sum[k], (double)aerr);
        }
    }
}

// Block reduction of max |err| (exact as bits of non-negative floats) and sum |err| into
// iteration k's totals: FP32 within a warp (at most 32 x particles-per-thread terms), FP64
// across warps and blocks.  All threads call it.
__device__ __forceinline__ void error_reduce(StepState *st, float amax, float asum, int k) {
    __shared__ unsigned smax[kMaxTile / 32];
    __shared__ double ssum[kMaxTile / 32];
    const unsigned m = warp_max_u(__float_as_uint(amax));
    const double s = (double)warp_sum_f(asum);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { smax[wid] = m; ssum[wid] = s; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned bm = 0;
        double bs = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { bm = max(bm, smax[w]); bs += ssum[w]; }
        if (bm) atomicMax(&st->err_bits[k], bm);
        atomicAdd(&st->err_sum[k], bs);
    }
}

// k < 0: iteration index from the device counter (the graph's WHILE loop only runs
// unconverged iterations); k >= 0: host-launched sequence, skip after convergence.
__device__ __forceinline__ bool corrector_iteration(const Params &P, const StepState *st, int &k) {
    if (k < 0) {
        k = st->iter;
        return true;
    }
    return !converged_before(P, st, k);
}

// Work item w of the batch's list: the tile (segment of the scene found by binary search
// over the segment offsets).
__device__ __forceinline__ int worklist_tile(const Params &P, int w) {
    int lo = 0, hi = P.nscenes;   // wl_off[lo] <= w < wl_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&P.wl_off[mid]) <= w) lo = mid;
        else hi = mid;
    }
    return __ldg(&P.wl_tile[lo]) + (w - __ldg(&P.wl_off[lo]));
}

// Number of work items, at most the number of tiles (of `slots` slots).
__device__ __forceinline__ int worklist_total(const Params &P, int slots) {
    const int tiles = (P.n + slots - 1) / slots;
    const int total = __ldg(&P.wl_off[P.nscenes]);
    return total < tiles ? total : tiles;
}

// Next work item of a persistent block (counter c; two shared slots alternate so that one
// barrier per item keeps the slot being read apart from the one being written).
__device__ __forceinline__ int worklist_next(int *ctr, int *slot, int &parity) {
    if (threadIdx.x == 0) slot[parity] = atomicAdd(ctr, 1);
    __syncthreads();
    const int w = slot[parity];
    parity ^= 1;
    return w;
}

// First slot of the block's tile of `slots` slots: the block's own, or with a batch work
// list (wl) the tile of work item blockIdx.x; -1 for a block past the list's end.
__device__ __forceinline__ int block_tile(const Params &P, int wl, int slots) {
    if (!wl) return tile_of_block(P, blockIdx.x, (P.n + slots - 1) / slots) * slots;
    if ((int)blockIdx.x >= worklist_total(P, slots)) return -1;
    return worklist_tile(P, blockIdx.x) * slots;
}

// One block per tile (all tiles, or the work list's) of PPT x blockDim slots; thread t
// takes slots t, t + blockDim, ... (PPT particles per thread).
template <int NB, int PPT>
__global__ void __launch_bounds__(kMaxTile, kPdMinBlocks)
k_pred_density(Params P, float4 *pos, const float4 *__restrict__ xstar,
               const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
               const ListEntry *__restrict__ list, const int *__restrict__ nbr, float *__restrict__ press,
               float *__restrict__ rhostar, float *__restrict__ derr, StepState *st, int k,
               float delta, int clamp_total, int wl) {
    if (!corrector_iteration(P, st, k)) return;
    const int s0 = block_tile(P, wl, PPT * blockDim.x);
    if (s0 < 0 || s0 >= P.n) return;
    __shared__ TileMap T;
    float amax = 0.f, asum = 0.f;
#pragma unroll 1
    for (int u = 0; u < PPT; u++) {
        const int su = s0 + u * blockDim.x;
        tile_setup_at(P.g, cell, start, su < P.n ? su : s0, T);
        int sc;
        const float aerr = pred_density_one<NB>(P, pos, xstar, cell, start, T, list, nbr, press, rhostar, derr,
                                                k, delta, clamp_total, su + threadIdx.x, sc);
        amax = fmaxf(amax, aerr);
        asum += aerr;
        if (P.nscenes > 0) scene_error_reduce(P, sc, aerr, k);
    }
    error_reduce(st, amax, asum, k);
}

// Batch: persistent blocks over the work list of the tiles whose scenes still run
// (launch_worklist), the same per-particle work as k_pred_density.
template <int NB>
__global__ void __launch_bounds__(kMaxTile, kPdWlMinBlocks)
k_pred_density_wl(Params P, float4 *pos, const float4 *__restrict__ xstar,
                  const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
                  const ListEntry *__restrict__ list, const int *__restrict__ nbr, float *__restrict__ press,
                  float *__restrict__ rhostar, float *__restrict__ derr, StepState *st, int k,
                  float delta, int clamp_total) {
    if (!corrector_iteration(P, st, k)) return;
    __shared__ TileMap T;
    __shared__ int slot[2];
    int parity = 0;
    const int total = worklist_total(P, blockDim.x);
    float amax = 0.f, asum = 0.f;   // this thread's particles (a few tiles): FP32 partial sum
    for (;;) {
        const int w = worklist_next(&P.wl_ctr[0], slot, parity);
        if (w >= total) break;
        const int s0 = worklist_tile(P, w) * blockDim.x;
        if (s0 < 0 || s0 >= P.n) continue;   // never for a list built by k_worklist
        tile_setup_at(P.g, cell, start, s0, T);
        int sc;
        const float aerr = pred_density_one<NB>(P, pos, xstar, cell, start, T, list, nbr, press, rhostar, derr,
                                                k, delta, clamp_total, s0 + threadIdx.x, sc);
        amax = fmaxf(amax, aerr);
        asum += aerr;
        scene_error_reduce(P, sc, aerr, k);
    }
    error_reduce(st, amax, asum, k);
}

// PredictPressureForceFor (pcisph_equations3.cpp:114-155) of particle i at the current
// positions, then either the next prediction or AccumulateForcesFor + TimeIntegrationFor.
// `last`: iteration k ends the corrector (single scene); batches decide per scene.
template <int NB>
__device__ __forceinline__ void pressure_force_one(const Params &P, const float4 *__restrict__ pos,
                                                   const float4 *__restrict__ vel,
                                                   const unsigned *__restrict__ cell,
                                                   const unsigned *__restrict__ start, const TileMap &T,
                                                   const ListEntry *__restrict__ list,
                                                   const int *__restrict__ nbr, float4 *__restrict__ force,
                                                   float4 *__restrict__ pforce, float4 *__restrict__ xstar,
                                                   float4 *__restrict__ pos_out, float4 *__restrict__ vel_out,
                                                   int k, int max_it, float dt, float dt_over_m, int mode,
                                                   bool last, int i, unsigned &fbits, bool &bad) {
    bool active = i < P.n;
    if (active && P.nscenes > 0) {
        // batch: each scene stops at its own convergence
        const int sc = P.scene[i];
        active = !scene_converged_before(P, sc, k);
        last = mode == 0 && ((k == max_it - 1) ||
                             fdv(__uint_as_float(P.scene_st[sc].err_bits[k]), P.target_density) < P.max_err_ratio);
    }
    if (!active) return;
    const float4 pi = pos[i];
    const float ai = pi.w;   // p_i / rho*_i^2
    float tx = 0.f, ty = 0.f, tz = 0.f;
    const float kg = P.m2 * P.spiky_dw_c;
    tile_members<NB>(
        P, start, T, list, nbr, pos, cell[i], i, [&](unsigned j) { return __ldg(&pos[j]); },
        [&](const float4 pj) {   // pj.w = p_j / rho*_j^2
            const float r2 = dist2(pi, pj);
            const float inv_d = rsqrtf(r2);
            const float d = r2 > 0.f ? r2 * inv_d : 0.f;   // coincident particles: distance 0
            // IsWithinSpiky(d, h) and d > 0 && !IsZero(d)
            if (d - P.h <= -P.iz && d >= P.iz) {
                const float x = 1.f - d * P.inv_h;
                const float c = kg * (ai + pj.w) * x * x * inv_d;
                tx += (pj.x - pi.x) * c;
                ty += (pj.y - pi.y) * c;
                tz += (pj.z - pi.z) * c;
            }
        });
    const v3 fp = V(-tx, -ty, -tz);
    pforce[i] = F4(fp);
    const v3 f = V(force[i]);
    if (last) {
        const v3 ft = vadd(f, fp);
        force[i] = F4(ft);
        v3 x = V(pi), v = V(vel[i]);
        integrate_particle(P, dt, ft, &x, &v);
        pos_out[i] = F4(x);
        vel_out[i] = F4(v);
        fbits = max(fbits, __float_as_uint(vlen(ft)));
        bad = bad || !finite_state(x, v);
    } else if (mode != 1) {
        v3 xs;
        predict_particle(P, dt, dt_over_m, f, fp, V(pi), V(vel[i]), &xs);
        xstar[i] = F4(xs);
    }
}

__device__ __forceinline__ bool corrector_ends(const Params &P, const StepState *st, int k, int max_it, int mode) {
    return mode == 0 && ((k == max_it - 1) ||
                         fdv(__uint_as_float(st->err_bits[k]), P.target_density) < P.max_err_ratio);
}

template <int NB, int PPT>
__global__ void __launch_bounds__(kMaxTile, kPfMinBlocks)
k_pressure_force(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                 const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
                 const ListEntry *__restrict__ list, const int *__restrict__ nbr, float4 *__restrict__ force,
                 float4 *__restrict__ pforce,
                 float4 *__restrict__ xstar, float4 *__restrict__ pos_out,
                 float4 *__restrict__ vel_out, StepState *st, int k, int max_it, float dt,
                 float dt_over_m, int mode, int wl) {
    if (!corrector_iteration(P, st, k)) return;
    const bool last = corrector_ends(P, st, k, max_it, mode);
    const int s0 = block_tile(P, wl, PPT * blockDim.x);
    if (s0 < 0 || s0 >= P.n) return;
    __shared__ TileMap T;
    unsigned fbits = 0;
    bool bad = false;   // integrated position or velocity not finite
#pragma unroll 1
    for (int u = 0; u < PPT; u++) {
        const int su = s0 + u * blockDim.x;
        tile_setup_at(P.g, cell, start, su < P.n ? su : s0, T);
        pressure_force_one<NB>(P, pos, vel, cell, start, T, list, nbr, force, pforce, xstar, pos_out, vel_out,
                               k, max_it, dt, dt_over_m, mode, last, su + threadIdx.x, fbits, bad);
    }
    fbits = warp_max_u(fbits);
    if ((threadIdx.x & 31) == 0 && fbits) atomicMax(&st->max_force_bits, fbits);
    count_nonfinite(bad, st);
}

// Batch: persistent blocks over the same work list as k_pred_density_wl.
template <int NB>
__global__ void __launch_bounds__(kMaxTile, kPfWlMinBlocks)
k_pressure_force_wl(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                    const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
                    const ListEntry *__restrict__ list, const int *__restrict__ nbr, float4 *__restrict__ force,
                    float4 *__restrict__ pforce, float4 *__restrict__ xstar, float4 *__restrict__ pos_out,
                    float4 *__restrict__ vel_out, StepState *st, int k, int max_it, float dt, float dt_over_m,
                    int mode) {
    if (!corrector_iteration(P, st, k)) return;
    __shared__ TileMap T;
    __shared__ int slot[2];
    int parity = 0;
    const int total = worklist_total(P, blockDim.x);
    unsigned fbits = 0;
    bool bad = false;
    for (;;) {
        const int w = worklist_next(&P.wl_ctr[1], slot, parity);
        if (w >= total) break;
        const int s0 = worklist_tile(P, w) * blockDim.x;
        if (s0 < 0 || s0 >= P.n) continue;   // never for a list built by k_worklist
        tile_setup_at(P.g, cell, start, s0, T);
        pressure_force_one<NB>(P, pos, vel, cell, start, T, list, nbr, force, pforce, xstar, pos_out, vel_out, k,
                               max_it, dt, dt_over_m, mode, false, s0 + threadIdx.x, fbits, bad);
    }
    fbits = warp_max_u(fbits);
    if ((threadIdx.x & 31) == 0 && fbits) atomicMax(&st->max_force_bits, fbits);
    count_nonfinite(bad, st);
}

// Batch: first and last sorted slot of every scene (both arrays preset to 0x7f7f7f7f / -1).
// The layout keeps each scene's slots contiguous and the scenes in order (containers
// stacked along z, the slowest axis of the cell order, two empty cells apart).
__global__ void __launch_bounds__(kThreads)
k_scene_slots(Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int s = P.scene[i];
    if (i == 0 || P.scene[i - 1] != s) atomicMin(&P.scene_first[s], i);
    if (i == P.n - 1 || P.scene[i + 1] != s) atomicMax(&P.scene_last[s], i);
}

// Exclusive block scan (sum, or max with identity INT_MIN) of one int per thread; *total
// gets the whole block's result.  All threads call it; sh holds 32 ints.
template <bool MAX>
__device__ __forceinline__ int block_scan_excl(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    const int id = MAX ? INT_MIN : 0;
    auto op = [](int a, int b) { return MAX ? (a > b ? a : b) : a + b; };
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = op(x, y);
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < nw ? sh[lane] : id;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t = op(t, y);
        }
        sh[lane] = t;
    }
    __syncthreads();
    const int before = __shfl_up_sync(0xffffffffu, x, 1);
    const int r = op(wid > 0 ? sh[wid - 1] : id, lane > 0 ? before : id);
    *total = sh[nw - 1];
    __syncthreads();
    return r;
}

// Batch work list of corrector iteration k (k < 0: the device counter): for every scene
// whose corrector still runs, the segment of tiles (of `tile` slots) holding its slots,
// without the tiles an earlier segment already holds; a scene that met the tolerance gets
// an empty segment.  Resets the persistent passes' counters.  One block.
__global__ void __launch_bounds__(1024)
k_worklist(Params P, const StepState *st, int k, int tile) {
    __shared__ int sh[32];
    if (k < 0) k = st->iter;
    int carry_tile = -1;   // last tile of the segments so far
    int carry_off = 0;     // work items so far
    for (int c = 0; c < P.nscenes; c += blockDim.x) {
        const int s = c + threadIdx.x;
        int ta = 0, tb = -1;
        if (s < P.nscenes) {
            const int f = P.scene_first[s], l = P.scene_last[s];
            if (l >= f && l >= 0 && !scene_converged_before(P, s, k)) {
                ta = f / tile;
                tb = l / tile;
            }
        }
        int chunk_max, chunk_sum;
        const int before = block_scan_excl<true>(tb, sh, &chunk_max);
        const int prev = max(carry_tile, before);
        if (ta <= prev) ta = prev + 1;
        const int len = tb >= ta ? tb - ta + 1 : 0;
        const int off = block_scan_excl<false>(len, sh, &chunk_sum);
        if (s < P.nscenes) {
            P.wl_off[s] = carry_off + off;
            P.wl_tile[s] = ta;
        }
        carry_tile = max(carry_tile, chunk_max);
        carry_off += chunk_sum;
    }
    if (threadIdx.x == 0) {
        P.wl_off[P.nscenes] = carry_off;
        P.wl_ctr[0] = 0;
        P.wl_ctr[1] = 0;
    }
}

// End of one corrector iteration in the graph-driven loop: stop when the density error
// of iteration k is below tolerance or k was the last allowed iteration (the break of
// ComputePressureForceAndIntegrate, pcisph_equations3.cpp:238-246).
__global__ void k_corrector_control(Params P, StepState *st, int max_it,
                                    cudaGraphConditionalHandle handle) {
    const int k = st->iter;
    const bool done = (k >= max_it - 1) ||
                      fdv(__uint_as_float(st->err_bits[k]), P.target_density) < P.max_err_ratio;
    st->iter = k + 1;
    cudaGraphSetConditional(handle, done ? 0u : 1u);
}

// ComputeAllForcesFor (sph_equations3.cpp:184-278, extended = 0) in Jacobi order: the
// reference integrates each particle inside the force loop (:277), racing with its
// neighbours' reads; here all forces read the step-start state and the integrated
// state goes to the other buffer.
__global__ void __launch_bounds__(kMaxTile)
k_sph_forces(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
             const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
             const ListEntry *__restrict__ list, const int *__restrict__ nbr, float4 *__restrict__ force,
             float4 *__restrict__ pos_out, float4 *__restrict__ vel_out, StepState *st, float dt) {
    __shared__ TileMap T;
    tile_setup(P.g, cell, start, P.n, T);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned fbits = 0;
    bool bad = false;   // integrated position or velocity not finite
    if (i < P.n) {
        const float4 pi = pos[i];
        const float4 vi = vel[i];
        const float ai = pi.w;   // p_i / rho_i^2
        float fx = P.mass * P.gx - P.drag * vi.x;
        float fy = P.mass * P.gy - P.drag * vi.y;
        float fz = P.mass * P.gz - P.drag * vi.z;
        float tx = 0.f, ty = 0.f, tz = 0.f;
        const float kg = P.m2 * P.spiky_dw_c;
        const float kv = P.visc_m2 * P.spiky_d2w_c;
        tile_members<(kGatherBatch < 4 ? kGatherBatch : 4)>(
            P, start, T, list, nbr, pos, cell[i], i,
            [&](unsigned j) { return PosVel{__ldg(&pos[j]), __ldg(&vel[j])}; },
            [&](const PosVel &nb) {
                const float4 pj = nb.p, vj = nb.v;   // vj.w = 1 / rho_j
                const float r2 = dist2(pi, pj);
                const float inv_d = rsqrtf(r2);
                const float d = r2 > 0.f ? r2 * inv_d : 0.f;   // coincident particles: distance 0
                if (d - P.h <= -P.iz) {
                    const float x = 1.f - d * P.inv_h;
                    if (d >= P.iz) {
                        const float c = kg * (ai + pj.w) * x * x * inv_d;
                        tx += (pj.x - pi.x) * c;
                        ty += (pj.y - pi.y) * c;
                        tz += (pj.z - pi.z) * c;
                    }
                    const float w = kv * x * vj.w;
                    fx += (vj.x - vi.x) * w;
                    fy += (vj.y - vi.y) * w;
                    fz += (vj.z - vi.z) * w;
                }
            });
        const v3 f = V(fx - tx, fy - ty, fz - tz);
        force[i] = F4(f);
        v3 x = V(pi), v = V(vi);
        integrate_particle(P, dt, f, &x, &v);
        pos_out[i] = F4(x);
        vel_out[i] = F4(v);
        fbits = __float_as_uint(vlen(f));
        bad = !finite_state(x, v);
    }
    fbits = warp_max_u(fbits);
    if ((threadIdx.x & 31) == 0 && fbits) atomicMax(&st->max_force_bits, fbits);
    count_nonfinite(bad, st);
}

// AccumulateForcesFor + TimeIntegrationFor (AccumulateAndIntegrateGPU,
// pcisph_equations3.cpp:179-212): F += Fp, then integrate into the other buffer.
__global__ void __launch_bounds__(kThreads)
k_accumulate_integrate(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                       float4 *__restrict__ force, const float4 *__restrict__ pforce,
                       float4 *__restrict__ pos_out, float4 *__restrict__ vel_out, float dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const v3 ft = vadd(V(force[i]), V(pforce[i]));
    force[i] = F4(ft);
    v3 x = V(pos[i]), v = V(vel[i]);
    integrate_particle(P, dt, ft, &x, &v);
    pos_out[i] = F4(x);
    vel_out[i] = F4(v);
}

// TimeIntegrationFor over all particles (TimeIntegrationGPU, sph_equations3.cpp:622-634)
__global__ void __launch_bounds__(kThreads)
k_integrate(Params P, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
            const float4 *__restrict__ force, float4 *__restrict__ pos_out,
            float4 *__restrict__ vel_out, float dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    v3 x = V(pos[i]), v = V(vel[i]);
    integrate_particle(P, dt, V(force[i]), &x, &v);
    pos_out[i] = F4(x);
    vel_out[i] = F4(v);
}

// ComputePseudoViscosityAggregationKernelFor (sph_equations3.cpp:341-371): membership
// from the step-start positions (the bucket), values at the integrated state.
__global__ void __launch_bounds__(kMaxTile)
k_pv_aggregate(Params P, const float4 *__restrict__ pos_old, const float4 *__restrict__ pos,
               const float4 *__restrict__ vel, const float *__restrict__ inv_rho,
               const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
               const ListEntry *__restrict__ list, const int *__restrict__ nbr, float4 *__restrict__ smoothed) {
    __shared__ TileMap T;
    tile_setup(P.g, cell, start, P.n, T);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float4 pi = pos[i];
    // the particle itself (distance 0): W_spiky(0) m / rho_i
    const float w0 = P.mass * __ldg(&inv_rho[i]) * P.spiky_w_c;
    const float4 v0 = vel[i];
    float ws = w0, sx = w0 * v0.x, sy = w0 * v0.y, sz = w0 * v0.z;
    tile_members(
        P, start, T, list, nbr, pos_old, cell[i], i, [&](unsigned j) { return j; },
        [&](unsigned j) {
            const float4 pj = __ldg(&pos[j]);
            const float d = sqrtf(dist2(pi, pj));
            if (d - P.h <= -P.iz) {
                const float x = 1.f - d * P.inv_h;
                const float wj = P.mass * __ldg(&inv_rho[j]) * (P.spiky_w_c * x * x * x);
                const float4 vj = __ldg(&vel[j]);
                ws += wj;
                sx += wj * vj.x;
                sy += wj * vj.y;
                sz += wj * vj.z;
            }
        });
    if (ws > 0.f) {
        const float inv = 1.f / ws;
        sx *= inv; sy *= inv; sz *= inv;
    }
    smoothed[i] = make_float4(sx, sy, sz, 0.f);
}

// ComputePseudoViscosityInterpolationKernelFor (sph_equations3.cpp:373-382)
__global__ void k_pv_interpolate(int n, float4 *__restrict__ vel, const float4 *__restrict__ smoothed,
                                 float t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = vel[i], s = smoothed[i];
    const float a = 1.f - t;
    vel[i] = make_float4(v.x * a + s.x * t, v.y * a + s.y * t, v.z * a + s.z * t, 0.f);
}

// Neighbour sets of the last density pass in caller order (bbg_neighbor_lists): every
// particle whose original id lies in [a, b) writes its members other than itself, as
// original ids in visit order (at most maxm of them, -1 after the last), into row id - a of
// out, and its full member count into counts[id - a].  pos0 holds the positions of that
// density pass (wide particles re-test their candidates there).
__global__ void __launch_bounds__(kThreads)
k_export_members(Params P, const unsigned *__restrict__ cell, const unsigned *__restrict__ start,
                 const ListEntry *__restrict__ list, const int *__restrict__ nbr,
                 const float4 *__restrict__ pos0, const int *__restrict__ pid, int a, int b, int maxm,
                 int *__restrict__ counts, int *__restrict__ out) {
    __shared__ TileMap T;
    tile_setup(P.g, cell, start, P.n, T);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int id = pid[i];
    if (id < a || id >= b) return;
    int *row = out + (size_t)(id - a) * (size_t)maxm;
    int c = 0;
    tile_members<1>(P, start, T, list, nbr, pos0, cell[i], i, [&](unsigned j) { return j; },
                    [&](unsigned j) {
                        if (c < maxm) row[c] = pid[j];
                        c++;
                    });
    for (int q = c; q < maxm; q++) row[q] = -1;
    counts[id - a] = c;
}

void launch_export_members(const Params &P, const DevBufs &B, int buf, int pid_buf, int a, int b, int maxm,
                           int *counts, int *out, cudaStream_t s) {
    k_export_members<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P, B.cell, B.start, B.list, B.nbr, B.pos[buf],
                                                                    B.pid[pid_buf], a, b, maxm, counts, out);
}

void launch_density(const Params &P, const DevBufs &B, int buf, int compute_pressure, cudaStream_t s) {
    BBG_PBEGIN(B, KID_DENSITY, s, -1);
    const int t = B.tune.block;
    if (kDensityX2 && !kListRelative) {
        k_soa<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P.n, B.pos[buf], B.soa);
        k_density_x2<<<blocks_for(P.n, t), t, 0, s>>>(P, B.pos[buf], B.vel[buf], B.cell, B.start, B.soa, B.rho,
                                                      B.inv_rho, B.press, B.nbr, B.list, compute_pressure, B.st,
                                                      B.tune.prune);
    } else {
        k_density<<<blocks_for(P.n, t), t, 0, s>>>(P, B.pos[buf], B.vel[buf], B.cell, B.start, B.rho, B.inv_rho,
                                                   B.press, B.nbr, B.list, compute_pressure, B.st);
    }
    if (P.nscenes > 0 && P.n > 0) {
        // batch: each scene's slot range (the scene of every slot was set just above)
        cudaMemsetAsync(P.scene_first, 0x7f, sizeof(int) * (size_t)P.nscenes, s);
        cudaMemsetAsync(P.scene_last, 0xff, sizeof(int) * (size_t)P.nscenes, s);
        k_scene_slots<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P);
    }
    BBG_PEND(B, s);
}

// Blocks of a member-walking pass over tiles of `slots` slots, in the tuned tile order
// (Params::tile_sms of the returned parameters).
static int tiled_grid(const Params &P, const DevBufs &B, int slots, Params *Q) {
    *Q = P;
    Q->tile_sms = 0;
    const int tiles = blocks_for(P.n, slots);
    if (B.tune.tile_order != 1 || P.nscenes > 0) return tiles;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) return tiles;
    Q->tile_sms = sms;
    return sms * ((tiles + sms - 1) / sms);
}

template <bool DIV, bool WARM>
static void non_pressure_nb(const Params &P0, const DevBufs &B, int buf, int predict, float dt,
                            float dt_over_m, cudaStream_t s, float *divsum) {
    const int t = B.tune.block;
    Params P;
    const int grid = tiled_grid(P0, B, t, &P);
#define NP_LAUNCH(NB)                                                                        \
    k_non_pressure<DIV, WARM, NB><<<grid, t, 0, s>>>(                                        \
        P, B.pos[buf], B.vel[buf], B.cell, B.start, B.list, B.nbr, B.force, B.xstar, B.pforce, \
        B.press, divsum, predict, dt, dt_over_m)
    switch (B.tune.batch_np) {
        case 2: NP_LAUNCH(2); break;
        case 8: NP_LAUNCH(8); break;
        default: NP_LAUNCH(4); break;
    }
#undef NP_LAUNCH
}

void launch_non_pressure(const Params &P, const DevBufs &B, int buf, int predict, float dt,
                         float dt_over_m, cudaStream_t s, float *divsum, bool warm) {
    BBG_PBEGIN(B, KID_NON_PRESSURE, s, -1);
    if (divsum) {
        if (warm) non_pressure_nb<true, true>(P, B, buf, predict, dt, dt_over_m, s, divsum);
        else non_pressure_nb<true, false>(P, B, buf, predict, dt, dt_over_m, s, divsum);
    } else {
        if (warm) non_pressure_nb<false, true>(P, B, buf, predict, dt, dt_over_m, s, nullptr);
        else non_pressure_nb<false, false>(P, B, buf, predict, dt, dt_over_m, s, nullptr);
    }
    BBG_PEND(B, s);
}

void launch_predict_first(const Params &P, const DevBufs &B, int buf, int is_first, float dt,
                          float dt_over_m, cudaStream_t s) {
    BBG_PBEGIN(B, KID_PREDICT_FIRST, s, -1);
    k_predict_first<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(
        P, B.pos[buf], B.vel[buf], B.force, B.xstar, B.pforce, B.press, B.rhostar, B.rho, B.derr,
        is_first, dt, dt_over_m);
    BBG_PEND(B, s);
}

// Resident blocks of a persistent kernel: every SM filled to the kernel's occupancy.
template <class K>
static int persistent_blocks(K kernel, int threads) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    return (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
}

template <int NB>
static int pd_grid(int t) { return persistent_blocks(k_pred_density_wl<NB>, t); }
template <int NB>
static int pf_grid(int t) { return persistent_blocks(k_pressure_force_wl<NB>, t); }

void update_worklist_grid(DevBufs &B) {
    const int t = B.tune.block;
    B.tune.wl_grid_pd = B.tune.batch_pd == 2 ? pd_grid<2>(t) : B.tune.batch_pd == 8 ? pd_grid<8>(t) : pd_grid<4>(t);
    B.tune.wl_grid_pf = B.tune.batch_pf == 2 ? pf_grid<2>(t) : B.tune.batch_pf == 8 ? pf_grid<8>(t) : pf_grid<4>(t);
}

// Particles per thread of the per-tile corrector passes (1 with tile-relative lists,
// whose entries are decoded against the block's own tile).
static int corrector_ppt(const DevBufs &B) { return kListRelative ? 1 : (B.tune.ppt == 2 ? 2 : 1); }

// Slots per tile of the corrector passes: the block, times the particles per thread for
// the per-tile kernels.
static int corrector_tile(const DevBufs &B) {
    return B.tune.block * (B.tune.worklist == 2 ? 1 : corrector_ppt(B));
}

void launch_worklist(const Params &P, const DevBufs &B, int k, cudaStream_t s) {
    k_worklist<<<1, 1024, 0, s>>>(P, B.st, k, corrector_tile(B));
}

void launch_pred_density(const Params &P, const DevBufs &B, int buf, int k, float delta,
                         cudaStream_t s, int clamp_total) {
    BBG_PBEGIN(B, KID_PRED_DENSITY, s, k);
    const int t = B.tune.block;
    const int wl = P.nscenes > 0 ? B.tune.worklist : 0;
    if (wl) launch_worklist(P, B, k, s);   // batch: the tiles of the scenes still running
    if (wl == 2) {
        // persistent blocks over the work list
#define PD_LAUNCH(NB)                                                                               \
    k_pred_density_wl<NB><<<B.tune.wl_grid_pd > 0 ? B.tune.wl_grid_pd : pd_grid<NB>(t), t, 0, s>>>(  \
        P, B.pos[buf], B.xstar, B.cell, B.start, B.list, B.nbr, B.press, B.rhostar, B.derr, B.st, k, \
        delta, clamp_total)
        switch (B.tune.batch_pd) {
            case 2: PD_LAUNCH(2); break;
            case 8: PD_LAUNCH(8); break;
            default: PD_LAUNCH(4); break;
        }
#undef PD_LAUNCH
    } else {
        const int ppt = corrector_ppt(B);
        Params Q;
        const int grid = wl ? blocks_for(P.n, t * ppt) : tiled_grid(P, B, t * ppt, &Q);
        if (wl) Q = P;
#define PD_LAUNCH(NB, PPT)                                                                        \
    k_pred_density<NB, PPT><<<grid, t, 0, s>>>(Q, B.pos[buf], B.xstar, B.cell, B.start, B.list, B.nbr, \
                                               B.press, B.rhostar, B.derr, B.st, k, delta, clamp_total, wl)
        switch (B.tune.batch_pd * 10 + ppt) {
            case 21: PD_LAUNCH(2, 1); break;
            case 81: PD_LAUNCH(8, 1); break;
            case 22: PD_LAUNCH(2, 2); break;
            case 42: PD_LAUNCH(4, 2); break;
            case 82: PD_LAUNCH(8, 2); break;
            default: PD_LAUNCH(4, 1); break;
        }
#undef PD_LAUNCH
    }
    BBG_PEND(B, s);
}

void launch_warm_start(const Params &P, const DevBufs &B, int buf, float scale, cudaStream_t s) {
    k_warm_start<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P.n, B.pos[buf], B.rho, B.pprev,
                                                                B.press, B.rhostar, B.derr, scale);
}

void launch_pack_acoef(const Params &P, const DevBufs &B, int buf, cudaStream_t s) {
    k_pack_acoef<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P.n, B.pos[buf], B.press, B.rhostar);
}

void launch_pressure_force(const Params &P, const DevBufs &B, int buf, int k, int max_it, float dt,
                           float dt_over_m, cudaStream_t s, int mode) {
    BBG_PBEGIN(B, KID_PRESSURE_FORCE, s, k);
    const int t = B.tune.block;
    const int wl = P.nscenes > 0 ? B.tune.worklist : 0;
    // batch: the work list launch_pred_density built for iteration k (built here when the
    // pass runs on its own)
    if (wl && mode == 1) launch_worklist(P, B, k, s);
    if (wl == 2) {
#define PF_LAUNCH(NB)                                                                                   \
    k_pressure_force_wl<NB><<<B.tune.wl_grid_pf > 0 ? B.tune.wl_grid_pf : pf_grid<NB>(t), t, 0, s>>>(    \
        P, B.pos[buf], B.vel[buf], B.cell, B.start, B.list, B.nbr, B.force, B.pforce, B.xstar,           \
        B.pos[1 - buf], B.vel[1 - buf], B.st, k, max_it, dt, dt_over_m, mode)
        switch (B.tune.batch_pf) {
            case 2: PF_LAUNCH(2); break;
            case 8: PF_LAUNCH(8); break;
            default: PF_LAUNCH(4); break;
        }
#undef PF_LAUNCH
    } else {
        const int ppt = corrector_ppt(B);
        Params Q;
        const int grid = wl ? blocks_for(P.n, t * ppt) : tiled_grid(P, B, t * ppt, &Q);
        if (wl) Q = P;
#define PF_LAUNCH(NB, PPT)                                                                             \
    k_pressure_force<NB, PPT><<<grid, t, 0, s>>>(                                                       \
        Q, B.pos[buf], B.vel[buf], B.cell, B.start, B.list, B.nbr, B.force, B.pforce, B.xstar,           \
        B.pos[1 - buf], B.vel[1 - buf], B.st, k, max_it, dt, dt_over_m, mode, wl)
        switch (B.tune.batch_pf * 10 + ppt) {
            case 21: PF_LAUNCH(2, 1); break;
            case 81: PF_LAUNCH(8, 1); break;
            case 22: PF_LAUNCH(2, 2); break;
            case 42: PF_LAUNCH(4, 2); break;
            case 82: PF_LAUNCH(8, 2); break;
            default: PF_LAUNCH(4, 1); break;
        }
#undef PF_LAUNCH
    }
    BBG_PEND(B, s);
}

void launch_corrector_control(const Params &P, const DevBufs &B, int max_it,
                              cudaGraphConditionalHandle handle, cudaStream_t s) {
    k_corrector_control<<<1, 1, 0, s>>>(P, B.st, max_it, handle);
}

void launch_sph_forces(const Params &P, const DevBufs &B, int buf, float dt, cudaStream_t s) {
    BBG_PBEGIN(B, KID_SPH_FORCES, s, -1);
    k_sph_forces<<<blocks_for(P.n, B.tune.block), B.tune.block, 0, s>>>(
        P, B.pos[buf], B.vel[buf], B.cell, B.start, B.list, B.nbr, B.force, B.pos[1 - buf],
        B.vel[1 - buf], B.st, dt);
    BBG_PEND(B, s);
}

void launch_accumulate_integrate(const Params &P, const DevBufs &B, int buf, float dt,
                                 cudaStream_t s) {
    BBG_PBEGIN(B, KID_INTEGRATE, s, -1);
    k_accumulate_integrate<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(
        P, B.pos[buf], B.vel[buf], B.force, B.pforce, B.pos[1 - buf], B.vel[1 - buf], dt);
    BBG_PEND(B, s);
}

void launch_integrate(const Params &P, const DevBufs &B, int buf, float dt, cudaStream_t s) {
    BBG_PBEGIN(B, KID_INTEGRATE, s, -1);
    k_integrate<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P, B.pos[buf], B.vel[buf], B.force,
                                                               B.pos[1 - buf], B.vel[1 - buf], dt);
    BBG_PEND(B, s);
}

// FP64 totals of the particle state: mass, kinetic energy, potential energy in the constant
// gravity field and momentum.  One partial row per block, summed by the host in block order,
// so the totals do not depend on scheduling.
constexpr int kEnergyBlocks = 1024;
__global__ void __launch_bounds__(kThreads)
k_energy(int n, const float4 *__restrict__ pos, const float4 *__restrict__ vel, double mass, double gx, double gy,
         double gz, double *__restrict__ partial) {
    double acc[kEnergyTerms] = {0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i], v = vel[i];
        const double vx = v.x, vy = v.y, vz = v.z;
        acc[0] += mass;
        acc[1] += 0.5 * mass * (vx * vx + vy * vy + vz * vz);
        acc[2] -= mass * (gx * (double)p.x + gy * (double)p.y + gz * (double)p.z);
        acc[3] += mass * vx;
        acc[4] += mass * vy;
        acc[5] += mass * vz;
    }
    __shared__ double red[kThreads / 32][kEnergyTerms];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < kEnergyTerms; t++) {
        const double v = warp_sum_d(acc[t]);
        if (lane == 0) red[wid][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < kEnergyTerms) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w][threadIdx.x];
        partial[blockIdx.x * kEnergyTerms + threadIdx.x] = v;
    }
}

int energy_blocks(int n) {
    const int b = blocks_for(n, kThreads);
    return b < kEnergyBlocks ? (b > 0 ? b : 1) : kEnergyBlocks;
}

void launch_energy(const Params &P, const DevBufs &B, int buf, const double g[3], double *partial, cudaStream_t s) {
    k_energy<<<energy_blocks(P.n), kThreads, 0, s>>>(P.n, B.pos[buf], B.vel[buf], (double)P.mass, g[0], g[1], g[2],
                                                     partial);
}

void launch_pseudo_viscosity(const Params &P, const DevBufs &B, int new_buf, float factor,
                             cudaStream_t s) {
    BBG_PBEGIN(B, KID_PSEUDO_VISCOSITY, s, -1);
    k_pv_aggregate<<<blocks_for(P.n, B.tune.block), B.tune.block, 0, s>>>(
        P, B.pos[1 - new_buf], B.pos[new_buf], B.vel[new_buf], B.inv_rho, B.cell, B.start, B.list, B.nbr,
        B.smoothed);
    k_pv_interpolate<<<blocks_for(P.n, kThreads), kThreads, 0, s>>>(P.n, B.vel[new_buf], B.smoothed,
                                                                    factor);
    BBG_PEND(B, s);
}

}  // namespace bbg
