// bbg_internal.cuh -- device-side definitions shared by the bubbles_gb300 kernels.
//
// Device state is FP32 structure-of-arrays in HBM: float4 position / velocity /
// force / predicted position / pressure force (w unused, 16-byte aligned loads),
// float density / pressure / predicted density, int original ids.  Particles are
// stored sorted by grid cell (x fastest, then y, then z; inside a cell by original
// id), so the 27 neighbour cells of a particle are 9 contiguous slot ranges.
//
// Exactness: the grid hash (src/core/grid.h:259-298), the bucket membership test
// IsWithinStd (src/core/kernel.cpp:229-233), the collider code and the integrator
// are evaluated with explicitly rounded operations (__fadd_rn, __fmul_rn, ...) in
// the reference's operand order, so they give the same bits as the reference built
// with `typedef float Float`.  The neighbour sums use contracted FP32 arithmetic in
// sorted-slot order and agree with the reference to about 1e-6 relative.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bbg {

constexpr int kMaxColliders = 16;
constexpr int kMaxIterations = 64;
constexpr int kBucketCap = 100;   // MaximumParticlesPerBucket, src/core/particle.h:10

struct GridDev {
    int nx, ny, nz;
    unsigned total;
    float minp[3], len[3], bmin[3], bmax[3];
};

struct ShapeDev {
    int type, reverse;   // type 1: box, 2: sphere, 3: a shape given by its field alone
    float t[3];          // translation
    float hx, hy, hz;    // box half sizes, sizex / 2.0 rounded to float
    float radius;        // sphere radius
    float friction;
    int sdf;             // index of the shape's signed-distance field in Params::sdf, or -1
};

// A signed-distance field on a vertex-centred grid (FieldGrid3f, src/core/grid.h:950-1240,
// built by GenerateShapeSDF or given), sampled trilinearly.
constexpr int kMaxSdf = 4;
struct SdfDev {
    const float *v;      // nodes, x fastest (LinearIndex)
    int nx, ny, nz;      // nodes per axis (resolution + 1)
    float org[3];        // minPoint
    float sp[3];         // spacing
    float inv2[3];       // (float)(1.0 / (2.0 * spacing)): Gradient's central difference
    int bounded;         // a mesh's field: positions outside [lo, hi] never collide
    float lo[3], hi[3];  // (Collider3::OptmizedClosestPointCheck, IsPenetrating)
};

// Corrector state of one scene of a batch.
struct SceneState {
    unsigned err_bits[kMaxIterations];   // max |density error| of each iteration
    double err_sum[kMaxIterations];      // sum |density error| of each iteration (FP64)
};

// Scalars every pass needs; passed by value as a kernel parameter.
struct Params {
    GridDev g;
    int n;
    int nshapes;
    ShapeDev shapes[kMaxColliders];
    float mass, radius, h, h2, inv_h, inv_h2, target_density;
    float iz;        // IsZero(x) <=> |x| < iz  (smallest float above 1e-8)
    float iz6;       // IsUnsafeZero(x) <=> |x| < iz6  (smallest float above 1e-6)
    float nb_lo;     // r^2 < nb_lo => IsWithinStd holds for sure
    float nb_hi;     // r^2 > nb_hi => IsWithinStd fails for sure
    float h2mz;      // h^2 - iz: W_std(r) > 0 <=> r^2 < h2mz (to FP32 rounding)
    float prune_m;   // margin of the density pass's reach test (far above position rounding)
    float std_c;     // 315 / (64 pi h^3)
    float spiky_dw_c;   // 45 / (pi h^4)
    float spiky_d2w_c;  // 90 / (pi h^5)
    float spiky_w_c;    // 15 / (pi h^3)
    float visc_m2;   // viscosity * m^2
    float m2;
    float drag;
    float gx, gy, gz;
    float eos_scale_over_exp, eos_exp, neg_scale;
    float rest_c1_int;   // (float)(-1.0 - 0.6): integrate restitution term
    float rest_int;      // (float)0.6
    float max_err_ratio; // corrector tolerance (float, as the reference compares)
    // batch of independent scenes stacked along z (nscenes = 0: one scene)
    int nscenes;
    const float *scene_zb;          // nscenes region starts along z (scene_zb[0] = -FLT_MAX)
    const ShapeDev *scene_box;      // container box of each scene
    SceneState *scene_st;           // per-scene corrector state (reset each substep)
    unsigned short *scene;          // scene of each sorted slot (density pass)
    // batch corrector work list: the tiles that hold particles of scenes whose corrector
    // still runs, rebuilt before every iteration and taken by persistent blocks
    int *scene_first, *scene_last;  // lowest / highest sorted slot of each scene
    int *wl_off;                    // nscenes + 1 offsets of the scenes' tile segments
    int *wl_tile;                   // first tile of each scene's segment
    int *wl_ctr;                    // next work item of the two persistent passes
    int tile_sms;                   // > 0: blocks dealt to tiles SM-strided (tile_of_block)
    int has_sdf;                    // some collider has a signed-distance field
    SdfDev sdf[kMaxSdf];
};

// Per-substep device scalars (reset each substep).
struct StepState {
    unsigned err_bits[kMaxIterations];   // max |density error| of each corrector iteration
    double err_sum[kMaxIterations];      // sum |density error| of each iteration (FP64)
    unsigned max_force_bits;             // max |F| after integration
    unsigned out_of_grid;
    unsigned nbr_overflow;
    unsigned nonfinite;
    unsigned crowded;                    // cells / particles past the work caps (see below)
    int iter;                            // corrector iteration (graph-driven loop)
};

// Work caps that keep a degenerate state (e.g. a blown-up simulation that piles particles
// into a few cells) from turning the per-cell rank and the candidate search quadratic:
// a cell with more than kRankCap particles keeps its arrival order instead of the order
// by id, and a particle with more than kMaxCandidates candidates in its 27 cells gets no
// neighbours.  Both are counted in StepState::crowded; normal states are far below them
// (about 8 particles per cell, 216 candidates).
constexpr unsigned kRankCap = 512;
constexpr unsigned kMaxCandidates = 1024;

// ----------------------------------------------------------------------------
// explicitly rounded FP32 helpers (no contraction)
// ----------------------------------------------------------------------------
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }

struct v3 { float x, y, z; };
__device__ __forceinline__ v3 V(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ v3 V(float4 a) { return V(a.x, a.y, a.z); }
__device__ __forceinline__ float4 F4(v3 a) { return make_float4(a.x, a.y, a.z, 0.f); }
__device__ __forceinline__ v3 vadd(v3 a, v3 b) { return V(fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)); }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return V(fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z)); }
__device__ __forceinline__ v3 vmul(v3 a, float s) { return V(fm(a.x, s), fm(a.y, s), fm(a.z, s)); }
__device__ __forceinline__ v3 vdiv(v3 a, float f) {
    float inv = fdv(1.0f, f);
    return vmul(a, inv);
}
__device__ __forceinline__ float vdot(v3 a, v3 b) { return fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)); }
__device__ __forceinline__ float vlen2(v3 a) { return vdot(a, a); }
__device__ __forceinline__ float vlen(v3 a) { return __fsqrt_rn(vlen2(a)); }
__device__ __forceinline__ float rmax(float a, float b) { return a < b ? b : a; }   // reference Max
__device__ __forceinline__ float rmin(float a, float b) { return a < b ? a : b; }   // reference Min
__device__ __forceinline__ float rclamp(float v, float lo, float hi) {
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}
__device__ __forceinline__ v3 vclamp(v3 v, v3 lo, v3 hi) {
    return V(rclamp(v.x, lo.x, hi.x), rclamp(v.y, lo.y, hi.y), rclamp(v.z, lo.z, hi.z));
}

// Inside(vec3, Bounds3) with its 1e-6 face tolerance, src/core/geometry.h:1773-1783
__device__ __forceinline__ bool inside3(v3 p, v3 mn, v3 mx, float iz6) {
    bool rv = (p.x >= mn.x && p.x <= mx.x && p.y >= mn.y && p.y <= mx.y && p.z >= mn.z &&
               p.z <= mx.z);
    if (!rv) {
        float ox = rmin(fabsf(fs(mn.x, p.x)), fabsf(fs(mx.x, p.x)));
        float oy = rmin(fabsf(fs(mn.y, p.y)), fabsf(fs(mx.y, p.y)));
        float oz = rmin(fabsf(fs(mn.z, p.z)), fabsf(fs(mx.z, p.z)));
        rv = fabsf(ox) < iz6 || fabsf(oy) < iz6 || fabsf(oz) < iz6;
    }
    return rv;
}

// ----------------------------------------------------------------------------
// grid hash: Grid::ExtremeEpsilon + GetHashedPosition + LinearIndex
// ----------------------------------------------------------------------------
__device__ __forceinline__ int hash_axis(float p, float bmin, float bmax, float minp, float len,
                                         int dim, float iz, unsigned *bad) {
    float eps = 0.f;
    if (fabsf(fs(p, bmin)) < iz) eps = 0.0001f;
    else if (fabsf(fs(p, bmax)) < iz) eps = -0.0001f;
    float pi = fa(p, eps);
    float dp = fdv(fs(pi, minp), len);
    int id = (int)floorf(dp);
    if (id < 0) { id = 0; *bad = 1; }
    if (id >= dim) { id = dim - 1; *bad = 1; }
    return id;
}

__device__ __forceinline__ unsigned grid_hash(const GridDev &g, float4 p, float iz, unsigned *bad) {
    int ux = hash_axis(p.x, g.bmin[0], g.bmax[0], g.minp[0], g.len[0], g.nx, iz, bad);
    int uy = hash_axis(p.y, g.bmin[1], g.bmax[1], g.minp[1], g.len[1], g.ny, iz, bad);
    int uz = hash_axis(p.z, g.bmin[2], g.bmax[2], g.minp[2], g.len[2], g.nz, iz, bad);
    return (unsigned)ux + (unsigned)uy * (unsigned)g.nx + (unsigned)uz * (unsigned)g.nx * (unsigned)g.ny;
}

// ----------------------------------------------------------------------------
// bucket membership: IsWithinStd(Distance(xi, xj), h) exactly as the FP32 reference,
// with a contracted fast path that only defers to the exact test in a 1e-6 band.
// ----------------------------------------------------------------------------
__device__ __forceinline__ bool std_member_exact(const Params &P, float4 a, float4 b) {
    float ex = fs(a.x, b.x), ey = fs(a.y, b.y), ez = fs(a.z, b.z);
    float e2 = fa(fa(fm(ex, ex), fm(ey, ey)), fm(ez, ez));
    float d = __fsqrt_rn(e2);
    float of = fs(fm(d, d), P.h2);
    return of <= -P.iz;   // !(IsZero(of) || of > 0)
}

__device__ __forceinline__ bool std_member(const Params &P, float4 a, float4 b, float r2) {
    if (r2 < P.nb_lo) return true;
    if (r2 > P.nb_hi) return false;
    return std_member_exact(P, a, b);
}

__device__ __forceinline__ float dist2(float4 a, float4 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}

// A particle whose neighbour set does not fit the compact list (tile.cuh) has kWide set
// in its cell word and is re-tested exactly on every pass instead.
constexpr unsigned kWide = 0x80000000u;
constexpr int kMaxList = 64;

// ----------------------------------------------------------------------------
// colliders: exact FP32 restatement of CollisionHandle / ColliderSet3::ResolveCollision
// (src/core/collider.cpp:3-44, 238-264), Shape::BoxClosestPoint / BoxClosestDistance
// (src/shapes/box.cpp:74-172), Shape::SphereClosestPoint (src/shapes/sphere.cpp:47-70),
// Shape::IsInside (src/core/shape.cpp:275-282); translation-only transforms.
// ----------------------------------------------------------------------------
__device__ __forceinline__ v3 plane_closest(v3 pp, v3 pn, v3 p) {
    v3 r = vsub(p, pp);
    return vadd(vsub(r, vmul(pn, vdot(r, pn))), pp);
}

__device__ __forceinline__ void box_plane(const ShapeDev &s, int i, v3 *pp, v3 *pn) {
    v3 mx = V(s.hx, s.hy, s.hz), mn = V(-s.hx, -s.hy, -s.hz);
    switch (i) {
        case 0: *pp = mx; *pn = V(1.f, 0.f, 0.f); break;
        case 1: *pp = mx; *pn = V(0.f, 1.f, 0.f); break;
        case 2: *pp = mx; *pn = V(0.f, 0.f, 1.f); break;
        case 3: *pp = mn; *pn = V(-1.f, 0.f, 0.f); break;
        case 4: *pp = mn; *pn = V(0.f, -1.f, 0.f); break;
        default: *pp = mn; *pn = V(0.f, 0.f, -1.f); break;
    }
}

__device__ __forceinline__ float box_closest_distance(const ShapeDev &s, v3 point, float iz6) {
    v3 pl = vsub(point, V(s.t[0], s.t[1], s.t[2]));
    v3 mx = V(s.hx, s.hy, s.hz), mn = V(-s.hx, -s.hy, -s.hz);
    v3 closest;
    bool isNeg = false;
    if (inside3(pl, mn, mx, iz6)) {
        v3 pp, pn;
        box_plane(s, 0, &pp, &pn);
        closest = plane_closest(pp, pn, pl);
        float d2 = vlen2(vsub(closest, pl));
        for (int i = 1; i < 6; i++) {
            box_plane(s, i, &pp, &pn);
            v3 local = plane_closest(pp, pn, pl);
            float ld2 = vlen2(vsub(local, pl));
            if (ld2 < d2) { closest = local; d2 = ld2; }
        }
        isNeg = true;
    } else {
        closest = vclamp(pl, mn, mx);
    }
    float d = vlen(vsub(pl, closest));
    return isNeg ? -d : d;
}

struct Cpq { v3 point, normal; float sd; };

__device__ __forceinline__ Cpq box_closest_point(const ShapeDev &s, v3 point, float iz6) {
    v3 t = V(s.t[0], s.t[1], s.t[2]);
    v3 pl = vsub(point, t);
    v3 mx = V(s.hx, s.hy, s.hz), mn = V(-s.hx, -s.hy, -s.hz);
    v3 closest, normal = V(1.f, 0.f, 0.f), pp, pn;
    bool isNeg = false;
    if (inside3(pl, mn, mx, iz6)) {
        box_plane(s, 0, &pp, &pn);
        closest = plane_closest(pp, pn, pl);
        float d2 = vlen2(vsub(closest, pl));
        for (int i = 1; i < 6; i++) {
            box_plane(s, i, &pp, &pn);
            v3 local = plane_closest(pp, pn, pl);
            float ld2 = vlen2(vsub(local, pl));
            if (ld2 < d2) { closest = local; normal = pn; d2 = ld2; }
        }
        isNeg = true;
    } else {
        closest = vclamp(pl, mn, mx);
        v3 cov = vsub(pl, closest);
        float maxCos = vdot(cov, normal);
        for (int i = 1; i < 6; i++) {
            box_plane(s, i, &pp, &pn);
            float c = vdot(pn, cov);
            if (c > maxCos) { normal = pn; maxCos = c; }
        }
    }
    float distance = vlen(vsub(closest, pl));
    if (isNeg) distance = -distance;
    if (s.reverse) normal = V(-normal.x, -normal.y, -normal.z);
    Cpq q;
    q.point = vadd(closest, t);
    q.normal = normal;
    q.sd = distance;
    return q;
}

__device__ __forceinline__ float sphere_closest_distance(const ShapeDev &s, v3 point) {
    v3 pl = vsub(point, V(s.t[0], s.t[1], s.t[2]));
    return fs(vlen(pl), s.radius);
}

__device__ __forceinline__ Cpq sphere_closest_point(const ShapeDev &s, v3 point, float iz) {
    float d = sphere_closest_distance(s, point);
    v3 t = V(s.t[0], s.t[1], s.t[2]);
    v3 pl = vsub(point, t);
    v3 N = V(0.f, 1.f, 0.f);
    if (!(fabsf(pl.x) < iz && fabsf(pl.y) < iz && fabsf(pl.z) < iz)) N = vdiv(pl, vlen(pl));
    v3 pN = vmul(N, s.radius);
    if (s.reverse) N = V(-N.x, -N.y, -N.z);
    Cpq q;
    q.point = vadd(pN, t);
    q.normal = N;
    q.sd = d;
    return q;
}

__device__ __forceinline__ Cpq shape_closest_point(const ShapeDev &s, v3 p, float iz, float iz6) {
    return s.type == 1 ? box_closest_point(s, p, iz6) : sphere_closest_point(s, p, iz);
}

// Conservative test that shape s cannot penetrate particle p of radius r: true only when
// the exact test (IsInside || |signed distance| < r) is false by a margin far above FP32
// rounding, so skipping the exact evaluation never changes a result.
__device__ __forceinline__ bool clearly_clear(const ShapeDev &s, v3 p, float r) {
    const float m = r * 1.0001f + 1e-6f;
    const float x = p.x - s.t[0], y = p.y - s.t[1], z = p.z - s.t[2];
    if (s.type == 1) {
        if (s.reverse)   // container: well inside on every axis
            return fabsf(x) <= s.hx - m && fabsf(y) <= s.hy - m && fabsf(z) <= s.hz - m;
        return fabsf(x) >= s.hx + m || fabsf(y) >= s.hy + m || fabsf(z) >= s.hz + m;
    }
    if (s.reverse) return false;
    const float R = s.radius + m;
    return x * x + y * y + z * z >= R * R * 1.0001f;
}

// ColliderSet3::ResolveCollision with restitution r (rc1 = (float)(-1.0 - r)).  The
// reference evaluates each shape's closest distance, then the chosen shape's closest
// point and IsInside (two more distance evaluations); Shape::ClosestDistance equals the
// closest-point query's signed distance bit for bit for boxes and spheres, so one query
// per shape gives the same answer.
__device__ __forceinline__ void resolve_against(const Params &P, const ShapeDev *shapes, int nshapes, float r,
                                                float rc1, v3 *pos, v3 *vel) {
    if (nshapes <= 0) return;
    bool all_clear = true;
    for (int i = 0; i < nshapes; i++) all_clear = all_clear && clearly_clear(shapes[i], *pos, P.radius);
    if (all_clear) return;
    int target = -1;
    float minD = 3.402823466e+38f;   // Infinity = FLT_MAX
    Cpq q;
    for (int i = 0; i < nshapes; i++) {
        const Cpq qi = shape_closest_point(shapes[i], *pos, P.iz, P.iz6);
        const float d = fabsf(qi.sd);
        if (d < minD) { target = i; minD = d; q = qi; }
    }
    if (target < 0) return;
    const ShapeDev &s = shapes[target];
    const bool inside = (s.reverse != 0) == !(q.sd < 0.f);
    if (!(inside || minD < P.radius)) return;
    v3 n = q.normal;
    v3 targetPoint = vadd(q.point, vmul(n, P.radius));
    v3 rel = *vel;   // collider velocity is zero for static shapes
    float ndr = vdot(n, rel);
    v3 relN = vmul(n, ndr);
    v3 relT = vsub(rel, relN);
    if (ndr < 0.f) {
        v3 dRelN = vmul(relN, rc1);
        relN = vmul(relN, -r);
        if (vlen2(relT) > 0.f) {
            float scale = fdv(vlen(dRelN), vlen(relT));
            float fScale = fs(1.0f, fm(s.friction, scale));
            float frictionScale = rmax(0.f, fScale);
            relT = vmul(relT, frictionScale);
        }
        *vel = vadd(vadd(relN, relT), V(0.f, 0.f, 0.f));
    }
    *pos = targetPoint;
}

// TimeIntegrationFor, src/equations/sph_equations3.cpp:283-339 (extended = 0).
// Scene of a batch whose region along z holds z (binary search over the region starts).
__device__ __forceinline__ int scene_of(const Params &P, float z) {
    int lo = 0, hi = P.nscenes;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&P.scene_zb[mid]) <= z) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ---- colliders with signed-distance fields ----
// GetBarycentric (src/core/sampling.h:7-31) of x over nodes [0, high]; a float outside
// the int range converts as on the host (the lowest int).
__device__ __forceinline__ void barycentric(float x, int high, int *i, float *f) {
    const float s = floorf(x);
    int k = (s >= -2147483648.f && s < 2147483648.f) ? (int)s : (int)0x80000000;
    if (high == 0) {
        *i = 0;
        *f = 0.f;
    } else if (k < 0) {
        *i = 0;
        *f = 0.f;
    } else if (k > high - 1) {
        *i = high - 1;
        *f = 1.f;
    } else {
        *i = k;
        *f = fs(x, s);
    }
}

// Lerp (src/core/geometry.h:1087-1089): (1 - t) p0 + t p1
__device__ __forceinline__ float rlerp(float p0, float p1, float t) { return fa(fm(fs(1.f, t), p0), fm(t, p1)); }

// FieldGrid3f::Sample (src/core/grid.h:1093-1133) of a vertex-centred grid
__device__ __forceinline__ float sdf_sample(const SdfDev &g, v3 p) {
    const int n[3] = {g.nx, g.ny, g.nz};
    const float pc[3] = {p.x, p.y, p.z};
    int ii[3], jj[3];
    float w[3];
    for (int k = 0; k < 3; k++) {
        const float origin = fa(g.org[k], fm(g.sp[k], 0.f));   // GetDataPosition(0)
        const float x = fdv(fs(pc[k], origin), g.sp[k]);
        barycentric(x, n[k] - 1, &ii[k], &w[k]);
        jj[k] = ii[k] + 1 < n[k] - 1 ? ii[k] + 1 : n[k] - 1;
    }
    const unsigned sx = (unsigned)g.nx, sxy = (unsigned)g.nx * (unsigned)g.ny;
    auto at = [&](int a, int b, int c) {
        return __ldg(&g.v[(unsigned)a + (unsigned)b * sx + (unsigned)c * sxy]);
    };
    const float f000 = at(ii[0], ii[1], ii[2]), f100 = at(jj[0], ii[1], ii[2]);
    const float f010 = at(ii[0], jj[1], ii[2]), f110 = at(jj[0], jj[1], ii[2]);
    const float f001 = at(ii[0], ii[1], jj[2]), f101 = at(jj[0], ii[1], jj[2]);
    const float f011 = at(ii[0], jj[1], jj[2]), f111 = at(jj[0], jj[1], jj[2]);
    const float b0 = rlerp(rlerp(f000, f100, w[0]), rlerp(f010, f110, w[0]), w[1]);
    const float b1 = rlerp(rlerp(f001, f101, w[0]), rlerp(f011, f111, w[0]), w[1]);
    return rlerp(b0, b1, w[2]);
}

// FieldGrid3f::Gradient (grid.h:1153-1169): central differences one spacing apart
__device__ __forceinline__ v3 sdf_gradient(const SdfDev &g, v3 p) {
    float d[3];
    for (int k = 0; k < 3; k++) {
        const v3 s = V(k == 0 ? g.sp[0] : 0.f, k == 1 ? g.sp[1] : 0.f, k == 2 ? g.sp[2] : 0.f);
        d[k] = fm(fs(sdf_sample(g, vadd(p, s)), sdf_sample(g, vsub(p, s))), g.inv2[k]);
    }
    return V(d[0], d[1], d[2]);
}

// Transform::Point of a translation ((1 x + 0 y) + 0 z) + t, in the host's operation order
__device__ __forceinline__ v3 translate_point(v3 p, float tx, float ty, float tz) {
    return V(fa(fa(fa(fm(1.f, p.x), fm(0.f, p.y)), fm(0.f, p.z)), tx),
             fa(fa(fa(fm(0.f, p.x), fm(1.f, p.y)), fm(0.f, p.z)), ty),
             fa(fa(fa(fm(0.f, p.x), fm(0.f, p.y)), fm(1.f, p.z)), tz));
}

// Shape::ClosestPointBySDF (src/shapes/bvh.cpp:666-707): the object-space point marched
// onto the zero level along the normalised gradient (at most 5 steps, stop at |sdf| <
// 0.001); the distance is unsigned.
__device__ __forceinline__ Cpq sdf_closest_point(const ShapeDev &s, const SdfDev &g, v3 pw) {
    const v3 point = translate_point(pw, -s.t[0], -s.t[1], -s.t[2]);   // WorldToObject
    v3 tn = V(0.f, 1.f, 0.f), tp = point;
    bool has_gradient = false;
    for (int i = 0; i < 5; i++) {
        const float sdf = sdf_sample(g, tp);
        if ((double)fabsf(sdf) < 0.001) break;
        tn = sdf_gradient(g, tp);
        const float len = vlen(tn);
        if (len > 0.f) tn = vdiv(tn, len);
        tp = vsub(tp, vmul(tn, sdf));
        has_gradient = true;
    }
    if (!has_gradient) {
        tn = sdf_gradient(g, tp);
        const float len = vlen(tn);
        if (len > 0.f) tn = vdiv(tn, len);
    }
    Cpq q;
    q.sd = vlen(vsub(point, tp));
    q.point = translate_point(tp, s.t[0], s.t[1], s.t[2]);   // ObjectToWorld
    // ObjectToWorld.Normal: the inverse's transpose, identity for a translation
    q.normal = V(fa(fa(fm(1.f, tn.x), fm(0.f, tn.y)), fm(0.f, tn.z)),
                 fa(fa(fm(0.f, tn.x), fm(1.f, tn.y)), fm(0.f, tn.z)),
                 fa(fa(fm(0.f, tn.x), fm(0.f, tn.y)), fm(1.f, tn.z)));
    return q;
}

// ColliderSet3::ResolveCollision + CollisionHandle (src/core/collider.cpp:3-44, 238-264)
// when a collider has a field: the target is the least |ClosestDistance| (the analytic
// distance, or the field's sample for a field-only shape), its closest point comes from
// ClosestPointBySDF and IsInside from the field's sample; a mesh's field skips positions
// outside the mesh bounds.  Kept out of line: the fast path above serves analytic shapes.
struct Contact { v3 pos, vel; };
static __device__ __noinline__ Contact resolve_with_fields(const Params &P, float r, float rc1, v3 p, v3 v) {
    Contact out;
    out.pos = p;
    out.vel = v;
    v3 *pos = &out.pos, *vel = &out.vel;
    int target = -1;
    float minD = 3.402823466e+38f;
    for (int i = 0; i < P.nshapes; i++) {
        const ShapeDev &s = P.shapes[i];
        if (s.sdf >= 0 && P.sdf[s.sdf].bounded &&
            !inside3(p, V(P.sdf[s.sdf].lo[0], P.sdf[s.sdf].lo[1], P.sdf[s.sdf].lo[2]),
                     V(P.sdf[s.sdf].hi[0], P.sdf[s.sdf].hi[1], P.sdf[s.sdf].hi[2]), P.iz6))
            continue;
        const float d = s.type == 3 ? sdf_sample(P.sdf[s.sdf], p) : shape_closest_point(s, p, P.iz, P.iz6).sd;
        if (fabsf(d) < minD) {
            target = i;
            minD = fabsf(d);
        }
    }
    if (target < 0) return out;
    const ShapeDev &s = P.shapes[target];
    Cpq q;
    bool inside;
    if (s.sdf >= 0) {
        q = sdf_closest_point(s, P.sdf[s.sdf], p);
        inside = sdf_sample(P.sdf[s.sdf], p) < 0.f;   // Shape::IsInside of a filled field
    } else {
        q = shape_closest_point(s, p, P.iz, P.iz6);
        inside = (s.reverse != 0) == !(q.sd < 0.f);
    }
    if (!(inside || fabsf(q.sd) < P.radius)) return out;
    v3 n = q.normal;
    v3 targetPoint = vadd(q.point, vmul(n, P.radius));
    v3 rel = *vel;
    float ndr = vdot(n, rel);
    v3 relN = vmul(n, ndr);
    v3 relT = vsub(rel, relN);
    if (ndr < 0.f) {
        v3 dRelN = vmul(relN, rc1);
        relN = vmul(relN, -r);
        if (vlen2(relT) > 0.f) {
            float scale = fdv(vlen(dRelN), vlen(relT));
            float fScale = fs(1.0f, fm(s.friction, scale));
            float frictionScale = rmax(0.f, fScale);
            relT = vmul(relT, frictionScale);
        }
        *vel = vadd(vadd(relN, relT), V(0.f, 0.f, 0.f));
    }
    *pos = targetPoint;
    return out;
}

// ColliderSet3::ResolveCollision over the scene's colliders: the global shapes of a
// single scene, or the container box of the particle's scene in a batch.
__device__ __forceinline__ void resolve_collision(const Params &P, float r, float rc1, v3 *pos, v3 *vel) {
    if (P.has_sdf) {
        const Contact c = resolve_with_fields(P, r, rc1, *pos, *vel);
        *pos = c.pos;
        *vel = c.vel;
        return;
    }
    if (P.nscenes > 0) {
        const ShapeDev box = P.scene_box[scene_of(P, pos->z)];
        resolve_against(P, &box, 1, r, rc1, pos, vel);
        return;
    }
    resolve_against(P, P.shapes, P.nshapes, r, rc1, pos, vel);
}

__device__ __forceinline__ void integrate_particle(const Params &P, float dt, v3 f, v3 *pos, v3 *vel) {
    v3 aFi = vdiv(f, P.mass);
    v3 at = vadd(V(0.f, 0.f, 0.f), aFi);
    v3 vi = vadd(*vel, vmul(at, dt));
    v3 pi = vadd(*pos, vmul(vi, dt));
    resolve_collision(P, P.rest_int, P.rest_c1_int, &pi, &vi);
    v3 mn = V(P.g.bmin[0], P.g.bmin[1], P.g.bmin[2]);
    v3 mx = V(P.g.bmax[0], P.g.bmax[1], P.g.bmax[2]);
    if (!inside3(pi, mn, mx, P.iz6)) {
        float r = P.radius;
        pi = vclamp(pi, vadd(mn, V(r, r, r)), vsub(mx, V(r, r, r)));
    }
    *pos = pi;
    *vel = vi;
}

// PredictVelocityAndPositionFor, src/equations/pcisph_equations3.cpp:21-27.
__device__ __forceinline__ void predict_particle(const Params &P, float dt, float dt_over_m, v3 f,
                                                 v3 fp, v3 x, v3 v, v3 *xs) {
    v3 tv = vadd(v, vmul(vadd(f, fp), dt_over_m));
    v3 tp = vadd(x, vmul(tv, dt));
    resolve_collision(P, 0.f, -1.0f, &tp, &tv);
    *xs = tp;
}

// ----------------------------------------------------------------------------
// warp/block reductions
// ----------------------------------------------------------------------------
__device__ __forceinline__ unsigned warp_max_u(unsigned v) { return __reduce_max_sync(0xffffffffu, v); }

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace bbg
