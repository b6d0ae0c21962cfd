// mesh.cu -- the signed-distance field of a triangle mesh on the device: GenerateShapeSDF of
// a mesh shape (src/core/shape.cpp:409-424, 479-510).
//
// One thread per grid node.  The distance is the least DistanceTriangle over the triangles
// (src/shapes/bvh.cpp:212-242; the reference's BVH only prunes, the minimum is the same
// value); the sign comes from MeshIsPointInside (shape.cpp:349-369): a ray from the node
// towards the mesh bounds' centre, the closest hit found (IntersectTriangle, bvh.cpp:244-
// 373, a watertight ray-triangle test with floating-point error bounds), the ray re-spawned
// past it (SpawnRayInDirection / OffsetRayOrigin, interaction.h:51-55, geometry.h:1843-
// 1858), hits counted until none is left; odd means inside.  Every operation is an
// explicitly rounded float or double operation in the reference's order, so the node values
// are the reference's except where two triangles tie for the closest hit (the reference's
// BVH order picks one of them, here the last by index does).  Triangles are read by all
// threads of a warp together (broadcast loads through L1).
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

#include <algorithm>
#include <utility>
#include <vector>

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

namespace {

__device__ __forceinline__ v3 tri_vertex(const float *__restrict__ tri, int t, int k) {
    const float *p = tri + 9 * (size_t)t + 3 * k;
    return V(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

__device__ __forceinline__ float sgn(float a) { return a > 0.f ? 1.f : (a < 0.f ? -1.f : 0.f); }

// Cross in double, rounded to float per component (geometry.h:906-914)
__device__ __forceinline__ v3 cross_d(v3 a, v3 b) {
    const double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return V(__double2float_rn(__dsub_rn(__dmul_rn(ay, bz), __dmul_rn(az, by))),
             __double2float_rn(__dsub_rn(__dmul_rn(az, bx), __dmul_rn(ax, bz))),
             __double2float_rn(__dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx))));
}

// Clamp(v, 0.0001, 1.0) with the double bounds returned as floats
__device__ __forceinline__ float clamp_edge(float v) {
    if ((double)v < 0.0001) return 0.0001f;
    if ((double)v > 1.0) return 1.f;
    return v;
}

// DistanceTriangle (bvh.cpp:212-242)
__device__ float distance_triangle(v3 p, v3 a, v3 b, v3 c) {
    const v3 ba = vsub(b, a), pa = vsub(p, a);
    const v3 cb = vsub(c, b), pb = vsub(p, b);
    const v3 ac = vsub(a, c), pc = vsub(p, c);
    const v3 nor = cross_d(ba, ac);
    const float s = fa(fa(sgn(vdot(cross_d(ba, nor), pa)), sgn(vdot(cross_d(cb, nor), pb))),
                       sgn(vdot(cross_d(ac, nor), pc)));
    float q;
    if ((double)s < 2.0) {
        const float e0 = vlen2(vsub(vmul(ba, clamp_edge(fdv(vdot(ba, pa), vlen2(ba)))), pa));
        const float e1 = vlen2(vsub(vmul(cb, clamp_edge(fdv(vdot(cb, pb), vlen2(cb)))), pb));
        const float e2 = vlen2(vsub(vmul(ac, clamp_edge(fdv(vdot(ac, pc), vlen2(ac)))), pc));
        q = rmin(rmin(e0, e1), e2);
    } else {
        const float d = vdot(nor, pa);
        q = fdv(fm(d, d), vlen2(nor));
    }
    return __fsqrt_rn(q);
}

__device__ __forceinline__ float comp(v3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ v3 permute(v3 v, int x, int y, int z) { return V(comp(v, x), comp(v, y), comp(v, z)); }
__device__ __forceinline__ float max3abs(float a, float b, float c) {   // MaxComponent(Abs(v))
    return rmax(fabsf(a), rmax(fabsf(b), fabsf(c)));
}
__device__ __forceinline__ bool is_zero(float a) { return (double)fabsf(a) < 1e-8; }

struct Gammas { float g2, g3, g5, g7; };

struct Hit { v3 p, err, n; float t; };

// IntersectTriangle (bvh.cpp:244-373) against a ray with tMax; on a hit, tmax and hit
// are updated.
__device__ bool intersect_triangle(v3 o, v3 dir, float &tmax, v3 p0, v3 p1, v3 p2, const Gammas &G, Hit &hit) {
    v3 p0t = vsub(p0, o), p1t = vsub(p1, o), p2t = vsub(p2, o);
    const v3 ad = V(fabsf(dir.x), fabsf(dir.y), fabsf(dir.z));
    const int kz = (ad.x > ad.y) ? ((ad.x > ad.z) ? 0 : 2) : ((ad.y > ad.z) ? 1 : 2);
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    const v3 d = permute(dir, kx, ky, kz);
    p0t = permute(p0t, kx, ky, kz);
    p1t = permute(p1t, kx, ky, kz);
    p2t = permute(p2t, kx, ky, kz);
    const float sx = fdv(-d.x, d.z), sy = fdv(-d.y, d.z), sz = fdv(1.f, d.z);
    p0t.x = fa(p0t.x, fm(sx, p0t.z));
    p0t.y = fa(p0t.y, fm(sy, p0t.z));
    p1t.x = fa(p1t.x, fm(sx, p1t.z));
    p1t.y = fa(p1t.y, fm(sy, p1t.z));
    p2t.x = fa(p2t.x, fm(sx, p2t.z));
    p2t.y = fa(p2t.y, fm(sy, p2t.z));
    float e0 = fs(fm(p1t.x, p2t.y), fm(p1t.y, p2t.x));
    float e1 = fs(fm(p2t.x, p0t.y), fm(p2t.y, p0t.x));
    float e2 = fs(fm(p0t.x, p1t.y), fm(p0t.y, p1t.x));
    if (is_zero(e0) || is_zero(e1) || is_zero(e2)) {
        e0 = __double2float_rn(__dsub_rn(__dmul_rn((double)p2t.y, (double)p1t.x), __dmul_rn((double)p2t.x, (double)p1t.y)));
        e1 = __double2float_rn(__dsub_rn(__dmul_rn((double)p0t.y, (double)p2t.x), __dmul_rn((double)p0t.x, (double)p2t.y)));
        e2 = __double2float_rn(__dsub_rn(__dmul_rn((double)p1t.y, (double)p0t.x), __dmul_rn((double)p1t.x, (double)p0t.y)));
    }
    if ((e0 < 0.f || e1 < 0.f || e2 < 0.f) && (e0 > 0.f || e1 > 0.f || e2 > 0.f)) return false;
    const float det = fa(fa(e0, e1), e2);
    if (is_zero(det)) return false;
    p0t.z = fm(p0t.z, sz);
    p1t.z = fm(p1t.z, sz);
    p2t.z = fm(p2t.z, sz);
    const float ts = fa(fa(fm(e0, p0t.z), fm(e1, p1t.z)), fm(e2, p2t.z));
    if (det < 0.f && (ts >= 0.f || ts < fm(tmax, det))) return false;
    if (det > 0.f && (ts <= 0.f || ts > fm(tmax, det))) return false;
    const float inv = fdv(1.f, det);
    const float b0 = fm(e0, inv), b1 = fm(e1, inv), b2 = fm(e2, inv);
    const float t = fm(ts, inv);
    const float maxzt = max3abs(p0t.z, p1t.z, p2t.z);
    const float dz = fm(G.g3, maxzt);
    const float maxxt = max3abs(p0t.x, p1t.x, p2t.x);
    const float maxyt = max3abs(p0t.y, p1t.y, p2t.y);
    const float dx = fm(G.g5, fa(maxxt, maxzt));
    const float dy = fm(G.g5, fa(maxyt, maxzt));
    const float de = fm(2.f, fa(fa(fm(fm(G.g2, maxxt), maxyt), fm(dy, maxxt)), fm(dx, maxyt)));
    const float maxe = max3abs(e0, e1, e2);
    const float dt = fm(fm(3.f, fa(fa(fm(fm(G.g3, maxe), maxzt), fm(de, maxzt)), fm(dz, maxe))), fabsf(inv));
    if (t <= dt) return false;
    const float xs = fa(fa(fabsf(fm(b0, p0.x)), fabsf(fm(b1, p1.x))), fabsf(fm(b2, p2.x)));
    const float ys = fa(fa(fabsf(fm(b0, p0.y)), fabsf(fm(b1, p1.y))), fabsf(fm(b2, p2.y)));
    const float zs = fa(fa(fabsf(fm(b0, p0.z)), fabsf(fm(b1, p1.z))), fabsf(fm(b2, p2.z)));
    hit.err = vmul(V(xs, ys, zs), G.g7);
    hit.p = vadd(vadd(vmul(p0, b0), vmul(p1, b1)), vmul(p2, b2));
    const v3 nn = cross_d(vsub(p0, p2), vsub(p1, p2));
    hit.n = vdiv(nn, vlen(nn));
    hit.t = t;
    tmax = t;
    return true;
}

// Bounds3::Intersect of the mesh bounds (geometry.h:1881-1898)
__device__ bool hits_bounds(v3 lo, v3 hi, v3 o, v3 d, float tmax, float g3) {
    float t0 = 0.f, t1 = tmax;
    const float grow = fa(1.f, fm(2.f, g3));
    for (int k = 0; k < 3; k++) {
        const float inv = fdv(1.f, comp(d, k));
        float tn = fm(fs(comp(lo, k), comp(o, k)), inv);
        float tf = fm(fs(comp(hi, k), comp(o, k)), inv);
        if (tn > tf) {
            const float x = tn;
            tn = tf;
            tf = x;
        }
        tf = fm(tf, grow);
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return false;
    }
    return true;
}

__device__ __forceinline__ float next_up(float v) {
    if (isinf(v) && v > 0.f) return v;
    if (v == -0.f) v = 0.f;
    unsigned u = __float_as_uint(v);
    u = v >= 0.f ? u + 1u : u - 1u;
    return __uint_as_float(u);
}

__device__ __forceinline__ float next_down(float v) {
    if (isinf(v) && v < 0.f) return v;
    if (v == 0.f) v = -0.f;
    unsigned u = __float_as_uint(v);
    u = v > 0.f ? u - 1u : u + 1u;
    return __uint_as_float(u);
}

// OffsetRayOrigin (geometry.h:1843-1858): past the hit by the error bound + 0.0001 along n
__device__ v3 offset_origin(const Hit &h, v3 w) {
    const float d = __double2float_rn((double)vdot(V(fabsf(h.n.x), fabsf(h.n.y), fabsf(h.n.z)), h.err) + 0.0001);
    v3 off = vmul(h.n, d);
    if (vdot(w, h.n) < 0.f) off = V(-off.x, -off.y, -off.z);
    v3 po = vadd(h.p, off);
    po.x = off.x > 0.f ? next_up(po.x) : (off.x < 0.f ? next_down(po.x) : po.x);
    po.y = off.y > 0.f ? next_up(po.y) : (off.y < 0.f ? next_down(po.y) : po.y);
    po.z = off.z > 0.f ? next_up(po.z) : (off.z < 0.f ? next_down(po.z) : po.z);
    return po;
}

constexpr int kMaxRayHits = 256;   // a ray stuck on degenerate geometry gives up (outside)

// Triangles are visited in tiles of kMeshTile consecutive triangles, each split into
// kMeshTile / kMeshSub sub-tiles, every tile and sub-tile with its bounding box: one is
// skipped when its box cannot hold a better answer, which leaves every result equal to the
// scan over all triangles.
//  - distance: skipped when the box lies farther than the best distance so far by more than
//    1 % plus an absolute margin (1e-3 of the mesh's bounding diagonal), so a skipped
//    triangle's computed distance cannot be below the best despite rounding;
//  - rays: skipped when the conservative ray-box test (Bounds3::IntersectP with the gamma
//    growth, the test of the reference's BVH) rejects the box for the current tMax, which
//    never rejects a box holding a hit at or before tMax.
constexpr int kMeshTile = 64;
constexpr int kMeshSub = 8;

// The box tests of the two passes.
__device__ __forceinline__ bool box_near(const float *__restrict__ bx, v3 p, float d, float margin) {
    const float ex = fmaxf(fmaxf(__ldg(&bx[0]) - p.x, p.x - __ldg(&bx[3])), 0.f);
    const float ey = fmaxf(fmaxf(__ldg(&bx[1]) - p.y, p.y - __ldg(&bx[4])), 0.f);
    const float ez = fmaxf(fmaxf(__ldg(&bx[2]) - p.z, p.z - __ldg(&bx[5])), 0.f);
    return !(sqrtf(ex * ex + ey * ey + ez * ez) > d * 1.01f + margin);
}

__device__ __forceinline__ bool box_on_ray(const float *__restrict__ bx, v3 o, v3 dir, float tmax, float g3) {
    return hits_bounds(V(__ldg(&bx[0]), __ldg(&bx[1]), __ldg(&bx[2])), V(__ldg(&bx[3]), __ldg(&bx[4]), __ldg(&bx[5])), o,
                       dir, tmax, g3);
}

// f(t) for every triangle t of the tiles and sub-tiles that keep(box) accepts, in order
template <class Keep, class F>
__device__ __forceinline__ void mesh_walk(const float *__restrict__ tiles, int ntri, Keep &&keep, F &&f) {
    const int ntiles = (ntri + kMeshTile - 1) / kMeshTile, nsub = (ntri + kMeshSub - 1) / kMeshSub;
    const float *sub = tiles + 6 * ntiles;
    for (int b = 0; b < ntiles; b++) {
        if (!keep(tiles + 6 * b)) continue;
        const int s1 = min(nsub, (b + 1) * (kMeshTile / kMeshSub));
        for (int q = b * (kMeshTile / kMeshSub); q < s1; q++) {
            if (!keep(sub + 6 * q)) continue;
            const int t1 = min(ntri, (q + 1) * kMeshSub);
            for (int t = q * kMeshSub; t < t1; t++) f(t);
        }
    }
}

__global__ void k_mesh_sdf(const float *__restrict__ tri, int ntri, const float *__restrict__ tiles,
                           const float *__restrict__ dtri, const float *__restrict__ dtiles, float margin,
                           SdfDev g, v3 lo, v3 hi, Gammas G, float *__restrict__ out, unsigned *__restrict__ stuck) {
    const unsigned total = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz;
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= total) return;
    const unsigned plane = (unsigned)g.nx * (unsigned)g.ny;
    const unsigned k = id / plane, rem = id - k * plane;
    const unsigned j = rem / (unsigned)g.nx, i = rem % (unsigned)g.nx;
    const v3 p = V(fa(g.org[0], fm(g.sp[0], (float)i)), fa(g.org[1], fm(g.sp[1], (float)j)),
                   fa(g.org[2], fm(g.sp[2], (float)k)));
    // MeshClosestDistance: the least DistanceTriangle (strictly smaller replaces; the least
    // value does not depend on the order, so this pass walks the Morton-ordered copy)
    float d = 3.1622776601683794e+18f;   // SqrtInfinity
    mesh_walk(dtiles, ntri, [&](const float *bx) { return box_near(bx, p, d, margin); }, [&](int t) {
        const float dt = distance_triangle(p, tri_vertex(dtri, t, 0), tri_vertex(dtri, t, 1), tri_vertex(dtri, t, 2));
        if (dt < d) d = dt;
    });
    // MeshIsPointInside: ray towards the bounds' centre, closest hits counted
    const v3 center = vmul(vadd(lo, hi), 0.5f);
    const v3 to = vsub(center, p);
    const v3 dir = vdiv(to, vlen(to));
    v3 o = p;
    int hits = 0;
    bool done = false;
    for (int it = 0; it < kMaxRayHits && !done; it++) {
        float tmax = 3.402823466e+38f;   // Infinity
        Hit h;
        bool any = false;
        if (hits_bounds(lo, hi, o, dir, tmax, G.g3)) {
            mesh_walk(tiles, ntri, [&](const float *bx) { return box_on_ray(bx, o, dir, tmax, G.g3); }, [&](int t) {
                any |= intersect_triangle(o, dir, tmax, tri_vertex(tri, t, 0), tri_vertex(tri, t, 1),
                                          tri_vertex(tri, t, 2), G, h);
            });
        }
        if (!any) {
            done = true;
        } else {
            hits++;
            o = offset_origin(h, dir);
        }
    }
    if (!done) {
        atomicAdd(stuck, 1u);
        hits = 0;
    }
    const bool interior = (hits % 2) != 0 && hits > 0;
    const float psd = rmax(fabsf(d), 0.00001f);
    out[id] = interior ? -psd : psd;
}

}  // namespace

// boxes of the tiles, then of the sub-tiles (6 floats each)
int mesh_tiles(int ntri) { return (ntri + kMeshTile - 1) / kMeshTile + (ntri + kMeshSub - 1) / kMeshSub; }

static void tile_boxes(const float *tri, int ntri, int size, float *tiles) {
    for (int b = 0; b < (ntri + size - 1) / size; b++) {
        float *bx = tiles + 6 * b;
        for (int k = 0; k < 3; k++) {
            bx[k] = 3.402823466e+38f;
            bx[3 + k] = -3.402823466e+38f;
        }
        for (int t = b * size; t < ntri && t < (b + 1) * size; t++)
            for (int c = 0; c < 3; c++)
                for (int k = 0; k < 3; k++) {
                    const float x = tri[9 * (size_t)t + 3 * c + k];
                    bx[k] = x < bx[k] ? x : bx[k];
                    bx[3 + k] = x > bx[3 + k] ? x : bx[3 + k];
                }
    }
}

void mesh_tile_bounds(const float *tri, int ntri, float *tiles) {
    tile_boxes(tri, ntri, kMeshTile, tiles);
    tile_boxes(tri, ntri, kMeshSub, tiles + 6 * ((ntri + kMeshTile - 1) / kMeshTile));
}

// The triangles in the Morton order of their centroids (30-bit codes in the mesh bounds,
// ties by index), for the distance pass's tiles.
void mesh_morton_order(const float *tri, int ntri, const float lo[3], const float hi[3], float *sorted) {
    std::vector<std::pair<unsigned, int>> key((size_t)ntri);
    for (int t = 0; t < ntri; t++) {
        unsigned code = 0;
        unsigned q[3];
        for (int k = 0; k < 3; k++) {
            const float c = (tri[9 * (size_t)t + k] + tri[9 * (size_t)t + 3 + k] + tri[9 * (size_t)t + 6 + k]) / 3.f;
            const float ext = hi[k] - lo[k];
            float u = ext > 0.f ? (c - lo[k]) / ext : 0.f;
            u = u < 0.f ? 0.f : (u > 1.f ? 1.f : u);
            q[k] = (unsigned)(u * 1023.f);
        }
        for (int bit = 9; bit >= 0; bit--)
            for (int k = 0; k < 3; k++) code = (code << 1) | ((q[k] >> bit) & 1u);
        key[(size_t)t] = std::make_pair(code, t);
    }
    std::sort(key.begin(), key.end());
    for (int r = 0; r < ntri; r++)
        for (int q = 0; q < 9; q++) sorted[9 * (size_t)r + q] = tri[9 * (size_t)key[(size_t)r].second + q];
}

void launch_mesh_sdf(const float *tri, int ntri, const float *tiles, const float *dtri, const float *dtiles,
                     float margin, const SdfDev &g, const float lo[3], const float hi[3], const float gamma[4],
                     float *out, unsigned *stuck, cudaStream_t s) {
    const long long total = (long long)g.nx * g.ny * g.nz;
    Gammas G;
    G.g2 = gamma[0];
    G.g3 = gamma[1];
    G.g5 = gamma[2];
    G.g7 = gamma[3];
    v3 l, h;
    l.x = lo[0]; l.y = lo[1]; l.z = lo[2];
    h.x = hi[0]; h.y = hi[1]; h.z = hi[2];
    k_mesh_sdf<<<blocks_for(total, 128), 128, 0, s>>>(tri, ntri, tiles, dtri, dtiles, margin, g, l, h, G, out, stuck);
}

}  // namespace bbg
