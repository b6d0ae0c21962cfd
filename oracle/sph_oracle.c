/*
 * sph_oracle.c -- CPU oracle for the Bubbles 3D SPH / PCISPH particle step.
 *
 * TEST INFRASTRUCTURE ONLY: the reference result the CUDA path is compared with (see
 * sph_oracle.h for who may load it).  Build with -ffp-contract=off so that x86-64 and aarch64
 * produce the same bits (the reference itself is compiled without contraction on
 * x86-64).  -DORC_FLOAT=float gives the FP32 oracle, -DORC_FLOAT=double the FP64
 * one.
 *
 * Every function below names the reference function it restates.  Expressions
 * keep the reference's operand order and its float/double promotions (for
 * example `Float x = 1.0 - d2 / h2;` evaluates 1.0 - (float) in double), because
 * those decide the last bit of the FP32 results.
 */
#include "sph_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORC_FLOAT
#define ORC_FLOAT float
#endif
typedef ORC_FLOAT Float;

#define ORC_PI 3.14159265358979323846      /* Pi, src/core/geometry.h:45 */
#define ORC_EPSILON 0.0001f                /* Epsilon, src/core/geometry.h:44 */
#define ORC_BUCKET 100                     /* MaximumParticlesPerBucket, particle.h:10 */

/* ------------------------------------------------------------------------- */
/* threads: the reference's ParallelFor (src/cuda/cutil.h:294-338) spawns one  */
/* std::thread per slice on every call; this does the same with pthreads.     */
/* ------------------------------------------------------------------------- */
static int g_threads = 1;

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }
int orc_float_bytes(void) { return (int)sizeof(Float); }

typedef void (*range_fn)(void *ctx, int begin, int end);
typedef struct { range_fn fn; void *ctx; int b, e; } slice_t;

static void *slice_main(void *arg) {
    slice_t *s = (slice_t *)arg;
    s->fn(s->ctx, s->b, s->e);
    return NULL;
}

static void parallel_for(int n, range_fn fn, void *ctx) {
    if (n <= 0) return;
    int nt = g_threads;
    if (nt <= 1 || n < 2 * nt) { fn(ctx, 0, n); return; }
    pthread_t th[256];
    slice_t sl[256];
    if (nt > 256) nt = 256;
    int chunk = (n + nt - 1) / nt;
    int used = 0;
    for (int t = 0; t < nt; t++) {
        int b = t * chunk, e = b + chunk;
        if (b >= n) break;
        if (e > n) e = n;
        sl[t].fn = fn; sl[t].ctx = ctx; sl[t].b = b; sl[t].e = e;
        if (pthread_create(&th[t], NULL, slice_main, &sl[t]) != 0) {
            fn(ctx, b, e);
            sl[t].fn = NULL;
        }
        used++;
    }
    for (int t = 0; t < used; t++)
        if (sl[t].fn) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------- */
/* scalar helpers: src/core/geometry.h:107-126                                */
/* ------------------------------------------------------------------------- */
static inline Float absf_(Float v) { return v > 0 ? v : -v; }
static inline int is_zero(Float a) { return (double)absf_(a) < 1e-8; }
static inline int is_unsafe_zero(Float a) { return (double)absf_(a) < 1e-6; }
static inline Float max_(Float a, Float b) { return a < b ? b : a; }
static inline Float min_(Float a, Float b) { return a < b ? a : b; }
static inline Float clamp_(Float v, Float lo, Float hi) {
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}
static inline Float sqrt_(Float v) { return (Float)sqrt((double)v); }
/* std::pow(Float, Float): powf for float (libstdc++ overload), pow for double */
static inline Float pow_(Float a, Float b) {
    if (sizeof(Float) == sizeof(float)) return (Float)powf((float)a, (float)b);
    return (Float)pow((double)a, (double)b);
}

/* vec3<Float> with the reference's operator semantics (geometry.h:496-629) */
typedef struct { Float x, y, z; } v3;
static inline v3 V(Float x, Float y, Float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, Float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vdiv(v3 a, Float f) { Float inv = (Float)1 / f; return V(a.x * inv, a.y * inv, a.z * inv); }
static inline Float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline Float vlen2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline Float vlen(v3 a) { return sqrt_(vlen2(a)); }
static inline Float vdist(v3 a, v3 b) { return vlen(vsub(a, b)); }
static inline Float vget(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline v3 vclamp(v3 v, v3 lo, v3 hi) {
    return V(clamp_(v.x, lo.x, hi.x), clamp_(v.y, lo.y, hi.y), clamp_(v.z, lo.z, hi.z));
}

typedef struct { v3 mn, mx; } bounds3;
static inline bounds3 mkbounds(v3 a, v3 b) {
    bounds3 r;
    r.mn = V(min_(a.x, b.x), min_(a.y, b.y), min_(a.z, b.z));
    r.mx = V(max_(a.x, b.x), max_(a.y, b.y), max_(a.z, b.z));
    return r;
}

/* Inside(vec3, Bounds3) with its 1e-6 face tolerance, geometry.h:1773-1783 */
static inline int inside3(v3 p, bounds3 b) {
    int rv = (p.x >= b.mn.x && p.x <= b.mx.x && p.y >= b.mn.y &&
              p.y <= b.mx.y && p.z >= b.mn.z && p.z <= b.mx.z);
    if (!rv) {
        Float ox = min_(absf_(b.mn.x - p.x), absf_(b.mx.x - p.x));
        Float oy = min_(absf_(b.mn.y - p.y), absf_(b.mx.y - p.y));
        Float oz = min_(absf_(b.mn.z - p.z), absf_(b.mx.z - p.z));
        rv = is_unsafe_zero(ox) || is_unsafe_zero(oy) || is_unsafe_zero(oz);
    }
    return rv;
}

/* ------------------------------------------------------------------------- */
/* SPH kernels: src/core/kernel.cpp:112-233                                   */
/* ------------------------------------------------------------------------- */
typedef struct { Float h, h2, h3, h4, h5; } kern;

static inline kern kern_std(Float r) {      /* SphStdKernel3::SetRadius */
    kern k; k.h = r; k.h2 = k.h * k.h; k.h3 = k.h2 * k.h; k.h4 = 0; k.h5 = k.h2 * k.h3;
    return k;
}
static inline kern kern_spiky(Float r) {    /* SphSpikyKernel3::SetRadius */
    kern k; k.h = r; k.h2 = k.h * k.h; k.h3 = k.h2 * k.h; k.h4 = k.h2 * k.h2;
    k.h5 = k.h2 * k.h3;
    return k;
}

static inline Float std_W(const kern *k, Float distance) {           /* kernel.cpp:123-132 */
    Float d2 = distance * distance;
    Float of = d2 - k->h2;
    if (is_zero(of) || of > 0) return 0;
    Float x = 1.0 - d2 / k->h2;
    return 315.0 / (64.0 * ORC_PI * k->h3) * x * x * x;
}
static inline Float spiky_W(const kern *k, Float distance) {         /* kernel.cpp:181-189 */
    Float of = distance - k->h;
    if (is_zero(of) || of > 0) return 0;
    Float x = 1.0 - distance / k->h;
    return 15.0 / (ORC_PI * k->h3) * x * x * x;
}
static inline Float spiky_dW(const kern *k, Float distance) {        /* kernel.cpp:191-199 */
    Float of = distance - k->h;
    if (is_zero(of) || of > 0) return 0;
    Float x = 1.0 - distance / k->h;
    return -45.0 / (ORC_PI * k->h4) * x * x;
}
static inline Float spiky_d2W(const kern *k, Float distance) {       /* kernel.cpp:201-209 */
    Float of = distance - k->h;
    if (is_zero(of) || of > 0) return 0;
    Float x = 1.0 - distance / k->h;
    return 90.0 / (ORC_PI * k->h5) * x;
}
static inline v3 spiky_gradW(const kern *k, Float distance, v3 dir) { /* kernel.cpp:220-222 */
    return vmul(dir, -spiky_dW(k, distance));
}
static inline int within_spiky(Float distance, Float radius) {        /* kernel.cpp:224-227 */
    Float of = distance - radius;
    return !(is_zero(of) || of > 0);
}
static inline int within_std(Float distance, Float radius) {          /* kernel.cpp:229-233 */
    Float h2 = radius * radius;
    Float d2 = distance * distance;
    Float of = d2 - h2;
    return !(is_zero(of) || of > 0);
}

double orc_kernel_eval(int which, double h, double r) {
    kern ks = kern_std((Float)h), kp = kern_spiky((Float)h);
    switch (which) {
        case 0: return std_W(&ks, (Float)r);
        case 1: return spiky_W(&kp, (Float)r);
        case 2: return spiky_dW(&kp, (Float)r);
        case 3: return spiky_d2W(&kp, (Float)r);
        case 4: return within_std((Float)r, (Float)h);
        case 5: return within_spiky((Float)r, (Float)h);
        default: return 0;
    }
}

/* ------------------------------------------------------------------------- */
/* BCC lattice: src/generator/bcclattice.cpp:5-77                             */
/* ------------------------------------------------------------------------- */
static int bcc_generate(bounds3 domain, Float spacing, v3 *points, int maxn) {
    Float halfSpacing = spacing / 2;
    Float width = absf_(domain.mx.x - domain.mn.x);
    Float height = absf_(domain.mx.y - domain.mn.y);
    Float depth = absf_(domain.mx.z - domain.mn.z);
    int hasOff = 0, stop = 0, pi = 0;
    v3 pos = V(0, 0, 0);
    for (int k = 0; k * halfSpacing <= depth && !stop; k++) {
        pos.z = k * halfSpacing + domain.mn.z;
        Float offset = hasOff ? halfSpacing : 0;
        for (int j = 0; j * spacing + offset <= height && !stop; j++) {
            pos.y = j * spacing + offset + domain.mn.y;
            for (int i = 0; i * spacing + offset <= width && !stop; i++) {
                pos.x = i * spacing + offset + domain.mn.x;
                if (maxn < 0 || pi < maxn) {
                    if (points) points[pi] = pos;
                    pi++;
                } else {
                    stop = 1;
                    break;
                }
            }
        }
        hasOff = !hasOff;
    }
    return pi;
}

/* SphParticleSet3::ComputeMass, src/core/particle.h:557-582 */
static Float compute_mass_bcc(Float targetDensity, Float targetSpacing, Float kernelRadius) {
    v3 points[1024];
    kern k = kern_std(kernelRadius);
    Float a = -1.5 * kernelRadius, b = 1.5 * kernelRadius;
    bounds3 bnd = mkbounds(V(a, a, a), V(b, b, b));
    int c = bcc_generate(bnd, targetSpacing, points, 1024);
    Float nDen = 0;
    for (int i = 0; i < c; i++) {
        Float sum = 0;
        for (int j = 0; j < c; j++) sum += std_W(&k, vlen(vsub(points[i], points[j])));
        nDen = max_(nDen, sum);
    }
    return targetDensity / nDen;
}

double orc_compute_mass_bcc(double target_density, double spacing, double kernel_radius) {
    return compute_mass_bcc((Float)target_density, (Float)spacing, (Float)kernel_radius);
}

/* PciSphSolver3::ComputeDeltaDenom, src/solvers/pcisph_solver3.cpp:148-180 */
static Float compute_delta_denom(Float spacing, Float kernelRadius) {
    Float kernelRadius2 = kernelRadius * kernelRadius;
    Float a = -1.5 * kernelRadius, b = 1.5 * kernelRadius;
    bounds3 bnd = mkbounds(V(a, a, a), V(b, b, b));
    int c = bcc_generate(bnd, spacing, NULL, -1);
    v3 *pts = (v3 *)malloc(sizeof(v3) * (size_t)(c > 0 ? c : 1));
    bcc_generate(bnd, spacing, pts, -1);
    kern k = kern_spiky(kernelRadius);
    Float denom = 0, denom2 = 0;
    v3 denom1 = V(0, 0, 0);
    for (int i = 0; i < c; i++) {
        v3 point = pts[i];
        Float distanceSquared = vlen2(point);
        if (distanceSquared < kernelRadius2) {
            Float distance = sqrt_(distanceSquared);
            v3 direction = (distance > 0) ? vdiv(point, distance) : V(0, 0, 0);
            v3 gradij = spiky_gradW(&k, distance, direction);
            denom1 = vadd(denom1, gradij);
            denom2 += vdot(gradij, gradij);
        }
    }
    denom += -vdot(denom1, denom1) - denom2;
    free(pts);
    return denom;
}

double orc_compute_delta_denom(double spacing, double kernel_radius) {
    return compute_delta_denom((Float)spacing, (Float)kernel_radius);
}

/* ------------------------------------------------------------------------- */
/* Grid: UtilBuildGridForDomain (util.cpp:269-287) + Grid::Build (grid.h:627-666) */
/* ------------------------------------------------------------------------- */
typedef struct {
    int dims[3];
    unsigned total;
    Float len[3], minp[3];
    bounds3 b;
    int *nbr;      /* 27 per cell, reference order: y, then x, then z */
    int *nbr_n;
} ogrid;

static void grid_geometry(ogrid *g, v3 dmin, v3 dmax, Float spacing, Float spacingScale) {
    bounds3 domain = mkbounds(dmin, dmax);
    Float length = spacing * spacingScale;
    Float hlen = 0.5 * length;
    Float invLen = 1.0f / length;
    int mx = (int)ceil(absf_(domain.mx.x - domain.mn.x) * invLen);
    int my = (int)ceil(absf_(domain.mx.y - domain.mn.y) * invLen);
    int mz = (int)ceil(absf_(domain.mx.z - domain.mn.z) * invLen);
    mx += (mx % 2) * length;
    my += (my % 2) * length;
    mz += (mz % 2) * length;
    v3 half = V(mx * hlen, my * hlen, mz * hlen);
    v3 center = vmul(vadd(domain.mn, domain.mx), 0.5);
    v3 dp0 = vsub(center, half), dp1 = vadd(center, half);
    int res[3] = {mx, my, mz};
    /* Grid::Build */
    v3 lower = V(FLT_MAX, FLT_MAX, FLT_MAX), high = V(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    v3 p0 = V(max_(dp0.x, dp1.x), max_(dp0.y, dp1.y), max_(dp0.z, dp1.z));
    v3 p1 = V(min_(dp0.x, dp1.x), min_(dp0.y, dp1.y), min_(dp0.z, dp1.z));
    Float lo[3] = {lower.x, lower.y, lower.z}, hi[3] = {high.x, high.y, high.z};
    for (int k = 0; k < 3; k++) {
        Float dl = vget(p0, k), du = vget(p1, k);
        if (dl < lo[k]) lo[k] = dl;
        if (dl > hi[k]) hi[k] = dl;
        if (du > hi[k]) hi[k] = du;
        if (du < lo[k]) lo[k] = du;
    }
    Float maxp[3];
    g->total = 1;
    for (int k = 0; k < 3; k++) {
        Float s = hi[k] - lo[k];
        Float len = s / (Float)res[k];
        g->len[k] = len;
        g->dims[k] = (int)ceil(s / len);
        maxp[k] = lo[k] + (Float)g->dims[k] * g->len[k];
        g->total *= (unsigned)g->dims[k];
        g->minp[k] = lo[k];
    }
    g->b = mkbounds(V(lo[0], lo[1], lo[2]), V(maxp[0], maxp[1], maxp[2]));
}

/* Grid::GetNeighborListFor(id, 1, ...), grid.h:555-593 */
static int grid_neighbor_list(const ogrid *g, int id, int *out) {
    unsigned plane = (unsigned)g->dims[0] * (unsigned)g->dims[1];
    int u2 = (int)((unsigned)id / plane);
    unsigned rem = (unsigned)id - (unsigned)u2 * plane;
    int u1 = (int)(rem / (unsigned)g->dims[0]);
    int u0 = (int)(rem % (unsigned)g->dims[0]);
    int count = 0;
    for (int j = u1 - 1; j <= u1 + 1; j++) {
        if (j < 0 || j >= g->dims[1]) continue;
        for (int i = u0 - 1; i <= u0 + 1; i++) {
            if (i < 0 || i >= g->dims[0]) continue;
            for (int k = u2 - 1; k <= u2 + 1; k++) {
                if (k < 0 || k >= g->dims[2]) continue;
                out[count++] = i + j * g->dims[0] + k * g->dims[0] * g->dims[1];
            }
        }
    }
    return count;
}

static void grid_build_lists(ogrid *g) {
    g->nbr = (int *)malloc(sizeof(int) * 27 * (size_t)g->total);
    g->nbr_n = (int *)malloc(sizeof(int) * (size_t)g->total);
    for (unsigned c = 0; c < g->total; c++)
        g->nbr_n[c] = grid_neighbor_list(g, (int)c, &g->nbr[27 * (size_t)c]);
}

int orc_build_grid(const double dmin[3], const double dmax[3], double spacing, double scale,
                   int dims[3], double geo[12]) {
    ogrid g;
    grid_geometry(&g, V((Float)dmin[0], (Float)dmin[1], (Float)dmin[2]),
                  V((Float)dmax[0], (Float)dmax[1], (Float)dmax[2]), (Float)spacing,
                  (Float)scale);
    for (int k = 0; k < 3; k++) {
        dims[k] = g.dims[k];
        geo[k] = g.minp[k]; geo[3 + k] = g.len[k];
        geo[6 + k] = vget(g.b.mn, k); geo[9 + k] = vget(g.b.mx, k);
    }
    return (int)g.total;
}

/* Grid::ExtremeEpsilon + GetHashedPosition + LinearIndex, grid.h:183-193, 259-298 */
static inline Float extreme_eps(const ogrid *g, Float p, int axis) {
    Float eps = 0;
    Float p0 = vget(g->b.mn, axis), p1 = vget(g->b.mx, axis);
    if (is_zero(p - p0)) eps = ORC_EPSILON;
    else if (is_zero(p - p1)) eps = -ORC_EPSILON;
    return eps;
}

static inline int grid_hash_u(const ogrid *g, v3 p, int u[3]) {
    int bad = 0;
    for (int i = 0; i < 3; i++) {
        Float pi = vget(p, i);
        pi += extreme_eps(g, pi, i);
        Float dmin = g->minp[i];
        Float dlen = g->len[i];
        Float dp = (pi - dmin) / dlen;
        int id = (int)floor(dp);
        /* The reference asserts here (compiled out); clamp so the oracle stays memory safe. */
        if (id < 0) { id = 0; bad = 1; }
        if (id >= g->dims[i]) { id = g->dims[i] - 1; bad = 1; }
        u[i] = id;
    }
    return bad;
}

static inline unsigned grid_hash(const ogrid *g, v3 p) {
    int u[3];
    grid_hash_u(g, p, u);
    return (unsigned)u[0] + (unsigned)u[1] * (unsigned)g->dims[0] +
           (unsigned)u[2] * (unsigned)g->dims[0] * (unsigned)g->dims[1];
}

/* ------------------------------------------------------------------------- */
/* Shapes and colliders                                                        */
/* ------------------------------------------------------------------------- */
typedef struct {
    int type, reverse;
    v3 t;                 /* translation */
    Float sx, sy, sz;     /* box sizes */
    Float radius;         /* sphere */
    Float friction;
} oshape;

typedef struct { v3 point, normal, velocity; Float sd; } cpq;

/* Plane3::ClosestPoint, box.cpp:22-26 */
static inline v3 plane_closest(v3 ppoint, v3 pnormal, v3 p) {
    v3 r = vsub(p, ppoint);
    return vadd(vsub(r, vmul(pnormal, vdot(r, pnormal))), ppoint);
}

static void box_planes(const oshape *s, bounds3 *lb, v3 pp[6], v3 pn[6]) {
    Float hx = s->sx / 2.0, hy = s->sy / 2.0, hz = s->sz / 2.0;
    *lb = mkbounds(V(-hx, -hy, -hz), V(hx, hy, hz));
    pp[0] = lb->mx; pn[0] = V(1, 0, 0);
    pp[1] = lb->mx; pn[1] = V(0, 1, 0);
    pp[2] = lb->mx; pn[2] = V(0, 0, 1);
    pp[3] = lb->mn; pn[3] = V(-1, 0, 0);
    pp[4] = lb->mn; pn[4] = V(0, -1, 0);
    pp[5] = lb->mn; pn[5] = V(0, 0, -1);
}

/* Shape::BoxClosestDistance, box.cpp:74-109 */
static Float box_closest_distance(const oshape *s, v3 point) {
    v3 pLocal = vsub(point, s->t);
    bounds3 lb; v3 pp[6], pn[6];
    box_planes(s, &lb, pp, pn);
    v3 closest;
    int isNeg = 0;
    if (inside3(pLocal, lb)) {
        closest = plane_closest(pp[0], pn[0], pLocal);
        Float d2 = vlen2(vsub(closest, pLocal));
        for (int i = 1; i < 6; i++) {
            v3 local = plane_closest(pp[i], pn[i], pLocal);
            Float ld2 = vlen2(vsub(local, pLocal));
            if (ld2 < d2) { closest = local; d2 = ld2; }
        }
        isNeg = 1;
    } else {
        closest = vclamp(pLocal, lb.mn, lb.mx);
    }
    return isNeg ? -vdist(pLocal, closest) : vdist(pLocal, closest);
}

/* Shape::BoxClosestPoint, box.cpp:111-172 */
static cpq box_closest_point(const oshape *s, v3 point) {
    v3 pLocal = vsub(point, s->t);
    bounds3 lb; v3 pp[6], pn[6];
    box_planes(s, &lb, pp, pn);
    v3 closest, normal = pn[0];
    int isNeg = 0;
    if (inside3(pLocal, lb)) {
        closest = plane_closest(pp[0], pn[0], pLocal);
        Float d2 = vlen2(vsub(closest, pLocal));
        for (int i = 1; i < 6; i++) {
            v3 local = plane_closest(pp[i], pn[i], pLocal);
            Float ld2 = vlen2(vsub(local, pLocal));
            if (ld2 < d2) { closest = local; normal = pn[i]; d2 = ld2; }
        }
        isNeg = 1;
    } else {
        closest = vclamp(pLocal, lb.mn, lb.mx);
        v3 cov = vsub(pLocal, closest);
        Float maxCosine = vdot(cov, normal);
        for (int i = 1; i < 6; i++) {
            Float cosine = vdot(pn[i], cov);
            if (cosine > maxCosine) { normal = pn[i]; maxCosine = cosine; }
        }
    }
    Float distance = vdist(closest, pLocal);
    if (isNeg) distance *= -1;
    if (s->reverse) normal = vmul(normal, -1);
    cpq q;
    q.point = vadd(closest, s->t);
    q.normal = normal;
    q.sd = distance;
    q.velocity = V(0, 0, 0);
    return q;
}

/* Shape::SphereClosestDistance / SphereClosestPoint, sphere.cpp:47-70 */
static Float sphere_closest_distance(const oshape *s, v3 point) {
    v3 pLocal = vsub(point, s->t);
    return vlen(pLocal) - s->radius;
}

static cpq sphere_closest_point(const oshape *s, v3 point) {
    Float d = sphere_closest_distance(s, point);
    v3 pLocal = vsub(point, s->t);
    v3 N = V(0, 1, 0);
    if (!(is_zero(pLocal.x) && is_zero(pLocal.y) && is_zero(pLocal.z))) N = vdiv(pLocal, vlen(pLocal));
    v3 pN = vmul(N, s->radius);
    if (s->reverse) N = vmul(N, -1);
    cpq q;
    q.point = vadd(pN, s->t);
    q.normal = N;
    q.sd = d;
    q.velocity = V(0, 0, 0);
    return q;
}

static inline Float shape_closest_distance(const oshape *s, v3 p) {   /* shape.cpp:206-232 */
    return s->type == ORC_SHAPE_BOX ? box_closest_distance(s, p) : sphere_closest_distance(s, p);
}
static inline cpq shape_closest_point(const oshape *s, v3 p) {       /* shape.cpp:234-254 */
    return s->type == ORC_SHAPE_BOX ? box_closest_point(s, p) : sphere_closest_point(s, p);
}
static inline int shape_is_inside(const oshape *s, v3 p) {            /* shape.cpp:275-282 */
    return s->reverse == !(shape_closest_distance(s, p) < 0);
}

/* CollisionHandle, collider.cpp:3-44 */
static void collision_handle(const oshape *s, Float radius, Float restitution, v3 *position,
                             v3 *velocity) {
    cpq q = shape_closest_point(s, *position);
    int penetrating = shape_is_inside(s, *position) || absf_(q.sd) < radius;
    if (!penetrating) return;
    v3 targetNormal = q.normal;
    v3 targetPoint = vadd(q.point, vmul(targetNormal, radius));
    v3 colliderVelocity = q.velocity;
    v3 relativeVel = vsub(*velocity, colliderVelocity);
    Float normalDotRel = vdot(targetNormal, relativeVel);
    v3 relativeVelN = vmul(targetNormal, normalDotRel);
    v3 relativeVelT = vsub(relativeVel, relativeVelN);
    if (normalDotRel < 0) {
        v3 deltaRelN = vmul(relativeVelN, (Float)(-1.0 - restitution));
        relativeVelN = vmul(relativeVelN, -restitution);
        if (vlen2(relativeVelT) > 0) {
            Float scale = vlen(deltaRelN) / vlen(relativeVelT);
            Float fScale = 1.0 - s->friction * scale;
            Float frictionScale = max_(0, fScale);
            relativeVelT = vmul(relativeVelT, frictionScale);
        }
        *velocity = vadd(vadd(relativeVelN, relativeVelT), colliderVelocity);
    }
    *position = targetPoint;
}

/* ColliderSet3::ResolveCollision, collider.cpp:238-264 */
static void collider_resolve(const oshape *shapes, int n, Float radius, Float restitution,
                             v3 *position, v3 *velocity) {
    int target = -1;
    Float minDistance = FLT_MAX;
    for (int i = 0; i < n; i++) {
        Float distance = absf_(shape_closest_distance(&shapes[i], *position));
        if (distance < minDistance) { target = i; minDistance = distance; }
    }
    if (target < 0) return;
    collision_handle(&shapes[target], radius, restitution, position, velocity);
}

/* ------------------------------------------------------------------------- */
/* Simulation state                                                            */
/* ------------------------------------------------------------------------- */
struct orc_sim {
    int n;
    /* SphParticleSet3 / ParticleSet3 scalars */
    Float mass, radius, targetDensity, targetSpacing, kernelRadius, relRadius;
    /* SphSolverData3 */
    Float eosExponent, negScale, viscosity, pseudoViscosity, soundSpeed, drag;
    v3 gravity;
    /* PciSphSolver3 */
    Float massOverTargetDensitySquared, deltaDenom;
    Float stepScale;
    ogrid g;
    oshape shapes[ORC_MAX_COLLIDERS];
    int nshapes;
    v3 *pos, *vel, *force, *inter, *tpos, *tvel, *pforce, *smoothed;
    Float *density, *pressure, *dpred, *derr;
    /* double-buffered chains (grid.h:20-156); buffer 0 = head/chainNodes, 1 = aux */
    int active;
    int *head[2], *tail[2], *clen[2], *next[2];
    unsigned *cell_of;
    int32_t *bucket, *bcount, *bfull;
    int higher;
    int frame_index;
    int tol_mode;   /* PredictPressure stores densityErrors (tolerance mode) */
    int clamp_total; /* warm start: negative total pressure scaled instead of the increment */
    /* ContinuousParticleSetBuilder3::MapGrid: positions per cell in chain order */
    v3 *map_pos;
    int *map_start;
};

static v3 *alloc_v3(int n) { return (v3 *)calloc((size_t)(n > 0 ? n : 1), sizeof(v3)); }
static Float *alloc_f(int n) { return (Float *)calloc((size_t)(n > 0 ? n : 1), sizeof(Float)); }

int orc_count(const orc_sim *s) { return s->n; }
int orc_higher_level(const orc_sim *s) { return s->higher; }
void orc_set_higher_level(orc_sim *s, int v) { s->higher = v; }

/* Cell::AddToChain / AddToNextChain on buffer b */
static inline void chain_append(orc_sim *s, int b, unsigned c, int node) {
    if (s->head[b][c] < 0) {
        s->head[b][c] = node;
        s->tail[b][c] = node;
    } else {
        s->next[b][s->tail[b][c]] = node;
        s->tail[b][c] = node;
    }
    s->next[b][node] = -1;
    s->clen[b][c]++;
}

/* DistributeResetCell over all cells + DistributeByParticle, grid.h:324-328, 391-407 */
static void distribute_by_particle(orc_sim *s) {
    for (int b = 0; b < 2; b++)
        for (unsigned c = 0; c < s->g.total; c++) {
            s->head[b][c] = -1; s->tail[b][c] = -1; s->clen[b][c] = 0;
        }
    s->active = 0;
    for (int i = 0; i < s->n; i++) {
        unsigned h = grid_hash(&s->g, s->pos[i]);
        chain_append(s, 0, h, i);
    }
}

orc_sim *orc_create(const orc_params *p, int n, const double *pos, const double *vel) {
    if (n <= 0 || !p || !pos) return NULL;
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    s->n = n;
    s->pos = alloc_v3(n); s->vel = alloc_v3(n); s->force = alloc_v3(n); s->inter = alloc_v3(n);
    s->tpos = alloc_v3(n); s->tvel = alloc_v3(n); s->pforce = alloc_v3(n); s->smoothed = alloc_v3(n);
    s->density = alloc_f(n); s->pressure = alloc_f(n); s->dpred = alloc_f(n); s->derr = alloc_f(n);
    for (int i = 0; i < n; i++) {
        s->pos[i] = V((Float)pos[3 * i], (Float)pos[3 * i + 1], (Float)pos[3 * i + 2]);
        if (vel) s->vel[i] = V((Float)vel[3 * i], (Float)vel[3 * i + 1], (Float)vel[3 * i + 2]);
    }
    /* DefaultSphSolverData3 fields (sph_solver3.cpp:124-151), values from the caller */
    s->eosExponent = (Float)p->eos_exponent;
    s->negScale = (Float)p->negative_pressure_scale;
    s->viscosity = max_(0, (Float)p->viscosity);
    s->pseudoViscosity = (Float)p->pseudo_viscosity;
    s->soundSpeed = (Float)p->sound_speed;
    s->drag = (Float)p->drag_coefficient;
    s->gravity = V((Float)p->gravity[0], (Float)p->gravity[1], (Float)p->gravity[2]);
    s->stepScale = (Float)p->time_step_limit_scale;
    /* PciSphSolver3::Setup / SphSolver3::Setup: density, spacing, radius, each recomputing mass */
    s->targetDensity = 1000.0;
    s->targetSpacing = 0.1;
    s->relRadius = 2.0;
    s->kernelRadius = s->relRadius * s->targetSpacing;
    s->targetDensity = (Float)p->target_density;
    s->radius = max_(0, (Float)p->target_spacing);
    s->targetSpacing = (Float)p->target_spacing;
    s->kernelRadius = s->relRadius * s->targetSpacing;
    s->relRadius = (Float)p->relative_kernel_radius;
    s->kernelRadius = s->relRadius * s->targetSpacing;
    s->mass = max_(0, compute_mass_bcc(s->targetDensity, s->targetSpacing, s->kernelRadius));
    if (p->mass > 0) s->mass = max_(0, (Float)p->mass);
    s->massOverTargetDensitySquared = s->mass / s->targetDensity;
    s->massOverTargetDensitySquared *= s->massOverTargetDensitySquared;
    s->deltaDenom = compute_delta_denom(s->targetSpacing, s->kernelRadius);
    /* colliders */
    s->nshapes = p->n_colliders < ORC_MAX_COLLIDERS ? p->n_colliders : ORC_MAX_COLLIDERS;
    for (int i = 0; i < s->nshapes; i++) {
        const orc_shape *src = &p->colliders[i];
        oshape *d = &s->shapes[i];
        d->type = src->type;
        d->reverse = src->reverse ? 1 : 0;
        d->t = V((Float)src->center[0], (Float)src->center[1], (Float)src->center[2]);
        d->sx = (Float)src->size[0]; d->sy = (Float)src->size[1]; d->sz = (Float)src->size[2];
        d->radius = (Float)src->size[0];
        d->friction = (Float)src->friction;
    }
    /* grid */
    grid_geometry(&s->g, V((Float)p->domain_min[0], (Float)p->domain_min[1], (Float)p->domain_min[2]),
                  V((Float)p->domain_max[0], (Float)p->domain_max[1], (Float)p->domain_max[2]),
                  s->targetSpacing, (Float)p->grid_spacing_scale);
    grid_build_lists(&s->g);
    for (int b = 0; b < 2; b++) {
        s->head[b] = (int *)malloc(sizeof(int) * s->g.total);
        s->tail[b] = (int *)malloc(sizeof(int) * s->g.total);
        s->clen[b] = (int *)malloc(sizeof(int) * s->g.total);
        s->next[b] = (int *)malloc(sizeof(int) * (size_t)n);
    }
    s->cell_of = (unsigned *)malloc(sizeof(unsigned) * (size_t)n);
    s->bucket = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * ORC_BUCKET);
    s->bcount = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    s->bfull = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    distribute_by_particle(s);
    s->higher = 0;
    s->frame_index = 1;
    return s;
}

void orc_destroy(orc_sim *s) {
    if (!s) return;
    free(s->pos); free(s->vel); free(s->force); free(s->inter); free(s->tpos); free(s->tvel);
    free(s->pforce); free(s->smoothed); free(s->density); free(s->pressure); free(s->dpred);
    free(s->derr);
    for (int b = 0; b < 2; b++) { free(s->head[b]); free(s->tail[b]); free(s->clen[b]); free(s->next[b]); }
    free(s->g.nbr); free(s->g.nbr_n); free(s->cell_of); free(s->bucket); free(s->bcount);
    free(s->bfull);
    free(s->map_pos); free(s->map_start);
    free(s);
}

void orc_scalars(const orc_sim *s, double out[8]) {
    out[0] = s->mass; out[1] = s->kernelRadius; out[2] = s->deltaDenom;
    out[3] = s->massOverTargetDensitySquared; out[4] = s->targetSpacing;
    out[5] = s->targetDensity; out[6] = s->radius; out[7] = s->relRadius;
}

void orc_grid_info(const orc_sim *s, int dims[3], double geo[12]) {
    for (int k = 0; k < 3; k++) {
        dims[k] = s->g.dims[k];
        geo[k] = s->g.minp[k]; geo[3 + k] = s->g.len[k];
        geo[6 + k] = vget(s->g.b.mn, k); geo[9 + k] = vget(s->g.b.mx, k);
    }
}

int orc_cell_neighbors(const orc_sim *s, int cell, int out[27]) {
    if (cell < 0 || (unsigned)cell >= s->g.total) return 0;
    memcpy(out, &s->g.nbr[27 * (size_t)cell], sizeof(int) * 27);
    return s->g.nbr_n[cell];
}

void orc_hash_points(const orc_sim *s, int n, const double *pts, uint32_t *cell_ids,
                     uint32_t *ucoords) {
    for (int i = 0; i < n; i++) {
        v3 p = V((Float)pts[3 * i], (Float)pts[3 * i + 1], (Float)pts[3 * i + 2]);
        int u[3];
        grid_hash_u(&s->g, p, u);
        if (ucoords) { ucoords[3 * i] = u[0]; ucoords[3 * i + 1] = u[1]; ucoords[3 * i + 2] = u[2]; }
        if (cell_ids) cell_ids[i] = grid_hash(&s->g, p);
    }
}

/* ------------------------------------------------------------------------- */
/* UpdateGridDistributionCPU, sph_equations3.cpp:388-423                      */
/* ------------------------------------------------------------------------- */
static void k_hash(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    for (int i = b; i < e; i++) s->cell_of[i] = grid_hash(&s->g, s->pos[i]);
}

/* Grid::DistributeToCellOpt, grid.h:449-494 */
static void k_cell_opt(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    int cur = s->active ? 1 : 0, nxt = 1 - cur;
    for (int c = b; c < e; c++) {
        s->head[nxt][c] = -1; s->tail[nxt][c] = -1; s->clen[nxt][c] = 0;
        const int *nb = &s->g.nbr[27 * (size_t)c];
        for (int q = 0; q < s->g.nbr_n[c]; q++) {
            int nc = nb[q];
            int node = s->head[cur][nc];
            for (int j = 0; j < s->clen[cur][nc]; j++) {
                if (s->cell_of[node] == (unsigned)c) chain_append(s, nxt, (unsigned)c, node);
                node = s->next[cur][node];
            }
        }
    }
}

/* Grid::DistributeParticleBucket, grid.h:422-447 */
static void k_bucket(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    int cur = s->active ? 1 : 0;
    for (int i = b; i < e; i++) {
        v3 pi = s->pos[i];
        unsigned cellId = grid_hash(&s->g, pi);
        const int *nb = &s->g.nbr[27 * (size_t)cellId];
        int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
        int count = 0, full = 0;
        for (int q = 0; q < s->g.nbr_n[cellId]; q++) {
            int nc = nb[q];
            int node = s->head[cur][nc];
            for (int j = 0; j < s->clen[cur][nc]; j++) {
                Float distance = vdist(pi, s->pos[node]);
                if (within_std(distance, s->kernelRadius)) {
                    if (count < ORC_BUCKET) bk[count++] = node;
                    full++;
                }
                node = s->next[cur][node];
            }
        }
        s->bcount[i] = count;
        s->bfull[i] = full;
    }
}

void orc_update_grid_distribution(orc_sim *s) {
    parallel_for(s->n, k_hash, s);
    if (s->higher) {
        distribute_by_particle(s);
    } else {
        parallel_for((int)s->g.total, k_cell_opt, s);
        s->active = 1 - s->active;   /* SwapCellList on every cell */
    }
    parallel_for(s->n, k_bucket, s);
    s->frame_index = 1;
}

/* ComputeParticleInteraction, sph_equations3.cpp:63-78 (constant gravity only) */
static void k_interaction(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    for (int i = b; i < e; i++) s->inter[i] = vadd(V(0, 0, 0), s->gravity);
}
void orc_compute_particle_interaction(orc_sim *s) { parallel_for(s->n, k_interaction, s); }

/* ComputePressureValue, sph_equations3.cpp:7-18 */
static inline Float pressure_value(const orc_sim *s, Float di) {
    Float targetDensity = s->targetDensity;
    Float eosScale = targetDensity * s->soundSpeed * s->soundSpeed;
    Float eosExponent = s->eosExponent;
    Float p = eosScale / eosExponent * (pow_((di / targetDensity), eosExponent) - 1.0);
    if (p < 0) p *= s->negScale;
    return p;
}

/* ComputeDensityFor, sph_equations3.cpp:25-58 */
typedef struct { orc_sim *s; int flag; Float fval; } pass_ctx;
static void k_density(void *ctx, int b, int e) {
    pass_ctx *pc = (pass_ctx *)ctx;
    orc_sim *s = pc->s;
    kern k = kern_std(s->kernelRadius);
    for (int i = b; i < e; i++) {
        v3 pi = s->pos[i];
        const int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
        Float sum = 0;
        for (int q = 0; q < s->bcount[i]; q++) sum += std_W(&k, vdist(pi, s->pos[bk[q]]));
        Float di = sum * s->mass;
        if (pc->flag != 0) s->pressure[i] = pressure_value(s, di);
        s->density[i] = di;
    }
}
void orc_compute_density(orc_sim *s, int compute_pressure) {
    pass_ctx pc = {s, compute_pressure, 0};
    parallel_for(s->n, k_density, &pc);
}

/* ComputeNonPressureForceFor, sph_equations3.cpp:80-110 */
static void k_nonpressure(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    kern k = kern_spiky(s->kernelRadius);
    Float mass = s->mass, mass2 = mass * mass;
    for (int i = b; i < e; i++) {
        v3 intr = s->inter[i], pi = s->pos[i], vi = s->vel[i];
        v3 fi = V(0, 0, 0);
        fi = vadd(fi, vmul(intr, mass));
        fi = vadd(fi, vmul(vi, -s->drag));
        const int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
        for (int q = 0; q < s->bcount[i]; q++) {
            int j = bk[q];
            v3 pj = s->pos[j], vj = s->vel[j];
            Float dj = s->density[j];
            Float dist = vdist(pi, pj);
            fi = vadd(fi, vdiv(vmul(vmul(vsub(vj, vi), s->viscosity * mass2), spiky_d2W(&k, dist)), dj));
        }
        s->force[i] = fi;
    }
}
void orc_compute_non_pressure_force(orc_sim *s) { parallel_for(s->n, k_nonpressure, s); }

/* PciSphSolver3::ComputeDelta / ComputeBeta, pcisph_solver3.cpp:182-189 */
double orc_compute_delta(const orc_sim *s, double dt_in) {
    Float dt = (Float)dt_in;
    Float timeStepSquare = dt * dt;
    Float beta = 2.0 * s->massOverTargetDensitySquared * timeStepSquare;
    return absf_(s->deltaDenom) > 0 ? -1 / (beta * s->deltaDenom) : 0;
}

/* TimeIntegrationFor, sph_equations3.cpp:283-339 (extended = 0) */
static inline void integrate_one(orc_sim *s, int i, Float timeStep) {
    v3 vi = s->vel[i], fi = s->force[i], pi = s->pos[i];
    v3 oi = pi;
    v3 aTi = V(0, 0, 0);
    v3 aFi = vdiv(fi, s->mass);
    v3 at = vadd(aTi, aFi);
    vi = vadd(vi, vmul(at, timeStep));
    pi = vadd(pi, vmul(vi, timeStep));
    if (s->nshapes > 0) collider_resolve(s->shapes, s->nshapes, s->radius, (Float)0.6, &pi, &vi);
    if (!inside3(pi, s->g.b)) {
        Float r = s->radius;
        pi = vclamp(pi, vadd(s->g.b.mn, V(r, r, r)), vsub(s->g.b.mx, V(r, r, r)));
    }
    Float dist = vdist(pi, oi);
    Float minLen = min_(s->g.len[0], min_(s->g.len[1], s->g.len[2]));
    if (dist >= minLen * 0.9) __atomic_store_n(&s->higher, 1, __ATOMIC_RELAXED);
    s->pos[i] = pi;
    s->vel[i] = vi;
}

static void k_integrate(void *ctx, int b, int e) {
    pass_ctx *pc = (pass_ctx *)ctx;
    for (int i = b; i < e; i++) integrate_one(pc->s, i, pc->fval);
}
void orc_time_integration(orc_sim *s, double dt) {
    pass_ctx pc = {s, 0, (Float)dt};
    parallel_for(s->n, k_integrate, &pc);
}

/* PredictVelocityAndPositionFor, pcisph_equations3.cpp:3-28 */
static void k_predict(void *ctx, int b, int e) {
    pass_ctx *pc = (pass_ctx *)ctx;
    orc_sim *s = pc->s;
    Float dt = pc->fval;
    for (int i = b; i < e; i++) {
        v3 vi = s->vel[i], pi = s->pos[i], fi = s->force[i];
        if (pc->flag) {
            s->dpred[i] = s->density[i];
            s->pforce[i] = V(0, 0, 0);
            s->derr[i] = 0;
            s->pressure[i] = 0;
        }
        v3 tmpVi = vadd(vi, vmul(vadd(fi, s->pforce[i]), dt / s->mass));
        v3 tmpPi = vadd(pi, vmul(tmpVi, dt));
        if (s->nshapes > 0) collider_resolve(s->shapes, s->nshapes, s->radius, (Float)0, &tmpPi, &tmpVi);
        s->tvel[i] = tmpVi;
        s->tpos[i] = tmpPi;
    }
}

/* PredictPressureFor, pcisph_equations3.cpp:60-90 */
static void k_pred_pressure(void *ctx, int b, int e) {
    pass_ctx *pc = (pass_ctx *)ctx;
    orc_sim *s = pc->s;
    Float delta = pc->fval;
    kern k = kern_std(s->kernelRadius);
    for (int i = b; i < e; i++) {
        v3 pi = s->tpos[i];
        Float ppi = s->pressure[i];
        const int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
        Float weightSum = 0;
        for (int q = 0; q < s->bcount[i]; q++) weightSum += std_W(&k, vdist(pi, s->tpos[bk[q]]));
        Float density = weightSum * s->mass;
        Float densityError = (density - s->targetDensity);
        Float pressure = delta * densityError;
        if (s->clamp_total) {
            if (densityError < 0) densityError *= s->negScale;
            ppi += pressure;
            if (ppi < 0) ppi *= s->negScale;
        } else {
            if (pressure < 0) {
                pressure *= s->negScale;
                densityError *= s->negScale;
            }
            ppi += pressure;
        }
        s->pressure[i] = ppi;
        s->dpred[i] = density;
        if (s->tol_mode) s->derr[i] = densityError;
    }
}

/* PredictPressureForceFor, pcisph_equations3.cpp:114-155 */
static void k_pred_force(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    Float mass = s->mass, mass2 = s->mass * s->mass, sphRadius = s->kernelRadius;
    kern k = kern_spiky(sphRadius);
    for (int i = b; i < e; i++) {
        v3 pi = s->pos[i];
        Float poi = s->pressure[i];
        Float di = s->dpred[i];
        Float di2 = di * di;
        v3 fi = V(0, 0, 0), ti = V(0, 0, 0);
        const int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
        for (int q = 0; q < s->bcount[i]; q++) {
            int j = bk[q];
            if (i == j) continue;
            v3 pj = s->pos[j];
            Float dj = s->dpred[j];
            Float dj2 = dj * dj;
            Float poj = s->pressure[j];
            Float dist = vdist(pi, pj);
            int valid = within_spiky(dist, sphRadius);
            if (valid && !is_zero(dj2)) {
                if (dist > 0 && !is_zero(dist)) {
                    v3 dir = vdiv(vsub(pj, pi), dist);
                    v3 gradij = spiky_gradW(&k, dist, dir);
                    ti = vadd(ti, vmul(gradij, mass2 * (poi / di2 + poj / dj2)));
                }
            }
        }
        (void)mass;
        fi = vsub(fi, ti);
        s->pforce[i] = fi;
    }
}

/* AccumulateForcesFor + TimeIntegrationFor, pcisph_equations3.cpp:179-197 */
static void k_accumulate_integrate(void *ctx, int b, int e) {
    pass_ctx *pc = (pass_ctx *)ctx;
    orc_sim *s = pc->s;
    for (int i = b; i < e; i++) {
        s->force[i] = vadd(s->force[i], s->pforce[i]);
        integrate_one(s, i, pc->fval);
    }
}

/* ComputePseudoViscosityAggregationKernelFor / InterpolationKernelFor, sph_equations3.cpp:341-382 */
static void k_pv_aggregate(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    kern k = kern_spiky(s->kernelRadius);
    Float mass = s->mass;
    for (int i = b; i < e; i++) {
        v3 pi = s->pos[i];
        v3 smoothedVi = V(0, 0, 0);
        Float weightSum = 0;
        const int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
        for (int q = 0; q < s->bcount[i]; q++) {
            int j = bk[q];
            v3 pj = s->pos[j];
            Float dj = s->density[j];
            v3 vj = s->vel[j];
            Float dist = vdist(pi, pj);
            Float wj = mass / dj * spiky_W(&k, dist);
            weightSum += wj;
            smoothedVi = vadd(smoothedVi, vmul(vj, wj));
        }
        if (weightSum > 0) smoothedVi = vmul(smoothedVi, (Float)(1.0 / weightSum));
        s->smoothed[i] = smoothedVi;
    }
}
static void k_pv_interpolate(void *ctx, int b, int e) {
    pass_ctx *pc = (pass_ctx *)ctx;
    orc_sim *s = pc->s;
    Float t = pc->fval * s->pseudoViscosity;
    Float smoothFactor = t < 0.0 ? (Float)0.0 : (t > 1.0 ? (Float)1.0 : t);
    for (int i = b; i < e; i++) {
        v3 vi = s->vel[i];
        vi = vadd(vmul(vi, (Float)(1 - smoothFactor)), vmul(s->smoothed[i], smoothFactor));
        s->vel[i] = vi;
    }
}

/* ComputePseudoViscosityInterpolationCPU, sph_equations3.cpp:469-482 */
void orc_pseudo_viscosity(orc_sim *s, double dt_in) {
    Float timeStep = (Float)dt_in;
    Float scale = s->pseudoViscosity * timeStep;
    if (scale > 0.1) {
        pass_ctx pc = {s, 0, timeStep};
        parallel_for(s->n, k_pv_aggregate, s);
        parallel_for(s->n, k_pv_interpolate, &pc);
    }
}

/* PredictVelocityAndPositionCPU / PredictPressureCPU / PredictPressureForceCPU /
 * AccumulateAndIntegrateCPU, pcisph_equations3.cpp:30-38, 92-98, 157-163, 190-197 */
void orc_predict_velocity_and_position(orc_sim *s, double dt, int is_first) {
    pass_ctx pp = {s, is_first != 0, (Float)dt};
    parallel_for(s->n, k_predict, &pp);
}
void orc_predict_pressure(orc_sim *s, double delta) {
    s->tol_mode = 1;
    pass_ctx pr = {s, 0, (Float)delta};
    parallel_for(s->n, k_pred_pressure, &pr);
}
void orc_predict_pressure_force(orc_sim *s) { parallel_for(s->n, k_pred_force, s); }
void orc_accumulate_and_integrate(orc_sim *s, double dt) {
    pass_ctx pi = {s, 0, (Float)dt};
    parallel_for(s->n, k_accumulate_integrate, &pi);
}

/* ComputePressureForceAndIntegrate, pcisph_equations3.cpp:218-256 */
int orc_pressure_force_and_integrate(orc_sim *s, double dt_in, double max_err_ratio,
                                     double delta_in, int max_it, int mode, double *final_err) {
    Float dt = (Float)dt_in, delta = (Float)delta_in;
    Float maxDensityErrorRatio = (Float)max_err_ratio;
    Float targetDensity = s->targetDensity;
    Float densityErrorRatio = 0;
    int it = 0;
    s->tol_mode = (mode != ORC_PCISPH_AS_SHIPPED);
    const int warm = (mode == ORC_PCISPH_WARM || mode == ORC_PCISPH_WARM_MONOTONE);
    s->clamp_total = (mode == ORC_PCISPH_WARM);
    if (warm) {
        /* warm start: keep each particle's pressure from the previous substep, rho* = rho,
         * and predict the first positions from F + Fp(p) instead of F alone */
        for (int i = 0; i < s->n; i++) { s->dpred[i] = s->density[i]; s->derr[i] = 0; }
        parallel_for(s->n, k_pred_force, s);
    }
    for (int k = 0; k < max_it; k++) {
        pass_ctx pp = {s, k == 0 && !warm, dt};
        parallel_for(s->n, k_predict, &pp);
        pass_ctx pr = {s, 0, delta};
        parallel_for(s->n, k_pred_pressure, &pr);
        parallel_for(s->n, k_pred_force, s);
        it = k + 1;
        Float maxDensityError = 0;
        for (int i = 0; i < s->n; i++) {
            Float y = s->derr[i];
            maxDensityError = (maxDensityError * maxDensityError > y * y) ? maxDensityError : y;
        }
        densityErrorRatio = maxDensityError / targetDensity;
        if (absf_(densityErrorRatio) < maxDensityErrorRatio) break;
    }
    pass_ctx pi = {s, 0, dt};
    parallel_for(s->n, k_accumulate_integrate, &pi);
    orc_pseudo_viscosity(s, dt_in);
    if (final_err) *final_err = densityErrorRatio;
    return it;
}

/* ComputeAllForcesFor (extended = 0), sph_equations3.cpp:184-278 */
static inline void all_forces_one(orc_sim *s, int i, const kern *k) {
    Float mass = s->mass, mass2 = s->mass * s->mass, sphRadius = s->kernelRadius;
    v3 intr = s->inter[i], pi = s->pos[i];
    v3 fi = V(0, 0, 0);
    Float poi = s->pressure[i], di = s->density[i], di2 = di * di;
    v3 vi = s->vel[i];
    fi = vadd(fi, vmul(intr, mass));
    fi = vadd(fi, vmul(vi, -s->drag));
    v3 ti = V(0, 0, 0), ni = V(0, 0, 0);
    const int32_t *bk = &s->bucket[(size_t)i * ORC_BUCKET];
    for (int q = 0; q < s->bcount[i]; q++) {
        int j = bk[q];
        if (i == j) continue;
        v3 pj = s->pos[j];
        Float dj = s->density[j], dj2 = dj * dj;
        v3 vj = s->vel[j];
        Float poj = s->pressure[j];
        Float dist = vdist(pi, pj);
        if (within_spiky(dist, sphRadius)) {
            if (dist > 0 && !is_zero(dist)) {
                v3 dir = vdiv(vsub(pj, pi), dist);
                v3 gradij = spiky_gradW(k, dist, dir);
                ti = vadd(ti, vmul(gradij, mass2 * (poi / di2 + poj / dj2)));
                ni = vadd(ni, vmul(gradij, mass / dj));
            }
            fi = vadd(fi, vdiv(vmul(vmul(vsub(vj, vi), s->viscosity * mass2), spiky_d2W(k, dist)), dj));
        }
    }
    (void)ni;
    fi = vsub(fi, ti);
    s->force[i] = fi;
}

static void k_all_forces(void *ctx, int b, int e) {
    orc_sim *s = (orc_sim *)ctx;
    kern k = kern_spiky(s->kernelRadius);
    for (int i = b; i < e; i++) all_forces_one(s, i, &k);
}

void orc_sph_all_forces(orc_sim *s, double dt, int inplace) {
    if (inplace) {
        /* as shipped: each particle integrates right after its own force sum, so later
         * particles see updated neighbours (single thread, index order). */
        kern k = kern_spiky(s->kernelRadius);
        for (int i = 0; i < s->n; i++) {
            all_forces_one(s, i, &k);
            integrate_one(s, i, (Float)dt);
        }
    } else {
        parallel_for(s->n, k_all_forces, s);
        orc_time_integration(s, dt);
    }
}

/* SphParticleSet3::ComputeNumberOfTimeSteps, particle.h:584-608 */
unsigned orc_number_of_time_steps(const orc_sim *s, double remaining, double scale) {
    Float timeStep = (Float)remaining, timeStepScale = (Float)scale;
    Float mass = s->mass, maxForce = 0.0, refDist = s->kernelRadius;
    for (int i = 0; i < s->n; i++) maxForce = max_(maxForce, vlen(s->force[i]));
    Float timeStepLimit = 0.40 * refDist / s->soundSpeed;
    if (!is_zero(maxForce)) {
        Float timeStepLimitbyForce = 0.25 * sqrt((double)(refDist * mass / maxForce));
        timeStepLimit = min_(timeStepLimitbyForce, timeStepLimit);
    }
    Float targetTimeStep = timeStepScale * timeStepLimit;
    return (unsigned)ceil(timeStep / targetTimeStep);
}

/* AdvanceTimeStep (PCISPH), pcisph_solver3.cpp:42-65 */
int orc_pcisph_substep(orc_sim *s, double dt, double max_err_ratio, int max_it, int mode,
                       double *final_err) {
    orc_update_grid_distribution(s);
    s->higher = 0;   /* ResetHigherLevel */
    orc_compute_particle_interaction(s);
    /* the equation-of-state pressure written here is dead in the corrector (its first
     * prediction zeroes the pressure); the warm start keeps the previous substep's instead */
    orc_compute_density(s, mode != ORC_PCISPH_WARM && mode != ORC_PCISPH_WARM_MONOTONE);
    orc_compute_non_pressure_force(s);
    double delta = orc_compute_delta(s, dt);
    if (mode == ORC_PCISPH_AS_SHIPPED) { max_err_ratio = 0.01; max_it = 5; }
    return orc_pressure_force_and_integrate(s, dt, max_err_ratio, delta, max_it, mode, final_err);
}

/* AdvanceTimeStep (SPH), sph_solver3.cpp:48-67 */
void orc_sph_substep(orc_sim *s, double dt, int inplace) {
    orc_update_grid_distribution(s);
    s->higher = 0;
    orc_compute_particle_interaction(s);
    orc_compute_density(s, 1);
    orc_sph_all_forces(s, dt, inplace);
    orc_pseudo_viscosity(s, dt);
}

/* PciSphSolver3::Advance, pcisph_solver3.cpp:67-89 */
int orc_advance_pcisph(orc_sim *s, double dt, double max_err_ratio, int max_it, int mode,
                       int *total_iters) {
    Float remainingTime = (Float)dt;
    int steps = 0, iters = 0;
    while (remainingTime > ORC_EPSILON) {
        unsigned n = orc_number_of_time_steps(s, remainingTime, s->stepScale);
        Float timeStep = remainingTime / (Float)n;
        iters += orc_pcisph_substep(s, timeStep, max_err_ratio, max_it, mode, NULL);
        remainingTime -= timeStep;
        steps++;
    }
    if (total_iters) *total_iters = iters;
    return steps;
}

/* SphSolver3::Advance, sph_solver3.cpp:69-93 */
int orc_advance_sph(orc_sim *s, double dt, int inplace) {
    Float remainingTime = (Float)dt;
    int steps = 0;
    while (remainingTime > ORC_EPSILON) {
        unsigned n = orc_number_of_time_steps(s, remainingTime, s->stepScale);
        Float timeStep = remainingTime / (Float)n;
        orc_sph_substep(s, timeStep, inplace);
        remainingTime -= timeStep;
        steps++;
    }
    return steps;
}

/* ------------------------------------------------------------------------- */
/* field access                                                                */
/* ------------------------------------------------------------------------- */
static v3 *vec_field(const orc_sim *s, int f) {
    switch (f) {
        case ORC_POSITION: return s->pos;
        case ORC_VELOCITY: return s->vel;
        case ORC_FORCE: return s->force;
        case ORC_INTERACTION: return s->inter;
        case ORC_PRED_POSITION: return s->tpos;
        case ORC_PRED_VELOCITY: return s->tvel;
        case ORC_PRESSURE_FORCE: return s->pforce;
        case ORC_SMOOTHED_VELOCITY: return s->smoothed;
        default: return NULL;
    }
}
static Float *scalar_field(const orc_sim *s, int f) {
    switch (f) {
        case ORC_DENSITY: return s->density;
        case ORC_PRESSURE: return s->pressure;
        case ORC_PRED_DENSITY: return s->dpred;
        case ORC_DENSITY_ERROR: return s->derr;
        default: return NULL;
    }
}

void orc_get_field(const orc_sim *s, int f, double *out) {
    v3 *v = vec_field(s, f);
    if (v) {
        for (int i = 0; i < s->n; i++) { out[3 * i] = v[i].x; out[3 * i + 1] = v[i].y; out[3 * i + 2] = v[i].z; }
        return;
    }
    Float *sc = scalar_field(s, f);
    if (sc) for (int i = 0; i < s->n; i++) out[i] = sc[i];
}

void orc_set_field(orc_sim *s, int f, const double *in) {
    v3 *v = vec_field(s, f);
    if (v) {
        for (int i = 0; i < s->n; i++) v[i] = V((Float)in[3 * i], (Float)in[3 * i + 1], (Float)in[3 * i + 2]);
        return;
    }
    Float *sc = scalar_field(s, f);
    if (sc) for (int i = 0; i < s->n; i++) sc[i] = (Float)in[i];
}

int orc_get_cells(const orc_sim *s, uint32_t *cell_of_particle, uint32_t *cell_counts,
                  uint32_t *chain_concat) {
    int cur = s->active ? 1 : 0;
    if (cell_of_particle)
        for (int i = 0; i < s->n; i++) cell_of_particle[i] = grid_hash(&s->g, s->pos[i]);
    size_t w = 0;
    for (unsigned c = 0; c < s->g.total; c++) {
        if (cell_counts) cell_counts[c] = (uint32_t)s->clen[cur][c];
        if (chain_concat) {
            int node = s->head[cur][c];
            for (int j = 0; j < s->clen[cur][c] && w < (size_t)s->n; j++) {
                chain_concat[w++] = (uint32_t)node;
                node = s->next[cur][node];
            }
        }
    }
    return (int)s->g.total;
}

int orc_get_buckets(const orc_sim *s, int32_t *counts, int32_t *ids) {
    int over = 0;
    for (int i = 0; i < s->n; i++) {
        if (counts) counts[i] = s->bcount[i];
        if (ids) {
            for (int q = 0; q < ORC_BUCKET; q++)
                ids[(size_t)i * ORC_BUCKET + q] = q < s->bcount[i] ? s->bucket[(size_t)i * ORC_BUCKET + q] : -1;
        }
        if (s->bfull[i] > ORC_BUCKET) over++;
    }
    return over;
}

/* ------------------------------------------------------------------------------------ */
/* Particle frames (src/third/serializer.cpp:20-45, 813-923)                             */
/* ------------------------------------------------------------------------------------ */
typedef struct {
    char *buf;
    size_t cap, len;
} frame_out;

static void frame_put(frame_out *o, const char *fmt, ...) {
    char tmp[128];
    va_list ap;
    va_start(ap, fmt);
    int k = vsnprintf(tmp, sizeof(tmp), fmt, ap);
    va_end(ap);
    for (int j = 0; j < k; j++, o->len++)
        if (o->len < o->cap) o->buf[o->len] = tmp[j];
}

size_t orc_frame_text(int n, int flags, const double *pos, const double *vel, const double *rho,
                      double mass, double spacing, char *buf, size_t capacity) {
    frame_out o = {buf, buf ? capacity : 0, 0};
    char fmt[8];
    int k = 0;
    if (flags & 0x01) fmt[k++] = 'p';
    if (flags & 0x02) fmt[k++] = 'v';
    if (flags & 0x04) fmt[k++] = 'd';
    if (flags & 0x20) fmt[k++] = 'm';
    fmt[k] = 0;
    frame_put(&o, "FluidBegin\n");
    frame_put(&o, "\t\"Type\" particles\n");
    frame_put(&o, "\t\"Count\" %d\n", n);
    frame_put(&o, "\t\"Format\" %s\n", fmt);
    frame_put(&o, "\t\"Spacing\" %g\n", (double)(Float)spacing);
    frame_put(&o, "\tDataBegin\n");
    for (int i = 0; i < n; i++) {
        int space = 0;
        frame_put(&o, "\t\t");
        if (flags & 0x01) {
            frame_put(&o, "%g %g %g", (double)(Float)pos[3 * i], (double)(Float)pos[3 * i + 1],
                      (double)(Float)pos[3 * i + 2]);
            space = 1;
        }
        if (flags & 0x02) {
            frame_put(&o, space ? " %g %g %g" : "%g %g %g", (double)(Float)vel[3 * i],
                      (double)(Float)vel[3 * i + 1], (double)(Float)vel[3 * i + 2]);
            space = 1;
        }
        if (flags & 0x04) {
            frame_put(&o, space ? " %g" : "%g", (double)(Float)rho[i]);
            space = 1;
        }
        if (flags & 0x20) frame_put(&o, space ? " %g" : "%g", (double)(Float)mass);
        frame_put(&o, "\n");
    }
    frame_put(&o, "\tDataEnd\n");
    frame_put(&o, "FluidEnd\n");
    return o.len;
}

/* ParseFloat's number reader (src/third/obj_loader.cpp:56-168): decimal mantissa summed in
 * double, exponent applied as ldexp(m * pow(5, e), e); a malformed token leaves 0. */
static double frame_parse_double(const char *s, const char *end) {
    static const double lut[] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
    double mantissa = 0.0;
    int exponent = 0, read = 0;
    char sign = '+', exp_sign = '+';
    const char *c = s;
    if (s >= end) return 0.0;
#define DIGIT(x) ((unsigned)((x) - '0') < 10u)
    if (*c == '+' || *c == '-') {
        sign = *c;
        c++;
    } else if (!DIGIT(*c)) {
        return 0.0;
    }
    while (c != end && DIGIT(*c)) {
        mantissa *= 10;
        mantissa += (int)(*c - '0');
        c++;
        read++;
    }
    if (read == 0) return 0.0;
    if (c == end) goto assemble;
    if (*c == '.') {
        c++;
        read = 1;
        while (c != end && DIGIT(*c)) {
            mantissa += (int)(*c - '0') * (read < 8 ? lut[read] : pow(10.0, -read));
            read++;
            c++;
        }
    } else if (*c != 'e' && *c != 'E') {
        goto assemble;
    }
    if (c == end) goto assemble;
    if (*c == 'e' || *c == 'E') {
        c++;
        if (c != end && (*c == '+' || *c == '-')) {
            exp_sign = *c;
            c++;
        } else if (c == end || !DIGIT(*c)) {   /* the character at the end is a delimiter */
            return 0.0;
        }
        read = 0;
        while (c != end && DIGIT(*c)) {
            exponent *= 10;
            exponent += (int)(*c - '0');
            c++;
            read++;
        }
        exponent *= (exp_sign == '+' ? 1 : -1);
        if (read == 0) return 0.0;
    }
assemble:
#undef DIGIT
    return (sign == '+' ? 1 : -1) * (exponent ? ldexp(mantissa * pow(5.0, exponent), exponent) : mantissa);
}

/* ParseFloat: skip spaces/tabs, the token ends at a space, tab, '\r' or the line's end. */
static Float frame_parse_float(const char **t, const char *line_end) {
    const char *p = *t;
    while (p < line_end && (*p == ' ' || *p == '\t')) p++;
    const char *e = p;
    while (e < line_end && *e != ' ' && *e != '\t' && *e != '\r') e++;
    *t = e;
    return (Float)frame_parse_double(p, e);
}

static void frame_skip_blanks(const char **t, const char *line_end) {
    while (*t < line_end && (**t == ' ' || **t == '\t')) (*t)++;
}

/* GetLine (src/third/obj_loader.cpp:253-268): a line ends at "\n", "\r\n" or "\r". */
static int frame_next_line(const char *text, size_t length, size_t *pos, size_t *a, size_t *b) {
    size_t i = *pos;
    if (i >= length) return 0;
    *a = i;
    while (i < length && text[i] != '\n' && text[i] != '\r') i++;
    *b = i;
    if (i < length) i += (text[i] == '\r' && i + 1 < length && text[i + 1] == '\n') ? 2 : 1;
    *pos = i;
    return 1;
}

/* The line's characters as a C string sees them (up to an embedded NUL). */
static size_t frame_c_end(const char *text, size_t a, size_t b) {
    size_t i = a;
    while (i < b && text[i] != '\0') i++;
    return i;
}

static int frame_flags_from(const char *f, size_t len) {
    int flags = 0;
    for (size_t i = 0; i < len; i++) {
        switch (f[i]) {
            case 'p': case 'P': flags |= 0x01; break;
            case 'v': case 'V': flags |= 0x02; break;
            case 'd': case 'D': flags |= 0x04; break;
            case 'm': case 'M': flags |= 0x20; break;
            case 'b': case 'B': flags |= 0x08; break;
            case 'n': case 'N': flags |= 0x10; break;
            case 'l': case 'L': flags |= 0x40; break;
            case 'o': case 'O': flags |= 0x100; break;
            case 'z': case 'Z': flags |= 0x80; break;
            default: return -1;
        }
    }
    return flags;
}

long orc_frame_parse(const char *text, size_t length, int *flags, int *count, double *pos, double *vel,
                     double *rho, int *boundary, long capacity) {
    size_t at = 0, a, b;
    int in_region = 0, pcount = 0, found = 0;
    const char *fmt = NULL;
    size_t fmt_len = 0;
    /* header: tokens split at spaces, tabs and the line end */
    while (!found && frame_next_line(text, length, &at, &a, &b)) {
        const size_t ce = frame_c_end(text, a, b);
        size_t tok = a;
        for (size_t i = a; i <= b && !found; i++) {
            const int sep = i == b || text[i] == ' ' || text[i] == '\t' || text[i] == '\0';
            if (!sep) continue;
            const size_t tl = i - tok;
            if (tl > 0) {
                const char *t = text + tok;
                if (!in_region) {
                    if (tl == 10 && !memcmp(t, "FluidBegin", 10)) in_region = 1;
                } else if (tl == 7 && !memcmp(t, "\"Count\"", 7)) {
                    /* the value follows the separator; a token ending the line is processed
                       with index 0, so its value is read from the line's second character */
                    const char *v = text + (i < b ? i + 1 : a + 1);
                    while (v < text + ce && (*v == ' ' || *v == '\t')) v++;
                    pcount = (int)frame_parse_float(&v, text + ce);
                } else if (tl == 8 && !memcmp(t, "\"Format\"", 8)) {
                    const char *v = text + (i < b ? i + 1 : a + 1);
                    while (v < text + ce && (*v == ' ' || *v == '\t')) v++;
                    fmt = v;
                    fmt_len = 0;
                    while (v + fmt_len < text + ce && v[fmt_len] != ' ' && v[fmt_len] != '\t') fmt_len++;
                } else if (tl == 9 && !memcmp(t, "DataBegin", 9)) {
                    found = 1;
                } else if (tl == 8 && !memcmp(t, "FluidEnd", 8)) {
                    in_region = 0;
                }
            }
            tok = i + 1;
        }
    }
    if (count) *count = pcount;
    if (fmt && fmt_len > 0) {
        const int f = frame_flags_from(fmt, fmt_len);
        if (f < 0) return -1;
        *flags = f;
    }
    if (!found) return -2;
    const int fl = *flags;
    long size = 0;
    int ended = 0;
    while (frame_next_line(text, length, &at, &a, &b)) {
        const char *end = text + frame_c_end(text, a, b);
        const char *t = text + a;
        if (t == end) continue;
        frame_skip_blanks(&t, end);
        if (t == end || *t == '#') continue;
        {
            int has_end = 0;
            for (const char *q = t; q + 7 <= end && !has_end; q++) has_end = !memcmp(q, "DataEnd", 7);
            if (has_end) {
                ended = 1;
                break;
            }
        }
        Float p3[3] = {0, 0, 0}, v3[3] = {0, 0, 0}, d = 0;
        int bnd = 0;
        if (fl & 0x01) {
            for (int k = 0; k < 3; k++) p3[k] = frame_parse_float(&t, end);
            frame_skip_blanks(&t, end);
        }
        if (fl & 0x02) {
            for (int k = 0; k < 3; k++) v3[k] = frame_parse_float(&t, end);
            frame_skip_blanks(&t, end);
        }
        if (fl & 0x04) {
            d = frame_parse_float(&t, end);
            frame_skip_blanks(&t, end);
        }
        if (fl & 0x20) {
            (void)frame_parse_float(&t, end);
            frame_skip_blanks(&t, end);
        }
        if (fl & 0x08) {
            bnd = (int)frame_parse_float(&t, end);
            frame_skip_blanks(&t, end);
            if ((fl & 0x100) && !bnd) continue;
        }
        if (size < capacity) {
            for (int k = 0; k < 3; k++) {
                if (pos) pos[3 * size + k] = (double)p3[k];
                if (vel) vel[3 * size + k] = (double)v3[k];
            }
            if (rho) rho[size] = (double)d;
            if (boundary) boundary[size] = bnd;
        }
        size++;
    }
    return ended ? size : -2;
}

/* ------------------------------------------------------------------------------------ */
/* Volume emission (src/core/emitter.cpp:8-12, 241-330; bcclattice.cpp:6-36)           */
/* ------------------------------------------------------------------------------------ */
/* rand_float (src/core/geometry.h:1900-1902): a float quotient in both builds */
static Float emit_rand_float(void) { return (Float)((float)rand() / ((float)RAND_MAX + 1.f)); }
/* std::sqrt / std::cos / std::sin of a Float: the float functions in the FP32 build */
#define FSQRT(x) _Generic((x), float: sqrtf, default: sqrt)(x)
#define FCOS(x) _Generic((x), float: cosf, default: cos)(x)
#define FSIN(x) _Generic((x), float: sinf, default: sin)(x)

long orc_emit_volume(const orc_shape *shape, int use_bounds, const double bmin[3], const double bmax[3],
                     double spacing, double jitter, const double vel[3], long max_particles, double *pos,
                     double *vel_out, long capacity) {
    oshape s;
    s.type = shape->type;
    s.reverse = shape->reverse ? 1 : 0;
    s.t = V((Float)shape->center[0], (Float)shape->center[1], (Float)shape->center[2]);
    s.sx = (Float)shape->size[0]; s.sy = (Float)shape->size[1]; s.sz = (Float)shape->size[2];
    s.radius = (Float)shape->size[0];
    s.friction = (Float)shape->friction;
    v3 lo, hi;
    if (use_bounds) {
        for (int k = 0; k < 3; k++) {
            Float a = (Float)bmin[k], b = (Float)bmax[k];
            ((Float *)&lo)[k] = a < b ? a : b;
            ((Float *)&hi)[k] = a > b ? a : b;
        }
    } else {
        /* ObjectToWorld of the object bounds (box.cpp:59-64, sphere.cpp:43-45): a translation */
        Float hx, hy, hz;
        if (s.type == ORC_SHAPE_BOX) {
            hx = s.sx / 2.0; hy = s.sy / 2.0; hz = s.sz / 2.0;
        } else {
            hx = hy = hz = s.radius;
        }
        lo = V(-hx + s.t.x, -hy + s.t.y, -hz + s.t.z);
        hi = V(hx + s.t.x, hy + s.t.y, hz + s.t.z);
    }
    const Float sp = (Float)spacing;
    const Float half = sp / 2;
    const Float width = hi.x - lo.x, height = hi.y - lo.y, depth = hi.z - lo.z;
    const Float max_jitter = (Float)(0.5 * (double)(Float)jitter * (double)sp);
    const v3 v0 = V((Float)0 + (Float)vel[0], (Float)0 + (Float)vel[1], (Float)0 + (Float)vel[2]);
    long emitted = 0;
    int has_off = 0, stop = 0;
    for (int k = 0; (Float)k * half <= depth && !stop; k++) {
        const Float pz = (Float)k * half + lo.z;
        const Float off = has_off ? half : 0;
        for (int j = 0; (Float)j * sp + off <= height && !stop; j++) {
            const Float py = (Float)j * sp + off + lo.y;
            for (int i = 0; (Float)i * sp + off <= width && !stop; i++) {
                const Float px = (Float)i * sp + off + lo.x;
                /* vec2f u(rand_float(), rand_float()): the second call lands in u[0] */
                const Float u1 = emit_rand_float();
                const Float u0 = emit_rand_float();
                const Float usqrt = 2 * FSQRT(u1 * (1 - u1));
                const Float utheta = (Float)(2 * 3.14159265358979323846 * (double)u0);
                const v3 dir = V(FCOS(utheta) * usqrt, FSIN(utheta) * usqrt, 1 - 2 * u1);
                const v3 target = vadd(V(px, py, pz), vmul(dir, max_jitter));
                const Float d = shape_closest_distance(&s, target);
                const Float sd = shape_is_inside(&s, target) ? -absf_(d) : absf_(d);
                if (sd <= 0) {
                    if (emitted < max_particles) {
                        if (emitted < capacity) {
                            pos[3 * emitted] = target.x; pos[3 * emitted + 1] = target.y; pos[3 * emitted + 2] = target.z;
                            vel_out[3 * emitted] = v0.x; vel_out[3 * emitted + 1] = v0.y;
                            vel_out[3 * emitted + 2] = v0.z;
                        }
                        emitted++;
                    } else {
                        stop = 1;
                    }
                }
            }
        }
        has_off = !has_off;
    }
    return emitted;
}

void orc_shape_distance(const orc_shape *shape, int n, const double *pts, double *distance, int *inside) {
    oshape s;
    s.type = shape->type;
    s.reverse = shape->reverse ? 1 : 0;
    s.t = V((Float)shape->center[0], (Float)shape->center[1], (Float)shape->center[2]);
    s.sx = (Float)shape->size[0]; s.sy = (Float)shape->size[1]; s.sz = (Float)shape->size[2];
    s.radius = (Float)shape->size[0];
    s.friction = 0;
    for (int i = 0; i < n; i++) {
        const v3 p = V((Float)pts[3 * i], (Float)pts[3 * i + 1], (Float)pts[3 * i + 2]);
        distance[i] = shape_closest_distance(&s, p);
        inside[i] = shape_is_inside(&s, p);
    }
}

/* ------------------------------------------------------------------------------------ */
/* Continuous emission (src/core/grid.h:1289-1402)                                       */
/* ------------------------------------------------------------------------------------ */
void orc_map_grid(orc_sim *s) {
    const int cur = s->active ? 1 : 0;
    free(s->map_pos);
    free(s->map_start);
    s->map_pos = alloc_v3(s->n);
    s->map_start = (int *)calloc((size_t)s->g.total + 1, sizeof(int));
    int w = 0;
    for (unsigned c = 0; c < s->g.total; c++) {
        s->map_start[c] = w;
        int node = s->head[cur][c];
        for (int j = 0; j < s->clen[cur][c] && w < s->n; j++) {
            s->map_pos[w++] = s->pos[node];
            node = s->next[cur][node];
        }
    }
    s->map_start[s->g.total] = w;
}

long orc_map_grid_emit(const orc_sim *s, double d, double *out, long capacity) {
    if (!s->map_pos) return -1;
    const int cur = s->active ? 1 : 0;
    const Float dd = (Float)d;
    long count = 0;
    for (unsigned c = 0; c < s->g.total; c++) {
        const int mapped = s->map_start[c + 1] - s->map_start[c];
        if (mapped == 0) continue;
        const int held = s->clen[cur][c];
        if (held >= ORC_BUCKET) continue;
        const int to_insert = ORC_BUCKET - held < mapped ? ORC_BUCKET - held : mapped;
        for (int i = 0; i < to_insert; i++) {
            const v3 pi = s->map_pos[s->map_start[c] + i];
            int ok = 1;
            int node = s->head[cur][c];
            for (int j = 0; j < held && ok; j++) {
                if (vlen(vsub(s->pos[node], pi)) < dd) ok = 0;
                node = s->next[cur][node];
            }
            if (!ok) continue;
            if (count < capacity) {
                out[3 * count] = pi.x;
                out[3 * count + 1] = pi.y;
                out[3 * count + 2] = pi.z;
            }
            count++;
        }
    }
    return count;
}

/* ------------------------------------------------------------------------------------ */
/* LNM boundary classification, fast variant (src/boundaries/lnm.h:24-33, 96-139, 245-275) */
/* ------------------------------------------------------------------------------------ */
void orc_lnm(const orc_sim *s, double h, int unbounded, int *levels) {
    const int cur = s->active ? 1 : 0;
    const unsigned total = s->g.total;
    int *level = (int *)malloc(sizeof(int) * (total ? total : 1));
    for (unsigned c = 0; c < total; c++) level[c] = -1;   /* UpdateQueryState */
    /* LNMComputeDelta: (min cell length / h)^3 as a float power, truncated to int */
    Float minlen = s->g.len[0] < s->g.len[1] ? s->g.len[0] : s->g.len[1];
    minlen = minlen < s->g.len[2] ? minlen : s->g.len[2];
    const float pd = powf((float)minlen / (float)h, 3.0f);
    const int delta = (!unbounded && pd > 0) ? (int)pd : 2147483647;
    /* L1: a cell with particles on the grid's border or next to an empty cell */
    for (unsigned c = 0; c < total; c++) {
        if (s->clen[cur][c] < 1) continue;
        const int cnt = s->g.nbr_n[c];
        if (cnt != 27) {
            level[c] = 1;
            continue;
        }
        for (int k = 0; k < cnt; k++)
            if (s->clen[cur][s->g.nbr[27 * (size_t)c + k]] == 0) {
                level[c] = 1;
                break;
            }
    }
    /* L2: a cell with particles next to an L1 cell holding at most delta particles */
    for (unsigned c = 0; c < total; c++) {
        if (s->clen[cur][c] < 1 || level[c] == 1) continue;
        for (int k = 0; k < s->g.nbr_n[c]; k++) {
            const int nb = s->g.nbr[27 * (size_t)c + k];
            if (level[nb] == 1 && s->clen[cur][nb] <= delta) {
                level[c] = 2;
                break;
            }
        }
    }
    for (int i = 0; i < s->n; i++) levels[i] = 0;
    for (unsigned c = 0; c < total; c++) {
        if (level[c] != 1 && level[c] != 2) continue;
        int node = s->head[cur][c];
        for (int j = 0; j < s->clen[cur][c]; j++) {
            levels[node] = level[c];
            node = s->next[cur][node];
        }
    }
    free(level);
}

/* LNMComputeDelta (lnm.h:24-33): (min cell length / h)^3 as a float power */
static float lnm_pre_delta(const orc_sim *s, double h) {
    Float minlen = s->g.len[0] < s->g.len[1] ? s->g.len[0] : s->g.len[1];
    minlen = minlen < s->g.len[2] ? minlen : s->g.len[2];
    return powf((float)minlen / (float)h, 3.0f);
}

/* the levels of cells at or below 2 written to their chains' particles */
static void lnm_set_chain(const orc_sim *s, unsigned c, int L, int *levels) {
    const int cur = s->active ? 1 : 0;
    int node = s->head[cur][c];
    for (int j = 0; j < s->clen[cur][c]; j++) {
        levels[node] = L;
        node = s->next[cur][node];
    }
}

static void cell_coords(const ogrid *g, unsigned c, int u[3]) {
    u[0] = (int)(c % (unsigned)g->dims[0]);
    u[1] = (int)((c / (unsigned)g->dims[0]) % (unsigned)g->dims[1]);
    u[2] = (int)(c / ((unsigned)g->dims[0] * (unsigned)g->dims[1]));
}

/* LNMBoundaryAreCoords1x1 (lnm.h:144-160): distinct cells at most one step apart per axis */
static int lnm_1x1(const int a[3], const int b[3]) {
    int eval = 0;
    for (int q = 0; q < 3; q++) {
        int ef = abs(a[q] - b[q]);
        if (ef < 2) eval += ef;
        else return 0;
    }
    return eval > 0 && eval <= 3;
}

/* LNMBoundarySingle (lnm.h:167-256): per cell with particles, L1 on the border; otherwise the
 * 5x5x5 neighbourhood in the reference's order (y, x, z) stops at the first empty adjacent
 * cell (L1) or the first adjacent cell with at most delta particles on the border (L2);
 * without a stop, L2 when an adjacent cell with at most delta particles touches one of the
 * empty cells met. */
void orc_lnm_single(const orc_sim *s, double h, int unbounded, int *levels) {
    const int cur = s->active ? 1 : 0;
    const ogrid *g = &s->g;
    const float pd = lnm_pre_delta(s, h);
    const int pre = unbounded ? -1 : (int)pd;   /* the kernel's int parameter */
    const int delta = pre > 0 ? pre : 2147483647;
    for (int i = 0; i < s->n; i++) levels[i] = 0;
    for (unsigned c = 0; c < g->total; c++) {
        if (s->clen[cur][c] == 0) continue;
        if (g->nbr_n[c] != 27) {
            lnm_set_chain(s, c, 1, levels);
            continue;
        }
        int u[3], src[125][3], cand[125][3], nsrc = 0, ncand = 0, is_l1 = 0, is_l2 = 0, stop = 0;
        cell_coords(g, c, u);
        for (int j = u[1] - 2; j <= u[1] + 2 && !stop; j++) {
            if (j < 0 || j >= g->dims[1]) continue;
            for (int i = u[0] - 2; i <= u[0] + 2 && !stop; i++) {
                if (i < 0 || i >= g->dims[0]) continue;
                for (int k = u[2] - 2; k <= u[2] + 2 && !stop; k++) {
                    if (k < 0 || k >= g->dims[2]) continue;
                    const int f[3] = {i, j, k};
                    const unsigned fid = (unsigned)i + (unsigned)j * g->dims[0] + (unsigned)k * g->dims[0] * g->dims[1];
                    if (fid == c) continue;
                    const int n = s->clen[cur][fid];
                    const int adj = lnm_1x1(f, u);
                    if (n == 0) {
                        if (adj) {
                            is_l1 = 1;
                            stop = 1;
                        } else {
                            memcpy(src[nsrc++], f, sizeof f);
                        }
                    } else if (adj && n <= delta) {
                        if (g->nbr_n[fid] != 27) {
                            is_l2 = 1;
                            nsrc = ncand = 0;
                            stop = 1;
                        } else if (!is_l2) {
                            memcpy(cand[ncand++], f, sizeof f);
                        }
                    }
                }
            }
        }
        if (is_l1) {
            lnm_set_chain(s, c, 1, levels);
        } else if (nsrc > 0 && ncand > 0) {
            for (int a = 0; a < nsrc && !is_l2; a++)
                for (int b = 0; b < ncand && !is_l2; b++) is_l2 = lnm_1x1(src[a], cand[b]);
        }
        if (is_l2) lnm_set_chain(s, c, 2, levels);
    }
}

/* LNMBoundaryExtended (lnm.h:291-462): voxel levels by LNMComputeOnce sweeps (0: empty,
 * 1: border or next to an empty cell, k: next to a level k-1 cell) for levels 0..max_level
 * (or until a sweep changes nothing when max_level < 0); particle attributes from the cell
 * of their hashed position; then the LK filter (a non-L1 cell next to an L1 cell holding at
 * most delta particles: 2) and unfiltered level-2 cells promoted to 3. */
void orc_lnm_extended(const orc_sim *s, double h, int max_level, int unbounded, int *levels) {
    const int cur = s->active ? 1 : 0;
    const ogrid *g = &s->g;
    int *level = (int *)malloc(sizeof(int) * (g->total ? g->total : 1));
    for (unsigned c = 0; c < g->total; c++) level[c] = -1;
    int L = 0;
    for (;;) {
        int changed = 0;
        for (unsigned c = 0; c < g->total; c++) {
            if (level[c] > -1) continue;
            if (s->clen[cur][c] == 0) {
                level[c] = 0;
                changed = 1;
            } else if (g->nbr_n[c] != 27) {
                level[c] = 1;
                changed = 1;
            } else if (L > 0) {
                for (int q = 0; q < g->nbr_n[c]; q++) {
                    const int nb = g->nbr[27 * (size_t)c + q];
                    if ((unsigned)nb != c && level[nb] == L - 1) {
                        level[c] = L;
                        changed = 1;
                        break;
                    }
                }
            }
        }
        int done = !changed;
        if (max_level > -1) done = L >= max_level;
        if (done) break;
        L++;
    }
    for (int i = 0; i < s->n; i++) {
        const int lv = level[grid_hash(g, s->pos[i])];
        levels[i] = lv > 0 ? lv : 0;
    }
    const float pd = unbounded ? -1.f : lnm_pre_delta(s, h);
    const int delta = pd > 0 ? (int)pd : 2147483647;
    for (unsigned c = 0; c < g->total; c++) {
        if (s->clen[cur][c] > 0 && level[c] != 1) {
            for (int q = 0; q < g->nbr_n[c]; q++) {
                const int nb = g->nbr[27 * (size_t)c + q];
                if (level[nb] == 1 && s->clen[cur][nb] <= delta) {
                    level[c] = -2;
                    lnm_set_chain(s, c, 2, levels);
                    break;
                }
            }
        } else if (level[c] == 1) {
            lnm_set_chain(s, c, 1, levels);
        }
    }
    for (unsigned c = 0; c < g->total; c++)
        if (s->clen[cur][c] > 0 && level[c] == 2) lnm_set_chain(s, c, 3, levels);
    free(level);
}

/* XiaoweiParticleIsBoundary (xiaowei.h:21-78): density below 0.7 of water's, or the
 * std-kernel (radius 6h) weighted mean of the 27 cells' positions farther than 0.15 * 6h */
static int xiaowei_is_boundary(const orc_sim *s, Float h, int id) {
    const int cur = s->active ? 1 : 0;
    const Float rhot = 0.7 * 1000.0;
    const Float rho = 6.0 * h;
    if (s->density[id] < rhot) return 1;
    const v3 pi = s->pos[id];
    const unsigned c = grid_hash(&s->g, pi);
    const kern k = kern_std(rho);
    Float wsum = 0;
    v3 sum = V(0, 0, 0);
    for (int q = 0; q < s->g.nbr_n[c]; q++) {
        const int nb = s->g.nbr[27 * (size_t)c + q];
        int node = s->head[cur][nb];
        for (int j = 0; j < s->clen[cur][nb]; j++) {
            const v3 pj = s->pos[node];
            const Float w = std_W(&k, vlen(vsub(pi, pj)));
            sum = vadd(sum, vmul(pj, w));
            wsum += w;
            node = s->next[cur][node];
        }
    }
    const Float inv = (Float)1 / wsum;
    sum = V(sum.x * inv, sum.y * inv, sum.z * inv);
    const Float asym = vlen(vsub(pi, sum));
    return asym > 0.15 * rho ? 1 : 0;
}

/* DiltsSpokeTakeUniformPoint's angles (dilts.h:70-97) with the C library's float sine and
 * cosine: tab[0..64] sin u, [65..129] cos u, [130..194] sin v, [195..259] cos v */
static void dilts_table(Float *tab) {
    const Float samples = (Float)64;
    for (int i = 0; i <= 64; i++) {
        const Float u = i * ORC_PI / samples;
        const Float v = i * 6.283185307179586 / samples;
        tab[i] = FSIN(u);
        tab[65 + i] = FCOS(u);
        tab[130 + i] = FSIN(v);
        tab[195 + i] = FCOS(v);
    }
}

/* DiltsSpokeParticleIsBoundary (dilts.h:110-153): a spoke point of the sphere of radius
 * 0.75 * spacing around the particle outside every overlapping neighbour's sphere */
static int dilts_is_boundary(const orc_sim *s, int id, const Float *tab) {
    const int cur = s->active ? 1 : 0;
    const v3 pi = s->pos[id];
    const unsigned c = grid_hash(&s->g, pi);
    const Float rad = s->radius * 0.75;
    v3 cand[1024];
    int n = 0;
    for (int q = 0; q < s->g.nbr_n[c]; q++) {
        const int nb = s->g.nbr[27 * (size_t)c + q];
        int node = s->head[cur][nb];
        for (int j = 0; j < s->clen[cur][nb]; j++) {
            if (node != id) {
                const v3 pj = s->pos[node];
                const Float d = vlen(vsub(pi, pj));
                if (!(d > (rad + rad) - ORC_EPSILON) && n < 1024) cand[n++] = pj;
            }
            node = s->next[cur][node];
        }
    }
    for (int i = 0; i <= 64; i++)
        for (int j = 0; j <= 64; j++) {
            const Float su = tab[i], cu = tab[65 + i], sv = tab[130 + j], cv = tab[195 + j];
            const v3 dir = V(su * cv, su * sv, cu);
            const v3 pt = vadd(vmul(dir, rad), pi);
            int inside = 0;
            for (int q = 0; q < n && !inside; q++)
                if (vlen(vsub(cand[q], pt)) <= rad) inside = 1;
            if (!inside) return 1;
        }
    return 0;
}

/* The surface app's field (apps/surface.cpp:276-470, ParticlesToSDF_Surface with
 * ZhuBridsonSDF (method 0) or SphSDF (1)) over the sim's domain grid and densities.  The
 * field's grid: cells of 2 mc_spacing (by_res = 0) or res[k] nodes at the largest extent /
 * (res - 1); origin the domain's min corner plus half a cell.  Returns the node count
 * (values up to cap stored, x fastest). */
long orc_particle_sdf(const orc_sim *s, int method, double kernel, double mc_spacing, int by_res, const int *res,
                      int nodes[3], double origin[3], double *spacing, float *values, long cap) {
    const int cur = s->active ? 1 : 0;
    const ogrid *g = &s->g;
    const v3 mn = g->b.mn, mx = g->b.mx;
    Float ds;
    int cells[3];
    if (!by_res) {
        ds = (Float)mc_spacing;
        ds *= (Float)2.0;
        for (int k = 0; k < 3; k++) {
            const Float ext = vget(mx, k) - vget(mn, k);
            cells[k] = (int)ceil(ext / ds);
        }
    } else {
        Float dk[3];
        for (int k = 0; k < 3; k++) {
            cells[k] = res[k] - 1;
            dk[k] = (vget(mx, k) - vget(mn, k)) / (Float)cells[k];
        }
        const Float m12 = dk[1] < dk[2] ? dk[2] : dk[1];
        ds = dk[0] < m12 ? m12 : dk[0];
    }
    const Float half = ds * (Float)0.5;
    const v3 org = V(mn.x + half, mn.y + half, mn.z + half);
    for (int k = 0; k < 3; k++) {
        nodes[k] = cells[k] + 1;
        origin[k] = vget(org, k);
    }
    *spacing = ds;
    const long total = (long)nodes[0] * nodes[1] * nodes[2];
    const Float inf = vlen(vsub(mx, mn));
    const Float R = (Float)kernel;
    const kern kr = kern_std(R);
    for (long q = 0; q < total && q < cap; q++) {
        const unsigned ux = (unsigned)(q % nodes[0]), uy = (unsigned)((q / nodes[0]) % nodes[1]);
        const unsigned uz = (unsigned)(q / ((long)nodes[0] * nodes[1]));
        const v3 p = V(org.x + ds * (Float)ux, org.y + ds * (Float)uy, org.z + ds * (Float)uz);
        if (!inside3(p, g->b)) {
            values[q] = (float)inf;
            continue;
        }
        const unsigned c = grid_hash(g, p);
        Float wsum = 0;
        v3 avg = V(0, 0, 0);
        for (int k = 0; k < g->nbr_n[c]; k++) {
            const int nb = g->nbr[27 * (size_t)c + k];
            int node = s->head[cur][nb];
            for (int j = 0; j < s->clen[cur][nb]; j++) {
                const v3 xi = s->pos[node];
                const Float d = vlen(vsub(p, xi));
                if (method == 0) {
                    if (d < R) {
                        const Float t = d / R;
                        const double cube = (1.0 - t * t) * (1.0 - t * t) * (1.0 - t * t);
                        const Float cf = (Float)cube;
                        const Float w = (Float)0 < cf ? cf : (Float)0;
                        wsum += w;
                        avg = vadd(avg, vmul(xi, w));
                    }
                } else {
                    wsum += (s->mass / s->density[node]) * std_W(&kr, d);
                }
                node = s->next[cur][node];
            }
        }
        Float v;
        if (method != 0) {
            v = (Float)0.5 - wsum;
        } else if (wsum > 0) {
            const Float inv = 1.0 / wsum;
            avg = V(avg.x * inv, avg.y * inv, avg.z * inv);
            v = vlen(vsub(p, avg)) - R * (Float)0.25;
        } else {
            v = inf;
        }
        values[q] = (float)v;
    }
    return total;
}

void orc_xiaowei(const orc_sim *s, double h, int *flags) {
    for (int i = 0; i < s->n; i++) flags[i] = xiaowei_is_boundary(s, (Float)h, i);
}

void orc_dilts(const orc_sim *s, int *flags) {
    Float tab[260];
    dilts_table(tab);
    for (int i = 0; i < s->n; i++) flags[i] = dilts_is_boundary(s, i, tab);
}

/* LNMBoundary with a geometric L2 filter (lnm.h:57-112, 258-289): L1 as the fast variant;
 * the particles of L2 cells are queued and marked 2 only when the Xiaowei (1) or Dilts
 * spoke (2) test finds them on the boundary.  stats: queued, accepted. */
void orc_lnm_geometric(const orc_sim *s, double h, int algorithm, int unbounded, int *levels, int *stats) {
    const int cur = s->active ? 1 : 0;
    const ogrid *g = &s->g;
    int *level = (int *)malloc(sizeof(int) * (g->total ? g->total : 1));
    Float tab[260];
    dilts_table(tab);
    for (unsigned c = 0; c < g->total; c++) level[c] = -1;
    for (int i = 0; i < s->n; i++) levels[i] = 0;
    const float pd = unbounded ? -1.f : lnm_pre_delta(s, h);
    const int delta = pd > 0 ? (int)pd : 2147483647;
    for (unsigned c = 0; c < g->total; c++) {
        if (s->clen[cur][c] < 1) continue;
        int l1 = g->nbr_n[c] != 27;
        for (int k = 0; k < g->nbr_n[c] && !l1; k++)
            if (s->clen[cur][g->nbr[27 * (size_t)c + k]] == 0) l1 = 1;
        if (l1) {
            level[c] = 1;
            lnm_set_chain(s, c, 1, levels);
        }
    }
    stats[0] = stats[1] = 0;
    for (unsigned c = 0; c < g->total; c++) {
        if (s->clen[cur][c] < 1 || level[c] == 1) continue;
        for (int k = 0; k < g->nbr_n[c]; k++) {
            const int nb = g->nbr[27 * (size_t)c + k];
            if (level[nb] == 1 && s->clen[cur][nb] <= delta) {
                level[c] = 2;
                int node = s->head[cur][c];
                for (int j = 0; j < s->clen[cur][c]; j++) {
                    stats[0]++;
                    const int b = algorithm == 1 ? xiaowei_is_boundary(s, (Float)h, node)
                                                 : dilts_is_boundary(s, node, tab);
                    if (b > 0) {
                        levels[node] = 2;
                        stats[1]++;
                    }
                    node = s->next[cur][node];
                }
                break;
            }
        }
    }
    free(level);
}
