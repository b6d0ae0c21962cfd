// api_post.cu -- the C ABI of colliders with signed-distance fields, boundary
// classification (LNM and the tests it uses), the surface app's particle field and
// marching cubes.
#include "api_internal.h"

// ----------------------------------------------------------------------------
// colliders with signed-distance fields (FieldGrid3f; GenerateShapeSDF)
// ----------------------------------------------------------------------------
// Attaches device node values (owned by the solver from here on) to collider `index`.
bbg_status bbg_api::attach_field(bbg_solver s, int index, const bbg_sdf_grid &g, float *values) {
    int slot = s->P.shapes[index].sdf;
    if (slot < 0) {
        if (s->nsdf >= kMaxSdf) {
            cudaFree(values);
            return fail(BBG_ERR_CAPACITY, "at most %d colliders can have fields", kMaxSdf);
        }
        slot = s->nsdf++;
    } else if (s->sdf_values[slot]) {
        cudaFree(s->sdf_values[slot]);
    }
    s->sdf_values[slot] = values;
    s->sdf_grid[slot] = g;
    SdfDev &d = s->P.sdf[slot];
    d.v = values;
    d.nx = g.nodes[0];
    d.ny = g.nodes[1];
    d.nz = g.nodes[2];
    for (int k = 0; k < 3; k++) {
        d.org[k] = (float)g.origin[k];
        d.sp[k] = (float)g.spacing[k];
        d.inv2[k] = (float)(1.0 / (2.0 * (double)d.sp[k]));   // Gradient's Float inv
        d.lo[k] = (float)g.bounds_min[k];
        d.hi[k] = (float)g.bounds_max[k];
    }
    d.bounded = g.bounded ? 1 : 0;
    s->P.shapes[index].sdf = slot;
    s->P.has_sdf = 1;
    s->epoch++;   // captured launches hold the collider parameters
    return BBG_OK;
}

namespace {

// GenerateShapeSDF's grid over bounds [lo, hi] (shape.cpp:479-502): widened by margin x
// extent, ceil(width / dx) cells across, cubic cells, in the reference's float operations.
bbg_status field_grid_for(const float lo_in[3], const float hi_in[3], double dx, double margin, bbg_sdf_grid *g) {
    const float mg = (float)margin;
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        const float scale = hi_in[k] - lo_in[k];
        lo[k] = lo_in[k] - scale * mg;
        hi[k] = hi_in[k] + scale * mg;
    }
    const float width = hi[0] - lo[0], height = hi[1] - lo[1], depth = hi[2] - lo[2];
    const int res = (int)std::ceil(width / (float)dx);
    if (!(width > 0) || res < 1 || res > 4096) return fail(BBG_ERR_INVALID_ARGUMENT, "a field of %d cells across", res);
    const float cell = width / (float)res;
    const int res_y = (int)std::ceil((float)res * height / width);
    const int res_z = (int)std::ceil((float)res * depth / width);
    if (res_y < 0 || res_z < 0 || res_y > 4096 || res_z > 4096)
        return fail(BBG_ERR_INVALID_ARGUMENT, "a field of %d x %d x %d cells", res, res_y, res_z);
    memset(g, 0, sizeof(*g));
    g->nodes[0] = res + 1;
    g->nodes[1] = res_y + 1;
    g->nodes[2] = res_z + 1;
    for (int k = 0; k < 3; k++) {
        g->origin[k] = lo[k];
        g->spacing[k] = cell;
    }
    return BBG_OK;
}

SdfDev field_dev(const bbg_sdf_grid &g, float *values) {
    SdfDev d;
    memset(&d, 0, sizeof(d));
    d.v = values;
    d.nx = g.nodes[0];
    d.ny = g.nodes[1];
    d.nz = g.nodes[2];
    for (int k = 0; k < 3; k++) {
        d.org[k] = (float)g.origin[k];
        d.sp[k] = (float)g.spacing[k];
    }
    return d;
}

bbg_status check_field_target(bbg_solver s, int index) {
    if (bbg_status r = check_solver(s)) return r;
    if (s->nscenes > 0) return fail(BBG_ERR_STATE, "fields are not supported on a batch of scenes");
    if (index < 0 || index >= s->P.nshapes) return fail(BBG_ERR_INVALID_ARGUMENT, "no collider %d", index);
    return BBG_OK;
}

}  // namespace

bbg_status bbg_collider_set_sdf(bbg_solver s, int index, const bbg_sdf_grid *grid, const float *values) {
    if (bbg_status r = check_field_target(s, index)) return r;
    if (!grid || !values) return fail(BBG_ERR_INVALID_ARGUMENT, "null grid or values");
    size_t total = 1;
    for (int k = 0; k < 3; k++) {
        if (grid->nodes[k] < 1 || !(grid->spacing[k] > 0) || !std::isfinite(grid->origin[k]))
            return fail(BBG_ERR_INVALID_ARGUMENT, "a field needs >= 1 node, spacing > 0 and a finite origin per axis");
        total *= (size_t)grid->nodes[k];
    }
    if (total >= 0xffffffffull) return fail(BBG_ERR_CAPACITY, "the field has %zu nodes", total);
    float *d = nullptr;
    CK(cudaMalloc((void **)&d, sizeof(float) * total));
    cudaError_t e = cudaMemcpy(d, values, sizeof(float) * total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return fail(BBG_ERR_CUDA, "field upload: %s", cudaGetErrorString(e));
    }
    return attach_field(s, index, *grid, d);
}

bbg_status bbg_collider_generate_sdf(bbg_solver s, int index, double dx, double margin) {
    if (bbg_status r = check_field_target(s, index)) return r;
    const ShapeDev &sh = s->P.shapes[index];
    if (sh.type != BBG_SHAPE_BOX && sh.type != BBG_SHAPE_SPHERE)
        return fail(BBG_ERR_INVALID_ARGUMENT, "collider %d is not a box or a sphere", index);
    if (!(dx > 0) || !(margin >= 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "need dx > 0 and margin >= 0");
    // GetBounds of the translated object box
    const float h[3] = {sh.type == BBG_SHAPE_BOX ? sh.hx : sh.radius, sh.type == BBG_SHAPE_BOX ? sh.hy : sh.radius,
                        sh.type == BBG_SHAPE_BOX ? sh.hz : sh.radius};
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = -h[k] + sh.t[k];
        hi[k] = h[k] + sh.t[k];
    }
    bbg_sdf_grid g;
    if (bbg_status r = field_grid_for(lo, hi, dx, margin, &g)) return r;
    const size_t total = (size_t)g.nodes[0] * g.nodes[1] * g.nodes[2];
    float *d = nullptr;
    CK(cudaMalloc((void **)&d, sizeof(float) * total));
    const SdfDev gd = field_dev(g, d);
    launch_sdf_generate(sh, gd, float_above(1e-8), float_above(1e-6), d, s->stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        cudaFree(d);
        return fail(BBG_ERR_CUDA, "field generation: %s", cudaGetErrorString(e));
    }
    return attach_field(s, index, g, d);
}

bbg_status bbg_collider_get_sdf(bbg_solver s, int index, bbg_sdf_grid *grid, float *values, size_t capacity,
                                size_t *count) {
    if (bbg_status r = check_field_target(s, index)) return r;
    const int slot = s->P.shapes[index].sdf;
    if (slot < 0) return fail(BBG_ERR_NOT_FOUND, "collider %d has no field", index);
    const bbg_sdf_grid &g = s->sdf_grid[slot];
    const size_t total = (size_t)g.nodes[0] * g.nodes[1] * g.nodes[2];
    if (grid) *grid = g;
    if (count) *count = total;
    if (values) {
        if (capacity < total) return fail(BBG_ERR_CAPACITY, "the field has %zu nodes", total);
        CK(cudaMemcpy(values, s->sdf_values[slot], sizeof(float) * total, cudaMemcpyDeviceToHost));
    }
    return BBG_OK;
}

bbg_status bbg_collider_query(bbg_solver s, int index, int n, const float *points, float *sample, float *gradient,
                              float *closest, float *normal, float *distance, int *inside) {
    if (bbg_status r = check_solver(s)) return r;
    if (index < 0 || index >= s->P.nshapes) return fail(BBG_ERR_INVALID_ARGUMENT, "no collider %d", index);
    if (s->P.shapes[index].type == BBG_SHAPE_SDF && s->P.shapes[index].sdf < 0)
        return fail(BBG_ERR_STATE, "collider %d is a field-only shape without a field", index);
    if (n <= 0 || !points) return fail(BBG_ERR_INVALID_ARGUMENT, "need n > 0 points");
    float *dp = nullptr;   // 3 in + 14 out floats per point
    CK(scratch_begin(s));
    CK(scratch_get(s, 17 * (size_t)n, &dp));
    float *dout = dp + 3 * (size_t)n;
    std::vector<float> o(14 * (size_t)n);
    cudaError_t e = cudaMemcpyAsync(dp, points, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        launch_shape_query(s->P, index, n, dp, dout, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(o.data(), dout, sizeof(float) * o.size(), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(BBG_ERR_CUDA, "collider query: %s", cudaGetErrorString(e));
    for (int q = 0; q < n; q++) {
        const float *r = &o[14 * (size_t)q];
        if (sample) sample[q] = r[0];
        for (int k = 0; k < 3; k++) {
            if (gradient) gradient[3 * q + k] = r[1 + k];
            if (closest) closest[3 * q + k] = r[4 + k];
            if (normal) normal[3 * q + k] = r[7 + k];
        }
        if (distance) distance[q] = r[10];
        if (inside) inside[q] = r[11] != 0.f;
    }
    return BBG_OK;
}

// ----------------------------------------------------------------------------
// the field of a triangle mesh (GenerateShapeSDF of a mesh shape)
// ----------------------------------------------------------------------------
namespace {

// Node values of the mesh's field into device memory (*values, owned by the caller).
bbg_status mesh_field(bbg_solver s, const float *vertices, int nv, const int *triangles, int nt, double dx,
                      double margin, bbg_sdf_grid *g, float **values, int *stuck) {
    if (!vertices || !triangles || nv < 3 || nt < 1) return fail(BBG_ERR_INVALID_ARGUMENT, "need a mesh");
    if (!(dx > 0) || !(margin >= 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "need dx > 0 and margin >= 0");
    std::vector<float> tri(9 * (size_t)nt);
    float lo[3] = {3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f};
    float hi[3] = {-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f};
    for (int t = 0; t < nt; t++) {
        for (int c = 0; c < 3; c++) {
            const int v = triangles[3 * (size_t)t + c];
            if (v < 0 || v >= nv) return fail(BBG_ERR_INVALID_ARGUMENT, "triangle %d: vertex %d out of range", t, v);
            for (int k = 0; k < 3; k++) {
                const float x = vertices[3 * (size_t)v + k];
                if (!std::isfinite(x)) return fail(BBG_ERR_INVALID_ARGUMENT, "vertex %d is not finite", v);
                tri[9 * (size_t)t + 3 * c + k] = x;
                // the BVH root bound: the union of the triangles' bounds
                lo[k] = x < lo[k] ? x : lo[k];
                hi[k] = x > hi[k] ? x : hi[k];
            }
        }
    }
    if (bbg_status r = field_grid_for(lo, hi, dx, margin, g)) return r;
    g->bounded = 1;
    for (int k = 0; k < 3; k++) {
        g->bounds_min[k] = lo[k];
        g->bounds_max[k] = hi[k];
    }
    // gamma(n) = n eps / (1 - n eps) with the reference's MachineEpsilon, in double
    float gam[4];
    const int ns[4] = {2, 3, 5, 7};
    for (int q = 0; q < 4; q++)
        gam[q] = (float)(((double)(float)ns[q] * 5.96046e-08) / (1 - (double)(float)ns[q] * 5.96046e-08));
    const size_t total = (size_t)g->nodes[0] * g->nodes[1] * g->nodes[2];
    // tiles of consecutive triangles with their boxes; the distance margin is 1e-3 of the
    // mesh's bounding diagonal
    const size_t ntile = (size_t)mesh_tiles(nt);
    std::vector<float> tiles(6 * ntile), dtri(9 * (size_t)nt), dtiles(6 * ntile);
    mesh_tile_bounds(tri.data(), nt, tiles.data());
    mesh_morton_order(tri.data(), nt, lo, hi, dtri.data());
    mesh_tile_bounds(dtri.data(), nt, dtiles.data());
    const double ex = (double)hi[0] - lo[0], ey = (double)hi[1] - lo[1], ez = (double)hi[2] - lo[2];
    const float margin_abs = (float)(1e-3 * std::sqrt(ex * ex + ey * ey + ez * ez));
    // one upload: triangles, their tiles, the Morton-ordered triangles, their tiles
    tri.insert(tri.end(), tiles.begin(), tiles.end());
    tri.insert(tri.end(), dtri.begin(), dtri.end());
    tri.insert(tri.end(), dtiles.begin(), dtiles.end());
    float *d_tri = nullptr, *d_out = nullptr;
    unsigned *d_stuck = nullptr;
    cudaError_t e = scratch_begin(s);
    if (e == cudaSuccess) e = scratch_get(s, tri.size(), &d_tri);
    if (e == cudaSuccess) e = scratch_get(s, 1, &d_stuck);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_out, sizeof(float) * total);   // the field: the caller's
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_tri, tri.data(), sizeof(float) * tri.size(), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_stuck, 0, sizeof(unsigned), s->stream);
    unsigned h_stuck = 0;
    if (e == cudaSuccess) {
        const float *d_tiles = d_tri + 9 * (size_t)nt, *d_dtri = d_tiles + 6 * ntile;
        launch_mesh_sdf(d_tri, nt, d_tiles, d_dtri, d_dtri + 9 * (size_t)nt, margin_abs, field_dev(*g, d_out), lo, hi,
                        gam, d_out, d_stuck, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_stuck, d_stuck, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        if (d_out) cudaFree(d_out);
        return fail(BBG_ERR_CUDA, "mesh field: %s", cudaGetErrorString(e));
    }
    if (stuck) *stuck = (int)h_stuck;
    *values = d_out;
    return BBG_OK;
}

}  // namespace

bbg_status bbg_mesh_sdf(bbg_solver s, const float *vertices, int nv, const int *triangles, int nt, double dx,
                        double margin, bbg_sdf_grid *grid, float *values, size_t capacity, size_t *count,
                        int *stuck) {
    if (bbg_status r = check_solver(s)) return r;
    bbg_sdf_grid g;
    float *d = nullptr;
    if (bbg_status r = mesh_field(s, vertices, nv, triangles, nt, dx, margin, &g, &d, stuck)) return r;
    const size_t total = (size_t)g.nodes[0] * g.nodes[1] * g.nodes[2];
    if (grid) *grid = g;
    if (count) *count = total;
    bbg_status r = BBG_OK;
    if (values) {
        if (capacity < total) {
            r = fail(BBG_ERR_CAPACITY, "the field has %zu nodes", total);
        } else {
            const cudaError_t e = cudaMemcpy(values, d, sizeof(float) * total, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) r = fail(BBG_ERR_CUDA, "mesh field: %s", cudaGetErrorString(e));
        }
    }
    cudaFree(d);
    return r;
}

bbg_status bbg_collider_set_mesh(bbg_solver s, int index, const float *vertices, int nv, const int *triangles,
                                 int nt, double dx, double margin) {
    if (bbg_status r = check_field_target(s, index)) return r;
    if (s->P.shapes[index].type != BBG_SHAPE_SDF)
        return fail(BBG_ERR_INVALID_ARGUMENT, "collider %d is not a field-only (BBG_SHAPE_SDF) collider", index);
    bbg_sdf_grid g;
    float *d = nullptr;
    if (bbg_status r = mesh_field(s, vertices, nv, triangles, nt, dx, margin, &g, &d, nullptr)) return r;
    return attach_field(s, index, g, d);
}

// ----------------------------------------------------------------------------
// boundary classification: LNMBoundary (src/boundaries/lnm.h:245-275)
// ----------------------------------------------------------------------------
// LNMComputeDelta (lnm.h:24-33): (min cell length / h)^dim as a float power
static float lnm_pre_delta(bbg_solver s, double h) {
    const float *len = s->P.g.len;
    const float minlen = len[0] < len[1] ? (len[0] < len[2] ? len[0] : len[2]) : (len[1] < len[2] ? len[1] : len[2]);
    return std::pow(minlen / (float)h, 3.0f);
}

// the kernels' delta from a float parameter (LNMBoundaryL2Kernel, LNMBoundaryLKKernel):
// truncated when positive, any count when unbounded
static int lnm_delta(bbg_solver s, double h, int unbounded) {
    const float pd = unbounded ? -1.f : lnm_pre_delta(s, h);
    return pd > 0 ? (int)pd : 0x7fffffff;
}

static bbg_status lnm_check(bbg_solver s, double h, const int *out) {
    if (bbg_status r = check_solver(s)) return r;
    if (!out || !(h > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "need h > 0 and an output");
    if (!s->setup_done || s->n <= 0) return fail(BBG_ERR_STATE, "no particles set up");
    if (!s->grid_valid)   // the reference classifies the grid's distribution: make one
        if (bbg_status r = grid_update(s)) return r;
    return BBG_OK;
}

// device scratch of the boundary passes (the solver's): cell levels, per-particle output
// and values, queue
struct LnmScratch {
    int *level = nullptr, *out = nullptr, *val = nullptr, *queue = nullptr, *counts = nullptr;
    cudaError_t alloc(bbg_solver s, size_t cells, size_t n) {
        cudaError_t e = scratch_begin(s);
        if (e == cudaSuccess) e = scratch_get(s, cells + 1, &level);
        if (e == cudaSuccess) e = scratch_get(s, n, &out);
        if (e == cudaSuccess) e = scratch_get(s, n, &val);
        if (e == cudaSuccess) e = scratch_get(s, n, &queue);
        if (e == cudaSuccess) e = scratch_get(s, 4, &counts);
        return e;
    }
};

static bbg_status lnm_finish(bbg_solver s, cudaError_t e, const LnmScratch &w, int *levels, const char *what) {
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(levels, w.out, sizeof(int) * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(BBG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return BBG_OK;
}

// The particle tests' arguments: Xiaowei at kernel radius 6h (xiaowei.h:26-33), Dilts at
// 0.75 x the set's radius (the target spacing, particle.h:536-541; dilts.h:30-33), the
// spoke angles i pi / 64 and j 2 pi / 64 rounded to float and their sines and cosines by
// the C library's float functions, as the reference computes them on the host.
static BoundaryArgs boundary_args(bbg_solver s, double h) {
    BoundaryArgs A;
    A.g = s->P.g;
    A.iz = s->P.iz;
    A.start = s->B.start;
    A.pos = s->B.pos[s->state];
    A.rho = s->B.rho;
    A.pid = s->B.pid[s->pid_cur];
    const float hf = (float)h;
    const float rho6 = (float)(6.0 * (double)hf);
    const float h2 = rho6 * rho6, h3 = h2 * rho6;
    A.x_rhot = (float)(0.7 * 1000.0);
    A.x_h2 = h2;
    A.x_wc = 315.0 / (64.0 * 3.14159265358979323846 * (double)h3);
    A.x_limit = 0.15 * (double)rho6;
    const float radius = (float)s->desc.target_spacing;
    A.d_rad = (float)((double)radius * 0.75);
    A.d_lim = (A.d_rad + A.d_rad) - 0.0001f;
    const float samples = (float)64;
    for (int i = 0; i <= 64; i++) {
        const float u = (float)(i * 3.14159265358979323846 / (double)samples);
        const float v = (float)(i * 6.283185307179586 / (double)samples);
        A.spoke[i] = sinf(u);
        A.spoke[65 + i] = cosf(u);
        A.spoke[130 + i] = sinf(v);
        A.spoke[195 + i] = cosf(v);
    }
    return A;
}

// ----------------------------------------------------------------------------
// boundary classification: LNMBoundary (src/boundaries/lnm.h:245-289) and its variants
// ----------------------------------------------------------------------------
bbg_status bbg_lnm_boundary(bbg_solver s, double h, int unbounded, int *levels) {
    if (bbg_status r = lnm_check(s, h, levels)) return r;
    LnmScratch w;
    cudaError_t e = w.alloc(s, s->P.g.total, (size_t)s->n);
    if (e == cudaSuccess)
        launch_lnm(s->P.g, s->B.start, s->B.cell, s->B.pid[s->pid_cur], s->n, lnm_delta(s, h, unbounded), w.level,
                   w.out, s->stream);
    return lnm_finish(s, e, w, levels, "LNM boundary");
}

bbg_status bbg_lnm_boundary_single(bbg_solver s, double h, int unbounded, int *levels) {
    if (bbg_status r = lnm_check(s, h, levels)) return r;
    // LNMBoundarySingleKernel takes delta as an int: truncated first, then any count unless positive
    const int pre = unbounded ? -1 : (int)lnm_pre_delta(s, h);
    LnmScratch w;
    cudaError_t e = w.alloc(s, s->P.g.total, (size_t)s->n);
    if (e == cudaSuccess)
        launch_lnm_single(s->P.g, s->B.start, s->B.cell, s->B.pid[s->pid_cur], s->n, pre > 0 ? pre : 0x7fffffff,
                          w.level, w.out, s->stream);
    return lnm_finish(s, e, w, levels, "LNM single-pass boundary");
}

bbg_status bbg_lnm_boundary_extended(bbg_solver s, double h, int max_level, int unbounded, int *levels) {
    if (bbg_status r = lnm_check(s, h, levels)) return r;
    LnmScratch w;
    cudaError_t e = w.alloc(s, s->P.g.total, (size_t)s->n);
    // LNMClassifyLazyGPU: levels 0..max_level, or until a sweep changes nothing
    const long cap = (long)s->P.g.total + 2;
    for (long L = 0; e == cudaSuccess; L++) {
        if (max_level < 0) e = cudaMemsetAsync(w.counts, 0, sizeof(int), s->stream);
        if (e == cudaSuccess) launch_lnm_once(s->P.g, s->B.start, w.level, (int)L, w.counts, s->stream);
        if (max_level > -1) {
            if (L >= max_level) break;
            continue;
        }
        int changed = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&changed, w.counts, sizeof(int), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (!changed || L >= cap) break;
    }
    if (e == cudaSuccess)
        launch_lnm_extended_finish(s->P.g, s->P.iz, s->B.pos[s->state], s->B.start, s->B.cell, s->B.pid[s->pid_cur],
                                   s->n, lnm_delta(s, h, unbounded), w.level, w.val, w.out, s->stream);
    return lnm_finish(s, e, w, levels, "LNM extended boundary");
}

bbg_status bbg_lnm_boundary_geometric(bbg_solver s, double h, int algorithm, int unbounded, int *levels,
                                      int *queued, int *accepted) {
    if (bbg_status r = lnm_check(s, h, levels)) return r;
    if (algorithm != BBG_BOUNDARY_XIAOWEI && algorithm != BBG_BOUNDARY_DILTS)
        return fail(BBG_ERR_INVALID_ARGUMENT, "unknown L2 filter %d", algorithm);
    if (algorithm == BBG_BOUNDARY_XIAOWEI && !(s->valid & bit(BBG_FIELD_DENSITY)))
        return fail(BBG_ERR_STATE, "the Xiaowei test reads the particle densities: none are valid");
    LnmScratch w;
    cudaError_t e = w.alloc(s, s->P.g.total, (size_t)s->n);
    if (e == cudaSuccess)
        launch_lnm_geometric(boundary_args(s, h), s->B.cell, s->n, lnm_delta(s, h, unbounded), algorithm, w.level,
                             w.queue, w.counts, w.out, s->stream);
    int counts[2] = {0, 0};
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, w.counts, sizeof counts, cudaMemcpyDeviceToHost, s->stream);
    if (bbg_status r = lnm_finish(s, e, w, levels, "LNM boundary with a geometric filter")) return r;
    if (queued) *queued = counts[0];
    if (accepted) *accepted = counts[1];
    return BBG_OK;
}

// XiaoweiBoundary (src/boundaries/xiaowei.h:80-87), DiltsSpokeBoundary (dilts.h:155-163)
bbg_status bbg_boundary_test(bbg_solver s, int method, double h, int *flags) {
    if (method == BBG_BOUNDARY_DILTS && !(h > 0)) h = 1.0;   // Dilts does not use h
    if (bbg_status r = lnm_check(s, h, flags)) return r;
    if (method != BBG_BOUNDARY_XIAOWEI && method != BBG_BOUNDARY_DILTS)
        return fail(BBG_ERR_INVALID_ARGUMENT, "unknown boundary test %d", method);
    if (method == BBG_BOUNDARY_XIAOWEI && !(s->valid & bit(BBG_FIELD_DENSITY)))
        return fail(BBG_ERR_STATE, "the Xiaowei test reads the particle densities: none are valid");
    LnmScratch w;
    cudaError_t e = w.alloc(s, s->P.g.total, (size_t)s->n);
    if (e == cudaSuccess) launch_boundary_test(boundary_args(s, h), method, s->n, w.out, s->stream);
    return lnm_finish(s, e, w, flags, "boundary test");
}

// ----------------------------------------------------------------------------
// the surface app's particle-to-field step: ParticlesToSDF_Surface (apps/surface.cpp:388-470)
// ----------------------------------------------------------------------------
// The field's grid from the domain grid's bounds: by spacing, cells of 2 x mc_spacing from
// pMin + half a cell, ceil(extent / cell) cells per axis; by resolution, that many nodes at
// the largest of extent / (nodes - 1), from pMin + half of it.  Float operations as the app.
static bbg_status particle_sdf_grid(bbg_solver s, double mc_spacing, const int *resolution, bbg_sdf_grid *g) {
    const GridDev &d = s->P.g;
    int cells[3];
    float ds;
    if (!resolution) {
        if (!(mc_spacing > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "need a positive marching-cubes spacing");
        ds = (float)mc_spacing * 2.0f;
        for (int k = 0; k < 3; k++) {
            const float c = std::ceil((d.bmax[k] - d.bmin[k]) / ds);
            if (!(c >= 0 && c <= 4096)) return fail(BBG_ERR_INVALID_ARGUMENT, "a field of %g cells across", (double)c);
            cells[k] = (int)c;
        }
    } else {
        float dk[3];
        for (int k = 0; k < 3; k++) {
            if (resolution[k] < 2 || resolution[k] > 4097)
                return fail(BBG_ERR_INVALID_ARGUMENT, "resolution must be in [2, 4097] nodes per axis");
            cells[k] = resolution[k] - 1;
            dk[k] = (d.bmax[k] - d.bmin[k]) / (float)cells[k];
        }
        const float m12 = dk[1] < dk[2] ? dk[2] : dk[1];
        ds = dk[0] < m12 ? m12 : dk[0];
    }
    memset(g, 0, sizeof(*g));
    for (int k = 0; k < 3; k++) {
        g->nodes[k] = cells[k] + 1;
        g->origin[k] = d.bmin[k] + ds * 0.5f;
        g->spacing[k] = ds;
    }
    return BBG_OK;
}

bbg_status bbg_particle_sdf(bbg_solver s, int method, double kernel_radius, double mc_spacing, const int *resolution,
                            bbg_sdf_grid *grid, float *values, size_t capacity) {
    if (bbg_status r = check_solver(s)) return r;
    if (!grid) return fail(BBG_ERR_INVALID_ARGUMENT, "null grid");
    if (method != BBG_SURFACE_ZHU_BRIDSON && method != BBG_SURFACE_SPH)
        return fail(BBG_ERR_INVALID_ARGUMENT, "unknown particle field method %d", method);
    if (!(kernel_radius > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "need a positive kernel radius");
    if (bbg_status r = particle_sdf_grid(s, mc_spacing, resolution, grid)) return r;
    const size_t total = (size_t)grid->nodes[0] * grid->nodes[1] * grid->nodes[2];
    if (!values) return BBG_OK;
    if (capacity < total) return fail(BBG_ERR_CAPACITY, "the field has %zu nodes, room for %zu", total, capacity);
    if (!s->setup_done || s->n <= 0) return fail(BBG_ERR_STATE, "no particles set up");
    if (!s->grid_valid)
        if (bbg_status r = grid_update(s)) return r;
    if (method == BBG_SURFACE_SPH && !(s->valid & bit(BBG_FIELD_DENSITY)))
        return fail(BBG_ERR_STATE, "the SPH field reads the particle densities: none are valid");
    SurfaceArgs A;
    memset(&A, 0, sizeof(A));
    A.g = s->P.g;
    A.iz = s->P.iz;
    A.iz6 = s->P.iz6;
    A.start = s->B.start;
    A.pos = s->B.pos[s->state];
    A.rho = s->B.rho;
    A.method = method;
    for (int k = 0; k < 3; k++) {
        A.nodes[k] = grid->nodes[k];
        A.org[k] = (float)grid->origin[k];
        A.sp[k] = (float)grid->spacing[k];
    }
    const float dx = A.g.bmax[0] - A.g.bmin[0], dy = A.g.bmax[1] - A.g.bmin[1], dz = A.g.bmax[2] - A.g.bmin[2];
    A.inf = std::sqrt(dx * dx + dy * dy + dz * dz);
    A.radius = (float)kernel_radius;
    A.offset = A.radius * 0.25f;
    A.mass = s->mass;
    A.r2 = A.radius * A.radius;
    A.wc = 315.0 / (64.0 * 3.14159265358979323846 * (double)(A.r2 * A.radius));
    float *d_out = nullptr;
    cudaError_t e = scratch_begin(s);
    if (e == cudaSuccess) e = scratch_get(s, total, &d_out);
    if (e == cudaSuccess) {
        launch_particle_sdf(A, d_out, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(values, d_out, sizeof(float) * total, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(BBG_ERR_CUDA, "particle field: %s", cudaGetErrorString(e));
    return BBG_OK;
}

// ----------------------------------------------------------------------------
// marching cubes (MarchingCubes, src/reconstruction/marching_cubes.cpp:204-457)
// ----------------------------------------------------------------------------
bbg_status bbg_marching_cubes(bbg_solver s, const bbg_sdf_grid *grid, const float *values, double iso,
                              int rotate_faces, float *points, float *normals, size_t point_capacity,
                              int *triangles, size_t triangle_capacity, size_t *npoints, size_t *ntriangles) {
    if (bbg_status r = check_solver(s)) return r;
    if (!grid || !values) return fail(BBG_ERR_INVALID_ARGUMENT, "null grid or values");
    for (int k = 0; k < 3; k++)
        if (grid->nodes[k] < 2 || !(grid->spacing[k] > 0))
            return fail(BBG_ERR_INVALID_ARGUMENT, "a field needs >= 2 nodes and spacing > 0 per axis");
    const long long nodes = (long long)grid->nodes[0] * grid->nodes[1] * grid->nodes[2];
    const long long cubes = (long long)(grid->nodes[0] - 1) * (grid->nodes[1] - 1) * (grid->nodes[2] - 1);
    if (3 * nodes >= (1ll << 31)) return fail(BBG_ERR_CAPACITY, "the field has %lld nodes", nodes);
    CK(mc_prepare());
    McInput in;
    in.nodes[0] = grid->nodes[0];
    in.nodes[1] = grid->nodes[1];
    in.nodes[2] = grid->nodes[2];
    for (int k = 0; k < 3; k++) {
        in.origin[k] = (float)grid->origin[k];
        in.spacing[k] = (float)grid->spacing[k];
        in.inv[k] = (float)(1.0 / (double)in.spacing[k]);   // invGridSize
    }
    in.iso = (float)iso;
    float *d_vals = nullptr, *d_pts = nullptr, *d_nrm = nullptr;
    int *d_tri = nullptr;
    unsigned *b[7] = {};
    const size_t sz[7] = {(size_t)cubes + 1, (size_t)cubes + 1, scan_partials_needed((unsigned)(cubes + 1)),
                          (size_t)(3 * nodes) + 1, (size_t)(3 * nodes) + 1, (size_t)(3 * nodes) + 1,
                          scan_partials_needed((unsigned)(3 * nodes + 1))};
    cudaError_t e = scratch_begin(s);
    if (e == cudaSuccess) e = scratch_get(s, (size_t)nodes, &d_vals);
    for (int q = 0; q < 7 && e == cudaSuccess; q++) e = scratch_get(s, sz[q], &b[q]);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_vals, values, sizeof(float) * (size_t)nodes, cudaMemcpyHostToDevice, s->stream);
    in.values = d_vals;
    size_t ntri = 0, nvert = 0;
    unsigned *h = s->h_u;
    if (e == cudaSuccess) e = mc_count(in, b[0], b[1], b[2], b[3], b[4], b[5], b[6], h, &ntri, &nvert, s->stream);
    bbg_status r = BBG_OK;
    if (e != cudaSuccess) {
        r = fail(BBG_ERR_CUDA, "marching cubes: %s", cudaGetErrorString(e));
    } else {
        if (npoints) *npoints = nvert;
        if (ntriangles) *ntriangles = ntri;
        if (!points || !normals || !triangles || point_capacity < nvert || triangle_capacity < ntri) {
            r = fail(BBG_ERR_CAPACITY, "the mesh has %zu points and %zu triangles", nvert, ntri);
        } else {
            e = scratch_get(s, 3 * nvert, &d_pts);
            if (e == cudaSuccess) e = scratch_get(s, 3 * nvert, &d_nrm);
            if (e == cudaSuccess) e = scratch_get(s, 3 * ntri, &d_tri);
            if (e == cudaSuccess) {
                mc_emit(in, b[1], b[3], b[5], rotate_faces ? 1 : 0, d_pts, d_nrm, d_tri, s->stream);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaMemcpyAsync(points, d_pts, sizeof(float) * 3 * nvert, cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(normals, d_nrm, sizeof(float) * 3 * nvert, cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(triangles, d_tri, sizeof(int) * 3 * ntri, cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) r = fail(BBG_ERR_CUDA, "marching cubes: %s", cudaGetErrorString(e));
        }
    }
    return r;
}
