// api_batch.cu -- the C ABI of batches of independent scenes (include/bbg.h):
// one solver over scenes stacked along z, their layout, transfers and per-scene statistics.
#include "api_internal.h"

// ----------------------------------------------------------------------------
// batches of independent scenes
// ----------------------------------------------------------------------------
bbg_status bbg_batch_create(const bbg_solver_desc *desc, const bbg_scene_desc *scenes, int count,
                            bbg_solver *out) {
    if (!desc || !scenes || !out || count <= 0)
        return fail(BBG_ERR_INVALID_ARGUMENT, "invalid batch arguments");
    if (count > 65535) return fail(BBG_ERR_INVALID_ARGUMENT, "at most 65535 scenes");
    *out = nullptr;
    const double cell = desc->target_spacing * desc->grid_spacing_scale;
    if (!(cell > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "spacing and grid scale must be > 0");
    // scenes stacked along z (the slowest axis of the cell order, so each scene's
    // particles stay contiguous), each container's min corner on a cell boundary, two
    // empty cells between consecutive containers
    double xmax = 0, ymax = 0, z = 0;
    long long total = 0;
    std::vector<double> off(3 * (size_t)count);
    std::vector<float> zb(count);
    std::vector<ShapeDev> boxes(count);
    for (int i = 0; i < count; i++) {
        const bbg_scene_desc &sc = scenes[i];
        double ext[3];
        for (int k = 0; k < 3; k++) {
            ext[k] = sc.box_max[k] - sc.box_min[k];
            if (!(ext[k] > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "scene %d: empty container", i);
        }
        if (sc.count <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "scene %d: no particles", i);
        total += sc.count;
        xmax = ext[0] > xmax ? ext[0] : xmax;
        ymax = ext[1] > ymax ? ext[1] : ymax;
        off[3 * i + 0] = -sc.box_min[0];
        off[3 * i + 1] = -sc.box_min[1];
        off[3 * i + 2] = z - sc.box_min[2];
        zb[i] = i == 0 ? -3.402823466e+38f : (float)(z - cell);
        bbg_shape box;
        memset(&box, 0, sizeof(box));
        box.type = BBG_SHAPE_BOX;
        box.reverse = 1;
        box.center[0] = 0.5 * ext[0];
        box.center[1] = 0.5 * ext[1];
        box.center[2] = z + 0.5 * ext[2];
        for (int k = 0; k < 3; k++) box.size[k] = ext[k];
        boxes[i] = shape_dev(box);
        z = ceil((z + ext[2]) / cell) * cell + 2.0 * cell;
    }
    if (total > 0x7fffffff) return fail(BBG_ERR_INVALID_ARGUMENT, "too many particles");
    bbg_solver_desc d = *desc;
    for (int k = 0; k < 3; k++) d.domain_min[k] = 0.0;
    d.domain_max[0] = ceil(xmax / cell) * cell;
    d.domain_max[1] = ceil(ymax / cell) * cell;
    d.domain_max[2] = z - 2.0 * cell;
    bbg_solver s = nullptr;
    bbg_status r = bbg_create(&d, (int)total, &s);
    if (r) return r;
    s->nscenes = count;
    s->scene_offset = off;
    s->scene_first.resize(count);
    s->scene_count.resize(count);
    int first = 0;
    for (int i = 0; i < count; i++) {
        s->scene_first[i] = first;
        s->scene_count[i] = scenes[i].count;
        first += scenes[i].count;
    }
    if (!r) r = dalloc(&s->d_zb, (size_t)count);
    if (!r) r = dalloc(&s->d_box, (size_t)count);
    if (!r) r = dalloc(&s->d_sst, (size_t)count);
    if (!r) r = dalloc(&s->d_scene, (size_t)total);
    if (!r) r = dalloc(&s->d_wl, 4 * (size_t)count + 3);
    if (!r && cudaMemset(s->d_wl, 0, sizeof(int) * (4 * (size_t)count + 3)) != cudaSuccess)
        r = fail(BBG_ERR_CUDA, "batch upload failed");
    if (!r && cudaMemcpy(s->d_zb, zb.data(), sizeof(float) * count, cudaMemcpyHostToDevice) != cudaSuccess)
        r = fail(BBG_ERR_CUDA, "batch upload failed");
    if (!r && cudaMemcpy(s->d_box, boxes.data(), sizeof(ShapeDev) * count, cudaMemcpyHostToDevice) != cudaSuccess)
        r = fail(BBG_ERR_CUDA, "batch upload failed");
    if (!r && cudaMemset(s->d_sst, 0, sizeof(SceneState) * count) != cudaSuccess)
        r = fail(BBG_ERR_CUDA, "batch upload failed");
    if (r) {
        bbg_destroy(s);
        return r;
    }
    s->P.nscenes = count;
    s->P.scene_zb = s->d_zb;
    s->P.scene_box = s->d_box;
    s->P.scene_st = s->d_sst;
    s->P.scene = s->d_scene;
    s->P.scene_first = s->d_wl;
    s->P.scene_last = s->d_wl + count;
    s->P.wl_off = s->d_wl + 2 * (size_t)count;        // count + 1 entries
    s->P.wl_tile = s->d_wl + 3 * (size_t)count + 1;
    s->P.wl_ctr = s->d_wl + 4 * (size_t)count + 1;    // 2 entries
    update_worklist_grid(s->B);
    s->epoch++;
    *out = s;
    return BBG_OK;
}

namespace {
bbg_status require_batch(bbg_solver s) {
    if (s->nscenes <= 0) return fail(BBG_ERR_STATE, "not a batch solver");
    return BBG_OK;
}
}  // namespace

bbg_status bbg_batch_scene_count(bbg_solver s, int *count) {
    if (bbg_status r = check_solver(s)) return r;
    if (!count) return fail(BBG_ERR_INVALID_ARGUMENT, "null count");
    *count = s->nscenes;
    return BBG_OK;
}

bbg_status bbg_batch_layout(bbg_solver s, double *offsets) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_batch(s)) return r;
    if (!offsets) return fail(BBG_ERR_INVALID_ARGUMENT, "null offsets");
    memcpy(offsets, s->scene_offset.data(), sizeof(double) * 3 * (size_t)s->nscenes);
    return BBG_OK;
}

bbg_status bbg_batch_upload(bbg_solver s, const float *pos, const float *vel) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_batch(s)) return r;
    if (!pos) return fail(BBG_ERR_INVALID_ARGUMENT, "null positions");
    const int n = s->capacity;
    std::vector<float> packed(3 * (size_t)n);
    for (int i = 0; i < s->nscenes; i++)
        for (int q = s->scene_first[i]; q < s->scene_first[i] + s->scene_count[i]; q++)
            for (int k = 0; k < 3; k++)
                packed[3 * (size_t)q + k] = (float)((double)pos[3 * (size_t)q + k] + s->scene_offset[3 * i + k]);
    bbg_status r = bbg_upload_particles(s, packed.data(), vel, n);
    if (r) return r;
    CK(cudaStreamSynchronize(s->stream));   // the host staging is released here
    return BBG_OK;
}

bbg_status bbg_batch_download(bbg_solver s, float *pos, float *vel) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_batch(s)) return r;
    bbg_status r = bbg_download(s, pos, vel);
    if (r) return r;
    if (pos)
        for (int i = 0; i < s->nscenes; i++)
            for (int q = s->scene_first[i]; q < s->scene_first[i] + s->scene_count[i]; q++)
                for (int k = 0; k < 3; k++)
                    pos[3 * (size_t)q + k] = (float)((double)pos[3 * (size_t)q + k] - s->scene_offset[3 * i + k]);
    return BBG_OK;
}

bbg_status bbg_batch_scene_stats(bbg_solver s, int *iterations, double *max_err) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_batch(s)) return r;
    std::vector<SceneState> st(s->nscenes);
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(st.data(), s->d_sst, sizeof(SceneState) * (size_t)s->nscenes, cudaMemcpyDeviceToHost));
    for (int i = 0; i < s->nscenes; i++) {
        int it = s->last_max_it;
        float err = 0;
        for (int k = 0; k < s->last_max_it; k++) {
            float e;
            memcpy(&e, &st[i].err_bits[k], 4);
            err = e / s->P.target_density;
            if (err < s->last_tol) {
                it = k + 1;
                break;
            }
        }
        if (iterations) iterations[i] = it;
        if (max_err) max_err[i] = err;
    }
    return BBG_OK;
}
