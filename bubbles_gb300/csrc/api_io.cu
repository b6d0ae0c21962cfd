// api_io.cu -- the C ABI of particle frames in the reference's text format
// (SerializerSaveSphDataSet3 / SerializerLoadSphDataSet3) and of binary checkpoints.
#include "api_internal.h"

// ----------------------------------------------------------------------------
// particle frames (SerializerSaveSphDataSet3 format)
// ----------------------------------------------------------------------------
namespace {
// Formats the frame's particle lines on the device; *head receives the header text and
// *body the byte count of the lines waiting in s->frame.out.
bbg_status frame_build(bbg_solver s, int flags, std::string *head, size_t *body) {
    if (bbg_status r = check_solver(s)) return r;
    if (!(flags & kFrameSupported) || (flags & ~kFrameSupported))
        return fail(BBG_ERR_INVALID_ARGUMENT, "frame flags must combine position, velocity, density and mass");
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    if ((flags & kFrameDensity) && !(s->valid & bit(BBG_FIELD_DENSITY)))
        return fail(BBG_ERR_STATE, "density is not valid in the current particle order");
    FrameBufs &F = s->frame;
    if (F.capacity < s->capacity) {
        free_frame(s);
        const size_t n = (size_t)s->capacity;
        bbg_status r = BBG_OK;
        if (!r) r = dalloc(&F.lines, n * kFrameLineCap);
        if (!r) r = dalloc(&F.lens, n);
        if (!r) r = dalloc(&F.scan_in, n);
        if (!r) r = dalloc(&F.offset, n + 1);
        if (!r) r = dalloc(&F.partials, scan_partials_needed((unsigned)n));
        if (!r) r = dalloc(&F.out, n * kFrameLineCap);
        if (r) {
            free_frame(s);
            return r;
        }
        F.capacity = s->capacity;
    }
    launch_frame_lines(s->n, flags, s->B.pos[s->state], s->B.vel[s->state], s->B.rho, s->B.slot, s->mass, F,
                       s->stream);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(s->h_u, &F.offset[s->n], sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    unsigned lines_bytes = 0;
    memcpy(&lines_bytes, s->h_u, sizeof(unsigned));
    *body = lines_bytes;
    char fmt[16];
    int k = 0;
    if (flags & kFramePosition) fmt[k++] = 'p';
    if (flags & kFrameVelocity) fmt[k++] = 'v';
    if (flags & kFrameDensity) fmt[k++] = 'd';
    if (flags & kFrameMass) fmt[k++] = 'm';
    fmt[k] = 0;
    char h[256];
    const int hl = snprintf(h, sizeof(h),
                            "FluidBegin\n\t\"Type\" particles\n\t\"Count\" %d\n\t\"Format\" %s\n"
                            "\t\"Spacing\" %g\n\tDataBegin\n",
                            s->n, fmt, (double)(float)s->desc.target_spacing);   // Float spacing
    head->assign(h, (size_t)hl);
    return BBG_OK;
}

const char kFrameTail[] = "\tDataEnd\nFluidEnd\n";
constexpr size_t kFrameTailLen = sizeof(kFrameTail) - 1;
}  // namespace

bbg_status bbg_frame_text(bbg_solver s, int flags, char *buf, size_t capacity, size_t *length) {
    std::string head;
    size_t body = 0;
    if (bbg_status r = frame_build(s, flags, &head, &body)) return r;
    const size_t total = head.size() + body + kFrameTailLen;
    if (length) *length = total;
    if (!buf || capacity < total) return fail(BBG_ERR_CAPACITY, "the frame needs %zu bytes", total);
    memcpy(buf, head.data(), head.size());
    CK(cudaMemcpy(buf + head.size(), s->frame.out, body, cudaMemcpyDeviceToHost));
    memcpy(buf + head.size() + body, kFrameTail, kFrameTailLen);
    return BBG_OK;
}

bbg_status bbg_frame_append(bbg_solver s, int flags, const char *path) {
    if (!path) return fail(BBG_ERR_INVALID_ARGUMENT, "null path");
    std::string head;
    size_t body = 0;
    if (bbg_status r = frame_build(s, flags, &head, &body)) return r;
    std::vector<char> text(head.size() + body + kFrameTailLen);
    memcpy(text.data(), head.data(), head.size());
    CK(cudaMemcpy(text.data() + head.size(), s->frame.out, body, cudaMemcpyDeviceToHost));
    memcpy(text.data() + head.size() + body, kFrameTail, kFrameTailLen);
    FILE *fp = fopen(path, "a+");
    if (!fp) return fail(BBG_ERR_INVALID_ARGUMENT, "cannot open %s", path);
    const size_t w = fwrite(text.data(), 1, text.size(), fp);
    const int closed = fclose(fp);
    if (w != text.size() || closed != 0) return fail(BBG_ERR_INVALID_ARGUMENT, "short write to %s", path);
    return BBG_OK;
}

bbg_status bbg_format_g(float value, char *out, int *length) {
    if (!out || !length) return fail(BBG_ERR_INVALID_ARGUMENT, "null output");
    *length = gfmt::format_g(value, out);
    return BBG_OK;
}

// ----------------------------------------------------------------------------
// checkpoint: binary snapshot of the solver state for exact resume
// ----------------------------------------------------------------------------
namespace {

constexpr char kCkptMagic[8] = {'B', 'B', 'G', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t kCkptVersion = 2;
// per-particle fields a snapshot carries when they are valid, in file order
constexpr int kCkptFields[] = {BBG_FIELD_POSITION,       BBG_FIELD_VELOCITY,      BBG_FIELD_FORCE,
                               BBG_FIELD_DENSITY,        BBG_FIELD_PRESSURE,      BBG_FIELD_PRED_POSITION,
                               BBG_FIELD_PRESSURE_FORCE, BBG_FIELD_PRED_DENSITY,  BBG_FIELD_DENSITY_ERROR,
                               BBG_FIELD_DIVERGENCE};

struct CkptHeader {
    char magic[8];
    uint32_t version, header_bytes, desc_bytes, shape_bytes, mlp_desc_bytes;
    int32_t nfields;   // colliders' signed-distance fields stored (grid + node values each)
    int32_t n, nshapes, nscenes, mlp;
    uint32_t fields;   // bit f set: field f stored
    uint32_t valid;    // the solver's valid-field mask
    float mass;
    int32_t mlp_trained;
    int64_t mlp_since;
    double mlp_loss_count;
    double mlp_loss;
    uint32_t adam_step, reserved1;
};


bool same_desc(const bbg_solver_desc &a, const bbg_solver_desc &b) {
#define EQ(f) (a.f == b.f)
    bool same = EQ(solver_kind) && EQ(eos_exponent) && EQ(negative_pressure_scale) && EQ(viscosity) &&
                EQ(pseudo_viscosity) && EQ(sound_speed) && EQ(drag_coefficient) && EQ(target_density) &&
                EQ(target_spacing) && EQ(relative_kernel_radius) && EQ(mass) && EQ(grid_spacing_scale) &&
                EQ(time_step_limit_scale) && EQ(pcisph_mode) && EQ(max_iterations) &&
                EQ(max_density_error_ratio) && EQ(pressure_init) && EQ(warm_rule) && EQ(warm_scale);
    for (int k = 0; k < 3; k++) same = same && EQ(gravity[k]) && EQ(domain_min[k]) && EQ(domain_max[k]);
#undef EQ
    return same;
}

struct Writer {
    std::vector<char> *out;
    void put(const void *p, size_t bytes) {
        const char *c = static_cast<const char *>(p);
        out->insert(out->end(), c, c + bytes);
    }
};

struct Reader {
    const char *p;
    size_t left;
    bool get(void *dst, size_t bytes) {
        if (bytes > left) return false;
        memcpy(dst, p, bytes);
        p += bytes;
        left -= bytes;
        return true;
    }
};

bbg_status ckpt_build(bbg_solver s, std::vector<char> *out) {
    if (bbg_status r = check_solver(s)) return r;
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    CkptHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kCkptMagic, sizeof(h.magic));
    h.version = kCkptVersion;
    h.header_bytes = sizeof(CkptHeader);
    h.desc_bytes = sizeof(bbg_solver_desc);
    h.shape_bytes = sizeof(ShapeDev);
    h.mlp_desc_bytes = sizeof(bbg_mlp_desc);
    h.n = s->n;
    h.nshapes = s->P.nshapes;
    h.nscenes = s->nscenes;
    for (int i = 0; i < s->P.nshapes; i++) h.nfields += s->P.shapes[i].sdf >= 0 ? 1 : 0;
    h.mlp = s->mlp_alloc ? 1 : 0;
    h.valid = s->valid;
    h.mass = s->mass;
    for (int f : kCkptFields) {
        const bool have = f == BBG_FIELD_DIVERGENCE ? s->mlp_alloc : (s->valid & bit(f)) != 0;
        if (have) h.fields |= bit(f);
    }
    if (s->mlp_alloc) {
        h.mlp_trained = s->mlp_trained;
        h.mlp_since = s->mlp_since;
        h.mlp_loss_count = s->mlp_loss_count;
        CK(cudaMemcpyAsync(s->h_u, s->mlp.step, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(&h.mlp_loss, s->mlp.loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        memcpy(&h.adam_step, s->h_u, sizeof(unsigned));
    }
    out->clear();
    Writer w{out};
    w.put(&h, sizeof(h));
    w.put(&s->desc, sizeof(bbg_solver_desc));
    w.put(s->P.shapes, sizeof(ShapeDev) * (size_t)s->P.nshapes);
    w.put(s->scene_count.data(), sizeof(int) * (size_t)s->nscenes);
    std::vector<float> buf;
    // each collider's field, in collider order: its grid, then its node values
    for (int i = 0; i < s->P.nshapes; i++) {
        const int slot = s->P.shapes[i].sdf;
        if (slot < 0) continue;
        const bbg_sdf_grid &g = s->sdf_grid[slot];
        buf.resize((size_t)g.nodes[0] * g.nodes[1] * g.nodes[2]);
        CK(cudaMemcpy(buf.data(), s->sdf_values[slot], sizeof(float) * buf.size(), cudaMemcpyDeviceToHost));
        w.put(&g, sizeof(g));
        w.put(buf.data(), sizeof(float) * buf.size());
    }
    for (int f : kCkptFields) {
        if (!(h.fields & bit(f))) continue;
        buf.resize((size_t)field_components(f) * (size_t)s->n);
        if (bbg_status r = bbg_get_field(s, f, buf.data())) return r;
        w.put(buf.data(), sizeof(float) * buf.size());
    }
    if (s->mlp_alloc) {
        w.put(&s->mdesc, sizeof(bbg_mlp_desc));
        buf.resize(3 * (size_t)kParams + kTail);
        float *b = buf.data();
        CK(cudaMemcpyAsync(b, s->mlp.theta, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(b + kParams, s->mlp.m1, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(b + 2 * kParams, s->mlp.m2, sizeof(float) * kParams, cudaMemcpyDeviceToHost,
                           s->stream));
        CK(cudaMemcpyAsync(b + 3 * kParams, s->mlp.tail, sizeof(float) * kTail, cudaMemcpyDeviceToHost,
                           s->stream));
        CK(cudaStreamSynchronize(s->stream));
        w.put(b, sizeof(float) * buf.size());
    }
    return BBG_OK;
}

bbg_status ckpt_restore(bbg_solver s, const char *data, size_t length) {
    if (bbg_status r = check_solver(s)) return r;
    if (!data) return fail(BBG_ERR_INVALID_ARGUMENT, "null checkpoint");
    Reader rd{data, length};
    CkptHeader h;
    if (!rd.get(&h, sizeof(h)) || memcmp(h.magic, kCkptMagic, sizeof(h.magic)) != 0)
        return fail(BBG_ERR_INVALID_ARGUMENT, "not a solver checkpoint");
    if (h.version != kCkptVersion || h.header_bytes != sizeof(CkptHeader) ||
        h.desc_bytes != sizeof(bbg_solver_desc) || h.shape_bytes != sizeof(ShapeDev) ||
        h.mlp_desc_bytes != sizeof(bbg_mlp_desc))
        return fail(BBG_ERR_INVALID_ARGUMENT, "checkpoint written by an incompatible library version");
    if (h.n <= 0 || h.nshapes < 0 || h.nshapes > kMaxColliders || h.nscenes < 0)
        return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint header");
    if (h.n > s->capacity) return fail(BBG_ERR_CAPACITY, "%d particles exceed capacity %d", h.n, s->capacity);
    bbg_solver_desc desc;
    if (!rd.get(&desc, sizeof(desc))) return fail(BBG_ERR_INVALID_ARGUMENT, "truncated checkpoint");
    if (!same_desc(desc, s->desc))
        return fail(BBG_ERR_STATE, "the checkpoint was written by a solver with another description");
    std::vector<ShapeDev> shapes((size_t)h.nshapes);
    std::vector<int> counts((size_t)h.nscenes);
    if (!rd.get(shapes.data(), sizeof(ShapeDev) * shapes.size()) ||
        !rd.get(counts.data(), sizeof(int) * counts.size()))
        return fail(BBG_ERR_INVALID_ARGUMENT, "truncated checkpoint");
    if (h.nscenes != s->nscenes || counts != s->scene_count)
        return fail(BBG_ERR_STATE, "the checkpoint's scene layout differs from this batch");
    // colliders: known types, field slots in range and used once, a field-only collider
    // with its field, and as many stored fields as colliders that have one
    int with_field = 0;
    unsigned slots_used = 0;
    for (const ShapeDev &sh : shapes) {
        if (sh.type != BBG_SHAPE_BOX && sh.type != BBG_SHAPE_SPHERE && sh.type != BBG_SHAPE_SDF)
            return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint: collider type %d", sh.type);
        if (sh.sdf < -1 || sh.sdf >= kMaxSdf || (sh.sdf >= 0 && (slots_used >> sh.sdf) & 1u))
            return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint: collider field slot %d", sh.sdf);
        if (sh.type == BBG_SHAPE_SDF && sh.sdf < 0)
            return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint: a field-only collider without its field");
        if (sh.sdf >= 0) {
            slots_used |= 1u << sh.sdf;
            with_field++;
        }
    }
    if (h.nfields != with_field) return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint: field count");
    if (with_field > 0 && s->nscenes > 0)
        return fail(BBG_ERR_STATE, "fields are not supported on a batch of scenes");
    std::vector<bbg_sdf_grid> grids((size_t)with_field);
    std::vector<std::vector<float>> values((size_t)with_field);
    for (int k = 0; k < with_field; k++) {
        bbg_sdf_grid &g = grids[(size_t)k];
        if (!rd.get(&g, sizeof(g))) return fail(BBG_ERR_INVALID_ARGUMENT, "truncated checkpoint");
        size_t total = 1;
        for (int a = 0; a < 3; a++) {
            if (g.nodes[a] < 1 || g.nodes[a] > 4097 || !(g.spacing[a] > 0) || !std::isfinite(g.origin[a]))
                return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint: field grid");
            total *= (size_t)g.nodes[a];
        }
        if (total >= 0xffffffffull) return fail(BBG_ERR_INVALID_ARGUMENT, "corrupt checkpoint: field grid");
        values[(size_t)k].resize(total);
        if (!rd.get(values[(size_t)k].data(), sizeof(float) * total))
            return fail(BBG_ERR_INVALID_ARGUMENT, "truncated checkpoint");
    }
    if ((h.mlp != 0) != s->mlp_alloc)
        return fail(BBG_ERR_STATE, "learned warm start %s in the checkpoint but %s in this solver",
                    h.mlp ? "present" : "absent", s->mlp_alloc ? "present" : "absent");
    const uint32_t need = bit(BBG_FIELD_POSITION) | bit(BBG_FIELD_VELOCITY);
    if ((h.fields & need) != need) return fail(BBG_ERR_INVALID_ARGUMENT, "checkpoint without positions");
    // every field before anything changes: a truncated file leaves the solver as it was
    std::vector<std::vector<float>> fields;
    for (int f : kCkptFields) {
        if (!(h.fields & bit(f))) continue;
        fields.emplace_back((size_t)field_components(f) * (size_t)h.n);
        if (!rd.get(fields.back().data(), sizeof(float) * fields.back().size()))
            return fail(BBG_ERR_INVALID_ARGUMENT, "truncated checkpoint");
    }
    bbg_mlp_desc md;
    std::vector<float> mlp;
    if (h.mlp) {
        mlp.resize(3 * (size_t)kParams + kTail);
        if (!rd.get(&md, sizeof(md)) || !rd.get(mlp.data(), sizeof(float) * mlp.size()))
            return fail(BBG_ERR_INVALID_ARGUMENT, "truncated checkpoint");
    }
    // the fields' device copies, then the particles; the colliders change only after both
    std::vector<float *> dev((size_t)with_field, nullptr);
    auto drop = [&]() {
        for (float *d : dev)
            if (d) cudaFree(d);
    };
    for (int k = 0; k < with_field; k++) {
        const std::vector<float> &v = values[(size_t)k];
        if (bbg_status r = dalloc(&dev[(size_t)k], v.size())) {
            drop();
            return r;
        }
        cudaError_t e = cudaMemcpy(dev[(size_t)k], v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            drop();
            return fail(BBG_ERR_CUDA, "field upload: %s", cudaGetErrorString(e));
        }
    }
    const float *pos = fields[0].data(), *vel = fields[1].data();
    if (bbg_status r = bbg_upload_particles(s, pos, vel, h.n)) {
        drop();
        return r;
    }
    free_fields(s);
    for (int i = 0; i < h.nshapes; i++) {
        s->P.shapes[i] = shapes[(size_t)i];
        s->P.shapes[i].sdf = -1;
    }
    s->P.nshapes = h.nshapes;
    for (int i = 0, k = 0; i < h.nshapes; i++) {
        if (shapes[(size_t)i].sdf < 0) continue;
        // cannot fail: at most kMaxSdf fields, all slots free after free_fields
        attach_field(s, i, grids[(size_t)k], dev[(size_t)k]);
        dev[(size_t)k++] = nullptr;
    }
    s->epoch++;
    if (!s->setup_done)
        if (bbg_status r = bbg_setup(s)) return r;
    s->mass = h.mass;
    const float mo = s->mass / (float)s->desc.target_density;
    s->mod2 = mo * mo;
    fill_params(s);
    s->epoch++;
    if (h.mlp) {
        if (bbg_status r = mlp_allocate(s, md)) return r;
        const float *b = mlp.data();
        MlpBufs &M = s->mlp;
        CK(cudaMemcpyAsync(M.theta, b, sizeof(float) * kParams, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(M.m1, b + kParams, sizeof(float) * kParams, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(M.m2, b + 2 * kParams, sizeof(float) * kParams, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(M.tail, b + 3 * kParams, sizeof(float) * kTail, cudaMemcpyHostToDevice, s->stream));
        memcpy(s->h_u, &h.adam_step, sizeof(unsigned));
        CK(cudaMemcpyAsync(M.step, s->h_u, sizeof(unsigned), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(M.loss, &h.mlp_loss, sizeof(double), cudaMemcpyHostToDevice, s->stream));
        launch_mlp_pack(M, s->stream);
        CK_LAUNCH();
        CK(cudaStreamSynchronize(s->stream));
        s->mlp_trained = h.mlp_trained;
        s->mlp_since = h.mlp_since;
        s->mlp_loss_count = h.mlp_loss_count;
    }
    size_t k = 0;
    for (int f : kCkptFields) {
        if (!(h.fields & bit(f))) continue;
        const std::vector<float> &v = fields[k++];
        if (f == BBG_FIELD_POSITION || f == BBG_FIELD_VELOCITY) continue;
        if (bbg_status r = bbg_set_field(s, f, v.data())) return r;
    }
    s->valid = h.valid;
    s->grid_valid = false;
    s->epoch++;
    return BBG_OK;
}

}  // namespace

bbg_status bbg_checkpoint_write(bbg_solver s, void *buf, size_t capacity, size_t *length) {
    std::vector<char> data;
    if (bbg_status r = ckpt_build(s, &data)) return r;
    if (length) *length = data.size();
    if (!buf || capacity < data.size())
        return fail(BBG_ERR_CAPACITY, "the checkpoint needs %zu bytes", data.size());
    memcpy(buf, data.data(), data.size());
    return BBG_OK;
}

bbg_status bbg_checkpoint_read(bbg_solver s, const void *buf, size_t length) {
    return ckpt_restore(s, static_cast<const char *>(buf), length);
}

bbg_status bbg_checkpoint_save(bbg_solver s, const char *path) {
    if (!path) return fail(BBG_ERR_INVALID_ARGUMENT, "null path");
    std::vector<char> data;
    if (bbg_status r = ckpt_build(s, &data)) return r;
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail(BBG_ERR_INVALID_ARGUMENT, "cannot open %s", path);
    const size_t w = fwrite(data.data(), 1, data.size(), fp);
    const int closed = fclose(fp);
    if (w != data.size() || closed != 0) return fail(BBG_ERR_INVALID_ARGUMENT, "short write to %s", path);
    return BBG_OK;
}

bbg_status bbg_checkpoint_load(bbg_solver s, const char *path) {
    if (!path) return fail(BBG_ERR_INVALID_ARGUMENT, "null path");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(BBG_ERR_NOT_FOUND, "cannot open %s", path);
    std::vector<char> data;
    char chunk[1 << 16];
    size_t got;
    while ((got = fread(chunk, 1, sizeof(chunk), fp)) > 0) data.insert(data.end(), chunk, chunk + got);
    fclose(fp);
    return ckpt_restore(s, data.data(), data.size());
}

// ----------------------------------------------------------------------------
// particle frames: reading (SerializerLoadSphDataSet3 / SerializerLoadParticles3)
// ----------------------------------------------------------------------------
namespace {


bbg_status frame_load(bbg_solver s, const char *text, size_t length, int *flags) {
    if (bbg_status r = check_solver(s)) return r;
    if (!text || !flags) return fail(BBG_ERR_INVALID_ARGUMENT, "null text or flags");
    FrameSection sec;
    const int found_section = frame_find_section(text, length, *flags, &sec);
    if (found_section == 1) return fail(BBG_ERR_INVALID_ARGUMENT, "unknown letter in the section's \"Format\"");
    if (found_section == 2)
        return fail(BBG_ERR_INVALID_ARGUMENT, "no complete fluid section (FluidBegin, DataBegin, DataEnd)");
    if (sec.count <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "the section's \"Count\" is %d", sec.count);
    if (sec.count > s->capacity)
        return fail(BBG_ERR_CAPACITY, "%d particles exceed capacity %d", sec.count, s->capacity);
    const size_t bytes = sec.data_end - sec.data_begin;
    if (bytes == 0 || bytes >= 0xffffffffu)
        return fail(BBG_ERR_INVALID_ARGUMENT, "the section's data block has %zu bytes", bytes);
    FrameReadBufs &R = s->fread;
    const size_t chunks = (bytes + kLineChunk - 1) / kLineChunk;
    if (R.text_cap < bytes) {
        R.text_cap = 0;
        if (bbg_status r = reserve(&R.text, bytes)) return r;
        R.text_cap = bytes;
    }
    if (R.chunk_cap < chunks + 1) {
        const size_t need = chunks + 1;
        R.chunk_cap = 0;
        bbg_status r = reserve(&R.chunk, need);
        if (!r) r = reserve(&R.chunk_start, need);
        if (!r) r = reserve(&R.chunk_part, scan_partials_needed((unsigned)need));
        if (r) return r;
        R.chunk_cap = need;
    }
    if (!R.pow5) {
        std::vector<double> p5(kPow5Hi - kPow5Lo + 1), p10(kPow10Max + 1);
        static const double lut[] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
        for (int e = kPow5Lo; e <= kPow5Hi; e++) p5[(size_t)(e - kPow5Lo)] = std::pow(5.0, e);
        for (int r = 0; r <= kPow10Max; r++) p10[(size_t)r] = r < 8 ? lut[r] : std::pow(10.0, -r);
        bbg_status r = reserve(&R.pow10, p10.size());
        if (!r) r = reserve(&R.pow5, p5.size());
        if (r) return r;
        CK(cudaMemcpy(R.pow5, p5.data(), sizeof(double) * p5.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(R.pow10, p10.data(), sizeof(double) * p10.size(), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpyAsync(R.text, text + sec.data_begin, bytes, cudaMemcpyHostToDevice, s->stream));
    unsigned lines = 0;
    CK(frame_split_lines(bytes, R, &lines, s->h_u, s->stream));
    CK_LAUNCH();
    if (R.line_cap < (size_t)lines + 1) {
        const size_t need = (size_t)lines + 1;
        R.line_cap = 0;
        bbg_status r = reserve(&R.line, need);
        if (!r) r = reserve(&R.vals, 6 * need);
        if (!r) r = reserve(&R.valid, need);
        if (!r) r = reserve(&R.flag_copy, need);
        if (!r) r = reserve(&R.index, need);
        if (!r) r = reserve(&R.line_part, scan_partials_needed((unsigned)need));
        if (r) return r;
        R.line_cap = need;
    }
    unsigned found = 0;
    CK(frame_parse_lines(bytes, lines, sec.flags, R, &found, s->h_u, s->stream));
    CK_LAUNCH();
    if (found < (unsigned)sec.count)
        return fail(BBG_ERR_INVALID_ARGUMENT, "the section holds %u particle lines, fewer than its Count %d",
                    found, sec.count);
    float *dp = s->B.stage, *dv = s->B.stage + 3 * (size_t)s->capacity;
    launch_frame_scatter(lines, sec.count, R, dp, dv, s->stream);
    CK_LAUNCH();
    if (bbg_status r = upload_common(s, dp, dv, sec.count)) return r;
    CK(cudaStreamSynchronize(s->stream));
    *flags = sec.flags;
    return BBG_OK;
}

}  // namespace

bbg_status bbg_frame_load_text(bbg_solver s, const char *text, size_t length, int *flags) {
    return frame_load(s, text, length, flags);
}

bbg_status bbg_frame_find_section(const char *text, size_t length, int *flags, int *count, size_t *data_begin,
                                  size_t *data_end) {
    if (!text || !flags) return fail(BBG_ERR_INVALID_ARGUMENT, "null text or flags");
    FrameSection sec;
    const int st = frame_find_section(text, length, *flags, &sec);
    if (st == 1) return fail(BBG_ERR_INVALID_ARGUMENT, "unknown letter in the section's \"Format\"");
    if (st == 2) return fail(BBG_ERR_NOT_FOUND, "no complete fluid section (FluidBegin, DataBegin, DataEnd)");
    *flags = sec.flags;
    if (count) *count = sec.count;
    if (data_begin) *data_begin = sec.data_begin;
    if (data_end) *data_end = sec.data_end;
    return BBG_OK;
}

bbg_status bbg_frame_load(bbg_solver s, const char *path, int *flags) {
    if (bbg_status r = check_solver(s)) return r;
    if (!path || !flags) return fail(BBG_ERR_INVALID_ARGUMENT, "null path or flags");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(BBG_ERR_NOT_FOUND, "cannot open %s", path);
    // read until the first section is complete: files of appended frames can be long
    std::vector<char> data;
    size_t block = (size_t)16 << 20;
    FrameSection sec;
    int st = 2;
    for (;;) {
        const size_t old = data.size();
        data.resize(old + block);
        const size_t got = fread(data.data() + old, 1, block, fp);
        data.resize(old + got);
        st = frame_find_section(data.data(), data.size(), *flags, &sec);
        if (st != 2 || got < block) break;
        block *= 2;
    }
    fclose(fp);
    return frame_load(s, data.data(), data.size(), flags);
}
