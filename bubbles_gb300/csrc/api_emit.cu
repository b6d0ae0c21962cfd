// api_emit.cu -- the C ABI of particle seeding: the volume emitter and continuous
// emission over the grid (VolumeParticleEmitter3, ContinuousParticleSetBuilder3).
#include "api_internal.h"

// ----------------------------------------------------------------------------
// seeding: VolumeParticleEmitter3 (src/core/emitter.cpp:8-12, 241-330)
// ----------------------------------------------------------------------------
bbg_status bbg_emitter_desc_default(bbg_emitter_desc *d) {
    if (!d) return fail(BBG_ERR_INVALID_ARGUMENT, "null desc");
    memset(d, 0, sizeof(*d));
    d->shape.type = BBG_SHAPE_BOX;
    d->shape.size[0] = d->shape.size[1] = d->shape.size[2] = 1.0;
    d->spacing = 0.02;
    d->max_particles = 0x7fffffff;   // IntInfinity
    return BBG_OK;
}

namespace {

// rand_float (src/core/geometry.h:1900-1902): rand() over RAND_MAX + 1 as floats
float rand_float() { return (float)rand() / ((float)RAND_MAX + 1.f); }

// The emitter's lattice: bounds (the shape's, a translated object box, or the given ones,
// ordered like a Bounds3f) and BccLatticePointGenerator::ForEach's loop counts, in the
// reference's float operations.
Lattice emitter_lattice(const bbg_emitter_desc &e) {
    Lattice L;
    float lo[3], hi[3];
    if (e.use_bounds) {
        for (int k = 0; k < 3; k++) {
            const float a = (float)e.bounds_min[k], b = (float)e.bounds_max[k];
            lo[k] = a < b ? a : b;
            hi[k] = a > b ? a : b;
        }
    } else {
        for (int k = 0; k < 3; k++) {
            const float h = e.shape.type == BBG_SHAPE_BOX ? (float)((double)(float)e.shape.size[k] / 2.0)
                                                          : (float)e.shape.size[0];
            const float t = (float)e.shape.center[k];
            lo[k] = -h + t;
            hi[k] = h + t;
        }
    }
    const float sp = (float)e.spacing, half = sp / 2;
    const float width = hi[0] - lo[0], height = hi[1] - lo[1], depth = hi[2] - lo[2];
    auto count = [](float step, float off, float extent) {
        int c = 0;
        while ((float)c * step + off <= extent) c++;
        return c;
    };
    for (int k = 0; k < 3; k++) L.lo[k] = lo[k];
    L.spacing = sp;
    L.half = half;
    L.layers = count(half, 0.f, depth);
    L.i0 = count(sp, 0.f, width);
    L.j0 = count(sp, 0.f, height);
    L.i1 = count(sp, half, width);
    L.j1 = count(sp, half, height);
    const long long s0 = (long long)L.i0 * L.j0, s1 = (long long)L.i1 * L.j1;
    L.total = (long long)(L.layers / 2) * (s0 + s1) + (L.layers % 2 ? s0 : 0);
    return L;
}

// ContinuousParticleSetBuilder3::AddParticle + Commit (grid.h:1404-1437): `count` staged
// particles (positions at stage, velocities at stage + 3 capacity) follow the existing ones
// (ids n .. n + count - 1); the next substep's grid update sorts them in.
bbg_status append_staged(bbg_solver s, int count) {
    float *dp = s->B.stage, *dv = s->B.stage + 3 * (size_t)s->capacity;
    launch_append(s->B, s->state, s->pid_cur, dp, dv, s->n, count, s->stream);
    CK_LAUNCH();
    if (s->mlp_alloc) CK(cudaMemsetAsync(s->mlp.divsum + s->n, 0, sizeof(float) * (size_t)count, s->stream));
    s->n += count;
    s->P.n = s->n;
    s->grid_valid = false;
    s->valid &= kPosVel | bit(BBG_FIELD_FORCE) | bit(BBG_FIELD_PRESSURE_FORCE) | bit(BBG_FIELD_DENSITY) |
                bit(BBG_FIELD_PRESSURE) | bit(BBG_FIELD_INTERACTION);
    s->epoch++;
    return BBG_OK;
}

}  // namespace

bbg_status bbg_emit_volume(bbg_solver s, const bbg_emitter_desc *e, int append, int *emitted) {
    if (bbg_status r = check_solver(s)) return r;
    if (!e) return fail(BBG_ERR_INVALID_ARGUMENT, "null emitter");
    if (e->shape.type != BBG_SHAPE_BOX && e->shape.type != BBG_SHAPE_SPHERE)
        return fail(BBG_ERR_INVALID_ARGUMENT, "emitter shape must be a box or a sphere");
    if (!(e->spacing > 0) || e->max_particles < 0 || !(e->jitter >= 0))
        return fail(BBG_ERR_INVALID_ARGUMENT, "emitter needs spacing > 0, jitter >= 0, max_particles >= 0");
    if (append && s->n > 0 && s->nscenes > 0)
        return fail(BBG_ERR_STATE, "appending to a batch of scenes is not supported");
    // the lattice's extent in spacings, before its loops are counted
    for (int k = 0; k < 3; k++) {
        const double lo = e->use_bounds ? e->bounds_min[k] : e->shape.center[k] - e->shape.size[0] - e->shape.size[k];
        const double hi = e->use_bounds ? e->bounds_max[k] : e->shape.center[k] + e->shape.size[0] + e->shape.size[k];
        if (!std::isfinite(lo) || !std::isfinite(hi) || !(std::fabs(hi - lo) / e->spacing < 4.0e6))
            return fail(BBG_ERR_INVALID_ARGUMENT, "the emitter's bounds are not finite or too many spacings wide");
    }
    const Lattice L = emitter_lattice(*e);
    if (L.total > (1ll << 28))
        return fail(BBG_ERR_CAPACITY, "the emitter's lattice has %lld points (at most 2^28)", L.total);
    const float sp = (float)e->spacing;
    const float max_jitter = (float)(0.5 * (double)(float)e->jitter * (double)sp);
    // the rand() sequence of the reference's loop: two values per lattice point, the
    // second landing in u[0] (vec2f u(rand_float(), rand_float()) as built); the offsets
    // are max_jitter * SampleSphere(u) in float operations
    const size_t P = (size_t)L.total;
    const bool jitter = max_jitter != 0.f;
    std::vector<float> off(jitter ? 3 * P : 0);
    if (!jitter) {
        for (size_t t = 0; t < 2 * P; t++) (void)rand();   // the draws the reference makes anyway
    } else {
        // the draws are sequential; the offsets of disjoint point ranges are computed by
        // the host's threads
        for (size_t t = 0; t < P; t++) {
            off[3 * t + 1] = rand_float();   // u[1]
            off[3 * t] = rand_float();       // u[0]
        }
        auto sample_sphere = [&](size_t lo, size_t hi) {
            for (size_t t = lo; t < hi; t++) {
                const float u1 = off[3 * t + 1], u0 = off[3 * t];
                const float usqrt = 2 * std::sqrt(u1 * (1 - u1));
                const float utheta = (float)(2 * 3.14159265358979323846 * (double)u0);
                off[3 * t] = std::cos(utheta) * usqrt * max_jitter;
                off[3 * t + 1] = std::sin(utheta) * usqrt * max_jitter;
                off[3 * t + 2] = (1 - 2 * u1) * max_jitter;
            }
        };
        const size_t workers = std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), 32));
        if (workers == 1 || P < 65536) {
            sample_sphere(0, P);
        } else {
            std::vector<std::thread> pool;
            const size_t chunk = (P + workers - 1) / workers;
            for (size_t w = 0; w < workers; w++) {
                const size_t lo = w * chunk, hi = std::min(P, lo + chunk);
                if (lo < hi) pool.emplace_back(sample_sphere, lo, hi);
            }
            for (auto &th : pool) th.join();
        }
    }
    int count = 0;
    if (P > 0) {
        EmitBufs &E = s->emit;
        if (E.cap < P + 1) {
            E.cap = 0;
            bbg_status r = reserve(&E.target, 3 * (P + 1));
            if (!r) r = reserve(&E.offset, 3 * (P + 1));
            if (!r) r = reserve(&E.flag, P + 1);
            if (!r) r = reserve(&E.flag_copy, P + 1);
            if (!r) r = reserve(&E.index, P + 1);
            if (!r) r = reserve(&E.part, scan_partials_needed((unsigned)(P + 1)));
            if (r) return r;
            E.cap = P + 1;
        }
        if (jitter) CK(cudaMemcpyAsync(E.offset, off.data(), sizeof(float) * off.size(), cudaMemcpyHostToDevice,
                                       s->stream));
        ShapeDev sd = shape_dev(e->shape);
        unsigned inside = 0;
        CK(emit_test(L, sd, float_above(1e-8), float_above(1e-6), jitter, E, &inside, s->h_u, s->stream));
        CK_LAUNCH();
        count = (int)(inside < (unsigned)e->max_particles ? inside : (unsigned)e->max_particles);
    }
    const int first = append ? s->n : 0;
    if (first + count > s->capacity)
        return fail(BBG_ERR_CAPACITY, "%d particles exceed capacity %d", first + count, s->capacity);
    if (emitted) *emitted = count;
    if (count == 0) return BBG_OK;
    // velocity(target) + initVel with the zero velocity field
    const float3 v = make_float3(0.f + (float)e->initial_velocity[0], 0.f + (float)e->initial_velocity[1],
                                 0.f + (float)e->initial_velocity[2]);
    float *dp = s->B.stage, *dv = s->B.stage + 3 * (size_t)s->capacity;
    launch_emit_scatter(L, count, s->emit, v, dp, dv, s->stream);
    CK_LAUNCH();
    if (!append || s->n == 0) {
        if (bbg_status r = upload_common(s, dp, dv, count)) return r;
    } else if (bbg_status r = append_staged(s, count)) {
        return r;
    }
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

// ----------------------------------------------------------------------------
// continuous emission: ContinuousParticleSetBuilder3::MapGrid / MapGridEmit
// ----------------------------------------------------------------------------
bbg_status bbg_map_grid(bbg_solver s, int *mapped) {
    if (bbg_status r = check_solver(s)) return r;
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    if (s->nscenes > 0) return fail(BBG_ERR_STATE, "continuous emission into a batch of scenes is not supported");
    // the reference maps the cells of the grid's last distribution (its Setup distributes)
    if (!s->grid_valid)
        if (bbg_status r = grid_update(s)) return r;
    MapBufs &M = s->map;
    if (M.cap < s->n + 1) {
        const size_t need = (size_t)s->n + 1;
        M.cap = 0;
        bbg_status r = reserve(&M.pos, need);
        if (!r) r = reserve(&M.cell, need);
        if (!r) r = reserve(&M.rank, need);
        if (!r) r = reserve(&M.flag, need);
        if (!r) r = reserve(&M.flag_copy, need);
        if (!r) r = reserve(&M.index, need);
        if (!r) r = reserve(&M.part, scan_partials_needed((unsigned)need));
        if (r) return r;
        M.cap = (int)need;
    }
    launch_map(s->n, s->B.pos[s->state], s->B.cell, s->B.start, M, s->stream);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s->stream));
    s->map_full = false;
    if (mapped) *mapped = M.count;
    return BBG_OK;
}

bbg_status bbg_map_grid_emit(bbg_solver s, double distance, const double velocity[3], int *emitted) {
    if (bbg_status r = check_solver(s)) return r;
    if (!velocity) return fail(BBG_ERR_INVALID_ARGUMENT, "null velocity");
    MapBufs &M = s->map;
    if (M.count <= 0) return fail(BBG_ERR_STATE, "bbg_map_grid has not been called");
    if (emitted) *emitted = 0;
    if (s->map_full) return BBG_OK;   // the reference's builder stops once it hit its capacity
    // the cells' particles now: the last distribution's sorted ranges plus the particles
    // added since (their cells as Commit's DistributeByParticleList would give them)
    const bool sorted = s->members_ok;
    const int first = sorted ? s->grid_n : 0;
    const bool bucketed = s->n > first;
    BucketBufs &K = s->bucket;
    if (bucketed) {
        const size_t cells = s->P.g.total, m = (size_t)(s->n - first);
        if (K.cells != cells || K.cap < m) {
            K.cells = 0;
            K.cap = 0;
            const size_t mm = std::max(m, (size_t)s->capacity);
            bbg_status r = reserve(&K.count, cells + 1);
            if (!r) r = reserve(&K.start, cells + 1);
            if (!r) r = reserve(&K.part, scan_partials_needed((unsigned)(cells + 1)));
            if (!r) r = reserve(&K.cell, mm);
            if (!r) r = reserve(&K.sub, mm);
            if (!r) r = reserve(&K.list, mm);
            if (r) return r;
            CK(cudaMemsetAsync(K.count, 0, sizeof(unsigned) * (cells + 1), s->stream));
            K.cells = cells;
            K.cap = mm;
        }
        launch_buckets(s->P, s->B.pos[s->state], first, s->n, K, s->stream);
        CK_LAUNCH();
    }
    unsigned passed = 0;
    CK(map_emit_test(M, sorted, s->B.start, bucketed, K, s->B.pos[s->state], (float)distance, &passed, s->h_u,
                     s->stream));
    CK_LAUNCH();
    const unsigned room = (unsigned)(s->capacity - s->n);
    const int count = (int)(passed < room ? passed : room);
    if (passed > room) s->map_full = true;
    if (count > 0) {
        const float3 v = make_float3((float)velocity[0], (float)velocity[1], (float)velocity[2]);
        launch_map_scatter(M, count, v, s->B.stage, s->B.stage + 3 * (size_t)s->capacity, s->stream);
        CK_LAUNCH();
        if (bbg_status r = append_staged(s, count)) return r;
    }
    CK(cudaStreamSynchronize(s->stream));
    if (emitted) *emitted = count;
    return BBG_OK;
}
