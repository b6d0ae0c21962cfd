// api.cu -- the C ABI of bubbles_gb300 (include/bbg.h): solver lifetime, the substep
// launch sequences, field access, the learned warm start's controls and launch tuning.
// Host code only; kernels live in grid.cu and sph.cu.  Batches, frames and checkpoints,
// seeding and post-processing are in api_batch.cu, api_io.cu, api_emit.cu and api_post.cu.
#include "api_internal.h"

namespace bbg_api {

thread_local char g_err[512] = "";

bbg_status fail(bbg_status code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

// Host-side fault injection for tests, off unless the environment sets BBG_FAIL_ALLOC_AFTER:
// the device allocation after that many successful ones (counted per process) fails as
// cudaMalloc does when memory runs out.
long alloc_fault_budget() {
    static const long budget = [] {
        const char *e = getenv("BBG_FAIL_ALLOC_AFTER");
        return e ? atol(e) : -1L;
    }();
    return budget;
}
long alloc_count = 0;

}  // namespace bbg_api

namespace bbg {
int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
}  // namespace bbg

namespace bbg_api {

bbg_status check_solver(bbg_solver s) {
    if (!s) return fail(BBG_ERR_INVALID_ARGUMENT, "null solver");
    return BBG_OK;
}

void fill_params(bbg_solver s) {
    Params &P = s->P;
    const bbg_solver_desc &d = s->desc;
    P.n = s->n;
    P.mass = s->mass;
    P.radius = (float)d.target_spacing;
    P.h = s->kernel_radius;
    P.h2 = P.h * P.h;
    P.inv_h = 1.0f / P.h;
    P.inv_h2 = 1.0f / P.h2;
    P.target_density = (float)d.target_density;
    P.iz = float_above(1e-8);
    P.iz6 = float_above(1e-6);
    const double T = (double)P.h2 - (double)P.iz;
    float lo = (float)(T * (1.0 - 1e-6));
    if ((double)lo > T * (1.0 - 1e-6)) lo = nextafterf(lo, 0.f);
    float hi = (float)(T * (1.0 + 1e-6));
    if ((double)hi < T * (1.0 + 1e-6)) hi = nextafterf(hi, 3.4e38f);
    P.nb_lo = lo;
    P.nb_hi = hi;
    P.h2mz = (float)T;
    // margin of the density pass's reach test: far above the rounding of positions and cell
    // faces (64 ulps of the largest grid coordinate) and the reference hash's 1e-4 nudge of
    // particles on the grid's bounds
    float cmax = 0.f;
    const int dn[3] = {P.g.nx, P.g.ny, P.g.nz};
    for (int k = 0; k < 3; k++) {
        const float top = P.g.minp[k] + (float)dn[k] * P.g.len[k];
        cmax = fmaxf(cmax, fmaxf(fmaxf(fabsf(P.g.bmin[k]), fabsf(P.g.bmax[k])), fmaxf(fabsf(P.g.minp[k]), fabsf(top))));
    }
    P.prune_m = fmaxf(fmaxf(1e-3f * P.h, 1.5e-4f), 64.f * cmax * 1.1920929e-7f);
    const double kPi = 3.14159265358979323846;
    const float h3 = P.h2 * P.h, h4 = P.h2 * P.h2, h5 = P.h2 * h3;
    P.std_c = (float)(315.0 / (64.0 * kPi * (double)h3));
    P.spiky_dw_c = (float)(45.0 / (kPi * (double)h4));
    P.spiky_d2w_c = (float)(90.0 / (kPi * (double)h5));
    P.spiky_w_c = (float)(15.0 / (kPi * (double)h3));
    const float visc = (float)d.viscosity > 0 ? (float)d.viscosity : 0.f;
    P.m2 = P.mass * P.mass;
    P.visc_m2 = visc * P.m2;
    P.drag = (float)d.drag_coefficient;
    P.gx = (float)d.gravity[0];
    P.gy = (float)d.gravity[1];
    P.gz = (float)d.gravity[2];
    const float rho0 = (float)d.target_density, c = (float)d.sound_speed;
    const float eosScale = rho0 * c * c;
    P.eos_scale_over_exp = eosScale / (float)d.eos_exponent;
    P.eos_exp = (float)d.eos_exponent;
    P.neg_scale = (float)d.negative_pressure_scale;
    P.rest_int = 0.6f;
    P.rest_c1_int = (float)(-1.0 - (double)0.6f);
    P.max_err_ratio = (float)d.max_density_error_ratio;
}

cudaError_t scratch_begin(bbg_solver s) {
    ScratchArena &a = s->scratch;
    if (a.want > a.cap || !a.extra.empty()) {
        // the previous call overflowed: one block of its total from here on
        for (void *p : a.extra) cudaFree(p);
        a.extra.clear();
        const size_t need = a.want > a.cap ? a.want : a.cap;
        if (a.base) cudaFree(a.base);
        a.base = nullptr;
        a.cap = 0;
        const cudaError_t e = cudaMalloc((void **)&a.base, need);
        if (e != cudaSuccess) {
            a.base = nullptr;
            a.want = 0;
            return e;
        }
        a.cap = need;
    }
    a.used = 0;
    a.want = 0;
    return cudaSuccess;
}

cudaError_t scratch_bytes(bbg_solver s, size_t bytes, void **out) {
    ScratchArena &a = s->scratch;
    const size_t b = (bytes + 255) & ~(size_t)255;   // 256-byte aligned buffers
    a.want += b;
    if (a.base && a.used + b <= a.cap) {
        *out = a.base + a.used;
        a.used += b;
        return cudaSuccess;
    }
    void *p = nullptr;
    const cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        *out = nullptr;
        return e;
    }
    a.extra.push_back(p);
    *out = p;
    return cudaSuccess;
}

void scratch_free(bbg_solver s) {
    ScratchArena &a = s->scratch;
    for (void *p : a.extra) cudaFree(p);
    a.extra.clear();
    if (a.base) cudaFree(a.base);
    a = ScratchArena();
}

void drop_graphs(bbg_solver s) {
    for (auto &g : s->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
        g = bbg_solver_s::SubstepGraph();
    }
}

void free_mlp(bbg_solver s);

// Detaches and frees the colliders' signed-distance fields.
void free_fields(bbg_solver s) {
    for (int k = 0; k < kMaxSdf; k++) {
        if (s->sdf_values[k]) cudaFree(s->sdf_values[k]);
        s->sdf_values[k] = nullptr;
        s->P.sdf[k] = SdfDev();
    }
    for (int i = 0; i < kMaxColliders; i++) s->P.shapes[i].sdf = -1;
    s->nsdf = 0;
    s->P.has_sdf = 0;
}

void free_frame(bbg_solver s) {
    FrameBufs &F = s->frame;
    void *ptrs[] = {F.lines, F.lens, F.scan_in, F.offset, F.partials, F.out};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    F = FrameBufs();
    FrameReadBufs &R = s->fread;
    void *rptrs[] = {R.text, R.chunk, R.chunk_start, R.chunk_part, R.line, R.vals, R.valid, R.flag_copy,
                     R.index, R.line_part, R.pow5, R.pow10};
    for (void *p : rptrs)
        if (p) cudaFree(p);
    R = FrameReadBufs();
    EmitBufs &E = s->emit;
    void *eptrs[] = {E.target, E.offset, E.flag, E.flag_copy, E.index, E.part};
    for (void *p : eptrs)
        if (p) cudaFree(p);
    E = EmitBufs();
    MapBufs &M = s->map;
    void *mptrs[] = {M.pos, M.cell, M.rank, M.flag, M.flag_copy, M.index, M.part};
    for (void *p : mptrs)
        if (p) cudaFree(p);
    M = MapBufs();
    BucketBufs &K = s->bucket;
    void *kptrs[] = {K.count, K.start, K.part, K.cell, K.sub, K.list};
    for (void *p : kptrs)
        if (p) cudaFree(p);
    K = BucketBufs();
    free_fields(s);
}

bbg_status free_all(bbg_solver s) {
    drop_graphs(s);
    scratch_free(s);
    free_mlp(s);
    free_frame(s);
    if (s->d_stage2) cudaFree(s->d_stage2);
    s->d_stage2 = nullptr;
    void *batch[] = {s->d_zb, s->d_box, s->d_sst, s->d_scene, s->d_wl};
    for (void *p : batch)
        if (p) cudaFree(p);
    s->d_zb = nullptr;
    s->d_box = nullptr;
    s->d_sst = nullptr;
    s->d_scene = nullptr;
    s->d_wl = nullptr;
    DevBufs &B = s->B;
    void *ptrs[] = {B.pos[0], B.pos[1], B.vel[0], B.vel[1], B.pid[0], B.pid[1], B.slot, B.force,
                    B.xstar, B.pforce, B.smoothed, B.rho, B.press, B.rhostar, B.derr, B.cell,
                    B.cell_old, B.sub, B.count, B.start, B.partials, B.tmp, B.nbr, B.st, B.stage,
                    B.red, B.list, B.inv_rho, B.pprev, B.soa};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    Prof *keep = B.prof;
    const Tuning tune = B.tune;
    B = DevBufs();
    B.prof = keep;
    B.tune = tune;
    if (s->h_st) cudaFreeHost(s->h_st);
    if (s->h_u) cudaFreeHost(s->h_u);
    s->h_st = nullptr;
    s->h_u = nullptr;
    return BBG_OK;
}

void free_mlp(bbg_solver s) {
    MlpBufs &M = s->mlp;
    void *ptrs[] = {M.theta, M.grad, M.lpart, M.m1, M.m2, M.w1f, M.w2f, M.tail, M.step, M.loss, M.feat, M.divsum,
                    M.divprev, M.bx, M.bt};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    M = MlpBufs();
    s->mlp_alloc = false;
}

// Glorot-uniform weights, zero biases (FP32 master copy on the host, then uploaded).
std::vector<float> mlp_initial_params(unsigned long long seed) {
    std::vector<float> th(kParams, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fan_in, int fan_out, int count) {
        const float a = sqrtf(6.f / (float)(fan_in + fan_out));
        std::uniform_real_distribution<float> u(-a, a);
        for (int k = 0; k < count; k++) th[off + k] = u(rng);
    };
    fill(kOffW1, kIn, kHid, kIn * kHid);
    fill(kOffW2, kHid, kHid, kHid * kHid);
    fill(kOffW3, kHid, 1, kHid);
    return th;
}

bbg_status mlp_allocate(bbg_solver s, const bbg_mlp_desc &d) {
    if (d.batch < 1 || d.train_substeps < 0 || d.steps_per_substep < 0 || d.finetune_steps < 0 ||
        !(d.learning_rate > 0) ||
        !(d.expectile > 0 && d.expectile < 1))
        return fail(BBG_ERR_INVALID_ARGUMENT, "invalid MLP training settings");
    CK(cudaStreamSynchronize(s->stream));
    if (!s->mlp_alloc || s->mlp.batch != d.batch) {
        free_mlp(s);
        MlpBufs &M = s->mlp;
        const size_t n = (size_t)s->capacity;
        bbg_status r = BBG_OK;
#define ALLOC(ptr, cnt) if (!r) r = dalloc(&(ptr), (cnt))
        ALLOC(M.theta, kParams); ALLOC(M.grad, (size_t)kGradRows * kParams); ALLOC(M.lpart, kGradRows); ALLOC(M.m1, kParams); ALLOC(M.m2, kParams);
        ALLOC(M.w1f, 8 * 32); ALLOC(M.w2f, 64 * 32); ALLOC(M.tail, kTail); ALLOC(M.step, 1);
        ALLOC(M.loss, 1); ALLOC(M.feat, n); ALLOC(M.divsum, n); ALLOC(M.divprev, n);
        ALLOC(M.bx, (size_t)d.batch);
        ALLOC(M.bt, (size_t)d.batch);
#undef ALLOC
        if (r) {
            free_mlp(s);
            return r;
        }
        CK(mlp_prepare());
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->desc.device));
        M.infer_blocks = kMlpBlocksPerSm * (sms > 0 ? sms : 1);   // the blocks of 128 threads an SM holds
        M.batch = d.batch;
        s->mlp_alloc = true;
    }
    s->mdesc = d;
    const std::vector<float> th = mlp_initial_params(d.seed);
    MlpBufs &M = s->mlp;
    CK(cudaMemcpyAsync(M.theta, th.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(M.m1, 0, sizeof(float) * kParams, s->stream));
    CK(cudaMemsetAsync(M.m2, 0, sizeof(float) * kParams, s->stream));
    CK(cudaMemsetAsync(M.step, 0, sizeof(unsigned), s->stream));
    CK(cudaMemsetAsync(M.loss, 0, sizeof(double), s->stream));
    CK(cudaMemsetAsync(M.feat, 0, sizeof(float4) * (size_t)s->capacity, s->stream));
    CK(cudaMemsetAsync(M.divsum, 0, sizeof(float) * (size_t)s->capacity, s->stream));
    CK(cudaMemsetAsync(M.divprev, 0, sizeof(float) * (size_t)s->capacity, s->stream));
    CK(cudaMemsetAsync(M.tail, 0, sizeof(float) * kTail, s->stream));
    launch_mlp_pack(M, s->stream);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s->stream));
    s->mlp_trained = 0;
    s->mlp_since = 0;
    s->epoch++;
    return BBG_OK;
}

// MakeBox / MakeSphere parameters as the device evaluates them (FP32, half sizes from
// the FP32 size as Box3 computes them).
ShapeDev shape_dev(const bbg_shape &sh) {
    ShapeDev d;
    d.type = sh.type;
    d.reverse = sh.reverse ? 1 : 0;
    for (int k = 0; k < 3; k++) d.t[k] = (float)sh.center[k];
    d.hx = (float)((double)(float)sh.size[0] / 2.0);
    d.hy = (float)((double)(float)sh.size[1] / 2.0);
    d.hz = (float)((double)(float)sh.size[2] / 2.0);
    d.radius = (float)sh.size[0];
    d.friction = (float)sh.friction;
    d.sdf = -1;
    return d;
}

bbg_status require_grid(bbg_solver s) {
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    if (!s->grid_valid) return fail(BBG_ERR_STATE, "no grid distribution yet (call bbg_update_grid_distribution)");
    return BBG_OK;
}

bbg_status reset_step_state(bbg_solver s) {
    CK(cudaMemsetAsync(s->B.st, 0, sizeof(StepState), s->stream));
    if (s->nscenes > 0)
        CK(cudaMemsetAsync(s->d_sst, 0, sizeof(SceneState) * (size_t)s->nscenes, s->stream));
    return BBG_OK;
}

// The other ping-pong buffer becomes the current state (an integration wrote into it); if
// it held the positions of the last density pass, the neighbour sets can no longer be
// exported.
void flip_state(bbg_solver s) {
    s->state = 1 - s->state;
    if (s->list_state == s->state) s->list_state = -1;
}

bbg_status grid_update(bbg_solver s) {
    bbg_status r = reset_step_state(s);
    if (r) return r;
    launch_grid_update(s->P, s->B, s->state, s->pid_cur, s->stream, s->mlp.divsum, s->mlp.divprev);
    CK_LAUNCH();
    s->list_state = -1;
    s->state = 1 - s->state;
    s->pid_cur = 1 - s->pid_cur;
    s->grid_valid = true;
    s->grid_n = s->n;
    s->members_ok = true;
    s->valid = kPosVel | bit(BBG_FIELD_INTERACTION);
    return BBG_OK;
}

// Iterations used by the last corrector, from the per-iteration maxima (host copy).
int iterations_from(const bbg_solver s, const StepState *st, int max_it, float tol, float *err_out,
                    double *mean_out) {
    int it = max_it;
    for (int k = 0; k < max_it; k++) {
        float e;
        memcpy(&e, &st->err_bits[k], 4);
        if (e / s->P.target_density < tol || k == max_it - 1) {
            it = k + 1;
            *err_out = e / s->P.target_density;
            *mean_out = st->err_sum[k] / (double)s->n / (double)s->P.target_density;
            break;
        }
    }
    return it;
}

bbg_status read_step_state(bbg_solver s) {
    CK(cudaMemcpyAsync(s->h_st, s->B.st, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

void add_substep_stats(bbg_solver s, float dt) {
    bbg_step_stats &a = s->acc;
    const StepState *st = s->h_st;
    a.substeps += 1;
    a.last_dt = dt;
    if (s->desc.solver_kind == BBG_SOLVER_PCISPH) {
        float err = 0;
        double mean = 0;
        int it = iterations_from(s, st, s->last_max_it, s->last_tol, &err, &mean);
        s->prof.mark_iterations(it);
        a.iterations += it;
        if (it > a.max_iterations_in_substep) a.max_iterations_in_substep = it;
        if (!(err < s->last_tol) && s->desc.pcisph_mode == BBG_PCISPH_TOLERANCE) a.not_converged += 1;
        a.max_density_error_ratio = err;
        a.mean_density_error_ratio = mean;
    }
    a.neighbor_overflow = (int)st->nbr_overflow;
    a.out_of_grid = (int)st->out_of_grid;
    a.crowded = (int)st->crowded;
    a.nonfinite = (int)st->nonfinite;
    float f;
    memcpy(&f, &st->max_force_bits, 4);
    a.max_force = f;
}

// Learned warm start: 0 off, 1 a training substep (plain corrector, then training on its
// pairs), 2 an inference substep (corrector started from the model's estimate).
int mlp_mode(bbg_solver s) {
    if (s->desc.pressure_init != BBG_PRESSURE_INIT_LEARNED || s->desc.solver_kind != BBG_SOLVER_PCISPH)
        return 0;
    if (s->mlp_trained < s->mdesc.train_substeps) return 1;
    // refresh: every refresh_interval-th substep after training runs plain and trains again
    if (s->mdesc.refresh_interval > 0 && s->mlp_since >= s->mdesc.refresh_interval) return 1;
    return 2;
}

// Bookkeeping after a substep has been launched in mode mm.
void mlp_after_substep(bbg_solver s, int mm) {
    if (mm == 1) {
        if (s->mlp_trained < s->mdesc.train_substeps) s->mlp_trained++;
        s->mlp_since = 0;
    } else if (mm == 2) {
        s->mlp_since++;
    }
}

bool warm_active(bbg_solver s) {
    return s->desc.pressure_init == BBG_PRESSURE_INIT_PREVIOUS || mlp_mode(s) == 2;
}

// Warm-started correctors with the CLAMP_TOTAL rule let the pressure decrease.
int clamp_total(bbg_solver s) {
    return warm_active(s) && s->desc.warm_rule == BBG_WARM_CLAMP_TOTAL;
}

// Start pressure = warm_scale * estimate; a scale <= 0 picks the measured defaults (the
// monotone update cannot lower an overestimated start, so the estimate is damped: the
// carried pressure by half, the learned one by a tenth).
float warm_scale(bbg_solver s) {
    if (s->desc.warm_scale > 0) return (float)s->desc.warm_scale;
    return s->desc.pressure_init == BBG_PRESSURE_INIT_LEARNED ? 0.9f : 0.5f;
}

// Pressure a corrector step assigns to a 1 % density error (the MLP's pressure unit).
float pressure_unit(bbg_solver s, float delta) { return delta * s->P.target_density * 0.01f; }

// Launches of a substep between the density pass and the corrector loop.
void launch_prologue(bbg_solver s, int work, float dt, float delta, int max_it, cudaStream_t cs) {
    (void)max_it;
    const Params &P = s->P;
    const DevBufs &B = s->B;
    const int mm = mlp_mode(s);
    const bool warm = warm_active(s);
    // the warm start (start pressure, pos.w = p / rho^2) precedes the force pass, which then
    // also sums the start's pressure force and predicts x* from F + Fp
    if (mm) launch_mlp_features(P, B, s->mlp, work, dt, pressure_unit(s, delta), cs);
    if (warm) {
        if (mm == 2) launch_mlp_warm_start(P, B, s->mlp, work, pressure_unit(s, delta), warm_scale(s), cs);
        else launch_warm_start(P, B, work, warm_scale(s), cs);
    }
    launch_non_pressure(P, B, work, 1, dt, dt / s->mass, cs, mm ? s->mlp.divsum : nullptr, warm);
}

// After a training substep's corrector: Adam steps on pairs of the converged state.
// (A learned substep runs finetune_steps of them on its own converged pressure.)
int training_steps(bbg_solver s) {
    const int mm = mlp_mode(s);
    return mm == 1 ? s->mdesc.steps_per_substep : mm == 2 ? s->mdesc.finetune_steps : 0;
}

void launch_training(bbg_solver s, float delta, cudaStream_t cs) {
    const bbg_mlp_desc &d = s->mdesc;
    const int steps = training_steps(s);
    cudaMemsetAsync(s->mlp.loss, 0, sizeof(double), cs);
    s->mlp_loss_count = (double)s->mlp.batch * (double)(steps > 0 ? steps : 1);
    for (int k = 0; k < steps; k++) {
        launch_mlp_collect(s->P, s->B, s->mlp, pressure_unit(s, delta), cs);
        launch_mlp_train_step(s->mlp, s->mlp.bx, s->mlp.bt, s->mlp.batch, (float)d.learning_rate,
                              (float)d.beta1, (float)d.beta2, (float)d.epsilon, (float)d.expectile, cs);
    }
}

// Corrector loop of ComputePressureForceAndIntegrate launched from the host: after each
// iteration the host reads that iteration's max density error, as the reference's loop
// does (pcisph_equations3.cpp:238-246), and stops once it is below tolerance.  The
// kernels take the same decision on the device.  (Substeps normally run as CUDA graphs
// whose conditional WHILE node keeps this loop on the device.)
bbg_status corrector(bbg_solver s, float dt, float delta, int max_it) {
    if (max_it < 1) max_it = 1;
    if (max_it > kMaxIterations) max_it = kMaxIterations;
    const float dt_over_m = dt / s->mass;
    s->last_max_it = max_it;
    s->last_tol = s->P.max_err_ratio;
    for (int k = 0; k < max_it; k++) {
        launch_pred_density(s->P, s->B, s->state, k, delta, s->stream, clamp_total(s));
        launch_pressure_force(s->P, s->B, s->state, k, max_it, dt, dt_over_m, s->stream);
        CK_LAUNCH();
        if (k == max_it - 1) break;
        CK(cudaMemcpyAsync(s->h_u, &s->B.st->err_bits[k], 4, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        float e;
        memcpy(&e, s->h_u, 4);
        if (e / s->P.target_density < s->P.max_err_ratio) break;
    }
    flip_state(s);
    s->valid |= kPosVel | bit(BBG_FIELD_FORCE) | bit(BBG_FIELD_PRESSURE) |
                bit(BBG_FIELD_PRESSURE_FORCE) | bit(BBG_FIELD_PRED_DENSITY) |
                bit(BBG_FIELD_DENSITY_ERROR) | bit(BBG_FIELD_PRED_POSITION);
    return BBG_OK;
}

bbg_status pseudo_viscosity(bbg_solver s, float dt) {
    const float scale = (float)s->desc.pseudo_viscosity * dt;
    if (scale > 0.1) {
        float t = dt * (float)s->desc.pseudo_viscosity;
        t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
        launch_pseudo_viscosity(s->P, s->B, s->state, t, s->stream);
        CK_LAUNCH();
    }
    return BBG_OK;
}

unsigned fbits(float f) {
    unsigned u;
    memcpy(&u, &f, 4);
    return u;
}

// Capture one whole substep (grid rebuild, density, forces, the corrector as a
// conditional WHILE node driven by k_corrector_control, integration) into a graph.
bbg_status capture_substep(bbg_solver s, float dt, int max_it, float delta,
                           bbg_solver_s::SubstepGraph &g) {
    const int st0 = s->state, pid0 = s->pid_cur, work = 1 - st0;
    const Params &P = s->P;
    const DevBufs &B = s->B;
    cudaStream_t cs = s->stream;
    if (!s->aux) CK(cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(B.st, 0, sizeof(StepState), cs);
    if (e == cudaSuccess && s->nscenes > 0)
        e = cudaMemsetAsync(s->d_sst, 0, sizeof(SceneState) * (size_t)s->nscenes, cs);
    launch_grid_update(P, B, st0, pid0, cs, s->mlp.divsum, s->mlp.divprev);
    if (s->desc.solver_kind == BBG_SOLVER_SPH) {
        launch_density(P, B, work, 1, cs);
        launch_sph_forces(P, B, work, dt, cs);
    } else {
        launch_density(P, B, work, 0, cs);
        launch_prologue(s, work, dt, delta, max_it, cs);
        cudaStreamCaptureStatus status;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;
        size_t ndeps = 0;
        cudaGraphConditionalHandle handle = 0;
        cudaGraphNode_t cnode = nullptr;
        if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(cs, &status, nullptr, &cg, &deps, &edges, &ndeps);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&handle, cg, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
        np.conditional.handle = handle;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        if (e == cudaSuccess) e = cudaGraphAddNode(&cnode, cg, deps, edges, ndeps, &np);
        if (e == cudaSuccess) {
            cudaGraph_t body = np.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(s->aux, body, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                launch_pred_density(P, B, work, -1, delta, s->aux, clamp_total(s));
                launch_pressure_force(P, B, work, -1, max_it, dt, dt / s->mass, s->aux);
                launch_corrector_control(P, B, max_it, handle, s->aux);
                cudaError_t e2 = cudaStreamEndCapture(s->aux, &body);
                if (e == cudaSuccess) e = e2;
            }
        }
        if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cs, &cnode, nullptr, 1,
                                                                      cudaStreamSetCaptureDependencies);
        if (training_steps(s) > 0) launch_training(s, delta, cs);
    }
    const float pv = (float)s->desc.pseudo_viscosity * dt;
    if (pv > 0.1) {
        float t = dt * (float)s->desc.pseudo_viscosity;
        t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
        launch_pseudo_viscosity(P, B, st0, t, cs);
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e3 = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e3;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return fail(BBG_ERR_CUDA, "substep graph capture: %s", cudaGetErrorString(e));
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return fail(BBG_ERR_CUDA, "substep graph instantiate: %s", cudaGetErrorString(e));
    }
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    g.graph = graph;
    g.exec = exec;
    g.valid = true;
    return BBG_OK;
}

void after_substep(bbg_solver s, float dt) {
    (void)dt;
    s->pid_cur = 1 - s->pid_cur;
    s->grid_valid = true;
    s->grid_n = s->n;
    s->members_ok = true;
    s->list_state = 1 - s->state;   // the graph's density pass ran on the other buffer
    s->valid = kPosVel | bit(BBG_FIELD_INTERACTION) | bit(BBG_FIELD_DENSITY) | bit(BBG_FIELD_FORCE) |
               bit(BBG_FIELD_PRESSURE);
    if (s->desc.solver_kind == BBG_SOLVER_PCISPH)
        s->valid |= bit(BBG_FIELD_PRESSURE_FORCE) | bit(BBG_FIELD_PRED_DENSITY) |
                    bit(BBG_FIELD_DENSITY_ERROR) | bit(BBG_FIELD_PRED_POSITION);
}

bbg_status substep(bbg_solver s, float dt) {
    for (int i = 0; i < s->P.nshapes; i++)
        if (s->P.shapes[i].type == BBG_SHAPE_SDF && s->P.shapes[i].sdf < 0)
            return fail(BBG_ERR_STATE, "collider %d is a field-only shape without a field", i);
    s->prof.substep++;
    const bool shipped = s->desc.pcisph_mode == BBG_PCISPH_AS_SHIPPED;
    int max_it = shipped ? 1 : s->desc.max_iterations;
    if (max_it < 1) max_it = 1;
    if (max_it > kMaxIterations) max_it = kMaxIterations;
    s->P.max_err_ratio = shipped ? 0.01f : (float)s->desc.max_density_error_ratio;
    const float delta = compute_delta(s->mod2, s->delta_denom, dt);
    if (s->use_graphs && !s->prof.on) {
        bbg_solver_s::SubstepGraph *hit = nullptr;
        for (auto &g : s->graphs)
            if (g.valid && g.epoch == s->epoch && g.dt_bits == fbits(dt) && g.state == s->state &&
                g.pid == s->pid_cur && g.max_it == max_it && g.tol_bits == fbits(s->P.max_err_ratio) &&
                g.variant == mlp_mode(s))
                hit = &g;
        if (!hit) {
            hit = &s->graphs[s->graph_next];
            s->graph_next = (s->graph_next + 1) % 8;
            bbg_status r = capture_substep(s, dt, max_it, delta, *hit);
            if (r) return r;
            hit->epoch = s->epoch;
            hit->dt_bits = fbits(dt);
            hit->state = s->state;
            hit->pid = s->pid_cur;
            hit->max_it = max_it;
            hit->tol_bits = fbits(s->P.max_err_ratio);
            hit->variant = mlp_mode(s);
        }
        const int mm = mlp_mode(s);
        CK(cudaGraphLaunch(hit->exec, s->stream));
        mlp_after_substep(s, mm);
        s->last_max_it = max_it;
        s->last_tol = s->P.max_err_ratio;
        after_substep(s, dt);
        return BBG_OK;
    }
    bbg_status r = grid_update(s);
    if (r) return r;
    if (s->desc.solver_kind == BBG_SOLVER_SPH) {
        launch_density(s->P, s->B, s->state, 1, s->stream);
        launch_sph_forces(s->P, s->B, s->state, dt, s->stream);
        CK_LAUNCH();
        s->list_state = s->state;
        flip_state(s);
        s->valid |= kPosVel | bit(BBG_FIELD_DENSITY) | bit(BBG_FIELD_PRESSURE) | bit(BBG_FIELD_FORCE);
        return pseudo_viscosity(s, dt);
    }
    launch_density(s->P, s->B, s->state, 0, s->stream);
    launch_prologue(s, s->state, dt, delta, max_it, s->stream);
    CK_LAUNCH();
    s->list_state = s->state;
    s->valid |= bit(BBG_FIELD_DENSITY) | bit(BBG_FIELD_FORCE);
    r = corrector(s, dt, delta, max_it);
    if (r) return r;
    if (training_steps(s) > 0) {
        launch_training(s, delta, s->stream);
        CK_LAUNCH();
    }
    mlp_after_substep(s, mlp_mode(s));
    return pseudo_viscosity(s, dt);
}

bbg_status max_force(bbg_solver s, float *out) {
    if (!(s->valid & bit(BBG_FIELD_FORCE))) return fail(BBG_ERR_STATE, "forces not valid");
    launch_max_force(s->B.force, s->n, s->B.red, s->stream);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(s->h_u, s->B.red, 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    memcpy(out, s->h_u, 4);
    return BBG_OK;
}

int field_components(int f) {
    switch (f) {
        case BBG_FIELD_POSITION: case BBG_FIELD_VELOCITY: case BBG_FIELD_FORCE:
        case BBG_FIELD_INTERACTION: case BBG_FIELD_PRED_POSITION: case BBG_FIELD_PRESSURE_FORCE:
            return 3;
        case BBG_FIELD_DENSITY: case BBG_FIELD_PRESSURE: case BBG_FIELD_PRED_DENSITY:
        case BBG_FIELD_DENSITY_ERROR: case BBG_FIELD_DIVERGENCE:
            return 1;
        default:
            return 0;
    }
}

float4 *vec_field(bbg_solver s, int f) {
    switch (f) {
        case BBG_FIELD_POSITION: return s->B.pos[s->state];
        case BBG_FIELD_VELOCITY: return s->B.vel[s->state];
        case BBG_FIELD_FORCE: return s->B.force;
        case BBG_FIELD_PRED_POSITION: return s->B.xstar;
        case BBG_FIELD_PRESSURE_FORCE: return s->B.pforce;
        default: return nullptr;
    }
}

float *scalar_field(bbg_solver s, int f) {
    switch (f) {
        case BBG_FIELD_DENSITY: return s->B.rho;
        case BBG_FIELD_PRESSURE: return s->B.press;
        case BBG_FIELD_PRED_DENSITY: return s->B.rhostar;
        case BBG_FIELD_DENSITY_ERROR: return s->B.derr;
        case BBG_FIELD_DIVERGENCE: return s->mlp_alloc ? s->mlp.divsum : nullptr;
        default: return nullptr;
    }
}

}  // namespace bbg_api

// ============================================================================
// C ABI
// ============================================================================
bbg_status bbg_api::upload_common(bbg_solver s, const float *d_pos, const float *d_vel, int n) {
    launch_upload(s->B, s->state, s->pid_cur, d_pos, d_vel, n, s->stream);
    CK_LAUNCH();
    if (s->mlp_alloc)   // no previous substep: no divergence to carry (bbg_set_field can set it)
        CK(cudaMemsetAsync(s->mlp.divsum, 0, sizeof(float) * (size_t)n, s->stream));
    if (n != s->n) s->epoch++;   // captured launches depend on n, not on the data
    s->n = n;
    s->P.n = n;
    s->grid_valid = false;
    s->members_ok = false;
    s->list_state = -1;
    s->valid = kPosVel | bit(BBG_FIELD_FORCE) | bit(BBG_FIELD_PRESSURE_FORCE) |
               bit(BBG_FIELD_DENSITY) | bit(BBG_FIELD_PRESSURE) | bit(BBG_FIELD_INTERACTION);
    return BBG_OK;
}

extern "C" {

const char *bbg_version(void) { return "bubbles_gb300 0.1 (sm_103a)"; }

const char *bbg_status_string(bbg_status s) {
    switch (s) {
        case BBG_OK: return "ok";
        case BBG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case BBG_ERR_CUDA: return "CUDA error";
        case BBG_ERR_OUT_OF_MEMORY: return "out of device memory";
        case BBG_ERR_CAPACITY: return "capacity exceeded";
        case BBG_ERR_STATE: return "invalid solver state";
        case BBG_ERR_NO_DEVICE: return "no CUDA device";
        case BBG_ERR_NOT_FOUND: return "not found";
        default: return "unknown status";
    }
}

const char *bbg_last_error(void) { return g_err; }

bbg_status bbg_device_count(int *count) {
    if (!count) return fail(BBG_ERR_INVALID_ARGUMENT, "null count");
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        c = 0;
    }
    *count = c;
    return BBG_OK;
}

bbg_status bbg_solver_desc_default(bbg_solver_desc *d, int kind) {
    if (!d) return fail(BBG_ERR_INVALID_ARGUMENT, "null desc");
    if (kind != BBG_SOLVER_PCISPH && kind != BBG_SOLVER_SPH)
        return fail(BBG_ERR_INVALID_ARGUMENT, "unknown solver kind %d", kind);
    memset(d, 0, sizeof(*d));
    d->solver_kind = kind;
    d->eos_exponent = 7.0;
    d->negative_pressure_scale = 0.0;
    d->viscosity = 0.04;
    d->pseudo_viscosity = 10.0;
    d->sound_speed = 100.0;
    d->drag_coefficient = 0.0001;
    d->gravity[0] = 0.0;
    d->gravity[1] = (double)-9.8f;   // vec3f(0.f, -9.8f, 0.f)
    d->gravity[2] = 0.0;
    d->target_density = 1000.0;
    d->target_spacing = 0.1;
    d->relative_kernel_radius = 2.0;
    d->mass = 0.0;
    d->grid_spacing_scale = 2.0;
    d->time_step_limit_scale = kind == BBG_SOLVER_PCISPH ? 5.0 : 1.0;
    d->pcisph_mode = BBG_PCISPH_AS_SHIPPED;
    d->max_iterations = 5;
    d->max_density_error_ratio = 0.01;
    d->device = 0;
    d->pressure_init = BBG_PRESSURE_INIT_ZERO;
    d->warm_rule = BBG_WARM_MONOTONE;
    d->warm_scale = 0.0;   // automatic: 0.5 for PREVIOUS, 0.9 for LEARNED
    return BBG_OK;
}

bbg_status bbg_build_grid(const double dmin[3], const double dmax[3], double spacing, double scale,
                          int dims[3], double geo[12]) {
    if (!dmin || !dmax || !dims || !geo || !(spacing > 0) || !(scale > 0))
        return fail(BBG_ERR_INVALID_ARGUMENT, "invalid grid arguments");
    float minp[3], len[3], bmin[3], bmax[3];
    build_grid(dmin, dmax, spacing, scale, dims, minp, len, bmin, bmax);
    for (int k = 0; k < 3; k++) {
        geo[k] = minp[k];
        geo[3 + k] = len[k];
        geo[6 + k] = bmin[k];
        geo[9 + k] = bmax[k];
    }
    return BBG_OK;
}

bbg_status bbg_compute_mass(int lattice, double target_density, double spacing, double kernel_radius,
                            double *mass) {
    if (!mass || (lattice != 0 && lattice != 1) || !(spacing > 0) || !(kernel_radius > 0))
        return fail(BBG_ERR_INVALID_ARGUMENT, "invalid mass arguments");
    *mass = compute_mass(lattice, (float)target_density, (float)spacing, (float)kernel_radius);
    return BBG_OK;
}

bbg_status bbg_compute_delta_denom(double spacing, double kernel_radius, double *denom) {
    if (!denom || !(spacing > 0) || !(kernel_radius > 0))
        return fail(BBG_ERR_INVALID_ARGUMENT, "invalid delta arguments");
    *denom = compute_delta_denom((float)spacing, (float)kernel_radius);
    return BBG_OK;
}

bbg_status bbg_create(const bbg_solver_desc *desc, int capacity, bbg_solver *out) {
    if (!desc || !out || capacity <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "invalid create arguments");
    *out = nullptr;
    if (!(desc->target_spacing > 0) || !(desc->relative_kernel_radius > 0) ||
        !(desc->grid_spacing_scale > 0) || !(desc->target_density > 0))
        return fail(BBG_ERR_INVALID_ARGUMENT, "spacing, kernel radius, grid scale and density must be > 0");
    if (desc->solver_kind != BBG_SOLVER_PCISPH && desc->solver_kind != BBG_SOLVER_SPH)
        return fail(BBG_ERR_INVALID_ARGUMENT, "unknown solver kind");
    for (int k = 0; k < 3; k++)
        if (!(desc->domain_max[k] > desc->domain_min[k]))
            return fail(BBG_ERR_INVALID_ARGUMENT, "empty domain on axis %d", k);
    int ndev = 0;
    bbg_device_count(&ndev);
    if (ndev <= 0) return fail(BBG_ERR_NO_DEVICE, "no CUDA device visible; bubbles_gb300 has no CPU path");
    if (desc->device < 0 || desc->device >= ndev) return fail(BBG_ERR_INVALID_ARGUMENT, "bad device ordinal");
    CK(cudaSetDevice(desc->device));

    bbg_solver s = new (std::nothrow) bbg_solver_s();
    if (!s) return fail(BBG_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->B = DevBufs();
    memset(&s->P, 0, sizeof(s->P));
    memset(&s->acc, 0, sizeof(s->acc));
    s->desc = *desc;
    s->capacity = capacity;
    // grid in the reference's FP32 arithmetic
    float minp[3], len[3], bmin[3], bmax[3];
    build_grid(desc->domain_min, desc->domain_max, desc->target_spacing, desc->grid_spacing_scale,
               s->dims, minp, len, bmin, bmax);
    const unsigned long long total = (unsigned long long)s->dims[0] * s->dims[1] * s->dims[2];
    if (total == 0 || total > 0x7fffffffull) {
        delete s;
        return fail(BBG_ERR_INVALID_ARGUMENT, "grid of %llu cells is out of range", total);
    }
    s->cells = (unsigned)total;
    GridDev &g = s->P.g;
    g.nx = s->dims[0]; g.ny = s->dims[1]; g.nz = s->dims[2];
    g.total = s->cells;
    for (int k = 0; k < 3; k++) {
        g.minp[k] = minp[k]; g.len[k] = len[k]; g.bmin[k] = bmin[k]; g.bmax[k] = bmax[k];
        s->dims_geo[k] = minp[k]; s->dims_geo[3 + k] = len[k];
        s->dims_geo[6 + k] = bmin[k]; s->dims_geo[9 + k] = bmax[k];
    }
    s->kernel_radius = (float)desc->relative_kernel_radius * (float)desc->target_spacing;

    cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail(BBG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    s->stream = s->own_stream;
    DevBufs &B = s->B;
    B.prof = &s->prof;
    const size_t n = (size_t)capacity;
    bbg_status r = BBG_OK;
#define ALLOC(ptr, cnt) if (!r) r = dalloc(&(ptr), (cnt))
    ALLOC(B.pos[0], n); ALLOC(B.pos[1], n); ALLOC(B.vel[0], n); ALLOC(B.vel[1], n);
    ALLOC(B.pid[0], n); ALLOC(B.pid[1], n); ALLOC(B.slot, n);
    ALLOC(B.force, n); ALLOC(B.xstar, n); ALLOC(B.pforce, n); ALLOC(B.smoothed, n);
    ALLOC(B.rho, n); ALLOC(B.press, n); ALLOC(B.rhostar, n); ALLOC(B.derr, n);
    ALLOC(B.cell, n); ALLOC(B.cell_old, n); ALLOC(B.sub, n); ALLOC(B.tmp, n); ALLOC(B.nbr, n);
    ALLOC(B.list, (size_t)kMaxList * n); ALLOC(B.inv_rho, n); ALLOC(B.pprev, n);
    ALLOC(B.soa, 3 * (n + 1)); B.soa_stride = n + (n & 1);
    ALLOC(B.count, (size_t)s->cells); ALLOC(B.start, (size_t)s->cells + 1);
    ALLOC(B.partials, scan_partials_needed(s->cells));
    ALLOC(B.st, 1); ALLOC(B.stage, 6 * n); ALLOC(B.red, 4);
#undef ALLOC
    if (!r && cudaMallocHost((void **)&s->h_st, sizeof(StepState)) != cudaSuccess) {
        cudaGetLastError();
        r = fail(BBG_ERR_OUT_OF_MEMORY, "pinned allocation failed");
    }
    if (!r && cudaMallocHost((void **)&s->h_u, 64) != cudaSuccess) {
        cudaGetLastError();
        r = fail(BBG_ERR_OUT_OF_MEMORY, "pinned allocation failed");
    }
    if (!r && cudaMemsetAsync(B.count, 0, sizeof(unsigned) * s->cells, s->stream) != cudaSuccess)
        r = fail(BBG_ERR_CUDA, "memset failed");
    if (!r && cudaMemsetAsync(B.st, 0, sizeof(StepState), s->stream) != cudaSuccess)
        r = fail(BBG_ERR_CUDA, "memset failed");
    if (!r && cudaStreamSynchronize(s->stream) != cudaSuccess) r = fail(BBG_ERR_CUDA, "sync failed");
    if (r) {
        free_all(s);
        cudaStreamDestroy(s->own_stream);
        delete s;
        return r;
    }
    if (desc->pressure_init == BBG_PRESSURE_INIT_LEARNED) {
        bbg_mlp_desc md;
        bbg_mlp_desc_default(&md);
        r = mlp_allocate(s, md);
        if (r) {
            free_all(s);
            cudaStreamDestroy(s->own_stream);
            delete s;
            return r;
        }
    }
    *out = s;
    return BBG_OK;
}

bbg_status bbg_destroy(bbg_solver s) {
    if (!s) return BBG_OK;
    cudaSetDevice(s->desc.device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_all(s);
    if (s->aux) cudaStreamDestroy(s->aux);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
    return BBG_OK;
}

bbg_status bbg_set_stream(bbg_solver s, void *stream) {
    if (bbg_status r = check_solver(s)) return r;
    CK(cudaStreamSynchronize(s->stream));
    s->stream = stream ? (cudaStream_t)stream : s->own_stream;
    s->epoch++;
    return BBG_OK;
}

bbg_status bbg_synchronize(bbg_solver s) {
    if (bbg_status r = check_solver(s)) return r;
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_set_colliders(bbg_solver s, const bbg_shape *shapes, int count) {
    if (bbg_status r = check_solver(s)) return r;
    if (count < 0 || count > kMaxColliders || (count > 0 && !shapes))
        return fail(BBG_ERR_INVALID_ARGUMENT, "collider count must be in [0, %d]", kMaxColliders);
    for (int i = 0; i < count; i++) {
        const bbg_shape &sh = shapes[i];
        if (sh.type != BBG_SHAPE_BOX && sh.type != BBG_SHAPE_SPHERE && sh.type != BBG_SHAPE_SDF)
            return fail(BBG_ERR_INVALID_ARGUMENT, "collider %d: unknown shape type", i);
    }
    free_fields(s);   // fields belong to the previous colliders
    for (int i = 0; i < count; i++) {
        s->P.shapes[i] = shape_dev(shapes[i]);
        if (shapes[i].type == BBG_SHAPE_SDF)   // defined by its field alone: identity transform
            for (int k = 0; k < 3; k++) s->P.shapes[i].t[k] = 0.f;
    }
    s->P.nshapes = count;
    s->epoch++;
    return BBG_OK;
}

bbg_status bbg_upload_particles(bbg_solver s, const float *pos, const float *vel, int n) {
    if (bbg_status r = check_solver(s)) return r;
    if (!pos || n <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "need n > 0 positions");
    if (n > s->capacity) return fail(BBG_ERR_CAPACITY, "%d particles exceed capacity %d", n, s->capacity);
    float *dp = s->B.stage, *dv = s->B.stage + 3 * (size_t)s->capacity;
    CK(cudaMemcpyAsync(dp, pos, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    if (vel) CK(cudaMemcpyAsync(dv, vel, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    return upload_common(s, dp, vel ? dv : nullptr, n);
}

bbg_status bbg_upload_particles_device(bbg_solver s, const float *d_pos, const float *d_vel, int n) {
    if (bbg_status r = check_solver(s)) return r;
    if (!d_pos || n <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "need n > 0 positions");
    if (n > s->capacity) return fail(BBG_ERR_CAPACITY, "%d particles exceed capacity %d", n, s->capacity);
    return upload_common(s, d_pos, d_vel, n);
}

bbg_status bbg_setup(bbg_solver s) {
    if (bbg_status r = check_solver(s)) return r;
    if (s->n <= 0) return fail(BBG_ERR_STATE, "upload particles before bbg_setup");
    const bbg_solver_desc &d = s->desc;
    float mass = compute_mass(0, (float)d.target_density, (float)d.target_spacing, s->kernel_radius);
    if (d.mass > 0) mass = (float)d.mass;
    s->mass = mass > 0 ? mass : 0.f;
    const float mo = s->mass / (float)d.target_density;
    s->mod2 = mo * mo;
    s->delta_denom = compute_delta_denom((float)d.target_spacing, s->kernel_radius);
    fill_params(s);
    s->setup_done = true;
    s->epoch++;
    return BBG_OK;
}

bbg_status bbg_update_grid_distribution(bbg_solver s) {
    if (bbg_status r = check_solver(s)) return r;
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    return grid_update(s);
}

bbg_status bbg_compute_particle_interaction(bbg_solver s) {
    if (bbg_status r = check_solver(s)) return r;
    s->valid |= bit(BBG_FIELD_INTERACTION);
    return BBG_OK;
}

bbg_status bbg_compute_density(bbg_solver s, int compute_pressure) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    launch_density(s->P, s->B, s->state, compute_pressure ? 1 : 0, s->stream);
    CK_LAUNCH();
    s->list_state = s->state;
    s->valid |= bit(BBG_FIELD_DENSITY) | (compute_pressure ? bit(BBG_FIELD_PRESSURE) : 0u);
    return BBG_OK;
}

bbg_status bbg_compute_non_pressure_force(bbg_solver s) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_DENSITY))) return fail(BBG_ERR_STATE, "density not computed");
    launch_non_pressure(s->P, s->B, s->state, 0, 0.f, 0.f, s->stream);
    CK_LAUNCH();
    s->valid |= bit(BBG_FIELD_FORCE);
    return BBG_OK;
}

bbg_status bbg_compute_delta(bbg_solver s, double dt, double *delta) {
    if (bbg_status r = check_solver(s)) return r;
    if (!delta) return fail(BBG_ERR_INVALID_ARGUMENT, "null delta");
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    *delta = compute_delta(s->mod2, s->delta_denom, (float)dt);
    return BBG_OK;
}

bbg_status bbg_use_cuda_graphs(bbg_solver s, int enable) {
    if (bbg_status r = check_solver(s)) return r;
    s->use_graphs = enable != 0;
    return BBG_OK;
}

bbg_status bbg_profiler_enable(bbg_solver s, int enable) {
    if (bbg_status r = check_solver(s)) return r;
    s->prof.on = enable != 0;
    // create the events up front so none is created inside a timed region
    while (s->prof.on && s->prof.pool.size() < 8192) {
        cudaEvent_t e = nullptr;
        CK(cudaEventCreate(&e));
        s->prof.pool.push_back(e);
    }
    return BBG_OK;
}

bbg_status bbg_profiler_report(bbg_solver s, int max_kernels, char *names, double *total_ms,
                               int32_t *launches, int32_t *kernel_count, int64_t *total_launches) {
    if (bbg_status r = check_solver(s)) return r;
    if (max_kernels < 0 || (max_kernels > 0 && (!names || !total_ms || !launches)))
        return fail(BBG_ERR_INVALID_ARGUMENT, "invalid report buffers");
    CK(cudaStreamSynchronize(s->stream));
    double ms[KID_COUNT] = {0};
    int cnt[KID_COUNT] = {0};
    for (auto &r : s->prof.recs) {
        if (r.skipped) continue;
        float e = 0.f;
        CK(cudaEventElapsedTime(&e, r.a, r.b));
        ms[r.id] += e;
        cnt[r.id] += 1;
    }
    int k = 0;
    for (int id = 0; id < KID_COUNT && k < max_kernels; id++) {
        if (!cnt[id]) continue;
        memset(names + 32 * k, 0, 32);
        strncpy(names + 32 * k, kernel_name(id), 31);
        total_ms[k] = ms[id];
        launches[k] = cnt[id];
        k++;
    }
    if (kernel_count) *kernel_count = k;
    if (total_launches) *total_launches = (int64_t)s->prof.launches;
    s->prof.release();
    return BBG_OK;
}

bbg_status bbg_compute_pressure_force_and_integrate(bbg_solver s, double dt, double max_err,
                                                    double delta, int max_it,
                                                    bbg_step_stats *stats) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_FORCE)) || !(s->valid & bit(BBG_FIELD_DENSITY)))
        return fail(BBG_ERR_STATE, "density and non-pressure force must be computed first");
    if (max_it < 1 || max_it > kMaxIterations)
        return fail(BBG_ERR_INVALID_ARGUMENT, "max_iterations must be in [1, %d]", kMaxIterations);
    const float fdt = (float)dt;
    // PredictVelocityAndPositionFor with is_first = 1: p = 0, Fp = 0, x* from F only
    CK(cudaMemsetAsync(s->B.st->err_bits, 0, sizeof(s->B.st->err_bits), s->stream));
    CK(cudaMemsetAsync(s->B.st->err_sum, 0, sizeof(s->B.st->err_sum), s->stream));
    CK(cudaMemsetAsync(&s->B.st->max_force_bits, 0, 4, s->stream));
    s->P.max_err_ratio = (float)max_err;
    launch_predict_first(s->P, s->B, s->state, 1, fdt, fdt / s->mass, s->stream);
    CK_LAUNCH();
    bbg_status r = corrector(s, fdt, (float)delta, max_it);
    if (r) return r;
    r = pseudo_viscosity(s, fdt);
    if (r) return r;
    if (stats) {
        memset(&s->acc, 0, sizeof(s->acc));
        if ((r = read_step_state(s))) return r;
        add_substep_stats(s, fdt);
        *stats = s->acc;
    }
    return BBG_OK;
}

bbg_status bbg_predict_velocity_and_position(bbg_solver s, double dt, int is_first) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_FORCE))) return fail(BBG_ERR_STATE, "forces not valid");
    if (!is_first && !(s->valid & bit(BBG_FIELD_PRESSURE_FORCE)))
        return fail(BBG_ERR_STATE, "pressure force not valid");
    launch_predict_first(s->P, s->B, s->state, is_first ? 1 : 0, (float)dt, (float)dt / s->mass,
                         s->stream);
    CK_LAUNCH();
    s->valid |= bit(BBG_FIELD_PRED_POSITION);
    if (is_first)
        s->valid |= bit(BBG_FIELD_PRESSURE) | bit(BBG_FIELD_PRESSURE_FORCE) |
                    bit(BBG_FIELD_PRED_DENSITY) | bit(BBG_FIELD_DENSITY_ERROR);
    return BBG_OK;
}

bbg_status bbg_predict_pressure(bbg_solver s, double delta) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_PRED_POSITION)) || !(s->valid & bit(BBG_FIELD_PRESSURE)))
        return fail(BBG_ERR_STATE, "predicted positions and pressure must be valid");
    CK(cudaMemsetAsync(s->B.st->err_bits, 0, sizeof(s->B.st->err_bits), s->stream));
    CK(cudaMemsetAsync(s->B.st->err_sum, 0, sizeof(s->B.st->err_sum), s->stream));
    launch_pred_density(s->P, s->B, s->state, 0, (float)delta, s->stream);
    CK_LAUNCH();
    s->valid |= bit(BBG_FIELD_PRESSURE) | bit(BBG_FIELD_PRED_DENSITY) | bit(BBG_FIELD_DENSITY_ERROR);
    return BBG_OK;
}

bbg_status bbg_predict_pressure_force(bbg_solver s) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_PRESSURE)) || !(s->valid & bit(BBG_FIELD_PRED_DENSITY)))
        return fail(BBG_ERR_STATE, "pressure and predicted density must be valid");
    launch_pack_acoef(s->P, s->B, s->state, s->stream);
    CK(cudaMemsetAsync(s->B.st->err_bits, 0, sizeof(s->B.st->err_bits), s->stream));
    launch_pressure_force(s->P, s->B, s->state, 0, 1 << 30, 0.f, 0.f, s->stream, 1);
    CK_LAUNCH();
    s->valid |= bit(BBG_FIELD_PRESSURE_FORCE);
    return BBG_OK;
}

bbg_status bbg_accumulate_and_integrate(bbg_solver s, double dt) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_FORCE)) || !(s->valid & bit(BBG_FIELD_PRESSURE_FORCE)))
        return fail(BBG_ERR_STATE, "forces and pressure forces must be valid");
    launch_accumulate_integrate(s->P, s->B, s->state, (float)dt, s->stream);
    CK_LAUNCH();
    flip_state(s);
    return BBG_OK;
}

bbg_status bbg_compute_pressure_force(bbg_solver s, double dt) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    if (!(s->valid & bit(BBG_FIELD_DENSITY)) || !(s->valid & bit(BBG_FIELD_PRESSURE)))
        return fail(BBG_ERR_STATE, "density and pressure must be computed first");
    launch_sph_forces(s->P, s->B, s->state, (float)dt, s->stream);
    CK_LAUNCH();
    flip_state(s);
    s->valid |= kPosVel | bit(BBG_FIELD_FORCE);
    return BBG_OK;
}

bbg_status bbg_time_integration(bbg_solver s, double dt) {
    if (bbg_status r = check_solver(s)) return r;
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    if (!(s->valid & bit(BBG_FIELD_FORCE))) return fail(BBG_ERR_STATE, "forces not valid");
    launch_integrate(s->P, s->B, s->state, (float)dt, s->stream);
    CK_LAUNCH();
    // the other buffer now holds the integrated state in the same slot order
    flip_state(s);
    return BBG_OK;
}

bbg_status bbg_compute_pseudo_viscosity_interpolation(bbg_solver s, double dt) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    return pseudo_viscosity(s, (float)dt);
}

bbg_status bbg_compute_number_of_time_steps(bbg_solver s, double remaining, double scale,
                                            unsigned *count) {
    if (bbg_status r = check_solver(s)) return r;
    if (!count) return fail(BBG_ERR_INVALID_ARGUMENT, "null count");
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    float mf = 0;
    if (bbg_status r = max_force(s, &mf)) return r;
    *count = number_of_time_steps((float)remaining, (float)s->desc.sound_speed, (float)scale,
                                  s->kernel_radius, s->mass, mf);
    return BBG_OK;
}

bbg_status bbg_advance_time_step(bbg_solver s, double dt, bbg_step_stats *stats) {
    if (bbg_status r = check_solver(s)) return r;
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    if (!(dt > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "dt must be > 0");
    bbg_status r = substep(s, (float)dt);
    if (r) return r;
    if (stats) {
        memset(&s->acc, 0, sizeof(s->acc));
        if ((r = read_step_state(s))) return r;
        add_substep_stats(s, (float)dt);
        *stats = s->acc;
    }
    return BBG_OK;
}

// One substep with the state in host memory: the uploads, AdvanceTimeStep and the downloads
// of bbg_upload_particles, bbg_set_field, bbg_advance_time_step, bbg_download and
// bbg_get_field, queued on the solver's stream with one synchronisation at the end.
bbg_status bbg_step_host(bbg_solver s, double dt, int n, const float *pos, const float *vel, const float *pressure,
                         const float *divergence, float *pos_out, float *vel_out, float *pressure_out,
                         float *divergence_out, bbg_step_stats *stats) {
    if (bbg_status r = check_solver(s)) return r;
    if (!pos || !vel || n <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "need n > 0 positions and velocities");
    if (n > s->capacity) return fail(BBG_ERR_CAPACITY, "%d particles exceed capacity %d", n, s->capacity);
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    if (!(dt > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if ((divergence || divergence_out) && !s->mlp_alloc)
        return fail(BBG_ERR_STATE, "the divergence field belongs to the learned warm start");
    if ((pressure || divergence || pressure_out || divergence_out) && !s->d_stage2)
        CK(cudaMalloc((void **)&s->d_stage2, sizeof(float) * 2 * (size_t)s->capacity));
    const size_t nn = (size_t)n;
    float *dp = s->B.stage, *dv = s->B.stage + 3 * (size_t)s->capacity;
    float *sp = s->d_stage2, *sd = s->d_stage2 ? s->d_stage2 + s->capacity : nullptr;
    CK(cudaMemcpyAsync(dp, pos, sizeof(float) * 3 * nn, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(dv, vel, sizeof(float) * 3 * nn, cudaMemcpyHostToDevice, s->stream));
    if (bbg_status r = upload_common(s, dp, dv, n)) return r;
    if (pressure) {
        CK(cudaMemcpyAsync(sp, pressure, sizeof(float) * nn, cudaMemcpyHostToDevice, s->stream));
        launch_set_scalar(s->B.press, s->B.slot, sp, n, s->stream);
        CK_LAUNCH();
        s->valid |= bit(BBG_FIELD_PRESSURE);
    }
    if (divergence) {
        CK(cudaMemcpyAsync(sd, divergence, sizeof(float) * nn, cudaMemcpyHostToDevice, s->stream));
        launch_set_scalar(s->mlp.divsum, s->B.slot, sd, n, s->stream);
        CK_LAUNCH();
    }
    if (bbg_status r = substep(s, (float)dt)) return r;
    if (pos_out || vel_out) {
        launch_download(s->B, s->state, s->pid_cur, pos_out ? dp : nullptr, vel_out ? dv : nullptr, n, s->stream);
        CK_LAUNCH();
        if (pos_out) CK(cudaMemcpyAsync(pos_out, dp, sizeof(float) * 3 * nn, cudaMemcpyDeviceToHost, s->stream));
        if (vel_out) CK(cudaMemcpyAsync(vel_out, dv, sizeof(float) * 3 * nn, cudaMemcpyDeviceToHost, s->stream));
    }
    if (pressure_out) {
        launch_get_scalar(s->B.press, s->B.slot, sp, n, s->stream);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(pressure_out, sp, sizeof(float) * nn, cudaMemcpyDeviceToHost, s->stream));
    }
    if (divergence_out) {
        launch_get_scalar(s->mlp.divsum, s->B.slot, sd, n, s->stream);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(divergence_out, sd, sizeof(float) * nn, cudaMemcpyDeviceToHost, s->stream));
    }
    if (stats) {
        memset(&s->acc, 0, sizeof(s->acc));
        if (bbg_status r = read_step_state(s)) return r;   // synchronises the stream
        add_substep_stats(s, (float)dt);
        *stats = s->acc;
    } else {
        CK(cudaStreamSynchronize(s->stream));
    }
    return BBG_OK;
}

bbg_status bbg_advance(bbg_solver s, double dt, bbg_step_stats *stats) {
    if (bbg_status r = check_solver(s)) return r;
    if (!s->setup_done) return fail(BBG_ERR_STATE, "bbg_setup has not been called");
    if (!(dt > 0)) return fail(BBG_ERR_INVALID_ARGUMENT, "dt must be > 0");
    memset(&s->acc, 0, sizeof(s->acc));
    float remaining = (float)dt;
    while (remaining > 0.0001f) {   // Epsilon, src/core/geometry.h:44
        float mf = 0;
        bbg_status r = max_force(s, &mf);
        if (r) return r;
        unsigned nsteps = number_of_time_steps(remaining, (float)s->desc.sound_speed,
                                               (float)s->desc.time_step_limit_scale,
                                               s->kernel_radius, s->mass, mf);
        if (nsteps == 0) nsteps = 1;
        const float step = remaining / (float)nsteps;
        if ((r = substep(s, step))) return r;
        if ((r = read_step_state(s))) return r;
        add_substep_stats(s, step);
        remaining -= step;
    }
    if (stats) *stats = s->acc;
    return BBG_OK;
}

bbg_status bbg_get_stats(bbg_solver s, bbg_step_stats *stats) {
    if (bbg_status r = check_solver(s)) return r;
    if (!stats) return fail(BBG_ERR_INVALID_ARGUMENT, "null stats");
    memset(&s->acc, 0, sizeof(s->acc));
    if (bbg_status r = read_step_state(s)) return r;
    add_substep_stats(s, 0.f);
    s->acc.substeps = 0;
    *stats = s->acc;
    return BBG_OK;
}

bbg_status bbg_particle_count(bbg_solver s, int *n) {
    if (bbg_status r = check_solver(s)) return r;
    if (!n) return fail(BBG_ERR_INVALID_ARGUMENT, "null n");
    *n = s->n;
    return BBG_OK;
}

bbg_status bbg_get_field(bbg_solver s, int field, float *out) {
    if (bbg_status r = check_solver(s)) return r;
    const int comps = field_components(field);
    if (!comps || !out) return fail(BBG_ERR_INVALID_ARGUMENT, "unknown field %d", field);
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    if (field == BBG_FIELD_DIVERGENCE ? !s->mlp_alloc : !(s->valid & bit(field)))
        return fail(BBG_ERR_STATE, "field %d is not valid in the current particle order", field);
    const size_t n = (size_t)s->n;
    if (field == BBG_FIELD_INTERACTION) {
        for (size_t i = 0; i < n; i++) {
            out[3 * i] = (float)s->desc.gravity[0];
            out[3 * i + 1] = (float)s->desc.gravity[1];
            out[3 * i + 2] = (float)s->desc.gravity[2];
        }
        return BBG_OK;
    }
    if (comps == 3) launch_get_vec(vec_field(s, field), s->B.slot, s->B.stage, s->n, s->stream);
    else launch_get_scalar(scalar_field(s, field), s->B.slot, s->B.stage, s->n, s->stream);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(out, s->B.stage, sizeof(float) * comps * n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_set_field(bbg_solver s, int field, const float *in) {
    if (bbg_status r = check_solver(s)) return r;
    const int comps = field_components(field);
    if (!comps || !in || field == BBG_FIELD_INTERACTION)
        return fail(BBG_ERR_INVALID_ARGUMENT, "field %d cannot be set", field);
    if (field == BBG_FIELD_DIVERGENCE && !s->mlp_alloc)
        return fail(BBG_ERR_STATE, "the divergence field belongs to the learned warm start");
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    const size_t n = (size_t)s->n;
    CK(cudaMemcpyAsync(s->B.stage, in, sizeof(float) * comps * n, cudaMemcpyHostToDevice, s->stream));
    if (comps == 3) launch_set_vec(vec_field(s, field), s->B.slot, s->B.stage, s->n, s->stream);
    else launch_set_scalar(scalar_field(s, field), s->B.slot, s->B.stage, s->n, s->stream);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s->stream));
    s->valid |= bit(field);
    if (field == BBG_FIELD_POSITION && s->list_state == s->state) s->list_state = -1;
    return BBG_OK;
}

bbg_status bbg_download(bbg_solver s, float *pos, float *vel) {
    if (bbg_status r = check_solver(s)) return r;
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    const size_t n = (size_t)s->n;
    float *dp = s->B.stage, *dv = s->B.stage + 3 * (size_t)s->capacity;
    launch_download(s->B, s->state, s->pid_cur, pos ? dp : nullptr, vel ? dv : nullptr, s->n, s->stream);
    CK_LAUNCH();
    if (pos) CK(cudaMemcpyAsync(pos, dp, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s->stream));
    if (vel) CK(cudaMemcpyAsync(vel, dv, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_download_device(bbg_solver s, float *d_pos, float *d_vel) {
    if (bbg_status r = check_solver(s)) return r;
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    launch_download(s->B, s->state, s->pid_cur, d_pos, d_vel, s->n, s->stream);
    CK_LAUNCH();
    return BBG_OK;
}

bbg_status bbg_get_scalars(bbg_solver s, double out[8]) {
    if (bbg_status r = check_solver(s)) return r;
    if (!out) return fail(BBG_ERR_INVALID_ARGUMENT, "null out");
    out[0] = s->mass;
    out[1] = s->kernel_radius;
    out[2] = s->delta_denom;
    out[3] = s->mod2;
    out[4] = (float)s->desc.target_spacing;
    out[5] = (float)s->desc.target_density;
    out[6] = (float)s->desc.target_spacing;
    out[7] = (float)s->desc.relative_kernel_radius;
    return BBG_OK;
}

// FP64 totals of the state: mass, kinetic energy, potential energy and momentum
bbg_status bbg_energy(bbg_solver s, double out[6]) {
    if (bbg_status r = check_solver(s)) return r;
    if (!out) return fail(BBG_ERR_INVALID_ARGUMENT, "null output");
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    const int nb = energy_blocks(s->n);
    double *d = nullptr;
    std::vector<double> h((size_t)nb * kEnergyTerms);
    cudaError_t e = cudaMalloc((void **)&d, sizeof(double) * h.size());
    if (e == cudaSuccess) {
        launch_energy(s->P, s->B, s->state, s->desc.gravity, d, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(BBG_ERR_CUDA, "energy: %s", cudaGetErrorString(e));
    for (int t = 0; t < kEnergyTerms; t++) {
        double v = 0.0;
        for (int b = 0; b < nb; b++) v += h[(size_t)b * kEnergyTerms + t];
        out[t] = v;
    }
    return BBG_OK;
}

bbg_status bbg_get_grid(bbg_solver s, int dims[3], double geo[12]) {
    if (bbg_status r = check_solver(s)) return r;
    if (!dims || !geo) return fail(BBG_ERR_INVALID_ARGUMENT, "null output");
    for (int k = 0; k < 3; k++) dims[k] = s->dims[k];
    for (int k = 0; k < 12; k++) geo[k] = s->dims_geo[k];
    return BBG_OK;
}

bbg_status bbg_dump_grid(bbg_solver s, uint32_t *cell_of_particle, uint32_t *cell_counts,
                         uint32_t *sorted_ids) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_grid(s)) return r;
    const size_t n = (size_t)s->n;
    if (cell_of_particle) {
        launch_get_uint(s->B.cell, s->B.slot, (unsigned *)s->B.stage, s->n, s->stream);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(cell_of_particle, s->B.stage, 4 * n, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (sorted_ids) {
        CK(cudaMemcpyAsync(sorted_ids, s->B.pid[s->pid_cur], 4 * n, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (cell_counts) {
        unsigned *tmp = new (std::nothrow) unsigned[(size_t)s->cells + 1];
        if (!tmp) return fail(BBG_ERR_OUT_OF_MEMORY, "host allocation failed");
        cudaError_t e = cudaMemcpyAsync(tmp, s->B.start, 4 * ((size_t)s->cells + 1),
                                        cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            delete[] tmp;
            return fail(BBG_ERR_CUDA, "grid copy: %s", cudaGetErrorString(e));
        }
        for (unsigned c = 0; c < s->cells; c++) cell_counts[c] = tmp[c + 1] - tmp[c];
        delete[] tmp;
    }
    return BBG_OK;
}

bbg_status bbg_neighbor_counts(bbg_solver s, int32_t *counts) {
    if (bbg_status r = check_solver(s)) return r;
    if (!counts) return fail(BBG_ERR_INVALID_ARGUMENT, "null counts");
    if (!(s->valid & bit(BBG_FIELD_DENSITY))) return fail(BBG_ERR_STATE, "density not computed");
    launch_get_int(s->B.nbr, s->B.slot, (int *)s->B.stage, s->n, s->stream);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(counts, s->B.stage, 4 * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_neighbor_lists(bbg_solver s, int max_per_particle, int32_t *counts, int32_t *ids) {
    if (bbg_status r = check_solver(s)) return r;
    if (!counts || max_per_particle < 0 || (max_per_particle > 0 && !ids))
        return fail(BBG_ERR_INVALID_ARGUMENT, "need counts, max_per_particle >= 0 and ids when it is > 0");
    if (s->list_state < 0 || !s->grid_valid)
        return fail(BBG_ERR_STATE, "no neighbour sets: compute the density (or a substep) after the last grid update");
    const int n = s->n;
    const size_t width = (size_t)max_per_particle;
    // rows of a chunk of caller ids staged in the 6 x capacity words of the staging buffer
    size_t rows = 6 * (size_t)s->capacity / (width + 1);
    if (rows > (size_t)n) rows = (size_t)n;
    int *dc = reinterpret_cast<int *>(s->B.stage);
    for (size_t a = 0; a < (size_t)n; a += rows) {
        const size_t b = a + rows < (size_t)n ? a + rows : (size_t)n;
        int *dout = dc + (b - a);
        launch_export_members(s->P, s->B, s->list_state, s->pid_cur, (int)a, (int)b, max_per_particle, dc, dout,
                              s->stream);
        CK_LAUNCH();
        CK(cudaMemcpyAsync(counts + a, dc, sizeof(int) * (b - a), cudaMemcpyDeviceToHost, s->stream));
        if (width)
            CK(cudaMemcpyAsync(ids + a * width, dout, sizeof(int) * (b - a) * width, cudaMemcpyDeviceToHost,
                               s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return BBG_OK;
}

}  // extern "C"

// ----------------------------------------------------------------------------
// learned warm start
// ----------------------------------------------------------------------------
namespace {
bbg_status require_mlp(bbg_solver s) {
    if (!s->mlp_alloc) return fail(BBG_ERR_STATE, "the learned warm start is not configured");
    return BBG_OK;
}
}  // namespace

bbg_status bbg_mlp_desc_default(bbg_mlp_desc *d) {
    if (!d) return fail(BBG_ERR_INVALID_ARGUMENT, "null desc");
    memset(d, 0, sizeof(*d));
    d->train_substeps = 200;
    d->batch = 16384;
    d->steps_per_substep = 4;
    d->learning_rate = 1e-3;
    d->beta1 = 0.9;
    d->beta2 = 0.999;
    d->epsilon = 1e-8;
    d->seed = 20240601ull;
    d->expectile = 0.5;
    d->finetune_steps = 0;
    d->refresh_interval = 0;
    return BBG_OK;
}

bbg_status bbg_mlp_configure(bbg_solver s, const bbg_mlp_desc *d) {
    if (bbg_status r = check_solver(s)) return r;
    if (!d) return fail(BBG_ERR_INVALID_ARGUMENT, "null desc");
    return mlp_allocate(s, *d);
}

bbg_status bbg_mlp_get_params(bbg_solver s, float *theta) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    if (!theta) return fail(BBG_ERR_INVALID_ARGUMENT, "null output");
    CK(cudaMemcpyAsync(theta, s->mlp.theta, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_mlp_set_params(bbg_solver s, const float *theta) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    if (!theta) return fail(BBG_ERR_INVALID_ARGUMENT, "null input");
    CK(cudaMemcpyAsync(s->mlp.theta, theta, sizeof(float) * kParams, cudaMemcpyHostToDevice, s->stream));
    launch_mlp_pack(s->mlp, s->stream);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_mlp_set_trained(bbg_solver s, int trained) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    if (trained < 0) return fail(BBG_ERR_INVALID_ARGUMENT, "negative substep count");
    s->mlp_trained = trained;
    return BBG_OK;
}

bbg_status bbg_mlp_status(bbg_solver s, int *trained, int *adam_steps, double *last_loss) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    unsigned step = 0;
    double loss = 0;
    CK(cudaMemcpyAsync(s->h_u, s->mlp.step, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    memcpy(&step, s->h_u, sizeof(unsigned));
    CK(cudaMemcpy(&loss, s->mlp.loss, sizeof(double), cudaMemcpyDeviceToHost));
    if (trained) *trained = s->mlp_trained;
    if (adam_steps) *adam_steps = (int)step;
    if (last_loss) *last_loss = loss / s->mlp_loss_count;
    return BBG_OK;
}

bbg_status bbg_mlp_infer(bbg_solver s, const float *features, int n, float *out) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    if (!features || !out || n <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "need n > 0 features");
    if (n > s->capacity) return fail(BBG_ERR_CAPACITY, "%d rows exceed capacity %d", n, s->capacity);
    float *df = s->B.stage, *dout = s->B.stage + 4 * (size_t)s->capacity;
    CK(cudaMemcpyAsync(df, features, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    launch_mlp_infer_raw(s->mlp, reinterpret_cast<const float4 *>(df), n, dout, s->stream);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_mlp_train_batch(bbg_solver s, const float *features, const float *targets, int batch) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    if (!features || !targets || batch <= 0) return fail(BBG_ERR_INVALID_ARGUMENT, "need a batch");
    if (5 * (size_t)batch > 6 * (size_t)s->capacity)
        return fail(BBG_ERR_CAPACITY, "batch of %d exceeds the staging of capacity %d", batch, s->capacity);
    float *dx = s->B.stage, *dt = s->B.stage + 4 * (size_t)batch;
    CK(cudaMemcpyAsync(dx, features, sizeof(float) * 4 * (size_t)batch, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(dt, targets, sizeof(float) * (size_t)batch, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->mlp.loss, 0, sizeof(double), s->stream));
    s->mlp_loss_count = (double)batch;
    const bbg_mlp_desc &d = s->mdesc;
    launch_mlp_train_step(s->mlp, reinterpret_cast<const float4 *>(dx), dt, batch, (float)d.learning_rate,
                          (float)d.beta1, (float)d.beta2, (float)d.epsilon, (float)d.expectile, s->stream);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

bbg_status bbg_mlp_get_features(bbg_solver s, float *out) {
    if (bbg_status r = check_solver(s)) return r;
    if (bbg_status r = require_mlp(s)) return r;
    if (!out) return fail(BBG_ERR_INVALID_ARGUMENT, "null output");
    if (s->n <= 0) return fail(BBG_ERR_STATE, "no particles");
    launch_mlp_get_features(s->mlp, s->B.slot, s->B.stage, s->n, s->stream);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(out, s->B.stage, sizeof(float) * 4 * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BBG_OK;
}

// ----------------------------------------------------------------------------
// launch tuning
// ----------------------------------------------------------------------------
bbg_status bbg_get_tuning(bbg_solver s, bbg_tuning *t) {
    if (bbg_status r = check_solver(s)) return r;
    if (!t) return fail(BBG_ERR_INVALID_ARGUMENT, "null tuning");
    t->block_size = s->B.tune.block;
    t->batch_np = s->B.tune.batch_np;
    t->batch_pd = s->B.tune.batch_pd;
    t->batch_pf = s->B.tune.batch_pf;
    t->prune = s->B.tune.prune;
    t->particles_per_thread = s->B.tune.ppt;
    t->tile_order = s->B.tune.tile_order;
    t->batch_worklist = s->B.tune.worklist;
    return BBG_OK;
}

bbg_status bbg_set_tuning(bbg_solver s, const bbg_tuning *t) {
    if (bbg_status r = check_solver(s)) return r;
    if (!t) return fail(BBG_ERR_INVALID_ARGUMENT, "null tuning");
    if (t->block_size != 64 && t->block_size != 128 && t->block_size != 256)
        return fail(BBG_ERR_INVALID_ARGUMENT, "block size must be 64, 128 or 256");
    for (int b : {t->batch_np, t->batch_pd, t->batch_pf})
        if (b != 2 && b != 4 && b != 8) return fail(BBG_ERR_INVALID_ARGUMENT, "gather batches must be 2, 4 or 8");
    if (t->prune != 0 && t->prune != 1) return fail(BBG_ERR_INVALID_ARGUMENT, "prune must be 0 or 1");
    if (t->particles_per_thread != 1 && t->particles_per_thread != 2)
        return fail(BBG_ERR_INVALID_ARGUMENT, "particles_per_thread must be 1 or 2");
    if (t->tile_order != 0 && t->tile_order != 1) return fail(BBG_ERR_INVALID_ARGUMENT, "tile_order must be 0 or 1");
    if (t->batch_worklist < 0 || t->batch_worklist > 2)
        return fail(BBG_ERR_INVALID_ARGUMENT, "batch_worklist must be 0, 1 or 2");
    CK(cudaStreamSynchronize(s->stream));
    s->B.tune.block = t->block_size;
    s->B.tune.batch_np = t->batch_np;
    s->B.tune.batch_pd = t->batch_pd;
    s->B.tune.batch_pf = t->batch_pf;
    s->B.tune.prune = t->prune;
    s->B.tune.ppt = t->particles_per_thread;
    s->B.tune.tile_order = t->tile_order;
    s->B.tune.worklist = t->batch_worklist;
    if (s->nscenes > 0) update_worklist_grid(s->B);
    s->epoch++;   // captured graphs hold the old launch shapes
    return BBG_OK;
}
