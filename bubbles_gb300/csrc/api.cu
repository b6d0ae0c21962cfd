// api.cu -- the C ABI of bubbles_gb300 (include/bbg.h): solver lifetime, the
// substep launch sequences and field access.  Host code only; kernels live in
// grid.cu and sph.cu.
#include "../../include/bbg.h"
#include "bbg_kernels.h"
#include "emit.h"
#include "frame.h"
#include "gfmt.h"
#include "host_math.h"
#include "mlp.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <thread>
#include <vector>

using namespace bbg;

namespace {

thread_local char g_err[512] = "";

bbg_status fail(bbg_status code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            if (e_ == cudaErrorMemoryAllocation)                                           \
                return fail(BBG_ERR_OUT_OF_MEMORY, "%s: %s", #call, cudaGetErrorString(e_)); \
            return fail(BBG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));            \
        }                                                                                  \
    } while (0)

#define CK_LAUNCH() CK(cudaGetLastError())

// bit per field id: valid in the current sorted-slot order
constexpr unsigned bit(int f) { return 1u << f; }
constexpr unsigned kPosVel = bit(BBG_FIELD_POSITION) | bit(BBG_FIELD_VELOCITY);

}  // namespace

namespace bbg {
int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
}  // namespace bbg

struct bbg_solver_s {
    bbg_solver_desc desc;
    int capacity = 0, n = 0;
    Params P;
    DevBufs B;
    int state = 0;     // ping-pong buffer holding the current positions / velocities
    int pid_cur = 0;   // pid buffer of the current sorted order
    unsigned cells = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    bool setup_done = false, grid_valid = false;
    unsigned valid = 0;
    float mass = 0, kernel_radius = 0, delta_denom = 0, mod2 = 0;
    float dims_geo[12];
    int dims[3];
    StepState *h_st = nullptr;   // pinned host mirror of the device step state
    unsigned *h_u = nullptr;     // pinned scratch
    float *d_stage2 = nullptr;   // 2 x capacity floats: the carried scalars of bbg_step_host
    int last_max_it = 1;
    float last_tol = 0.01f;
    int pcisph_last_substep = 0;
    bbg_step_stats acc;          // accumulated over the current advance call
    Prof prof;
    // CUDA graphs of whole substeps, keyed by dt, corrector controls and ping-pong parity
    struct SubstepGraph {
        bool valid = false;
        unsigned epoch = 0, dt_bits = 0, tol_bits = 0;
        int state = -1, pid = -1, max_it = 0, variant = -1;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
    } graphs[8];   // ping-pong parities x corrector variants
    int graph_next = 0;
    unsigned epoch = 1;          // bumped whenever captured launch arguments may change
    bool use_graphs = true;
    cudaStream_t aux = nullptr;  // capture stream of the corrector loop body
    // learned warm start
    MlpBufs mlp;
    bbg_mlp_desc mdesc;
    bool mlp_alloc = false;
    int mlp_trained = 0;         // substeps used for training so far
    long long mlp_since = 0;     // learned substeps since the last refresh (refresh_interval)
    double mlp_loss_count = 1;   // samples behind the loss accumulator
    // batch of scenes stacked along z
    int nscenes = 0;
    std::vector<int> scene_first, scene_count;
    std::vector<double> scene_offset;   // 3 per scene: packed = scene coordinates + offset
    float *d_zb = nullptr;
    ShapeDev *d_box = nullptr;
    SceneState *d_sst = nullptr;
    unsigned short *d_scene = nullptr;
    int *d_wl = nullptr;   // batch work list: scene first / last slots, segment offsets and tiles, counters
    FrameBufs frame;             // particle-frame writer buffers (allocated on first use)
    FrameReadBufs fread;         // frame reader buffers (grown on use)
    EmitBufs emit;               // emitter buffers (grown on use)
    MapBufs map;                 // MapGrid's remembered cells
    BucketBufs bucket;           // cell lists of particles added since the last distribution
    int grid_n = 0;              // particles in the last grid distribution's sorted ranges
    bool members_ok = false;     // sorted ranges [0, grid_n) are the last distribution's cells
    int list_state = -1;         // buffer holding the positions of the last density pass, whose
                                 // neighbour sets the member lists hold (-1: none)
    bool map_full = false;       // MapGridEmit reached the capacity once (it stops emitting)
    // signed-distance fields of colliders (Params::sdf holds their device descriptors)
    float *sdf_values[kMaxSdf] = {};
    bbg_sdf_grid sdf_grid[kMaxSdf] = {};
    int nsdf = 0;
};

namespace {

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

// Host-side fault injection for tests, off unless the environment sets BBG_FAIL_ALLOC_AFTER:
// the device allocation after that many successful ones (counted per process) fails as
// cudaMalloc does when memory runs out.
static long alloc_fault_budget() {
    static const long budget = [] {
        const char *e = getenv("BBG_FAIL_ALLOC_AFTER");
        return e ? atol(e) : -1L;
    }();
    return budget;
}
static long alloc_count = 0;

template <class T>
bbg_status dalloc(T **p, size_t count) {
    const long budget = alloc_fault_budget();
    if (budget >= 0 && __atomic_fetch_add(&alloc_count, 1, __ATOMIC_SEQ_CST) >= budget) {
        *p = nullptr;
        return fail(BBG_ERR_OUT_OF_MEMORY, "device allocation failed (injected by BBG_FAIL_ALLOC_AFTER)");
    }
    const cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        cudaGetLastError();   // a failed allocation must not surface in a later call's launch check
        *p = nullptr;
        return fail(e == cudaErrorMemoryAllocation ? BBG_ERR_OUT_OF_MEMORY : BBG_ERR_CUDA,
                    "device allocation of %zu bytes: %s", sizeof(T) * count, cudaGetErrorString(e));
    }
    return BBG_OK;
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
        M.infer_blocks = 6 * (sms > 0 ? sms : 1);   // 6 blocks of 128 threads fit an SM
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
static int mlp_mode(bbg_solver s) {
    if (s->desc.pressure_init != BBG_PRESSURE_INIT_LEARNED || s->desc.solver_kind != BBG_SOLVER_PCISPH)
        return 0;
    if (s->mlp_trained < s->mdesc.train_substeps) return 1;
    // refresh: every refresh_interval-th substep after training runs plain and trains again
    if (s->mdesc.refresh_interval > 0 && s->mlp_since >= s->mdesc.refresh_interval) return 1;
    return 2;
}

// Bookkeeping after a substep has been launched in mode mm.
static void mlp_after_substep(bbg_solver s, int mm) {
    if (mm == 1) {
        if (s->mlp_trained < s->mdesc.train_substeps) s->mlp_trained++;
        s->mlp_since = 0;
    } else if (mm == 2) {
        s->mlp_since++;
    }
}

static bool warm_active(bbg_solver s) {
    return s->desc.pressure_init == BBG_PRESSURE_INIT_PREVIOUS || mlp_mode(s) == 2;
}

// Warm-started correctors with the CLAMP_TOTAL rule let the pressure decrease.
static int clamp_total(bbg_solver s) {
    return warm_active(s) && s->desc.warm_rule == BBG_WARM_CLAMP_TOTAL;
}

// Start pressure = warm_scale * estimate; a scale <= 0 picks the measured defaults (the
// monotone update cannot lower an overestimated start, so the estimate is damped: the
// carried pressure by half, the learned one by a tenth).
static float warm_scale(bbg_solver s) {
    if (s->desc.warm_scale > 0) return (float)s->desc.warm_scale;
    return s->desc.pressure_init == BBG_PRESSURE_INIT_LEARNED ? 0.9f : 0.5f;
}

// Pressure a corrector step assigns to a 1 % density error (the MLP's pressure unit).
static float pressure_unit(bbg_solver s, float delta) { return delta * s->P.target_density * 0.01f; }

// Launches of a substep between the density pass and the corrector loop.
static void launch_prologue(bbg_solver s, int work, float dt, float delta, int max_it, cudaStream_t cs) {
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
static int training_steps(bbg_solver s) {
    const int mm = mlp_mode(s);
    return mm == 1 ? s->mdesc.steps_per_substep : mm == 2 ? s->mdesc.finetune_steps : 0;
}

static void launch_training(bbg_solver s, float delta, cudaStream_t cs) {
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

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
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

static bbg_status upload_common(bbg_solver s, const float *d_pos, const float *d_vel, int n) {
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
    if (t->batch_worklist < 0 || t->batch_worklist > 2)
        return fail(BBG_ERR_INVALID_ARGUMENT, "batch_worklist must be 0, 1 or 2");
    CK(cudaStreamSynchronize(s->stream));
    s->B.tune.block = t->block_size;
    s->B.tune.batch_np = t->batch_np;
    s->B.tune.batch_pd = t->batch_pd;
    s->B.tune.batch_pf = t->batch_pf;
    s->B.tune.prune = t->prune;
    s->B.tune.ppt = t->particles_per_thread;
    s->B.tune.worklist = t->batch_worklist;
    if (s->nscenes > 0) update_worklist_grid(s->B);
    s->epoch++;   // captured graphs hold the old launch shapes
    return BBG_OK;
}

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

bbg_status attach_field(bbg_solver s, int index, const bbg_sdf_grid &g, float *values);

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

// frees and reallocates (no copy): the reader's buffers only grow
template <class T>
bbg_status reserve(T **p, size_t need) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    CK(cudaMalloc((void **)p, sizeof(T) * (need ? need : 1)));
    return BBG_OK;
}

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

// ----------------------------------------------------------------------------
// colliders with signed-distance fields (FieldGrid3f; GenerateShapeSDF)
// ----------------------------------------------------------------------------
namespace {

// Attaches device node values (owned by the solver from here on) to collider `index`.
bbg_status attach_field(bbg_solver s, int index, const bbg_sdf_grid &g, float *values) {
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
    float *dp = nullptr;   // a query buffer of its own: 3 in + 14 out floats per point
    CK(cudaMalloc((void **)&dp, sizeof(float) * 17 * (size_t)n));
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
    cudaFree(dp);
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
    cudaError_t e = cudaMalloc((void **)&d_tri, sizeof(float) * tri.size());
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_out, sizeof(float) * total);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_stuck, sizeof(unsigned));
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
    cudaFree(d_tri);
    cudaFree(d_stuck);
    if (e != cudaSuccess) {
        cudaFree(d_out);
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

// device scratch of the boundary passes: cell levels, per-particle output and values, queue
struct LnmScratch {
    int *level = nullptr, *out = nullptr, *val = nullptr, *queue = nullptr, *counts = nullptr;
    cudaError_t alloc(size_t cells, size_t n) {
        cudaError_t e = cudaMalloc((void **)&level, sizeof(int) * (cells + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&out, sizeof(int) * n);
        if (e == cudaSuccess) e = cudaMalloc((void **)&val, sizeof(int) * n);
        if (e == cudaSuccess) e = cudaMalloc((void **)&queue, sizeof(int) * n);
        if (e == cudaSuccess) e = cudaMalloc((void **)&counts, sizeof(int) * 4);
        return e;
    }
    ~LnmScratch() {
        cudaFree(level);
        cudaFree(out);
        cudaFree(val);
        cudaFree(queue);
        cudaFree(counts);
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
    cudaError_t e = w.alloc(s->P.g.total, (size_t)s->n);
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
    cudaError_t e = w.alloc(s->P.g.total, (size_t)s->n);
    if (e == cudaSuccess)
        launch_lnm_single(s->P.g, s->B.start, s->B.cell, s->B.pid[s->pid_cur], s->n, pre > 0 ? pre : 0x7fffffff,
                          w.level, w.out, s->stream);
    return lnm_finish(s, e, w, levels, "LNM single-pass boundary");
}

bbg_status bbg_lnm_boundary_extended(bbg_solver s, double h, int max_level, int unbounded, int *levels) {
    if (bbg_status r = lnm_check(s, h, levels)) return r;
    LnmScratch w;
    cudaError_t e = w.alloc(s->P.g.total, (size_t)s->n);
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
    cudaError_t e = w.alloc(s->P.g.total, (size_t)s->n);
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
    cudaError_t e = w.alloc(s->P.g.total, (size_t)s->n);
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
    cudaError_t e = cudaMalloc((void **)&d_out, sizeof(float) * total);
    if (e == cudaSuccess) {
        launch_particle_sdf(A, d_out, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(values, d_out, sizeof(float) * total, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d_out);
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
    cudaError_t e = cudaMalloc((void **)&d_vals, sizeof(float) * (size_t)nodes);
    for (int q = 0; q < 7 && e == cudaSuccess; q++) e = cudaMalloc((void **)&b[q], sizeof(unsigned) * sz[q]);
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
            e = cudaMalloc((void **)&d_pts, sizeof(float) * 3 * (nvert ? nvert : 1));
            if (e == cudaSuccess) e = cudaMalloc((void **)&d_nrm, sizeof(float) * 3 * (nvert ? nvert : 1));
            if (e == cudaSuccess) e = cudaMalloc((void **)&d_tri, sizeof(int) * 3 * (ntri ? ntri : 1));
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
    cudaFree(d_vals);
    cudaFree(d_pts);
    cudaFree(d_nrm);
    cudaFree(d_tri);
    for (unsigned *p : b) cudaFree(p);
    return r;
}

