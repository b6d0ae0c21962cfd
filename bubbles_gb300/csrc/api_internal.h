// api_internal.h -- the solver state and the helpers shared by the C-ABI translation
// units: api.cu (solver lifetime, substeps, fields, learned warm start, launch tuning),
// api_batch.cu (batches of scenes), api_io.cu (particle frames and checkpoints),
// api_emit.cu (seeding) and api_post.cu (colliders with fields, boundary classification,
// surface field, marching cubes).  Host code only.
#pragma once

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

namespace bbg_api {

// records the message returned by bbg_last_error() and returns the code
bbg_status fail(bbg_status code, const char *fmt, ...);
// device allocations made so far, and after how many the test hook makes the next fail
long alloc_fault_budget();
extern long alloc_count;

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

}  // namespace bbg_api

// Device scratch of the post-processing calls, owned by the solver and kept between calls:
// a bump allocator over one block.  A call that needs more than the block gets extra
// blocks, and the next call replaces them by one block of that call's total, so repeated
// calls of the same size allocate nothing.
struct ScratchArena {
    char *base = nullptr;
    size_t cap = 0, used = 0, want = 0;
    std::vector<void *> extra;
};

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
    ScratchArena scratch;        // device scratch of the post-processing calls
};

namespace bbg_api {

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

bbg_status check_solver(bbg_solver s);
void fill_params(bbg_solver s);
void drop_graphs(bbg_solver s);
void free_fields(bbg_solver s);
void free_frame(bbg_solver s);
bbg_status free_all(bbg_solver s);
void free_mlp(bbg_solver s);
std::vector<float> mlp_initial_params(unsigned long long seed);
bbg_status mlp_allocate(bbg_solver s, const bbg_mlp_desc &d);
ShapeDev shape_dev(const bbg_shape &sh);
bbg_status require_grid(bbg_solver s);
bbg_status reset_step_state(bbg_solver s);
void flip_state(bbg_solver s);
bbg_status grid_update(bbg_solver s);
int iterations_from(const bbg_solver s, const StepState *st, int max_it, float tol, float *err_out, double *mean_out);
bbg_status read_step_state(bbg_solver s);
void add_substep_stats(bbg_solver s, float dt);
int mlp_mode(bbg_solver s);
void mlp_after_substep(bbg_solver s, int mm);
bool warm_active(bbg_solver s);
int clamp_total(bbg_solver s);
float warm_scale(bbg_solver s);
float pressure_unit(bbg_solver s, float delta);
void launch_prologue(bbg_solver s, int work, float dt, float delta, int max_it, cudaStream_t cs);
int training_steps(bbg_solver s);
void launch_training(bbg_solver s, float delta, cudaStream_t cs);
bbg_status corrector(bbg_solver s, float dt, float delta, int max_it);
bbg_status pseudo_viscosity(bbg_solver s, float dt);
unsigned fbits(float f);
bbg_status capture_substep(bbg_solver s, float dt, int max_it, float delta, bbg_solver_s::SubstepGraph &g);
void after_substep(bbg_solver s, float dt);
bbg_status substep(bbg_solver s, float dt);
bbg_status max_force(bbg_solver s, float *out);
int field_components(int f);
float4 *vec_field(bbg_solver s, int f);
float *scalar_field(bbg_solver s, int f);
// device positions / velocities (d_vel may be null) as the solver's n particles
bbg_status upload_common(bbg_solver s, const float *d_pos, const float *d_vel, int n);

// attaches device node values (owned by the solver from here on) to collider `index`
bbg_status attach_field(bbg_solver s, int index, const bbg_sdf_grid &g, float *values);

// Scratch of one post-processing call: scratch_begin at its start (after the previous call
// synchronised its stream), then one scratch_bytes / scratch_get per buffer; the buffers
// stay valid until the next scratch_begin.
cudaError_t scratch_begin(bbg_solver s);
cudaError_t scratch_bytes(bbg_solver s, size_t bytes, void **out);
template <class T>
cudaError_t scratch_get(bbg_solver s, size_t count, T **out) {
    return scratch_bytes(s, sizeof(T) * (count ? count : 1), reinterpret_cast<void **>(out));
}
void scratch_free(bbg_solver s);

// frees and reallocates (no copy): buffers that only grow
template <class T>
bbg_status reserve(T **p, size_t need) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    CK(cudaMalloc((void **)p, sizeof(T) * (need ? need : 1)));
    return BBG_OK;
}

}  // namespace bbg_api

using namespace bbg_api;
