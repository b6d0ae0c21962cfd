// bbg_kernels.h -- host-callable launchers of the bubbles_gb300 kernels.
#pragma once

#include "bbg_internal.cuh"
#include "prof.h"
#include "tile.cuh"

namespace bbg {

// Launch tuning of the neighbour passes (bbg_set_tuning): block size (= tile) and how
// many members' records each thread requests together, per pass.
struct Tuning {
    int block = 128;       // 64, 128 or 256
    int batch_np = 4;      // non-pressure pass (two records per member)
    int batch_pd = 4;      // predicted-density pass
    int batch_pf = 4;      // pressure-force pass
    int prune = 0;         // density pass: walk only the cells each particle's sphere reaches (1)
    int ppt = 1;           // particles per thread of the predicted-density and pressure-force passes (1, 2)
    int tile_order = 0;    // member-walking passes: 0 block b takes tile b; 1 SM-strided (tile_of_block)
    int worklist = 1;      // batch corrector: 0 all tiles, 1 a block per listed tile, 2 persistent blocks
    int wl_grid_pd = 0;    // batch: resident blocks of the persistent predicted-density and
    int wl_grid_pf = 0;    // pressure-force passes for this shape (update_worklist_grid)
};

// Device buffers of one solver (all sized for `capacity` particles / grid cells).
struct DevBufs {
    float4 *pos[2], *vel[2];   // ping-pong particle state
    int *pid[2];               // original id of each sorted slot
    int *slot;                 // sorted slot of each original id
    float4 *force, *xstar, *pforce, *smoothed;
    float *rho, *press, *rhostar, *derr;
    unsigned *cell;            // cell id of each sorted slot (last grid update)
    unsigned *cell_old;        // scratch: cell id of each pre-sort slot
    unsigned *sub;             // scratch: arrival index inside the cell
    unsigned *count;           // per-cell counts (kept zero between updates)
    unsigned *start;           // cell start offsets, total + 1 entries
    unsigned *partials;        // scan partials
    uint2 *tmp;                // scratch: (original id, pre-sort slot) placed by cell
    int *nbr;                  // neighbour count of each sorted slot
    ListEntry *list;           // member lists: kMaxList entries per particle,
                               // member-major (list[q * n + i]; tile.cuh)
    float *inv_rho;            // 1 / density
    float *soa;                // density pass: step-start x, y, z as three arrays of soa_stride
    size_t soa_stride;
    float *pprev;              // pressure of the previous substep, in the current order
    StepState *st;
    float *stage;              // n * 3 floats of staging for host copies
    unsigned *red;             // reduction scratch (max |F|)
    Prof *prof;                // host-side launch profiler (may be null)
    Tuning tune;
};

#define BBG_PBEGIN(B, id, s, it) do { if ((B).prof) (B).prof->begin((id), (s), (it)); } while (0)
#define BBG_PEND(B, s) do { if ((B).prof) (B).prof->end(s); } while (0)

// api.cu: record the message returned by bbg_last_error()
int set_error(int code, const char *fmt, ...);

// grid.cu
size_t scan_partials_needed(unsigned cells);
// exclusive scan of per-cell counts into start[0..cells] (zeroes the counts)
void launch_cell_scan(unsigned *count, unsigned cells, unsigned *partials, unsigned *start,
                      cudaStream_t s);
// carry_in / carry_out (optional): one float per particle gathered into the new order
void launch_grid_update(const Params &P, const DevBufs &B, int src_buf, int pid_src,
                        cudaStream_t s, const float *carry_in = nullptr, float *carry_out = nullptr);
void launch_upload(const DevBufs &B, int buf, int pid_buf, const float *d_pos, const float *d_vel,
                   int n, cudaStream_t s);
void launch_download(const DevBufs &B, int buf, int pid_buf, float *d_pos, float *d_vel, int n,
                     cudaStream_t s);
// field gather/scatter between caller order (n*3 or n floats) and sorted slots
void launch_get_vec(const float4 *src, const int *slot, float *out, int n, cudaStream_t s);
void launch_set_vec(float4 *dst, const int *slot, const float *in, int n, cudaStream_t s);
void launch_get_scalar(const float *src, const int *slot, float *out, int n, cudaStream_t s);
void launch_set_scalar(float *dst, const int *slot, const float *in, int n, cudaStream_t s);
void launch_get_uint(const unsigned *src, const int *slot, unsigned *out, int n, cudaStream_t s);
void launch_get_int(const int *src, const int *slot, int *out, int n, cudaStream_t s);
void launch_fill_vec(float4 *dst, float x, float y, float z, int n, cudaStream_t s);
void launch_max_force(const float4 *force, int n, unsigned *out_bits, cudaStream_t s);

// sph.cu
void launch_density(const Params &P, const DevBufs &B, int buf, int compute_pressure,
                    cudaStream_t s);
// members (other than itself, as original ids) of every particle with original id in
// [a, b) at the last density pass on buffer buf: counts[id - a], maxm ids per row of out
void launch_export_members(const Params &P, const DevBufs &B, int buf, int pid_buf, int a, int b, int maxm,
                           int *counts, int *out, cudaStream_t s);
// divsum != null: also the velocity-divergence sum of each particle (learned warm start);
// warm: the corrector's start pressure is set, add its pressure force and predict from F + Fp
void launch_non_pressure(const Params &P, const DevBufs &B, int buf, int predict, float dt,
                         float dt_over_m, cudaStream_t s, float *divsum = nullptr, bool warm = false);
void launch_predict_first(const Params &P, const DevBufs &B, int buf, int is_first, float dt,
                          float dt_over_m, cudaStream_t s);
void launch_pack_acoef(const Params &P, const DevBufs &B, int buf, cudaStream_t s);
// clamp_total: warm-started corrector (the total pressure, not the increment, is clamped)
// batch: resident blocks of the persistent corrector passes for B.tune's launch shape
// (set outside stream capture: creation and bbg_set_tuning)
void update_worklist_grid(DevBufs &B);
void launch_pred_density(const Params &P, const DevBufs &B, int buf, int k, float delta,
                         cudaStream_t s, int clamp_total = 0);
// mode 0: pressure force, then the next prediction or (converged) integration;
// 1: pressure force only; 2: pressure force and prediction, never integration.
void launch_pressure_force(const Params &P, const DevBufs &B, int buf, int k, int max_it,
                           float dt, float dt_over_m, cudaStream_t s, int mode = 0);
// p = scale * previous pressure, rho* = rho, pos.w = p / rho^2
void launch_warm_start(const Params &P, const DevBufs &B, int buf, float scale, cudaStream_t s);
void launch_corrector_control(const Params &P, const DevBufs &B, int max_it,
                              cudaGraphConditionalHandle handle, cudaStream_t s);
void launch_sph_forces(const Params &P, const DevBufs &B, int buf, float dt, cudaStream_t s);
void launch_accumulate_integrate(const Params &P, const DevBufs &B, int buf, float dt,
                                 cudaStream_t s);
void launch_integrate(const Params &P, const DevBufs &B, int buf, float dt, cudaStream_t s);
// FP64 totals (mass, kinetic, potential, momentum x, y, z): energy_blocks(n) partial rows
constexpr int kEnergyTerms = 6;
int energy_blocks(int n);
void launch_energy(const Params &P, const DevBufs &B, int buf, const double g[3], double *partial, cudaStream_t s);
void launch_pseudo_viscosity(const Params &P, const DevBufs &B, int new_buf, float factor,
                             cudaStream_t s);

// GenerateShapeSDF of an analytic shape into the node values of grid g (sdf.cu)
void launch_sdf_generate(const ShapeDev &shape, const SdfDev &g, float iz, float iz6, float *out, cudaStream_t s);

// Shape queries of collider `index` at n points (xyz); 14 floats per point out (sdf.cu)
void launch_shape_query(const Params &P, int index, int n, const float *pts, float *out, cudaStream_t s);

// GenerateShapeSDF of a triangle mesh (9 floats per triangle) into g's node values; stuck
// counts rays that gave up (mesh.cu)
// mesh.cu: tiles of consecutive triangles with their bounding boxes (6 floats per tile)
int mesh_tiles(int ntri);
void mesh_tile_bounds(const float *tri, int ntri, float *tiles);
void mesh_morton_order(const float *tri, int ntri, const float lo[3], const float hi[3], float *sorted);
// tri/tiles: the caller's order (ray passes); dtri/dtiles: the Morton order (distance pass)
void launch_mesh_sdf(const float *tri, int ntri, const float *tiles, const float *dtri, const float *dtiles,
                     float margin, const SdfDev &g, const float lo[3], const float hi[3], const float gamma[4],
                     float *out, unsigned *stuck, cudaStream_t s);

// LNM boundary levels (1, 2, 0) of n sorted slots into out (caller order through pid);
// level: one int per cell (boundary.cu)
// boundary.cu: arguments of the particle tests of the boundary classification
struct BoundaryArgs {
    GridDev g;
    float iz;
    const unsigned *start;
    const float4 *pos;    // current positions, slot order
    const float *rho;     // densities, slot order (Xiaowei)
    const int *pid;
    float x_rhot;         // Xiaowei: 0.7 * water density; 6h squared; 315 / (64 pi (6h)^3);
    float x_h2;           // 0.15 * 6h (as double)
    double x_wc, x_limit;
    float d_rad, d_lim;   // Dilts: 0.75 * radius; 2 rad - Epsilon
    float spoke[260];     // sin u, cos u, sin v, cos v of the 65 spoke angles (host libm)
};
void launch_lnm_single(const GridDev &g, const unsigned *start, const unsigned *cell, const int *pid, int n,
                       int delta, int *level, int *out, cudaStream_t s);
void launch_lnm_once(const GridDev &g, const unsigned *start, int *level, int L, int *changed, cudaStream_t s);
void launch_lnm_extended_finish(const GridDev &g, float iz, const float4 *pos, const unsigned *start,
                                const unsigned *cell, const int *pid, int n, int delta, int *level, int *val,
                                int *out, cudaStream_t s);
void launch_lnm_geometric(const BoundaryArgs &A, const unsigned *cell, int n, int delta, int algorithm,
                          int *level, int *queue, int *counts, int *out, cudaStream_t s);
void launch_boundary_test(const BoundaryArgs &A, int algorithm, int n, int *out, cudaStream_t s);
// surface.cu: ParticlesToSDF_Surface's field (method 0 Zhu-Bridson, 1 SPH)
struct SurfaceArgs {
    GridDev g;
    float iz, iz6;
    const unsigned *start;
    const float4 *pos;
    const float *rho;
    int method;
    int nodes[3];
    float org[3], sp[3];
    float inf;            // the domain grid's diagonal length
    float radius;         // kernel radius
    float offset;         // Zhu-Bridson: radius x threshold
    float mass, r2;       // SPH: particle mass, radius squared,
    double wc;            // 315 / (64 pi radius^3)
};
void launch_particle_sdf(const SurfaceArgs &A, float *out, cudaStream_t s);
void launch_lnm(const GridDev &g, const unsigned *start, const unsigned *cell, const int *pid, int n, int delta,
                int *level, int *out, cudaStream_t s);

// Marching cubes of a vertex-centred field (mc.cu)
struct McInput {
    const float *values;   // device, x fastest
    int nodes[3];
    float origin[3], spacing[3];
    float inv[3];          // (float)(1.0 / spacing)
    float iso;
};
cudaError_t mc_prepare();
cudaError_t mc_count(const McInput &in, unsigned *ntri_cube, unsigned *tri_start, unsigned *tri_part,
                     unsigned *crossing, unsigned *flag_copy, unsigned *vindex, unsigned *v_part, unsigned *h,
                     size_t *ntri, size_t *nvert, cudaStream_t s);
void mc_emit(const McInput &in, const unsigned *tri_start, const unsigned *crossing, const unsigned *vindex,
             int rotate, float *points, float *normals, int *tris, cudaStream_t s);

}  // namespace bbg
