/*
 * bbg.h -- C ABI of bubbles_gb300, the GB300-native (sm_103a) Bubbles 3D SPH /
 * PCISPH particle step.
 *
 * The reference has no plugin or FFI layer; its seam is the free-function and class
 * layer of src/core/sph_solver.h:76-196 and src/core/pcisph_solver.h:56-99, with the
 * GPU/CPU choice made inside AdvanceTimeStep (src/solvers/pcisph_solver3.cpp:42-65,
 * src/solvers/sph_solver3.cpp:48-67).  Every entry point below replaces one of those
 * functions (cited beside it) with plain pointers, sizes and a status code.
 *
 * Conventions
 *  - All functions return bbg_status; BBG_OK is 0.  bbg_last_error() gives a message.
 *  - Host particle arrays are float xyz triples (n*3) in the caller's particle order
 *    (the reference's vec3f with Float=float); scalar fields are n floats.
 *  - "_device" variants take device pointers and never synchronise.
 *  - Device state is FP32 structure-of-arrays, re-sorted by grid cell every substep;
 *    the caller's particle order is kept through an id permutation.
 *  - The library has no CPU fallback: without a CUDA device every compute call fails
 *    with BBG_ERR_NO_DEVICE.
 */
#ifndef BBG_H
#define BBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int bbg_status;
#define BBG_OK 0
#define BBG_ERR_INVALID_ARGUMENT 1
#define BBG_ERR_CUDA 2
#define BBG_ERR_OUT_OF_MEMORY 3
#define BBG_ERR_CAPACITY 4
#define BBG_ERR_STATE 5
#define BBG_ERR_NO_DEVICE 6
#define BBG_ERR_NOT_FOUND 7

#define BBG_SOLVER_PCISPH 0
#define BBG_SOLVER_SPH 1

/* PCISPH corrector modes.  AS_SHIPPED reproduces the reference exactly: it never
 * stores densityErrors (pcisph_equations3.cpp:17,82-89), so its convergence test
 * always passes after one predict-correct pass.  TOLERANCE stores the per-particle
 * density error the reference computes and iterates until
 * max|err|/rho0 < max_density_error_ratio or max_iterations. */
#define BBG_PCISPH_AS_SHIPPED 0
#define BBG_PCISPH_TOLERANCE 1

/* Initial pressure of the corrector.  ZERO is the reference (p = 0, Fp = 0 at k = 0,
 * pcisph_equations3.cpp:13-19).  PREVIOUS starts from each particle's converged pressure
 * of the previous substep, and LEARNED from the per-particle MLP estimate; both then run
 * one pressure-force pass to predict positions and continue with the unchanged corrector
 * to the same tolerance, so only the number of iterations changes. */
#define BBG_PRESSURE_INIT_ZERO 0
#define BBG_PRESSURE_INIT_PREVIOUS 1
#define BBG_PRESSURE_INIT_LEARNED 2

/* Pressure update of a warm-started corrector.  MONOTONE (default): the reference update
 * (negative increments scaled by the negative-pressure scale) from the warm start, which
 * therefore has to underestimate: warm_scale damps it (0.5 for PREVIOUS and 0.9 for
 * LEARNED when warm_scale <= 0).  CLAMP_TOTAL: p += delta * err with either sign and the
 * total clamped like a negative pressure, so an overestimated start can come down; over
 * long runs it saves few iterations and with LEARNED starts it has diverged. */
#define BBG_WARM_CLAMP_TOTAL 0
#define BBG_WARM_MONOTONE 1

#define BBG_SHAPE_BOX 1
#define BBG_SHAPE_SPHERE 2
#define BBG_SHAPE_SDF 3      /* defined by a signed-distance field alone (MakeSDFShape) */
#define BBG_MAX_COLLIDERS 16

/* Field ids for bbg_get_field / bbg_set_field (ParticleSet3 accessors,
 * src/core/particle.h:154-401, and PciSphSolverData3, pcisph_solver.h:17-25). */
#define BBG_FIELD_POSITION 0
#define BBG_FIELD_VELOCITY 1
#define BBG_FIELD_FORCE 2
#define BBG_FIELD_INTERACTION 3
#define BBG_FIELD_DENSITY 4
#define BBG_FIELD_PRESSURE 5
#define BBG_FIELD_PRED_POSITION 6
#define BBG_FIELD_PRESSURE_FORCE 8
#define BBG_FIELD_PRED_DENSITY 9
#define BBG_FIELD_DENSITY_ERROR 10
/* Learned warm start only: each particle's velocity-divergence sum of the last substep,
 * a feature of the next one (the state a host round trip must carry, with the pressure). */
#define BBG_FIELD_DIVERGENCE 11

typedef struct bbg_solver_s *bbg_solver;

/* Scene description: SphSolverData3 (sph_solver.h:31-50), SphParticleSet3
 * (particle.h:508-609), the domain grid of UtilBuildGridForDomain (util.cpp:269-287)
 * and the PciSphSolver3 corrector controls (pcisph_solver.h:56-83). */
typedef struct {
    int solver_kind;                 /* BBG_SOLVER_PCISPH / BBG_SOLVER_SPH */
    double eos_exponent;             /* 7 */
    double negative_pressure_scale;  /* 0 */
    double viscosity;                /* 0.04 */
    double pseudo_viscosity;         /* 10 */
    double sound_speed;              /* 100 */
    double drag_coefficient;         /* 1e-4 */
    double gravity[3];               /* constant interaction; reference default (0,-9.8,0) */
    double target_density;           /* 1000 */
    double target_spacing;           /* particle spacing h0; also the particle radius */
    double relative_kernel_radius;   /* 2: kernel radius = 2 h0 */
    double mass;                     /* > 0 overrides the BCC-lattice mass of ComputeMass */
    double domain_min[3];            /* domain bounds handed to UtilBuildGridForDomain */
    double domain_max[3];
    double grid_spacing_scale;       /* 2: cell length = spacing * scale */
    double time_step_limit_scale;    /* Advance CFL scale: 5 (PCISPH), 1 (SPH) */
    int pcisph_mode;                 /* BBG_PCISPH_AS_SHIPPED / BBG_PCISPH_TOLERANCE */
    int max_iterations;              /* corrector cap (reference call site: 5) */
    double max_density_error_ratio;  /* corrector tolerance (reference: 0.01) */
    int device;                      /* CUDA device ordinal */
    int pressure_init;               /* BBG_PRESSURE_INIT_* (reference: ZERO) */
    int warm_rule;                   /* BBG_WARM_* for a non-zero pressure_init */
    double warm_scale;               /* start pressure = warm_scale * estimate; <= 0: default */
} bbg_solver_desc;

/* Analytic collider shape with a translation-only ObjectToWorld (MakeBox,
 * src/shapes/box.cpp:6-10; MakeSphere, src/shapes/sphere.cpp:5-9). */
typedef struct {
    int type;            /* BBG_SHAPE_BOX / BBG_SHAPE_SPHERE */
    int reverse;         /* reverseOrientation; 1 for a container box */
    double center[3];
    double size[3];      /* box edge lengths; size[0] is the sphere radius */
    double friction;     /* Collider3::frictionCoefficient */
} bbg_shape;

typedef struct {
    int substeps;                     /* substeps run by this call */
    int iterations;                   /* corrector iterations summed over substeps */
    int max_iterations_in_substep;
    int not_converged;                /* substeps that hit max_iterations above tolerance */
    double last_dt;                   /* last substep length */
    double max_density_error_ratio;   /* last substep's final max|err|/rho0 */
    double mean_density_error_ratio;  /* last substep's final mean|err|/rho0 (FP64 sum) */
    int neighbor_overflow;            /* particles with > 100 neighbours (reference bucket cap) */
    int out_of_grid;                  /* particles hashed outside the grid (clamped) */
    double max_force;                 /* max |F| after the last substep (CFL input) */
    int crowded;                      /* cells / particles past the work caps of a degenerate
                                         state (a cell of > 512 particles, > 1,024 candidates) */
    int nonfinite;                    /* particles whose integrated position or velocity is
                                         not finite (NaN or infinite) in the last substep */
} bbg_step_stats;

/* Learned warm start (pressure_init = BBG_PRESSURE_INIT_LEARNED): a per-particle MLP
 * 4 -> 64 -> 64 -> 1 (GELU, BF16 tensor-core inference with FP32 accumulation) maps
 * (100 (rho - rho0) / rho0, -100 dt div v, (neighbours - 1) / 32, p_prev / p_unit) to
 * p / p_unit, p_unit = delta rho0 / 100.  The first train_substeps substeps run the plain
 * corrector and train the model online (FP32 forward / backward, Adam) on their
 * (features, converged pressure) pairs; later substeps start the unchanged corrector from
 * the model's estimate.  No reference counterpart. */
#define BBG_MLP_PARAMS 4545   /* W1[4][64], b1[64], W2[64][64], b2[64], w3[64], b3 */
typedef struct {
    int train_substeps;        /* plain substeps that train the model before it is used (200) */
    int batch;                 /* training pairs per Adam step (16384) */
    int steps_per_substep;     /* Adam steps after each training substep (4) */
    double learning_rate;      /* 1e-3 */
    double beta1, beta2, epsilon;   /* 0.9, 0.999, 1e-8 */
    unsigned long long seed;   /* weight initialisation */
    double expectile;          /* training loss: squared error weighted (1 - tau) above and
                                  tau below the target (0.5: mean squared error); tau < 0.5
                                  biases estimates low, which suits the monotone update */
    int finetune_steps;        /* Adam steps after each learned substep on its own converged
                                  pressure (0: the model is fixed after training) */
    int refresh_interval;      /* after training, every refresh_interval-th substep runs the
                                  plain corrector and trains on it again (0: never) */
} bbg_mlp_desc;

/* ----- library ----------------------------------------------------------- */
const char *bbg_version(void);
const char *bbg_status_string(bbg_status s);
const char *bbg_last_error(void);
/* Number of CUDA devices visible (0 without a GPU). */
bbg_status bbg_device_count(int *count);

/* ----- host-side setup math (no GPU needed) ------------------------------- */
/* DefaultSphSolverData3 (sph_solver3.cpp:124-151) + PciSphSolver3::Initialize
 * (pcisph_solver3.cpp:9-14). */
bbg_status bbg_solver_desc_default(bbg_solver_desc *desc, int solver_kind);
/* UtilBuildGridForDomain + Grid::Build (util.cpp:269-287, grid.h:627-666) in the
 * reference's FP32 arithmetic.  geo = minPoint[3], cellsLen[3], bounds.pMin[3],
 * bounds.pMax[3]. */
bbg_status bbg_build_grid(const double domain_min[3], const double domain_max[3],
                          double spacing, double spacing_scale, int dims[3], double geo[12]);
/* SphParticleSet3::ComputeMass (particle.h:557-582): lattice 0 = BCC (the reference),
 * 1 = simple cubic at the same spacing. */
bbg_status bbg_compute_mass(int lattice, double target_density, double spacing,
                            double kernel_radius, double *mass);
/* PciSphSolver3::ComputeDeltaDenom (pcisph_solver3.cpp:148-180). */
bbg_status bbg_compute_delta_denom(double spacing, double kernel_radius, double *denom);

/* ----- solver lifetime (PciSphSolver3 / SphSolver3) ------------------------ */
/* Initialize: allocates device state for up to `capacity` particles. */
bbg_status bbg_create(const bbg_solver_desc *desc, int capacity, bbg_solver *out);
bbg_status bbg_destroy(bbg_solver s);
/* SetColliders (pcisph_solver3.cpp:27-31). */
bbg_status bbg_set_colliders(bbg_solver s, const bbg_shape *shapes, int count);
/* ParticleSetBuilder3::MakeParticleSet (particle.h:685-709): host xyz arrays. */
bbg_status bbg_upload_particles(bbg_solver s, const float *pos, const float *vel, int n);
bbg_status bbg_upload_particles_device(bbg_solver s, const float *d_pos, const float *d_vel,
                                       int n);
/* Setup (pcisph_solver3.cpp:103-146): mass, delta denominator, first distribution. */
bbg_status bbg_setup(bbg_solver s);
/* Use the caller's cudaStream_t (NULL = the solver's own stream). */
bbg_status bbg_set_stream(bbg_solver s, void *cuda_stream);
bbg_status bbg_synchronize(bbg_solver s);

/* ----- stepping ----------------------------------------------------------- */
/* One substep with the state in host memory, as a host that keeps its particles on the CPU
 * calls it every step: positions and velocities (n each, xyz) uploaded, optionally the warm
 * start's carried pressure and divergence (BBG_FIELD_PRESSURE / BBG_FIELD_DIVERGENCE,
 * caller order), AdvanceTimeStep(dt), then the same fields downloaded into the *_out arrays
 * that are not NULL.  Equivalent to bbg_upload_particles, bbg_set_field,
 * bbg_advance_time_step, bbg_download and bbg_get_field in sequence, queued on the solver's
 * stream with a single synchronisation at the end (stats as bbg_advance_time_step's). */
bbg_status bbg_step_host(bbg_solver s, double dt, int n, const float *pos, const float *vel, const float *pressure,
                         const float *divergence, float *pos_out, float *vel_out, float *pressure_out,
                         float *divergence_out, bbg_step_stats *stats);

/* Advance(dt) with the CFL substep loop (pcisph_solver3.cpp:67-89,
 * sph_solver3.cpp:69-93). */
bbg_status bbg_advance(bbg_solver s, double dt, bbg_step_stats *stats);
/* AdvanceTimeStep: one substep of length dt (pcisph_solver3.cpp:42-65,
 * sph_solver3.cpp:48-67).  Asynchronous when stats is NULL. */
bbg_status bbg_advance_time_step(bbg_solver s, double dt, bbg_step_stats *stats);
/* Replay whole substeps as CUDA graphs (default on): the corrector runs as a conditional
 * WHILE node whose condition the device sets after each iteration, so a substep is one
 * graph launch with no host round trip.  Graphs are cached per substep length, so the
 * first substep of a new dt pays for a capture.  Profiling uses direct launches. */
bbg_status bbg_use_cuda_graphs(bbg_solver s, int enable);
/* Read the statistics of the last substep (synchronises). */
bbg_status bbg_get_stats(bbg_solver s, bbg_step_stats *stats);

/* ----- particle frames --------------------------------------------------------- */
/* The block SerializerSaveSphDataSet3 (src/third/serializer.cpp:880-923) appends to a
 * frame file, for the caller-order particles: FluidBegin, "Type" particles, "Count",
 * "Format", "Spacing", DataBegin, one line per particle (two tabs, the selected fields as
 * %g numbers), DataEnd, FluidEnd.  Lines are formatted and packed on the device; the
 * numbers are exactly printf("%g") of the FP32 state.  Flags: the reference's
 * SERIALIZER_POSITION / VELOCITY / DENSITY / MASS (src/third/serializer.h:7-12). */
#define BBG_FRAME_POSITION 0x01
#define BBG_FRAME_VELOCITY 0x02
#define BBG_FRAME_DENSITY 0x04
#define BBG_FRAME_MASS 0x20
/* Into buf (not terminated); *length is the frame's size, also when buf is too small
 * (BBG_ERR_CAPACITY). */
bbg_status bbg_frame_text(bbg_solver s, int flags, char *buf, size_t capacity, size_t *length);
/* Appends the block to a file (fopen "a+", as the reference). */
bbg_status bbg_frame_append(bbg_solver s, int flags, const char *path);
/* printf("%g", (double)value) through the device formatter's code, on the host (at most
 * 14 characters, not terminated). */
bbg_status bbg_format_g(float value, char *out, int *length);
/* SerializerLoadSphDataSet3 (src/third/serializer.cpp:562-577): the particles of the
 * first fluid section of a frame become the solver's particles (positions and velocities;
 * zero where the section's format lacks them), as if built by a ParticleSetBuilder3 and
 * uploaded.  The header is read on the host (SerializerFindFluidSection, :145-181); the data
 * lines are split and parsed on the device with the reference's number reader
 * (src/third/obj_loader.cpp:56-168, 270-278) in the same double operations, so every value
 * equals the reference's (NaN payloads aside).  Lines are skipped as the reference skips
 * them (empty, blank, '#'; with the 'o' rule, boundary value 0); the data ends at the first
 * line holding "DataEnd".  *flags: in, the flags used when the section has no "Format";
 * out, the section's.  Errors: no complete section, an unknown format letter, fewer
 * particle lines than "Count" (the reference reads past its array there), more particles
 * than the capacity.  A file is read only up to the end of its first section. */
bbg_status bbg_frame_load(bbg_solver s, const char *path, int *flags);
bbg_status bbg_frame_load_text(bbg_solver s, const char *text, size_t length, int *flags);
/* The header step alone (host only, no GPU): the first fluid section's flags (in/out as
 * above), "Count", and its data lines [*data_begin, *data_end) as byte offsets. */
bbg_status bbg_frame_find_section(const char *text, size_t length, int *flags, int *count,
                                  size_t *data_begin, size_t *data_end);

/* ----- checkpoint (exact resume) ------------------------------------------------ */
/* The reference saves text frames only (SerializerSaveSphDataSet3,
 * src/third/serializer.cpp:1027) and reloads positions and velocities from them
 * (SerializerLoadSphDataSet3, :562-577), so its resume loses pressure, forces and the CFL
 * input.  A checkpoint holds the full state in binary: the solver description (checked
 * on load), the colliders with their signed-distance fields (grid and node values; the
 * fields attached to the loading solver are replaced by these), the scene layout of a
 * batch, every valid per-particle field in caller order (positions, velocities, forces,
 * density, pressure, predicted state, the carried divergence) and the learned warm start's
 * weights, Adam moments and training counters.  Loading it into a solver created with the
 * same description (any device, capacity >= the particle count) continues the run bit for
 * bit.  A file with an unknown collider type, a field slot out of range or used twice, a
 * field-only collider without its field or a truncated record is refused
 * (BBG_ERR_INVALID_ARGUMENT) before the solver changes.  Native byte order. */
bbg_status bbg_checkpoint_save(bbg_solver s, const char *path);
bbg_status bbg_checkpoint_load(bbg_solver s, const char *path);
/* The same bytes through memory; *length is the size, also when buf is too small
 * (BBG_ERR_CAPACITY). */
bbg_status bbg_checkpoint_write(bbg_solver s, void *buf, size_t capacity, size_t *length);
bbg_status bbg_checkpoint_read(bbg_solver s, const void *buf, size_t length);

/* ----- colliders with signed-distance fields ---------------------------------------- */
/* A vertex-centred FieldGrid3f (src/core/grid.h:950-1240): nodes[k] = cells + 1 per axis,
 * node (i, j, k) at origin + spacing * (i, j, k), values x fastest.  A collider with a
 * field resolves collisions as the reference's shapes with a filled grid do
 * (ColliderSet3::ResolveCollision, src/core/collider.cpp:238-264): the target is the least
 * |ClosestDistance| (analytic for a box or sphere, the field's trilinear sample for a
 * BBG_SHAPE_SDF collider), the closest point is Shape::ClosestPointBySDF
 * (src/shapes/bvh.cpp:666-707: five gradient steps at most), IsInside is sample < 0.  A
 * field with `bounded` set is a mesh's: positions outside [bounds_min, bounds_max] never
 * collide with it (Collider3::OptmizedClosestPointCheck); its target distance is the
 * field's sample where the reference measures the mesh itself.  At most 4 fields; setting
 * the colliders again drops them. */
typedef struct {
    int nodes[3];
    double origin[3];
    double spacing[3];
    int bounded;
    double bounds_min[3], bounds_max[3];
} bbg_sdf_grid;
bbg_status bbg_collider_set_sdf(bbg_solver s, int index, const bbg_sdf_grid *grid, const float *values);
/* GenerateShapeSDF (src/core/shape.cpp:479-510) of a box or sphere collider on the device:
 * the shape's bounds widened by margin x extent, ceil(width / dx) cells across, nodes set
 * to max(|ClosestDistance|, 1e-5) signed by IsInside; the field is attached to the
 * collider.  Reference defaults: dx 0.01, margin 0.1. */
bbg_status bbg_collider_generate_sdf(bbg_solver s, int index, double dx, double margin);
/* GenerateShapeSDF of a triangle mesh (MakeMesh + GenerateShapeSDF, src/shapes/bvh.cpp:51-56,
 * src/core/shape.cpp:479-510) on the device: vertices xyz (nv), triangles as vertex index
 * triples (nt).  The grid covers the mesh bounds widened by margin x extent; a node holds
 * max(least DistanceTriangle, 1e-5) (bvh.cpp:212-242), negative when a ray towards the
 * bounds' centre crosses the mesh an odd number of times (MeshIsPointInside,
 * shape.cpp:349-369, with the reference's watertight ray-triangle test and ray re-spawning).
 * Values equal the reference's except where two triangles tie for a closest hit.  *stuck
 * counts rays that met more than 256 surfaces (counted outside). */
bbg_status bbg_mesh_sdf(bbg_solver s, const float *vertices, int nv, const int *triangles, int nt,
                        double dx, double margin, bbg_sdf_grid *grid, float *values, size_t capacity,
                        size_t *count, int *stuck);
/* The same field attached to a BBG_SHAPE_SDF collider as a mesh's (bounded by the mesh):
 * MakeCollider3 of a mesh shape, which generates its field (src/core/collider.cpp:340-348). */
bbg_status bbg_collider_set_mesh(bbg_solver s, int index, const float *vertices, int nv, const int *triangles,
                                 int nt, double dx, double margin);
/* A collider's field: its grid, and its values when capacity (in floats) suffices;
 * *count = node count. */
bbg_status bbg_collider_get_sdf(bbg_solver s, int index, bbg_sdf_grid *grid, float *values, size_t capacity,
                                size_t *count);

/* Collider `index` queried at n points as the collision code sees it: its field's Sample
 * and Gradient (zeros without a field), Shape::ClosestPoint (point, normal, distance: signed
 * for an analytic shape, the marched distance with a field) and IsInside.  Any output may
 * be NULL. */
bbg_status bbg_collider_query(bbg_solver s, int index, int n, const float *points, float *sample,
                              float *gradient, float *closest, float *normal, float *distance,
                              int *inside);

/* ----- particle seeding (VolumeParticleEmitter3) --------------------------------- */
/* VolumeParticleEmitter3 (src/core/emitter.h:39-69, emitter.cpp:241-330) with a box or
 * sphere shape, one-shot, the zero velocity field: the BCC lattice of
 * BccLatticePointGenerator::ForEach (src/generator/bcclattice.cpp:6-36) over the shape's
 * bounds (or the given ones), each point moved by 0.5 * jitter * spacing *
 * SampleSphere(rand_float(), rand_float()), kept when Shape::SignedDistance <= 0, at most
 * max_particles, velocity = initial_velocity.  The lattice and the inside test run on the
 * device, one thread per lattice point, in the reference's float operations; the jitter
 * offsets are the C library's rand() sequence (seed it with srand as for the reference),
 * two values per lattice point like the reference's loop.  When max_particles stops the
 * reference's loop early it draws fewer values than this call (the emitted particles are
 * the same). */
typedef struct {
    bbg_shape shape;                 /* box or sphere (friction unused) */
    int use_bounds;                  /* 1: the lattice spans [bounds_min, bounds_max] */
    double bounds_min[3], bounds_max[3];
    double spacing;
    double jitter;                   /* 0: the exact lattice */
    double initial_velocity[3];
    int max_particles;               /* IntInfinity (2^31 - 1) by default */
} bbg_emitter_desc;
bbg_status bbg_emitter_desc_default(bbg_emitter_desc *desc);
/* append = 0: the emitted particles replace the solver's (a ParticleSetBuilder3 filled by
 * Emit, then MakeParticleSet and upload); append = 1: they follow the existing particles
 * (ContinuousParticleSetBuilder3::AddParticle and Commit), ids n .. n + emitted - 1. */
bbg_status bbg_emit_volume(bbg_solver s, const bbg_emitter_desc *desc, int append, int *emitted);

/* Continuous emission (ContinuousParticleSetBuilder3, src/core/grid.h:1246-1450).
 * bbg_map_grid = MapGrid (:1289-1321): remembers, for every occupied cell of the grid's last
 * distribution (one is made first when the particles were uploaded since), its particles'
 * positions in chain order; *mapped = how many.  bbg_map_grid_emit = MapGridEmit
 * (:1359-1402) with a constant velocity field: in every mapped cell holding fewer than 100
 * particles now (MaximumParticlesPerBucket), each of the first (100 - held) remembered
 * positions that no particle of the cell is closer to than `distance` becomes a new
 * particle after the existing ones, cells in ascending order, positions in chain order.
 * The cell's particles are those of the last distribution (at their current positions)
 * plus the ones added since, as Commit's DistributeByParticleList places them.  At the
 * capacity the call adds what fits and, like the reference's builder, later calls add
 * nothing.  One thread per remembered position on the device. */
bbg_status bbg_map_grid(bbg_solver s, int *mapped);
bbg_status bbg_map_grid_emit(bbg_solver s, double distance, const double velocity[3], int *emitted);

/* ----- boundary classification (LNM) ---------------------------------------------- */
/* LNMBoundary, fast variant (src/boundaries/lnm.h:24-139, 245-275) on the grid's last
 * distribution (one is made first when there is none): levels[i] of each particle (caller
 * order) is 1 when its cell lies on the grid's border or next to an empty cell, 2 when its
 * cell is next to a level-1 cell holding at most delta = (min cell length / h)^3 particles
 * (any number when unbounded), else 0.  One thread per cell, then one per particle. */
bbg_status bbg_lnm_boundary(bbg_solver s, double h, int unbounded, int *levels);

/* LNMBoundarySingle (lnm.h:167-256): the N2x2 classification in one pass.  A cell with
 * particles is L1 on the grid's border; otherwise its 5x5x5 neighbourhood, walked in the
 * reference's order (y, x, z), decides at the first adjacent empty cell (L1) or the first
 * adjacent cell holding at most delta particles that lies on the border (L2); without
 * either, L2 when an adjacent cell holding 1..delta particles touches an empty cell.
 * delta is (min cell length / h)^3 truncated to int, any count when that is 0 or unbounded. */
bbg_status bbg_lnm_boundary_single(bbg_solver s, double h, int unbounded, int *levels);

/* LNMBoundaryExtended (lnm.h:291-462): cell levels by sweeps (0 empty, 1 border or next to
 * an empty cell, k next to a level k-1 cell) for k up to max_level (max_level < 0: until a
 * sweep changes nothing); each particle takes its hashed cell's level (0 past max_level);
 * a non-L1 cell next to an L1 cell holding at most delta particles gives its particles 2,
 * the other level-2 cells 3; L1 cells 1. */
bbg_status bbg_lnm_boundary_extended(bbg_solver s, double h, int max_level, int unbounded, int *levels);

/* Particle tests of boundary.  XIAOWEI (xiaowei.h:21-78): density below 700, or the
 * std-kernel (radius 6h) weighted mean of the 27 cells' positions farther than 0.9h from
 * the particle; reads the set's densities (BBG_FIELD_DENSITY must be valid).  DILTS
 * (dilts.h:110-153): one of the 65 x 65 spoke points on the sphere of radius 0.75 x the
 * target spacing lies outside every overlapping neighbour's sphere (h unused). */
#define BBG_BOUNDARY_XIAOWEI 1
#define BBG_BOUNDARY_DILTS 2

/* LNMBoundary with a geometric L2 filter (algorithm XIAOWEI or DILTS; lnm.h:57-112,
 * 258-289): L1 as the fast variant; the particles of L2 cells are queued and marked 2 only
 * when the test finds them on the boundary, else 0.  queued / accepted (optional): the
 * work queue's size and accepted count, as the reference's bounds app reports them. */
bbg_status bbg_lnm_boundary_geometric(bbg_solver s, double h, int algorithm, int unbounded, int *levels,
                                      int *queued, int *accepted);

/* XiaoweiBoundary / DiltsSpokeBoundary (xiaowei.h:80-87, dilts.h:155-163): flags[i] = 1 for
 * each boundary particle, one thread per particle. */
bbg_status bbg_boundary_test(bbg_solver s, int method, double h, int *flags);

/* ----- the surface app's particle field ------------------------------------------ */
/* ParticlesToSDF_Surface (apps/surface.cpp:276-470): a vertex-centred field over the solver's
 * domain grid for marching cubes.  The field's grid: with resolution NULL, cells of
 * 2 x mc_spacing from the domain's min corner plus half a cell, ceil(extent / cell) cells
 * per axis; else resolution[k] nodes at the largest of extent / (resolution - 1).  Each
 * node outside the domain holds the domain's diagonal length; inside, over the particles of
 * the 27 cells around it:
 *   ZHU_BRIDSON: |p - x_avg| - 0.25 R, x_avg the mean of positions weighted by
 *                max(0, (1 - (d/R)^2)^3) for d < R (the diagonal length when no weight);
 *   SPH:         0.5 - sum (m / rho_j) W_std(d, R)  (BBG_FIELD_DENSITY must be valid).
 * The app builds its domain from the particles' bounds grown by the spacing, on cells of
 * twice the spacing, with an SPH set of that spacing and relative kernel radius 2.
 * With values NULL only *grid is filled; otherwise capacity must hold every node.  One
 * thread per node on the device. */
#define BBG_SURFACE_ZHU_BRIDSON 0
#define BBG_SURFACE_SPH 1
bbg_status bbg_particle_sdf(bbg_solver s, int method, double kernel_radius, double mc_spacing, const int *resolution,
                            bbg_sdf_grid *grid, float *values, size_t capacity);

/* ----- marching cubes ----------------------------------------------------------- */
/* MarchingCubes (src/reconstruction/marching_cubes.cpp:204-457) of a vertex-centred field
 * at iso on the device: a vertex on every grid edge whose ends straddle iso (at or below
 * counts as inside), placed and given a normal (interpolated central-difference gradients,
 * normalised) in the reference's float operations, so points and normals equal the
 * reference's; triangles face away from the inside (rotate_faces reverses them).  The
 * triangulation comes from a table derived here, not the reference's case table: in
 * ambiguous configurations the connectivity (and count) of triangles can differ.  Points
 * are ordered by edge (x edges, then y, then z, each by node), triangles by cube (x slowest,
 * z fastest).  With too small capacities (or NULL buffers) the counts are returned with
 * BBG_ERR_CAPACITY. */
bbg_status bbg_marching_cubes(bbg_solver s, const bbg_sdf_grid *grid, const float *values, double iso,
                              int rotate_faces, float *points, float *normals, size_t point_capacity,
                              int *triangles, size_t triangle_capacity, size_t *npoints, size_t *ntriangles);

/* ----- launch tuning ------------------------------------------------------------ */
/* Block size of the neighbour passes (each block walks one tile of consecutive cell-
 * sorted particles), how many members' records a thread requests together in the
 * non-pressure, predicted-density and pressure-force passes, and whether the density pass
 * leaves out the neighbour cells (and rows of cells) a particle's sphere cannot reach.
 * Results do not depend on them (bit for bit); bubbles_gb300.autotune measures and picks
 * them. */
typedef struct {
    int block_size;      /* 64, 128 (default) or 256 */
    int batch_np;        /* 2, 4 (default) or 8 */
    int batch_pd;
    int batch_pf;
    int prune;           /* 0 (default: measured faster on GB300) or 1 */
    int particles_per_thread;  /* predicted-density and pressure-force passes: 1 (default) or 2 */
    int tile_order;      /* member-walking passes: 0 (default) block b takes tile b; 1 blocks
                            b, b + S, b + 2S, ... (S = the SM count) take consecutive tiles */
    int batch_worklist;  /* batches: 0 one block per tile of every scene, 1 (default) one block
                            per tile of the scenes whose corrector still runs (a work list
                            rebuilt every iteration), 2 persistent blocks over that list */
} bbg_tuning;
bbg_status bbg_get_tuning(bbg_solver s, bbg_tuning *t);
bbg_status bbg_set_tuning(bbg_solver s, const bbg_tuning *t);

/* ----- batches of independent scenes ------------------------------------------ */
/* Many small scenes advanced together by one solver: every pass is one launch over all
 * of them.  The scenes share the solver description (spacing, density, corrector
 * controls, dt) and each has its own container, a reverse box collider (global colliders
 * of bbg_set_colliders are not used in a batch).  Containers are stacked along z with
 * two empty grid cells between them, so no particle has a neighbour in another scene;
 * each scene's corrector stops at its own convergence.  No reference counterpart. */
typedef struct {
    int count;                /* particles of the scene */
    double box_min[3];        /* its container in scene coordinates */
    double box_max[3];
} bbg_scene_desc;
bbg_status bbg_batch_create(const bbg_solver_desc *desc, const bbg_scene_desc *scenes, int count,
                            bbg_solver *out);
bbg_status bbg_batch_scene_count(bbg_solver s, int *count);
/* Translation of each scene into the packed domain (count x 3: packed = scene + offset). */
bbg_status bbg_batch_layout(bbg_solver s, double *offsets);
/* All particles, scene after scene, in scene coordinates (n x 3 each; vel may be NULL). */
bbg_status bbg_batch_upload(bbg_solver s, const float *pos, const float *vel);
bbg_status bbg_batch_download(bbg_solver s, float *pos, float *vel);
/* Corrector iterations and final max|err|/rho0 of each scene in the last substep. */
bbg_status bbg_batch_scene_stats(bbg_solver s, int *iterations, double *max_err);

/* ----- learned warm start ---------------------------------------------------- */
bbg_status bbg_mlp_desc_default(bbg_mlp_desc *desc);
/* (Re)initialise the model and its training schedule (allocates on first use). */
bbg_status bbg_mlp_configure(bbg_solver s, const bbg_mlp_desc *desc);
/* FP32 master parameters, BBG_MLP_PARAMS floats in the layout above. */
bbg_status bbg_mlp_get_params(bbg_solver s, float *theta);
bbg_status bbg_mlp_set_params(bbg_solver s, const float *theta);
/* Substeps already used for training; setting it to train_substeps or more switches a
 * model loaded with bbg_mlp_set_params straight to inference. */
bbg_status bbg_mlp_set_trained(bbg_solver s, int trained_substeps);
bbg_status bbg_mlp_status(bbg_solver s, int *trained_substeps, int *adam_steps, double *last_loss);
/* Raw network outputs (p / p_unit before the clamp at 0) for n host feature rows
 * (n x 4 floats), through the tensor-core inference kernel. */
bbg_status bbg_mlp_infer(bbg_solver s, const float *features, int n, float *out);
/* One forward / backward / Adam step on a host batch (batch x 4 features, batch targets). */
bbg_status bbg_mlp_train_batch(bbg_solver s, const float *features, const float *targets, int batch);
/* Features of the last substep in the caller's particle order (n x 4 floats). */
bbg_status bbg_mlp_get_features(bbg_solver s, float *out);

/* ----- individual passes (sph_solver.h:124-196, pcisph_solver.h:85-99) ------- */
bbg_status bbg_update_grid_distribution(bbg_solver s);          /* UpdateGridDistributionGPU */
bbg_status bbg_compute_particle_interaction(bbg_solver s);      /* ComputeParticleInteractionGPU */
bbg_status bbg_compute_density(bbg_solver s, int compute_pressure); /* ComputeDensityGPU */
bbg_status bbg_compute_non_pressure_force(bbg_solver s);        /* ComputeNonPressureForceGPU */
bbg_status bbg_compute_pressure_force(bbg_solver s, double dt); /* ComputePressureForceGPU (SPH,
                                                                   Jacobi order) */
bbg_status bbg_time_integration(bbg_solver s, double dt);       /* TimeIntegrationGPU */
bbg_status bbg_compute_pseudo_viscosity_interpolation(bbg_solver s, double dt);
/* ComputePressureForceAndIntegrate (pcisph_equations3.cpp:218-256). */
bbg_status bbg_compute_pressure_force_and_integrate(bbg_solver s, double dt,
                                                    double max_density_error_ratio,
                                                    double delta, int max_iterations,
                                                    bbg_step_stats *stats);
bbg_status bbg_compute_delta(bbg_solver s, double dt, double *delta);  /* ComputeDelta */
/* The corrector's passes on their own, for callers composing their own loop:
 * PredictVelocityAndPositionGPU (pcisph_equations3.cpp:50-56), PredictPressureGPU
 * (:108-112; the density error is stored), PredictPressureForceGPU (:173-177; from the
 * pressure and predicted-density fields) and AccumulateAndIntegrateGPU (:207-212). */
bbg_status bbg_predict_velocity_and_position(bbg_solver s, double dt, int is_first);
bbg_status bbg_predict_pressure(bbg_solver s, double delta);
bbg_status bbg_predict_pressure_force(bbg_solver s);
bbg_status bbg_accumulate_and_integrate(bbg_solver s, double dt);
/* SphParticleSet3::ComputeNumberOfTimeSteps (particle.h:584-608). */
bbg_status bbg_compute_number_of_time_steps(bbg_solver s, double remaining, double scale,
                                            unsigned *count);

/* ----- state access ------------------------------------------------------- */
bbg_status bbg_particle_count(bbg_solver s, int *n);
/* Host arrays in the caller's order.  Fields other than position and velocity are
 * permuted by every grid update; reading one that has not been recomputed since
 * returns BBG_ERR_STATE. */
bbg_status bbg_get_field(bbg_solver s, int field, float *out);
bbg_status bbg_set_field(bbg_solver s, int field, const float *in);
/* Position and velocity, host (synchronising) or device (asynchronous). */
bbg_status bbg_download(bbg_solver s, float *pos, float *vel);
bbg_status bbg_download_device(bbg_solver s, float *d_pos, float *d_vel);
/* Solver scalars: mass, kernel radius, delta denominator, (m/rho0)^2, spacing,
 * target density, particle radius, relative kernel radius. */
bbg_status bbg_get_scalars(bbg_solver s, double out[8]);
bbg_status bbg_get_grid(bbg_solver s, int dims[3], double geo[12]);
/* FP64 totals of the current state, reduced on the device (fixed block partials summed in
 * order, so repeatable): out = {mass, kinetic energy sum m|v|^2/2, potential energy
 * -sum m g.x in the scene's gravity, momentum x, y, z}.  The run logs of the large
 * configuration record them every 10 substeps. */
bbg_status bbg_energy(bbg_solver s, double out[6]);
/* Grid state after the last update: cell id of each particle (caller order),
 * particle count per cell, and particle ids in cell-sorted order (stable by id). */
bbg_status bbg_dump_grid(bbg_solver s, uint32_t *cell_of_particle, uint32_t *cell_counts,
                         uint32_t *sorted_ids);
/* Neighbour count of each particle (caller order) at the last grid update. */
bbg_status bbg_neighbor_counts(bbg_solver s, int32_t *counts);
/* Neighbour sets of the last density pass (Grid::DistributeParticleBucket's buckets,
 * src/core/grid.h:423-447, read back as ParticleSet3::GetParticleBucket would,
 * src/core/particle.h:22-60): counts[i] = members of particle i other than itself
 * (caller order, never truncated); ids[i * max_per_particle + q] = their caller ids in
 * the solver's visit order, -1 past the last, at most max_per_particle of them (0: counts
 * only).  BBG_ERR_STATE when no density pass ran on the current grid distribution or its
 * positions were overwritten since. */
bbg_status bbg_neighbor_lists(bbg_solver s, int max_per_particle, int32_t *counts, int32_t *ids);

/* ----- allocation-free grid sort ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc -- a host
 * application that owns the device-memory budget and loads this library as a plugin,
 * or code running where device allocation is forbidden.  It computes the grid of
 * bbg_update_grid_distribution + bbg_dump_grid on caller-owned device buffers:
 *   d_pos          n xyz float triples (caller order)
 *   d_cell_of      n cell ids (caller order)
 *   d_sorted_ids   n particle indices sorted by (cell id, index); a cell of more than
 *                  512 particles (a degenerate state) keeps the arrival order instead,
 *                  as the solver's grid does
 *   d_cell_start   cells + 1 offsets of each cell's range in d_sorted_ids
 *   d_out_of_grid  optional (NULL: not counted) one counter, set to the number of
 *                  particles outside the grid; like the solver's grid (and the
 *                  reference's hash), those are clamped into the edge cells
 * with the grid of UtilBuildGridForDomain(domain, spacing, spacing_scale).  It never
 * allocates: its scratch is one fixed __device__ array of BBG_NOALLOC_SCRATCH_BYTES
 * that every GPU loading the library holds until exit, so n and the cell count are
 * capped (BBG_ERR_CAPACITY beyond).  A call outside stream capture looks the array's
 * device address up (cudaGetSymbolAddress) on the current device, so a device reset
 * between calls is safe; a call inside a capture reuses the address of the last
 * uncaptured call there, so the first call on a device must not be captured
 * (BBG_ERR_STATE).  All calls share the array: calls whose GPU work overlaps race and
 * must be serialised.  Asynchronous on `cuda_stream` (NULL = the legacy default
 * stream). */
#define BBG_NOALLOC_MAX_PARTICLES 1048576
#define BBG_NOALLOC_MAX_CELLS 1048576
#define BBG_NOALLOC_SCRATCH_BYTES 20973576
bbg_status bbg_grid_sort_noalloc(const float *d_pos, int n, const double domain_min[3],
                                 const double domain_max[3], double spacing,
                                 double spacing_scale, uint32_t *d_cell_of,
                                 uint32_t *d_sorted_ids, uint32_t *d_cell_start,
                                 uint32_t *d_out_of_grid, void *cuda_stream);

/* ----- profiling (ProfilerPrepare / ProfilerFinish around every GPULaunch,
 *       src/cuda/cutil.h:237-244; ProfilerReport, src/core/profiler.cpp:175-247) ---- */
/* Record CUDA events around every kernel launch on the solver's stream. */
bbg_status bbg_profiler_enable(bbg_solver s, int enable);
/* Drain the records (synchronises): per kernel its name (32 chars each), total device
 * milliseconds and launch count over launches that did work, plus the number of
 * kernel launches of every kind, including corrector launches that returned at once
 * because an earlier iteration had converged. */
bbg_status bbg_profiler_report(bbg_solver s, int max_kernels, char *names, double *total_ms,
                               int32_t *launches, int32_t *kernel_count,
                               int64_t *total_launches);

#ifdef __cplusplus
}
#endif
#endif /* BBG_H */
