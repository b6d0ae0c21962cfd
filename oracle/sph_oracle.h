/*
 * sph_oracle.h -- CPU oracle for the Bubbles 3D SPH / PCISPH particle step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the reference result that the CUDA path is
 * compared against; nothing in the product links it.  Only tests/, __graft_entry__.smoke()
 * and bench.py (its cpu_baseline leg and its --impl reference arm) may load it.
 *
 * It restates, in plain C, the reference's CPU implementation of the step:
 *   - grid build and hashing        src/core/grid.h:259-298, 603-666; src/core/util.cpp:269-287
 *   - double-buffered cell chains   src/core/grid.h:20-156, 391-500
 *   - per-particle buckets (<=100)  src/core/grid.h:423-447; src/core/particle.h:22-60
 *   - SPH kernels                   src/core/kernel.cpp:113-233
 *   - density / EOS / forces        src/equations/sph_equations3.cpp:7-339
 *   - PCISPH predict-correct        src/equations/pcisph_equations3.cpp:3-256
 *   - colliders (box, sphere)       src/core/collider.cpp:4-45,238-264; src/shapes/box.cpp:74-172;
 *                                   src/shapes/sphere.cpp:47-70; src/core/shape.cpp:206-288
 *   - setup math                    src/core/particle.h:557-608; src/solvers/pcisph_solver3.cpp:103-189
 * The chain order, bucket order and every mixed float/double promotion of the
 * reference are kept, so that the FP32 build (-DORC_FLOAT=float) reproduces the
 * reference compiled with `typedef float Float` and the FP64 build reproduces the
 * reference as shipped (`typedef double Float`, src/core/geometry.h:68-69).
 *
 * Parity of this restatement is pinned against the reference itself, built
 * host-only by oracle/ref/Makefile, and against the golden fixtures under
 * tests/golden/ that were generated from that build.
 *
 * All arrays crossing this interface are double precision, xyz interleaved; they
 * are rounded to the oracle's Float on the way in.
 */
#ifndef BUBBLES_SPH_ORACLE_H
#define BUBBLES_SPH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_COLLIDERS 16
#define ORC_SHAPE_BOX 1
#define ORC_SHAPE_SPHERE 2

typedef struct {
    int type;            /* ORC_SHAPE_BOX / ORC_SHAPE_SPHERE */
    int reverse;         /* reverseOrientation (container boxes use 1) */
    double center[3];    /* translation of ObjectToWorld */
    double size[3];      /* box edge lengths; size[0] = sphere radius */
    double friction;     /* Collider3::frictionCoefficient */
} orc_shape;

typedef struct {
    /* SphSolverData3 (src/core/sph_solver.h:31-50; defaults sph_solver3.cpp:124-151) */
    double eos_exponent;
    double negative_pressure_scale;
    double viscosity;
    double pseudo_viscosity;
    double sound_speed;
    double drag_coefficient;
    double gravity[3];
    /* SphParticleSet3 */
    double target_density;
    double target_spacing;
    double relative_kernel_radius;
    double mass;                 /* > 0: ParticleSet::SetMass override after Setup */
    /* Grid: UtilBuildGridForDomain(domain, spacing, spacing_scale) */
    double domain_min[3];
    double domain_max[3];
    double grid_spacing_scale;
    /* colliders */
    int n_colliders;
    orc_shape colliders[ORC_MAX_COLLIDERS];
    /* Advance */
    double time_step_limit_scale;   /* kDefaultTimeStepLimitScale (5) for PCISPH, 1 for SPH */
} orc_params;

typedef struct orc_sim orc_sim;

/* field ids for orc_get_field / orc_set_field */
enum {
    ORC_POSITION = 0, ORC_VELOCITY = 1, ORC_FORCE = 2, ORC_INTERACTION = 3,
    ORC_DENSITY = 4, ORC_PRESSURE = 5, ORC_PRED_POSITION = 6, ORC_PRED_VELOCITY = 7,
    ORC_PRESSURE_FORCE = 8, ORC_PRED_DENSITY = 9, ORC_DENSITY_ERROR = 10,
    ORC_SMOOTHED_VELOCITY = 11
};

/* PCISPH corrector modes */
/* WARM / WARM_MONOTONE: tolerance mode started from the pressure the particles hold
 * (the previous substep's, or any start set with orc_set_field); WARM lets the pressure
 * decrease and clamps the total, WARM_MONOTONE keeps the reference update. */
enum { ORC_PCISPH_AS_SHIPPED = 0, ORC_PCISPH_TOLERANCE = 1, ORC_PCISPH_WARM = 2, ORC_PCISPH_WARM_MONOTONE = 3 };

int      orc_float_bytes(void);
void     orc_set_threads(int n);
int      orc_get_threads(void);

orc_sim *orc_create(const orc_params *p, int n, const double *pos, const double *vel);
void     orc_destroy(orc_sim *s);

/* Scalars after Setup: mass, kernel radius, delta denominator, (m/rho0)^2. */
void     orc_scalars(const orc_sim *s, double out[8]);
/* Grid: dims[3]; minp[3], len[3], bmin[3], bmax[3] packed into geo[12]. */
void     orc_grid_info(const orc_sim *s, int dims[3], double geo[12]);
/* Reference neighbour list of a cell (27 max), returns the count. */
int      orc_cell_neighbors(const orc_sim *s, int cell, int out[27]);
/* Hash arbitrary points with the grid rule (GetLinearHashedPosition). */
void     orc_hash_points(const orc_sim *s, int n, const double *pts, uint32_t *cell_ids,
                         uint32_t *ucoords);

/* Stand-alone setup math (no simulation needed). */
double   orc_compute_mass_bcc(double target_density, double spacing, double kernel_radius);
double   orc_compute_delta_denom(double spacing, double kernel_radius);
int      orc_build_grid(const double dmin[3], const double dmax[3], double spacing,
                        double scale, int dims[3], double geo[12]);
double   orc_kernel_eval(int which, double h, double r);

/* Passes (each the reference CPU wrapper of the same name). */
void     orc_update_grid_distribution(orc_sim *s);
void     orc_compute_particle_interaction(orc_sim *s);
void     orc_compute_density(orc_sim *s, int compute_pressure);
void     orc_compute_non_pressure_force(orc_sim *s);
double   orc_compute_delta(const orc_sim *s, double dt);
/* Returns iterations run; *final_err = last max density-error ratio. */
int      orc_pressure_force_and_integrate(orc_sim *s, double dt, double max_err_ratio,
                                          double delta, int max_it, int mode,
                                          double *final_err);
void     orc_time_integration(orc_sim *s, double dt);
/* The corrector's sub-passes on their own (tolerance mode stores densityErrors). */
void     orc_predict_velocity_and_position(orc_sim *s, double dt, int is_first);
void     orc_predict_pressure(orc_sim *s, double delta);
void     orc_predict_pressure_force(orc_sim *s);
void     orc_accumulate_and_integrate(orc_sim *s, double dt);
/* SPH all-forces pass. inplace=1: the reference as shipped (integrates each particle
 * inside the force loop, sph_equations3.cpp:277); inplace=0: Jacobi order. */
void     orc_sph_all_forces(orc_sim *s, double dt, int inplace);
void     orc_pseudo_viscosity(orc_sim *s, double dt);
unsigned orc_number_of_time_steps(const orc_sim *s, double remaining, double scale);
/* One AdvanceTimeStep (PCISPH); returns corrector iterations. */
int      orc_pcisph_substep(orc_sim *s, double dt, double max_err_ratio, int max_it, int mode,
                            double *final_err);
/* One AdvanceTimeStep (SPH). */
void     orc_sph_substep(orc_sim *s, double dt, int inplace);
/* Advance(dt) with the CFL substep loop; returns substeps taken. */
int      orc_advance_pcisph(orc_sim *s, double dt, double max_err_ratio, int max_it, int mode,
                            int *total_iters);
int      orc_advance_sph(orc_sim *s, double dt, int inplace);

/* Field access (n*3 for vectors, n for scalars). */
void     orc_get_field(const orc_sim *s, int field, double *out);
void     orc_set_field(orc_sim *s, int field, const double *in);
int      orc_count(const orc_sim *s);
int      orc_higher_level(const orc_sim *s);
void     orc_set_higher_level(orc_sim *s, int v);

/* Grid state: cell of each particle; per-cell chain length; chains concatenated in
 * cell order (n ids).  Returns the number of cells. */
int      orc_get_cells(const orc_sim *s, uint32_t *cell_of_particle, uint32_t *cell_counts,
                       uint32_t *chain_concat);
/* Buckets: counts[n], ids[n*100] (-1 padded).  Returns the number of particles whose
 * neighbour count exceeded the 100-slot bucket (truncated, as the reference does). */
int      orc_get_buckets(const orc_sim *s, int32_t *counts, int32_t *ids);

/* Particle frame of SerializerSaveSphDataSet3 (src/third/serializer.cpp:880-923 with
 * PushParticleSetToFile :813-878 and PrintToFile :20-45): header, one line per particle
 * (two tabs, the selected fields printed "%g" from Float values, separated by spaces),
 * trailer.  Flags are SERIALIZER_POSITION/VELOCITY/DENSITY/MASS (0x01/0x02/0x04/0x20);
 * vel and rho may be NULL when not selected.  Writes at most `capacity` bytes into buf and
 * returns the frame's full length (sequential, one thread, as the reference). */
size_t   orc_frame_text(int n, int flags, const double *pos, const double *vel, const double *rho,
                        double mass, double spacing, char *buf, size_t capacity);

/* ContinuousParticleSetBuilder3::MapGrid (src/core/grid.h:1289-1321) on the simulation's
 * current chains, and MapGridEmit (:1359-1402): the positions a refill would add, cells
 * ascending, chain order (at most `capacity` stored; the count is returned, -1 without a
 * map).  The oracle's particle arrays do not grow: the caller appends. */
void     orc_map_grid(orc_sim *s);
long     orc_map_grid_emit(const orc_sim *s, double distance, double *out, long capacity);

/* LNMBoundary, fast variant (src/boundaries/lnm.h:245-275) on the current chains: each
 * particle's level, 1 (a cell on the grid's border or next to an empty cell), 2 (next to
 * an L1 cell holding at most delta = (min cell length / h)^3 particles; unbounded: any)
 * or 0. */
void     orc_lnm(const orc_sim *s, double h, int unbounded, int *levels);
void     orc_lnm_single(const orc_sim *s, double h, int unbounded, int *levels);
void     orc_lnm_extended(const orc_sim *s, double h, int max_level, int unbounded, int *levels);
void     orc_lnm_geometric(const orc_sim *s, double h, int algorithm, int unbounded, int *levels, int *stats);
void     orc_xiaowei(const orc_sim *s, double h, int *flags);
void     orc_dilts(const orc_sim *s, int *flags);
long     orc_particle_sdf(const orc_sim *s, int method, double kernel, double mc_spacing, int by_res, const int *res,
                          int nodes[3], double origin[3], double *spacing, float *values, long cap);

/* Shape::ClosestDistance and IsInside of a box or sphere at n points (src/core/shape.cpp:
 * 206-232, 275-282): the values SetNodeSDFKernel (shape.cpp:409-424) signs into a field. */
void     orc_shape_distance(const orc_shape *shape, int n, const double *pts, double *distance, int *inside);

/* VolumeParticleEmitter3::Emit into a ParticleSetBuilder3 (src/core/emitter.cpp:8-12,
 * 241-330) for a box or sphere: the BCC lattice of BccLatticePointGenerator::ForEach
 * (src/generator/bcclattice.cpp:6-36) over the shape's bounds (or [bmin, bmax] when
 * use_bounds), each point moved by max_jitter * SampleSphere(rand(), rand()), kept when
 * Shape::SignedDistance <= 0, up to max_particles.  Two rand() values per visited lattice
 * point, as the reference; velocities = initial velocity.  Returns the count (at most
 * `capacity` stored). */
long     orc_emit_volume(const orc_shape *shape, int use_bounds, const double bmin[3], const double bmax[3],
                         double spacing, double jitter, const double vel[3], long max_particles, double *pos,
                         double *vel_out, long capacity);

/* SerializerLoadParticles3 (src/third/serializer.cpp:540-560): the first fluid section of a
 * frame text -- header tokens (SerializerFindFluidSection / SerializerFluidProcessToken,
 * :83-181), then one particle per data line up to the first non-comment line holding
 * "DataEnd" (_SerializerLoadParticles3, :450-538), every number read by ParseFloat
 * (src/third/obj_loader.cpp:56-168, 270-278).  *flags: in, the flags used when the
 * section has no "Format"; out, the section's.  Stores at most `capacity` particles
 * (pos/vel xyz, density, boundary; any may be NULL) and returns how many data lines were
 * read; *count receives the header's "Count".  Returns -1 for an unknown format letter,
 * -2 without a fluid section or without "DataEnd". */
long     orc_frame_parse(const char *text, size_t length, int *flags, int *count, double *pos,
                         double *vel, double *rho, int *boundary, long capacity);

#ifdef __cplusplus
}
#endif
#endif
