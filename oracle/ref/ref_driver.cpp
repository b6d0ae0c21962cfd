/*
 * ref_driver.cpp -- C entry points over the reference's own solver classes and CPU
 * passes, compiled together with the reference sources by build_ref.py (host-only,
 * single thread).  Test infrastructure only: it pins the CPU oracle and generates the
 * golden fixtures under tests/golden/.  Parameters use the oracle's orc_params layout.
 */
#include <collider.h>
#include <emitter.h>
#include <lnm.h>
#include <marching_cubes.h>
#include <cutil.h>
#include <interaction.h>
#include <pcisph_solver.h>
#include <serializer.h>
#include <shape.h>
#include <sph_solver.h>
#include <transform.h>
#include <util.h>
#include <statics.h>
#include <host_mesh.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../sph_oracle.h"

/* Normally defined by src/solvers/pcisph_solver2.cpp:7, which the host-only compile leaves out. */
extern const Float kDefaultTimeStepLimitScale = 5.0;

/* Non-static reference functions without a header declaration. */
void PredictVelocityAndPositionCPU(PciSphSolverData3 *data, Float timeIntervalInSeconds, int is_first);
void PredictPressureCPU(PciSphSolverData3 *data, Float delta);
void PredictPressureForceCPU(PciSphSolverData3 *data);
void AccumulateAndIntegrateCPU(PciSphSolverData3 *data, Float timeStep);
void AdvanceTimeStep(PciSphSolver3 *solver, Float timeStep, int use_cpu);
void AdvanceTimeStep(SphSolver3 *solver, Float timeStep, int use_cpu);

struct RefSim {
    int n = 0, kind = 0;
    PciSphSolver3 pci;
    SphSolver3 sph;
    SphSolverData3 *data = nullptr;
    SphParticleSet3 *sphSet = nullptr;
    ParticleSet3 *pSet = nullptr;
    Grid3 *grid = nullptr;
    ContinuousParticleSetBuilder3 *cont = nullptr;   // ref_create_continuous only
    ColliderSet3 *cs = nullptr;
};

static vec3f V3(const double *a) { return vec3f((Float)a[0], (Float)a[1], (Float)a[2]); }

extern "C" {

int ref_float_bytes(void) { return (int)sizeof(Float); }

static RefSim *finish_sim(RefSim *s, const orc_params *p, SphParticleSet3 *set, int kind) {
    SphSolverData3 *data = DefaultSphSolverData3(false);
    data->eosExponent = p->eos_exponent;
    data->negativePressureScale = p->negative_pressure_scale;
    data->viscosity = p->viscosity;
    data->pseudoViscosity = p->pseudo_viscosity;
    data->soundSpeed = p->sound_speed;
    data->dragCoefficient = p->drag_coefficient;
    InteractionsBuilder3 ib;
    AddConstantInteraction(ib, V3(p->gravity));
    data->cInteractions = ib.MakeConstantInteractions(data->cInteractionsCount);
    s->data = data;
    s->sphSet = set;
    Bounds3f domain(V3(p->domain_min), V3(p->domain_max));
    s->grid = UtilBuildGridForDomain(domain, p->target_spacing, p->grid_spacing_scale);
    if (kind == 0) {
        s->pci.Initialize(data);
        s->pci.Setup(p->target_density, p->target_spacing, p->relative_kernel_radius, s->grid, s->sphSet);
    } else {
        s->sph.Initialize(data);
        s->sph.Setup(p->target_density, p->target_spacing, p->relative_kernel_radius, s->grid, s->sphSet);
    }
    s->pSet = s->sphSet->GetParticleSet();
    if (p->mass > 0) {
        s->pSet->SetMass(p->mass);
        Float mo = s->pSet->GetMass() / s->sphSet->GetTargetDensity();
        s->pci.massOverTargetDensitySquared = mo * mo;
    }
    if (p->n_colliders > 0) {
        ColliderSetBuilder3 cb;
        for (int i = 0; i < p->n_colliders; i++) {
            const orc_shape &c = p->colliders[i];
            bool at_origin = c.center[0] == 0 && c.center[1] == 0 && c.center[2] == 0;
            Transform t = at_origin ? Transform() : Translate(V3(c.center));
            Shape *shape = c.type == ORC_SHAPE_BOX ? MakeBox(t, V3(c.size), c.reverse != 0)
                                                   : MakeSphere(t, (Float)c.size[0], c.reverse != 0);
            cb.AddCollider3(shape, c.friction);
        }
        ColliderSet3 *cs = cb.GetColliderSet();
        s->cs = cs;
        if (kind == 0) s->pci.SetColliders(cs);
        else s->sph.SetColliders(cs);
    }
    return s;
}

RefSim *ref_create(const orc_params *p, int n, const double *pos, const double *vel, int kind) {
    SetCPUThreads(1);
    SetSystemUseCPU();
    RefSim *s = new RefSim();
    s->n = n;
    s->kind = kind;
    ParticleSetBuilder3 builder;
    for (int i = 0; i < n; i++) {
        vec3f v = vel ? V3(&vel[3 * i]) : vec3f(0);
        builder.AddParticle(V3(&pos[3 * i]), v);
    }
    return finish_sim(s, p, SphParticleSet3FromBuilder(&builder), kind);
}

/* The same scene on a ContinuousParticleSetBuilder3 of `capacity` particles (the builder's
 * own particle set, so MapGrid / MapGridEmit can add to it). */
RefSim *ref_create_continuous(const orc_params *p, int n, const double *pos, const double *vel, int kind,
                              int capacity) {
    SetCPUThreads(1);
    SetSystemUseCPU();
    RefSim *s = new RefSim();
    s->n = n;
    s->kind = kind;
    s->cont = new ContinuousParticleSetBuilder3(capacity);
    s->cont->SetKernelRadius((Float)(p->relative_kernel_radius * p->target_spacing));
    for (int i = 0; i < n; i++) {
        vec3f v = vel ? V3(&vel[3 * i]) : vec3f(0);
        s->cont->AddParticle(V3(&pos[3 * i]), v);
    }
    s->cont->Commit();
    return finish_sim(s, p, SphParticleSet3FromContinuousBuilder(s->cont), kind);
}

/* ContinuousParticleSetBuilder3::MapGrid on the simulation grid. */
void ref_map_grid(RefSim *s) { s->cont->MapGrid(s->grid); }

/* ContinuousParticleSetBuilder3::MapGridEmit with a constant velocity field; returns the
 * particle count afterwards. */
int ref_map_grid_emit(RefSim *s, double d, const double *vel) {
    const vec3f v = V3(vel);
    s->cont->MapGridEmit([v](const vec3f &) -> vec3f { return v; }, (Float)d);
    s->n = s->pSet->GetParticleCount();
    return s->n;
}

void ref_destroy(RefSim *s) { delete s; /* reference buffers live in its memory regions */ }

void ref_scalars(RefSim *s, double out[8]) {
    out[0] = s->pSet->GetMass();
    out[1] = s->sphSet->GetKernelRadius();
    out[2] = s->pci.deltaDenom;
    out[3] = s->pci.massOverTargetDensitySquared;
    out[4] = s->sphSet->GetTargetSpacing();
    out[5] = s->sphSet->GetTargetDensity();
    out[6] = s->pSet->GetRadius();
    out[7] = s->sphSet->kernelRadiusOverTargetSpacing;
}

void ref_grid_info(RefSim *s, int dims[3], double geo[12]) {
    for (int k = 0; k < 3; k++) {
        dims[k] = s->grid->usizes[k];
        geo[k] = s->grid->minPoint[k];
        geo[3 + k] = s->grid->cellsLen[k];
        geo[6 + k] = s->grid->bounds.pMin[k];
        geo[9 + k] = s->grid->bounds.pMax[k];
    }
}

/* --- passes ------------------------------------------------------------------ */
void ref_update_grid_distribution(RefSim *s) { UpdateGridDistributionCPU(s->data); }
void ref_reset_higher_level(RefSim *s) { s->sphSet->ResetHigherLevel(); }
int ref_higher_level(RefSim *s) { return s->sphSet->requiresHigherLevelUpdate; }
void ref_compute_particle_interaction(RefSim *s) { ComputeParticleInteractionCPU(s->data); }
void ref_compute_density(RefSim *s, int cp) { ComputeDensityCPU(s->data, cp); }
void ref_compute_non_pressure_force(RefSim *s) { ComputeNonPressureForceCPU(s->data); }
double ref_compute_delta(RefSim *s, double dt) { return s->pci.ComputeDelta((Float)dt); }
void ref_pressure_force_and_integrate(RefSim *s, double dt, double tol, double delta, int max_it) {
    ComputePressureForceAndIntegrate(s->pci.solverData, dt, tol, delta, max_it, 1);
}
void ref_predict_velocity_and_position(RefSim *s, double dt, int first) {
    PredictVelocityAndPositionCPU(s->pci.solverData, dt, first);
}
void ref_predict_pressure(RefSim *s, double delta) { PredictPressureCPU(s->pci.solverData, delta); }
void ref_predict_pressure_force(RefSim *s) { PredictPressureForceCPU(s->pci.solverData); }
void ref_accumulate_and_integrate(RefSim *s, double dt) { AccumulateAndIntegrateCPU(s->pci.solverData, dt); }
void ref_pseudo_viscosity(RefSim *s, double dt) { ComputePseudoViscosityInterpolationCPU(s->data, dt); }
void ref_time_integration(RefSim *s, double dt) { TimeIntegrationCPU(s->data, dt); }
/* SPH ComputePressureForceCPU as shipped: all forces + in-place integration. */
void ref_sph_pressure_force(RefSim *s, double dt) { ComputePressureForceCPU(s->data, dt); }
unsigned ref_number_of_time_steps(RefSim *s, double remaining, double scale) {
    return s->sphSet->ComputeNumberOfTimeSteps(remaining, s->data->soundSpeed, scale);
}
void ref_advance_time_step(RefSim *s, double dt) {
    if (s->kind == 0) AdvanceTimeStep(&s->pci, dt, 1);
    else AdvanceTimeStep(&s->sph, dt, 1);
}
void ref_advance(RefSim *s, double dt) {
    if (s->kind == 0) s->pci.Advance(dt);
    else s->sph.Advance(dt);
}

/* --- state ------------------------------------------------------------------- */
static void put(const vec3f &v, double *o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
static vec3f get(const double *a) { return vec3f((Float)a[0], (Float)a[1], (Float)a[2]); }

void ref_get_field(RefSim *s, int f, double *out) {
    PciSphSolverData3 *pd = s->pci.solverData;
    for (int i = 0; i < s->n; i++) {
        switch (f) {
            case ORC_POSITION: put(s->pSet->GetParticlePosition(i), &out[3 * i]); break;
            case ORC_VELOCITY: put(s->pSet->GetParticleVelocity(i), &out[3 * i]); break;
            case ORC_FORCE: put(s->pSet->GetParticleForce(i), &out[3 * i]); break;
            case ORC_INTERACTION: put(s->pSet->GetParticleInteraction(i), &out[3 * i]); break;
            case ORC_DENSITY: out[i] = s->pSet->GetParticleDensity(i); break;
            case ORC_PRESSURE: out[i] = s->pSet->GetParticlePressure(i); break;
            case ORC_PRED_POSITION: put(pd->tempPositions[i], &out[3 * i]); break;
            case ORC_PRED_VELOCITY: put(pd->tempVelocities[i], &out[3 * i]); break;
            case ORC_PRESSURE_FORCE: put(pd->pressureForces[i], &out[3 * i]); break;
            case ORC_PRED_DENSITY: out[i] = pd->densityPredicted[i]; break;
            case ORC_DENSITY_ERROR: out[i] = pd->densityErrors[i]; break;
            default: break;
        }
    }
}

void ref_set_field(RefSim *s, int f, const double *in) {
    PciSphSolverData3 *pd = s->pci.solverData;
    for (int i = 0; i < s->n; i++) {
        switch (f) {
            case ORC_POSITION: s->pSet->SetParticlePosition(i, get(&in[3 * i])); break;
            case ORC_VELOCITY: s->pSet->SetParticleVelocity(i, get(&in[3 * i])); break;
            case ORC_FORCE: s->pSet->SetParticleForce(i, get(&in[3 * i])); break;
            case ORC_DENSITY: s->pSet->SetParticleDensity(i, (Float)in[i]); break;
            case ORC_PRESSURE: s->pSet->SetParticlePressure(i, (Float)in[i]); break;
            case ORC_PRESSURE_FORCE: pd->pressureForces[i] = get(&in[3 * i]); break;
            case ORC_PRED_DENSITY: pd->densityPredicted[i] = (Float)in[i]; break;
            default: break;
        }
    }
}

int ref_get_cells(RefSim *s, uint32_t *cell_of, uint32_t *counts, uint32_t *chains) {
    Grid3 *g = s->grid;
    for (int i = 0; i < s->n; i++) cell_of[i] = g->GetLinearHashedPosition(s->pSet->GetParticlePosition(i));
    size_t w = 0;
    for (unsigned c = 0; c < g->GetCellCount(); c++) {
        Cell3 *cell = g->GetCell(c);
        int len = cell->GetChainLength();
        counts[c] = (uint32_t)len;
        ParticleChain *node = cell->GetChain();
        for (int j = 0; j < len && node && w < (size_t)s->n; j++) {
            chains[w++] = node->pId;
            node = node->next;
        }
    }
    return (int)g->GetCellCount();
}

void ref_get_buckets(RefSim *s, int32_t *counts, int32_t *ids) {
    for (int i = 0; i < s->n; i++) {
        Bucket *b = s->pSet->GetParticleBucket(i);
        counts[i] = b->Count();
        for (int q = 0; q < 100; q++) ids[100 * i + q] = q < b->Count() ? b->Get(q) : -1;
    }
}

/* VolumeParticleEmitter3::Emit (src/core/emitter.cpp:241-330) of a box or sphere
 * (MakeBox / MakeSphere with a translation) into a ParticleSetBuilder3 after srand(seed):
 * the lattice spans the shape's bounds, or [bmin, bmax] when use_bounds.  Returns the
 * number emitted (at most `capacity` stored). */
int ref_emit_volume(int type, int reverse, const double *center, const double *size, int use_bounds,
                    const double *bmin, const double *bmax, double spacing, double jitter, const double *vel,
                    int max_particles, unsigned seed, double *pos, double *vel_out, int capacity) {
    Transform t = Translate(V3(center));
    Shape *shape = type == 1 ? MakeBox(t, V3(size), reverse != 0) : MakeSphere(t, (Float)size[0], reverse != 0);
    ParticleSetBuilder3 builder;
    VolumeParticleEmitter3 *em;
    if (use_bounds)
        em = new VolumeParticleEmitter3(shape, Bounds3f(V3(bmin), V3(bmax)), (Float)spacing, V3(vel), vec3f(0), 0,
                                        max_particles, (Float)jitter);
    else
        em = new VolumeParticleEmitter3(shape, (Float)spacing, V3(vel), vec3f(0), 0, max_particles, (Float)jitter);
    srand(seed);
    em->Emit(&builder);
    const int n = (int)builder.positions.size();
    for (int i = 0; i < n && i < capacity; i++) {
        for (int k = 0; k < 3; k++) {
            pos[3 * i + k] = (double)builder.positions[(size_t)i][k];
            vel_out[3 * i + k] = (double)builder.velocities[(size_t)i][k];
        }
    }
    delete em;
    return n;
}

/* GenerateShapeSDF(shape, dx, margin) of collider i's shape. */
void ref_generate_collider_sdf(RefSim *s, int i, double dx, double margin) {
    GenerateShapeSDF(s->cs->colliders[i]->shape, (Float)dx, (Float)margin);
}

/* Collider i's shape becomes MakeSDFShape over the sphere's bounds: a field-only shape
 * whose nodes hold Distance(p, center) - radius. */
void ref_make_sdf_sphere_collider(RefSim *s, int i, const double *center, double radius, double dx,
                                  double margin) {
    const vec3f c = V3(center);
    const Float r = (Float)radius;
    Bounds3f b(c - vec3f(r), c + vec3f(r));
    s->cs->colliders[i]->shape = MakeSDFShape(b, [c, r](const vec3f &p, Shape *, int) -> Float {
        return Distance(p, c) - r;
    }, (Float)dx, (Float)margin);
}

/* MakeMesh of a triangle mesh (vertices xyz, triangles as vertex index triples) with an
 * identity transform, then GenerateShapeSDF(shape, dx, margin): the grid and up to
 * `capacity` node values (x fastest).  Returns the node count. */
int ref_mesh_sdf(const double *verts, int nv, const int *tris, int nt, double dx, double margin, int *nodes,
                 double *origin, double *spacing, float *values, int capacity) {
    ParsedMesh *mesh = new ParsedMesh();
    mesh->p = new Point3f[(size_t)nv];
    mesh->indices = new Point3i[3 * (size_t)nt];
    for (int i = 0; i < nv; i++) mesh->p[i] = Point3f((Float)verts[3 * i], (Float)verts[3 * i + 1], (Float)verts[3 * i + 2]);
    for (int i = 0; i < 3 * nt; i++) mesh->indices[i] = Point3i(tris[i], -1, -1);
    mesh->nTriangles = nt;
    mesh->nVertices = nv;
    mesh->nUvs = 0;
    mesh->nNormals = 0;
    mesh->n = nullptr;
    mesh->s = nullptr;
    mesh->uv = nullptr;
    strcpy(mesh->name, "mesh");
    Shape *shape = MakeMesh(mesh, Transform(), false);
    GenerateShapeSDF(shape, (Float)dx, (Float)margin);
    FieldGrid3f *g = shape->grid;
    for (int k = 0; k < 3; k++) {
        nodes[k] = (int)g->resolution[k];
        origin[k] = g->minPoint[k];
        spacing[k] = g->spacing[k];
    }
    const int total = (int)g->total;
    for (int q = 0; q < total && q < capacity; q++) values[q] = (float)g->field[q];
    return total;
}

/* Collider i's field: nodes, origin, spacing; up to `capacity` values (x fastest). */
int ref_collider_sdf(RefSim *s, int i, int *nodes, double *origin, double *spacing, float *values, int capacity) {
    FieldGrid3f *g = s->cs->colliders[i]->shape->grid;
    if (!g) return 0;
    for (int k = 0; k < 3; k++) {
        nodes[k] = (int)g->resolution[k];
        origin[k] = g->minPoint[k];
        spacing[k] = g->spacing[k];
    }
    const int total = (int)g->total;
    for (int q = 0; q < total && q < capacity; q++) values[q] = (float)g->field[q];
    return total;
}

/* Collider i's field and shape queries at n points: FieldGrid3f::Sample, Gradient,
 * Shape::ClosestPoint (point, normal, signed distance) and IsInside. */
void ref_sdf_probe(RefSim *s, int i, int n, const double *pts, double *sample, double *grad, double *cp,
                   double *cn, double *cd, int *inside) {
    Shape *shape = s->cs->colliders[i]->shape;
    for (int q = 0; q < n; q++) {
        const vec3f p = V3(&pts[3 * q]);
        sample[q] = shape->grid->Sample(p);
        const vec3f gr = shape->grid->Gradient(p);
        ClosestPointQuery cq;
        shape->ClosestPoint(p, &cq);
        for (int k = 0; k < 3; k++) {
            grad[3 * q + k] = gr[k];
            cp[3 * q + k] = cq.point[k];
            cn[3 * q + k] = cq.normal[k];
        }
        cd[q] = cq.signedDistance;
        inside[q] = shape->IsInside(p) ? 1 : 0;
    }
}

/* LNMBoundary (src/boundaries/lnm.h:245-275, the fast variant) on the grid's current
 * chains with v0 reset to 0 first: each particle's level (1, 2, or 0 inside). */
void ref_lnm(RefSim *s, double h, int unbounded, int *levels) {
    for (int i = 0; i < s->n; i++) s->pSet->SetParticleV0(i, 0);
    s->grid->UpdateQueryState();
    LNMBoundary(s->pSet, s->grid, (Float)h, 0, nullptr, unbounded != 0);
    for (int i = 0; i < s->n; i++) levels[i] = s->pSet->GetParticleV0(i);
}

/* LNMBoundarySingle (src/boundaries/lnm.h:167-256): the N2x2 classification in one pass. */
void ref_lnm_single(RefSim *s, double h, int unbounded, int *levels) {
    for (int i = 0; i < s->n; i++) s->pSet->SetParticleV0(i, 0);
    s->grid->UpdateQueryState();
    LNMBoundarySingle(s->pSet, s->grid, (Float)h, unbounded != 0);
    for (int i = 0; i < s->n; i++) levels[i] = s->pSet->GetParticleV0(i);
}

/* LNMBoundaryExtended (src/boundaries/lnm.h:440-462): voxel levels up to max_level, the
 * LK filter and the L2 -> L3 promotion, as the bounds app calls it (cells invalidated,
 * v0 cleared). */
void ref_lnm_extended(RefSim *s, double h, int max_level, int unbounded, int *levels) {
    for (int i = 0; i < s->n; i++) s->pSet->SetParticleV0(i, 0);
    s->grid->UpdateQueryState();
    LNMInvalidateCells(s->grid);
    LNMBoundaryExtended(s->pSet, s->grid, (Float)h, max_level, 0, unbounded != 0);
    for (int i = 0; i < s->n; i++) levels[i] = s->pSet->GetParticleV0(i);
}

/* LNMBoundary with a geometric L2 filter (algorithm 1: Xiaowei, 2: Dilts spoke) through
 * the reference's work queue (lnm.h:57-79, 258-289).  stats[0] = particles queued (L2
 * cells), stats[1] = accepted as boundary. */
void ref_lnm_geometric(RefSim *s, double h, int algorithm, int unbounded, int *levels, int *stats) {
    for (int i = 0; i < s->n; i++) s->pSet->SetParticleV0(i, 0);
    s->grid->UpdateQueryState();
    LNMWorkQueue *q = cudaAllocateVx(LNMWorkQueue, 1);
    q->SetSlots(s->n);
    LNMBoundary(s->pSet, s->grid, (Float)h, algorithm, q, unbounded != 0);
    stats[0] = q->size;
    stats[1] = q->counter;
    for (int i = 0; i < s->n; i++) levels[i] = s->pSet->GetParticleV0(i);
}

/* XiaoweiBoundary (src/boundaries/xiaowei.h:21-88) on the stored densities: 1 boundary. */
void ref_xiaowei(RefSim *s, double h, int *flags) {
    for (int i = 0; i < s->n; i++) flags[i] = XiaoweiParticleIsBoundary(s->pSet, s->grid, (Float)h, i);
}

/* DiltsSpokeBoundary (src/boundaries/dilts.h:110-163): 1 boundary. */
void ref_dilts(RefSim *s, int *flags) {
    for (int i = 0; i < s->n; i++) flags[i] = DiltsSpokeParticleIsBoundary(s->grid, s->pSet, i);
}

/* The spoke sample points of DiltsSpokeTakeUniformPoint around the origin for r = 1, in
 * the reference's order; returns the count. */
int ref_dilts_points(float *out, int cap) {
    vec3f o(0, 0, 0);
    int done = 0, i = 0, j = 0, k = 0;
    while (!done) {
        vec3f p = DiltsSpokeTakeUniformPoint(o, (Float)1, done, i, j, DILTS_LINEAR_SAMPLE_COUNT);
        if (k < cap) {
            out[3 * k] = (float)p.x;
            out[3 * k + 1] = (float)p.y;
            out[3 * k + 2] = (float)p.z;
        }
        k++;
    }
    return k;
}

} /* extern "C" */

/* The surface app's options (apps/surface.cpp:19-32), declared here with the same layout so
 * ParticlesToSDF_Surface can be called as the app calls it. */
typedef struct {
    Float kernel;
    Float spacing;
    Float marchingCubeSpacing;
    Float iso;
    std::string input;
    std::string output;
    int method;
    int inflags;
    int legacy;
    bool byResolution;
    vec3ui resolution;
    TriangleMeshFormat outformat;
} surface_opts;

FieldGrid3f *ParticlesToSDF_Surface(ParticleSetBuilder3 *pBuilder, surface_opts *opts, TimerList &timer);
Float ZhuBridsonSDF(vec3f p, Grid3 *grid, ParticleSet3 *pSet, Float kernelRadius, Float threshold);
Float SphSDF(vec3f p, Grid3 *grid, ParticleSet3 *pSet, Float kernelRadius);

extern "C" {

/* The surface app's particle-to-field step (apps/surface.cpp:388-470, methods 0 Zhu-Bridson
 * and 1 SPH).  direct = 1 calls ParticlesToSDF_Surface itself; direct = 0 runs the same steps
 * with the reference's own pieces (UtilBuildGridForBuilder, SphSolver3::Setup, the grid
 * distribution and density passes, FieldGrid3f::Build, ZhuBridsonSDF / SphSDF) so that the
 * densities and the domain grid can be returned too.  Returns the node count (values up to
 * cap stored); nodes[3], origin[3], spacing[1]; dom[6] the domain bounds; dens[n]. */
long ref_surface_sdf(const double *pos, int n, double spacing, double kernel, double mc_spacing, int by_res,
                     const int *res, int method, int direct, int *nodes, double *origin, double *sdf_spacing,
                     float *values, long cap, double *dom, float *dens) {
    SetCPUThreads(1);
    SetSystemUseCPU();
    ParticleSetBuilder3 builder;
    for (int i = 0; i < n; i++) builder.AddParticle(V3(pos + 3 * i));
    FieldGrid3f *g = nullptr;
    if (direct) {
        surface_opts opts;
        opts.kernel = (Float)kernel;
        opts.spacing = (Float)spacing;
        opts.marchingCubeSpacing = (Float)mc_spacing;
        opts.iso = 0;
        opts.method = method;
        opts.inflags = 0;
        opts.legacy = 0;
        opts.byResolution = by_res != 0;
        opts.resolution = by_res ? vec3ui((unsigned)res[0], (unsigned)res[1], (unsigned)res[2]) : vec3ui(0);
        TimerList timer;
        g = ParticlesToSDF_Surface(&builder, &opts, timer);
    } else {
        const Float spacingScale = 2.0, threshold = 0.25, sp = (Float)spacing, radius = (Float)kernel;
        Float sdfSpacing = (Float)mc_spacing;
        Grid3 *grid = UtilBuildGridForBuilder(&builder, sp, spacingScale);
        Bounds3f b = grid->GetBounds();
        SphSolver3 solver;
        SphParticleSet3 *sphpSet = SphParticleSet3FromBuilder(&builder);
        ParticleSet3 *pSet = sphpSet->GetParticleSet();
        solver.Initialize(DefaultSphSolverData3());
        solver.Setup(WaterDensity, sp, spacingScale, grid, sphpSet);
        UpdateGridDistributionGPU(solver.solverData);
        ComputeDensityGPU(solver.solverData);
        grid->UpdateQueryState();
        g = cudaAllocateVx(FieldGrid3f, 1);
        if (!by_res) {
            sdfSpacing *= spacingScale;
            vec3f p0 = b.pMin + 0.5 * vec3f(sdfSpacing);
            int nx = std::ceil(b.ExtentOn(0) / sdfSpacing);
            int ny = std::ceil(b.ExtentOn(1) / sdfSpacing);
            int nz = std::ceil(b.ExtentOn(2) / sdfSpacing);
            g->Build(vec3ui(nx, ny, nz), sdfSpacing, p0, VertexCentered);
        } else {
            vec3ui r = vec3ui((unsigned)res[0], (unsigned)res[1], (unsigned)res[2]) - vec3ui(1);
            Float dx = b.ExtentOn(0) / (Float)r.x;
            Float dy = b.ExtentOn(1) / (Float)r.y;
            Float dz = b.ExtentOn(2) / (Float)r.z;
            Float ds = Max(dx, Max(dy, dz));
            vec3f p0 = b.pMin + 0.5 * vec3f(ds);
            g->Build(r, ds, p0, VertexCentered);
        }
        Float inf = b.Diagonal().Length();
        for (int i = 0; i < (int)g->total; i++) {
            vec3ui u = DimensionalIndex(i, g->resolution, 3);
            vec3f p = g->GetDataPosition(u);
            Float estimate = inf;
            if (method == 0) estimate = ZhuBridsonSDF(p, grid, pSet, radius, threshold);
            else if (method == 1) estimate = SphSDF(p, grid, pSet, radius);
            g->SetValueAt(estimate, u);
        }
        for (int k = 0; k < 3; k++) {
            dom[k] = b.pMin[k];
            dom[3 + k] = b.pMax[k];
        }
        for (int i = 0; i < n; i++) dens[i] = (float)pSet->GetParticleDensity(i);
    }
    for (int k = 0; k < 3; k++) {
        nodes[k] = (int)g->resolution[k];
        origin[k] = g->minPoint[k];
    }
    sdf_spacing[0] = g->spacing[0];
    for (long q = 0; q < (long)g->total && q < cap; q++) values[q] = (float)g->field[q];
    return (long)g->total;
}

/* MarchingCubes (src/reconstruction/marching_cubes.cpp:204-457) of a vertex-centred field
 * (nodes per axis, origin, spacing, values x fastest) at iso, single thread: the mesh's
 * points, normals and triangles (at most the capacities stored).  Returns the point count;
 * *ntri receives the triangle count. */
int ref_marching_cubes(const int *nodes, const double *origin, const double *spacing, const float *values,
                       double iso, int rotate, float *points, float *normals, int *tris, int pcap, int tcap,
                       int *ntri) {
    SetCPUThreads(1);
    SetSystemUseCPU();
    FieldGrid3f *g = cudaAllocateVx(FieldGrid3f, 1);
    g->Build(vec3ui((unsigned)(nodes[0] - 1), (unsigned)(nodes[1] - 1), (unsigned)(nodes[2] - 1)),
             vec3f((Float)spacing[0], (Float)spacing[1], (Float)spacing[2]), V3(origin), VertexCentered);
    for (unsigned q = 0; q < g->total; q++) g->field[q] = (Float)values[q];
    g->MarkFilled();
    HostTriangleMesh3 mesh;
    MarchingCubes(g, &mesh, (Float)iso, rotate != 0);
    const int np = (int)mesh.points.size(), nt = (int)mesh.pointIndices.size();
    for (int i = 0; i < np && i < pcap; i++)
        for (int k = 0; k < 3; k++) {
            points[3 * i + k] = (float)mesh.points[(size_t)i][k];
            normals[3 * i + k] = (float)mesh.normals[(size_t)i][k];
        }
    for (int i = 0; i < nt && i < tcap; i++)
        for (int k = 0; k < 3; k++) tris[3 * i + k] = (int)mesh.pointIndices[(size_t)i][k];
    *ntri = nt;
    return np;
}

/* SerializerLoadParticles3 on a frame file: the first fluid section's particles (at most
 * `capacity` stored; NULL outputs skipped).  Returns the number read (-1: no file). */
int ref_load_frame(const char *path, int *flags, double *pos, double *vel, double *rho, int *boundary,
                   int capacity) {
    std::vector<SerializedParticle> parts;
    int f = *flags;
    int n = SerializerLoadParticles3(&parts, path, f);
    *flags = f;
    for (int i = 0; i < n && i < capacity; i++) {
        const SerializedParticle &q = parts[(size_t)i];
        for (int k = 0; k < 3; k++) {
            if (pos) pos[3 * i + k] = (double)q.position[k];
            if (vel) vel[3 * i + k] = (double)q.velocity[k];
        }
        if (rho) rho[i] = (double)q.density;
        if (boundary) boundary[i] = q.boundary;
    }
    return n;
}

/* Appends SerializerSaveSphDataSet3's particle frame of the current state to `path`. */
void ref_save_frame(RefSim *s, const char *path, int flags) { SerializerSaveSphDataSet3(s->data, path, flags); }

}  // extern "C"
