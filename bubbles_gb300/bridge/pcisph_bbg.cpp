/*
 * pcisph_bbg.cpp -- see pcisph_bbg.h.  The reference stores FP64 AoS vec3f (Float =
 * double as shipped); the binding converts to and from the float xyz triples of the C ABI.
 */
#include "pcisph_bbg.h"

namespace {

int attach(SphSolverData3 *d, int kind, BbgBridge *b, Bounds3f domain, Float spacingScale, const bbg_shape *shapes,
           int nshapes, int mode) {
    SphParticleSet3 *sph = d->sphpSet;
    ParticleSet3 *p = sph->GetParticleSet();
    bbg_solver_desc desc;
    if (int r = bbg_solver_desc_default(&desc, kind)) return r;
    desc.eos_exponent = d->eosExponent;
    desc.negative_pressure_scale = d->negativePressureScale;
    desc.viscosity = d->viscosity;
    desc.pseudo_viscosity = d->pseudoViscosity;
    desc.sound_speed = d->soundSpeed;
    desc.drag_coefficient = d->dragCoefficient;
    vec3f g(0, 0, 0);
    for (int i = 0; i < d->cInteractionsCount; i++) g = g + d->cInteractions[i].value;
    desc.gravity[0] = g.x;
    desc.gravity[1] = g.y;
    desc.gravity[2] = g.z;
    desc.target_density = sph->GetTargetDensity();
    desc.target_spacing = sph->GetTargetSpacing();
    desc.relative_kernel_radius = sph->GetKernelRadius() / sph->GetTargetSpacing();
    desc.mass = p->GetMass();
    desc.grid_spacing_scale = spacingScale;
    for (int k = 0; k < 3; k++) {
        desc.domain_min[k] = domain.pMin[k];
        desc.domain_max[k] = domain.pMax[k];
    }
    if (kind == BBG_SOLVER_PCISPH) {
        desc.pcisph_mode = mode;
        desc.max_iterations = 5;               // the reference's call site (pcisph_solver3.cpp:62-63)
        desc.max_density_error_ratio = 0.01;
        desc.time_step_limit_scale = 5.0;      // kDefaultTimeStepLimitScale
    }
    const int n = p->GetParticleCount();
    if (int r = bbg_create(&desc, n, &b->h)) return r;
    if (int r = bbg_set_colliders(b->h, shapes, nshapes)) return r;
    b->pos.resize(3 * (size_t)n);
    b->vel.resize(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        const vec3f x = p->GetParticlePosition(i), v = p->GetParticleVelocity(i);
        for (int k = 0; k < 3; k++) {
            b->pos[3 * (size_t)i + k] = (float)x[k];
            b->vel[3 * (size_t)i + k] = (float)v[k];
        }
    }
    if (int r = bbg_upload_particles(b->h, b->pos.data(), b->vel.data(), n)) return r;
    return bbg_setup(b->h);
}

int advance(SphSolverData3 *d, BbgBridge *b, Float dt) {
    bbg_step_stats st;
    if (int r = bbg_advance(b->h, dt, &st)) return r;
    if (int r = bbg_download(b->h, b->pos.data(), b->vel.data())) return r;
    ParticleSet3 *p = d->sphpSet->GetParticleSet();
    for (int i = 0; i < p->GetParticleCount(); i++) {
        const float *x = &b->pos[3 * (size_t)i], *v = &b->vel[3 * (size_t)i];
        p->SetParticlePosition(i, vec3f(x[0], x[1], x[2]));
        p->SetParticleVelocity(i, vec3f(v[0], v[1], v[2]));
    }
    return 0;
}

}  // namespace

int BbgAttach(PciSphSolver3 *solver, BbgBridge *b, Bounds3f domain, Float spacingScale, const bbg_shape *shapes,
              int nshapes, int mode) {
    return attach(solver->GetSphSolverData(), BBG_SOLVER_PCISPH, b, domain, spacingScale, shapes, nshapes, mode);
}

int BbgAttach(SphSolver3 *solver, BbgBridge *b, Bounds3f domain, Float spacingScale, const bbg_shape *shapes,
              int nshapes) {
    return attach(solver->GetSphSolverData(), BBG_SOLVER_SPH, b, domain, spacingScale, shapes, nshapes, 0);
}

int BbgAdvance(PciSphSolver3 *solver, BbgBridge *b, Float dt) { return advance(solver->GetSphSolverData(), b, dt); }

int BbgAdvance(SphSolver3 *solver, BbgBridge *b, Float dt) { return advance(solver->GetSphSolverData(), b, dt); }
