/*
 * bridge_main.cpp -- a reference-side program using the binding of
 * bubbles_gb300/bridge/pcisph_bbg.cpp: it builds a PCISPH dam break with the reference's
 * own classes (ParticleSetBuilder3, DefaultSphSolverData3, UtilBuildGridForDomain,
 * PciSphSolver3::Setup, ColliderSetBuilder3), attaches libbbg and advances it.  With a
 * GPU it also advances a twin reference solver on its CPU path and prints the largest
 * position difference; without one it prints the status bbg_create returned.
 * Compiled by tests/test_bridge_cpu.py against the reference headers.
 */
#include <collider.h>
#include <cutil.h>
#include <interaction.h>
#include <pcisph_solver.h>
#include <shape.h>
#include <sph_solver.h>
#include <transform.h>
#include <util.h>

#include <cmath>
#include <cstdio>

#include "../../bubbles_gb300/bridge/pcisph_bbg.h"

static PciSphSolver3 *make(Grid3 **grid, Bounds3f domain, Float spacing) {
    ParticleSetBuilder3 builder;
    for (int z = 0; z < 12; z++)
        for (int y = 0; y < 10; y++)
            for (int x = 0; x < 12; x++)
                builder.AddParticle(vec3f(-0.28 + spacing * x, -0.23 + spacing * y, -0.28 + spacing * z));
    SphSolverData3 *data = DefaultSphSolverData3(true);
    *grid = UtilBuildGridForDomain(domain, spacing, 2.0);
    PciSphSolver3 *solver = new PciSphSolver3();
    solver->Initialize(data);
    solver->Setup(1000.0, spacing, 2.0, *grid, SphParticleSet3FromBuilder(&builder));
    ColliderSetBuilder3 cb;
    cb.AddCollider3(MakeBox(Transform(), vec3f(0.6, 0.5, 0.6), true), 0);
    cb.AddCollider3(MakeSphere(Translate(vec3f(0.05, -0.05, 0.05)), 0.08, false), 0);
    solver->SetColliders(cb.GetColliderSet());
    return solver;
}

int main() {
    SetCPUThreads(1);
    SetSystemUseCPU();
    const Float spacing = 0.02;
    Bounds3f domain(vec3f(-0.3, -0.25, -0.3), vec3f(0.3, 0.25, 0.3));
    Grid3 *grid = nullptr;
    PciSphSolver3 *solver = make(&grid, domain, spacing);
    bbg_shape shapes[2] = {};
    shapes[0].type = BBG_SHAPE_BOX;
    shapes[0].reverse = 1;
    shapes[0].size[0] = 0.6; shapes[0].size[1] = 0.5; shapes[0].size[2] = 0.6;
    shapes[1].type = BBG_SHAPE_SPHERE;
    shapes[1].center[0] = 0.05; shapes[1].center[1] = -0.05; shapes[1].center[2] = 0.05;
    shapes[1].size[0] = 0.08;
    BbgBridge bridge;
    int r = BbgAttach(solver, &bridge, domain, 2.0, shapes, 2, BBG_PCISPH_AS_SHIPPED);
    printf("attach %d\n", r);
    if (r) return 0;
    Grid3 *grid2 = nullptr;
    PciSphSolver3 *twin = make(&grid2, domain, spacing);
    r = BbgAdvance(solver, &bridge, 2e-3);
    printf("advance %d\n", r);
    if (r) return 1;
    twin->Advance(2e-3);
    ParticleSet3 *a = solver->GetSphParticleSet()->GetParticleSet();
    ParticleSet3 *b = twin->GetSphParticleSet()->GetParticleSet();
    double worst = 0;
    for (int i = 0; i < a->GetParticleCount(); i++) {
        vec3f d = a->GetParticlePosition(i) - b->GetParticlePosition(i);
        worst = fmax(worst, fmax(fabs(d.x), fmax(fabs(d.y), fabs(d.z))));
    }
    printf("max position difference %.3e\n", worst);
    return 0;
}
