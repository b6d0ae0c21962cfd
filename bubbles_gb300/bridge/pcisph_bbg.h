/*
 * pcisph_bbg.h -- the binding a Bubbles build adds to run its PciSphSolver3 / SphSolver3
 * step on libbbg: one bbg_solver per reference solver, the reference's particle set
 * copied in at attach time and back after each Advance.  Compiled inside the reference
 * tree (its headers: pcisph_solver.h, sph_solver.h), linked with -lbbg.
 */
#pragma once
#include <bbg.h>
#include <pcisph_solver.h>
#include <sph_solver.h>

#include <vector>

struct BbgBridge {
    bbg_solver h = nullptr;
    std::vector<float> pos, vel;
    ~BbgBridge() {
        if (h) bbg_destroy(h);
    }
};

/* After PciSphSolver3::Setup (pcisph_solver3.cpp:103-146): `domain` is the Bounds3f the
 * scene handed to UtilBuildGridForDomain (util.cpp:269-287) and `spacingScale` its scale;
 * the colliders are the scene's MakeBox / MakeSphere shapes as bbg_shape records;
 * `mode` is BBG_PCISPH_AS_SHIPPED (the reference) or BBG_PCISPH_TOLERANCE. */
int BbgAttach(PciSphSolver3 *solver, BbgBridge *b, Bounds3f domain, Float spacingScale, const bbg_shape *shapes,
              int nshapes, int mode);
/* The same after SphSolver3::Setup (sph_solver3.cpp). */
int BbgAttach(SphSolver3 *solver, BbgBridge *b, Bounds3f domain, Float spacingScale, const bbg_shape *shapes,
              int nshapes);
/* PciSphSolver3::Advance / SphSolver3::Advance (pcisph_solver3.cpp:67-89,
 * sph_solver3.cpp:69-93) on the device: the CFL substeps, then positions and velocities
 * back into the reference's particle set. */
int BbgAdvance(PciSphSolver3 *solver, BbgBridge *b, Float dt);
int BbgAdvance(SphSolver3 *solver, BbgBridge *b, Float dt);
