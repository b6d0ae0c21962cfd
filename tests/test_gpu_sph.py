"""Config 1 (plain SPH, SphSolver3) end to end, and the pseudo-viscosity pass.

SphSolver3::AdvanceTimeStep (src/solvers/sph_solver3.cpp:48-67) runs the grid update,
the constant interactions, density + EOS, ComputeAllForcesFor with its integration and
then, only when pseudoViscosity * dt > 0.1, the smoothed-velocity interpolation
(ComputePseudoViscosityInterpolation*, src/equations/sph_equations3.cpp:341-382,
469-482, 655-664).  The all-forces pass runs in Jacobi order here (the reference races:
it integrates inside the force loop), and the oracle's `inplace=0` mode is that order.

  - substeps through advance_time_step (the CUDA-graph path), each against the oracle
    re-seeded from the GPU's own state: density relative 1e-5, positions within
    1e-5 x spacing, velocities within 1e-5 of the largest speed;
  - Advance(dt)'s CFL loop: the same substep count;
  - pseudo-viscosity from identical inputs (bit-identical integrated state, identical
    densities and neighbour sets): |dv_i| <= 1e-5 x the largest speed among particle i
    and its neighbours (a convex combination of those velocities), and a whole substep
    with the pass active.
"""
import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5


@pytest.fixture(scope="module")
def sph_moving(gpu):
    """Config 1 (16,384 particles) after 40 substeps of 1e-3 / 7 on the GPU."""
    sc, pos = scenes.sph_16k(seed=5)
    sub = sc["dt"] / 7
    with bb.Solver(sc, pos=pos) as g:
        for _ in range(40):
            g.advance_time_step(sub)
        p, v = g.download()
    return sc, sub, p, v


def test_sph_substeps_through_advance_time_step(sph_moving):
    sc, sub, p, v = sph_moving
    g = bb.Solver(sc, pos=p, vel=v)
    worst = {"rho": 0.0, "x": 0.0, "v": 0.0}
    for _ in range(7):   # one Advance(1e-3) of the configuration
        pg, vg = g.download()
        o = O.OracleSim(sc, pg, vg, variant="f32")
        g.advance_time_step(sub)
        o.sph_substep(sub, inplace=0)
        rho_g, rho_o = g.get(bb.FIELD_DENSITY), o.get(O.DENSITY)
        p2, v2 = g.download()
        vmax = max(1.0, float(np.abs(o.get(O.VELOCITY)).max()))
        worst["rho"] = max(worst["rho"], float(np.max(np.abs(rho_g - rho_o) / rho_o)))
        worst["x"] = max(worst["x"], float(np.max(np.abs(p2 - o.get(O.POSITION)))) / sc["spacing"])
        worst["v"] = max(worst["v"], float(np.max(np.abs(v2 - o.get(O.VELOCITY)))) / vmax)
        o.close()
    g.close()
    print("SPH substeps vs oracle, worst per-particle: %s" % worst)
    assert worst["rho"] <= RTOL and worst["x"] <= RTOL and worst["v"] <= RTOL


def test_sph_advance_cfl_loop(sph_moving):
    sc, sub, p, v = sph_moving
    g = bb.Solver(sc, pos=p, vel=v)
    o = O.OracleSim(sc, p, v, variant="f32")
    g.advance_time_step(sub)            # forces for the CFL estimate on both sides
    o.sph_substep(sub, inplace=0)
    pg, vg = g.download()
    o.close()
    o = O.OracleSim(sc, pg, vg, variant="f32")
    o.update_grid_distribution()
    o.compute_particle_interaction()
    o.compute_density(1)
    o.set(O.FORCE, g.get(bb.FIELD_FORCE))
    steps_o = o.number_of_time_steps(sc["dt"], 1.0)
    st = g.advance(sc["dt"])
    assert st["substeps"] == steps_o
    g.close()
    o.close()


def _pv_pair(sc, p, v, sub):
    """GPU solver and oracle at the same integrated state, densities and buckets, just
    before the pseudo-viscosity pass of a substep of length sub."""
    g = bb.Solver(sc, pos=p, vel=v)
    o = O.OracleSim(sc, p, v, variant="f32")
    g.update_grid_distribution()
    g.compute_density(1)
    o.update_grid_distribution()
    rng = np.random.default_rng(11)
    m = g.scalars()["mass"]
    f = (rng.normal(size=p.shape) * 20 * m).astype(np.float32)
    g.set(bb.FIELD_FORCE, f)
    o.set(O.FORCE, f)
    g.time_integration(sub)
    o.time_integration(sub)
    p1, v1 = g.download()
    assert np.array_equal(p1, o.get(O.POSITION).astype(np.float32))
    assert np.array_equal(v1, o.get(O.VELOCITY).astype(np.float32))
    o.set(O.DENSITY, g.get(bb.FIELD_DENSITY))
    return g, o, v1


def test_pseudo_viscosity_from_identical_inputs(sph_moving):
    sc, sub, p, v = sph_moving
    scp = dict(sc, pseudo_viscosity=1000.0)   # pseudoViscosity x dt = 0.143 > 0.1: active
    assert scp["pseudo_viscosity"] * sub > 0.1
    g, o, v1 = _pv_pair(scp, p, v, sub)
    cnt, ids = g.neighbor_lists(64)
    g.compute_pseudo_viscosity_interpolation(sub)
    o.pseudo_viscosity(sub)
    _, vg = g.download()
    vo = o.get(O.VELOCITY)
    speed = np.linalg.norm(v1.astype(np.float64), axis=1)
    nb = np.where(ids >= 0, speed[np.maximum(ids, 0)], 0.0)
    scale = np.maximum(speed, nb.max(axis=1))
    dv = np.linalg.norm(vg - vo, axis=1)
    moved = np.linalg.norm(vo - v1, axis=1)
    print("pseudo-viscosity: mean |dv| applied %.3e, worst error / scale %.3e"
          % (moved.mean(), float(np.max(dv / np.maximum(scale, 1e-30)))))
    assert moved.mean() > 0                   # the pass did change the velocities
    assert np.all(dv <= RTOL * np.maximum(scale, 1e-30))
    g.close()
    o.close()


def test_pseudo_viscosity_inactive_below_threshold(sph_moving):
    sc, sub, p, v = sph_moving
    g, o, v1 = _pv_pair(sc, p, v, sub)        # 10 x 1.43e-4 < 0.1: the reference skips it
    g.compute_pseudo_viscosity_interpolation(sub)
    _, vg = g.download()
    assert np.array_equal(vg, v1)
    g.close()
    o.close()


def test_sph_substep_with_pseudo_viscosity(sph_moving):
    sc, sub, p, v = sph_moving
    scp = dict(sc, pseudo_viscosity=1000.0)
    g = bb.Solver(scp, pos=p, vel=v)
    o = O.OracleSim(scp, p, v, variant="f32")
    g.advance_time_step(sub)
    o.sph_substep(sub, inplace=0)
    pg, vg = g.download()
    vmax = max(1.0, float(np.abs(o.get(O.VELOCITY)).max()))
    assert np.max(np.abs(pg - o.get(O.POSITION))) <= RTOL * sc["spacing"]
    assert np.max(np.abs(vg - o.get(O.VELOCITY))) <= RTOL * vmax
    g.close()
    o.close()
