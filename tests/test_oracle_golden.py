"""The CPU oracle reproduces the reference bit for bit.

tests/golden/*.npz were produced by the reference's own CPU path built host-only
(tests/golden/make_golden.py); the oracle must match them exactly in FP32 and FP64:
setup math, grid geometry, cell chains (including the incremental DistributeToCellOpt
order), buckets, every field after three as-shipped substeps, a three-iteration
corrector, Advance(dt) with its CFL loop, and the as-shipped (in-place) SPH step.
Where the reference build is available, the same comparison also runs live on other
seeds.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refsim as R

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = {"pos": O.POSITION, "vel": O.VELOCITY, "force": O.FORCE, "density": O.DENSITY,
          "pressure": O.PRESSURE, "pred_density": O.PRED_DENSITY,
          "pressure_force": O.PRESSURE_FORCE, "pred_pos": O.PRED_POSITION}


def load(name):
    d = np.load(os.path.join(GOLD, name), allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["scene"]))


@pytest.mark.parametrize("variant", ["f32", "f64"])
def test_pcisph_golden(variant):
    g, sc = load("pcisph_%s.npz" % variant)
    o = O.OracleSim(sc, g["pos0"], variant=variant)
    s = o.scalars()
    assert [s["mass"], s["kernel_radius"], s["delta_denom"], s["mass_over_density_sq"]] == list(g["scalars"])
    dims, geo = o.grid_info()
    assert np.array_equal(dims, g["grid_dims"]) and np.array_equal(geo, g["grid_geo"])
    for got, want in zip(o.cells(), ("setup_cell_of", "setup_counts", "setup_chains")):
        assert np.array_equal(got, g[want]), want
    for _ in range(3):
        o.pcisph_substep(sc["dt"], 0.01, 5, O.PCISPH_AS_SHIPPED)
    for got, want in zip(o.cells(), ("step3_cell_of", "step3_counts", "step3_chains")):
        assert np.array_equal(got, g[want]), want
    counts, _, _ = o.buckets()
    assert np.array_equal(counts, g["step3_bucket_counts"])
    for name, f in FIELDS.items():
        assert np.array_equal(o.get(f), g["step3_" + name]), name
    o.update_grid_distribution()
    o.set_higher_level(0)
    o.compute_particle_interaction()
    o.compute_density(1)
    o.compute_non_pressure_force()
    delta = o.compute_delta(sc["dt"])
    assert delta == float(g["corr_delta"])
    for k in range(3):
        o.predict_velocity_and_position(sc["dt"], int(k == 0))
        o.predict_pressure(delta)
        o.predict_pressure_force()
    for name in ("pred_density", "pressure", "pressure_force", "pred_pos"):
        assert np.array_equal(o.get(FIELDS[name]), g["corr_" + name]), name
    o.accumulate_and_integrate(sc["dt"])
    assert np.array_equal(o.get(O.POSITION), g["corr_pos"])
    assert np.array_equal(o.get(O.VELOCITY), g["corr_vel"])
    o.advance_pcisph(2e-3, 0.01, 5, O.PCISPH_AS_SHIPPED)
    assert np.array_equal(o.get(O.POSITION), g["advance_pos"])


@pytest.mark.parametrize("variant", ["f32", "f64"])
def test_sph_golden_as_shipped(variant):
    g, sc = load("sph_%s.npz" % variant)
    o = O.OracleSim(sc, g["pos0"], variant=variant)
    for _ in range(3):
        o.sph_substep(sc["dt"], inplace=1)
    for name in ("pos", "vel", "force", "density", "pressure"):
        assert np.array_equal(o.get(FIELDS[name]), g["step3_" + name]), name


@pytest.mark.skipif(not R.available(), reason="reference checkout not present")
@pytest.mark.parametrize("variant", ["f32", "f64"])
@pytest.mark.parametrize("seed", [3, 11])
def test_oracle_matches_live_reference(variant, seed):
    from bubbles_gb300 import scenes
    sc, pos = scenes.small_pcisph(n_side=(9, 12, 8), seed=seed)
    sc["colliders"][1]["center"] = (-0.05, -0.12, 0.0)   # sphere inside the splash
    r = R.RefSim(sc, pos, variant=variant)
    o = O.OracleSim(sc, pos, variant=variant)
    for _ in range(6):
        r.advance_time_step(sc["dt"] * 2)
        o.pcisph_substep(sc["dt"] * 2, 0.01, 5, O.PCISPH_AS_SHIPPED)
    for name, f in FIELDS.items():
        assert np.array_equal(o.get(f), r.get(f)), name
    for a, b in zip(o.cells(), r.cells()):
        assert np.array_equal(a, b)
