"""Boundary classifications of src/boundaries/lnm.h, xiaowei.h and dilts.h on the sorted grid:
LNMBoundarySingle, LNMBoundaryExtended, LNMBoundary with the Xiaowei and Dilts L2 filters,
XiaoweiBoundary and DiltsSpokeBoundary.

The oracle's restatements (oracle/sph_oracle.c) are pinned against what the reference
computed for a jittered BCC sphere (tests/golden/boundary_f32.npz); the device is compared
with both, particle by particle, and at 1M particles with the oracle.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "boundary_f32.npz")


def golden():
    d = np.load(GOLDEN, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["scene"])), json.loads(str(d["cases"]))


@pytest.fixture(scope="module")
def oracle_sim():
    g, sc, cases = golden()
    o = O.OracleSim(sc, g["pos"])
    o.update_grid_distribution()
    o.set(O.DENSITY, g["density"])
    yield o, g, cases
    o.close()


def test_oracle_single_and_extended_are_the_reference(oracle_sim):
    o, g, cases = oracle_sim
    for i, (h, ub) in enumerate(cases["single"]):
        assert np.array_equal(o.lnm_single(h, ub), g["single_%d" % i]), (h, ub)
    for i, (h, ml, ub) in enumerate(cases["extended"]):
        assert np.array_equal(o.lnm_extended(h, ml, ub), g["extended_%d" % i]), (h, ml, ub)


def test_oracle_geometric_tests_are_the_reference(oracle_sim):
    o, g, cases = oracle_sim
    for i, (h, alg, ub) in enumerate(cases["geometric"]):
        lv, q, a = o.lnm_geometric(h, alg, ub)
        assert np.array_equal(lv, g["geometric_%d" % i]) and [q, a] == g["geometric_stats_%d" % i].tolist()
    for i, h in enumerate(cases["xiaowei"]):
        assert np.array_equal(o.xiaowei(h), g["xiaowei_%d" % i]), h
    d = o.dilts()
    assert np.array_equal(d, g["dilts"]) and 0 < d.sum() < len(d)


def test_fixture_exercises_every_outcome():
    g, _, cases = golden()
    assert all(np.isin([0, 1, 2], g["single_%d" % i]).all() for i in range(len(cases["single"])))
    assert np.isin([1, 2, 3], g["extended_0"]).all()
    assert all(g["geometric_stats_%d" % i][1] > 0 for i in range(len(cases["geometric"])))


def test_spoke_points_follow_the_float_sine():
    """The spoke points' angles use the C library's float sine and cosine (the reference's
    sin / cos of a float): the points for r = 1 are the products of those values."""
    g, _, _ = golden()
    f = np.float32
    u = np.array([f(i * np.pi / float(f(64))) for i in range(65)], f)
    v = np.array([f(i * 6.283185307179586 / float(f(64))) for i in range(65)], f)
    pts = g["dilts_points"]
    assert pts.shape == (65 * 65, 3)
    cosu = pts[::65, 2]
    assert np.allclose(cosu, np.cos(u), atol=1e-7) and np.allclose(pts[:65, 2], 1.0)


@pytest.mark.gpu
def test_device_matches_reference(gpu):
    g, sc, cases = golden()
    with bb.Solver(sc, pos=g["pos"]) as s:
        s.update_grid_distribution()
        s.set(bb.FIELD_DENSITY, g["density"])
        for i, (h, ub) in enumerate(cases["single"]):
            assert np.array_equal(s.lnm_boundary_single(h, ub), g["single_%d" % i]), (h, ub)
        for i, (h, ml, ub) in enumerate(cases["extended"]):
            assert np.array_equal(s.lnm_boundary_extended(h, ml, ub), g["extended_%d" % i]), (h, ml, ub)
        for i, (h, alg, ub) in enumerate(cases["geometric"]):
            lv, q, a = s.lnm_boundary_geometric(h, alg, ub)
            assert np.array_equal(lv, g["geometric_%d" % i]), (h, alg, ub)
            assert [q, a] == g["geometric_stats_%d" % i].tolist()
        for i, h in enumerate(cases["xiaowei"]):
            assert np.array_equal(s.boundary_test("xiaowei", h), g["xiaowei_%d" % i]), h
        assert np.array_equal(s.boundary_test("dilts"), g["dilts"])


@pytest.mark.gpu
def test_xiaowei_needs_densities(gpu):
    g, sc, _ = golden()
    with bb.Solver(sc, pos=g["pos"]) as s:
        with pytest.raises(bb.BbgError):
            s.boundary_test("xiaowei", 0.02)
        with pytest.raises(bb.BbgError):
            s.lnm_boundary_geometric(0.02, 7)


@pytest.mark.gpu
def test_full_size_against_oracle(gpu):
    """1,048,576 particles after a few substeps: every classification equals the oracle's on
    the same distribution and densities.  Dilts runs on a jittered BCC sphere of 95,362
    particles in the same container (the dam's cubic lattice leaves every particle on the
    boundary)."""
    sc, pos = bb.scenes.pcisph_1m()
    with bb.Solver(sc, pos=pos) as s:
        for _ in range(3):
            s.advance_time_step(sc["dt"])
        p, _ = s.download()
    o = O.OracleSim(sc, p)
    o.update_grid_distribution()
    o.compute_density(0)
    rho = o.get(O.DENSITY)
    h = sc["spacing"]
    want = {"single": o.lnm_single(h), "extended": o.lnm_extended(h, 5), "xiaowei": o.xiaowei(h),
            "geometric": o.lnm_geometric(h, 1)}
    o.close()
    with bb.Solver(sc, pos=p) as s:
        s.update_grid_distribution()
        s.set(bb.FIELD_DENSITY, rho)
        assert np.array_equal(s.lnm_boundary_single(h), want["single"])
        ext = s.lnm_boundary_extended(h, 5)
        assert np.array_equal(ext, want["extended"]) and np.isin([1, 2, 3, 4, 5], ext).all()
        assert np.array_equal(s.boundary_test("xiaowei", h), want["xiaowei"])
        lv, q, a = s.lnm_boundary_geometric(h, "xiaowei")
        assert np.array_equal(lv, want["geometric"][0]) and (q, a) == want["geometric"][1:]
    ctypes.CDLL(None).srand(3)
    sub, _ = O.emit_volume({"type": "sphere", "center": (0.0, 0.0, 0.0), "radius": 0.18}, sc["spacing"], jitter=0.2)
    o = O.OracleSim(sc, sub)
    o.update_grid_distribution()
    want = o.dilts()
    o.close()
    with bb.Solver(sc, pos=sub) as s:
        s.update_grid_distribution()
        got = s.boundary_test("dilts")
    assert np.array_equal(got, want) and 0 < got.sum() < len(got)
