"""LNM boundary classification (src/boundaries/lnm.h, fast variant) on the sorted grid.

The oracle's restatement (oracle/sph_oracle.c, orc_lnm) is pinned against the levels the
reference computed (tests/golden/lnm_f32.npz); the device classification is compared with
both, particle by particle, and at 1M particles with the oracle.
"""
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lnm_f32.npz")


def golden():
    d = np.load(GOLDEN, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["scene"])), json.loads(str(d["cases"]))


def test_oracle_lnm_is_the_reference():
    g, sc, cases = golden()
    o = O.OracleSim(sc, g["pos"])
    o.update_grid_distribution()
    for i, (h, unbounded) in enumerate(cases):
        assert np.array_equal(o.lnm(h, unbounded), g["levels_%d" % i]), (h, unbounded)
    o.close()


@pytest.mark.gpu
def test_lnm_matches_reference(gpu):
    g, sc, cases = golden()
    with bb.Solver(sc, pos=g["pos"]) as s:
        s.update_grid_distribution()
        for i, (h, unbounded) in enumerate(cases):
            assert np.array_equal(s.lnm_boundary(h, unbounded), g["levels_%d" % i]), (h, unbounded)


@pytest.mark.gpu
def test_lnm_full_size_against_oracle(gpu):
    """1,048,576 particles after a few substeps: the same levels as the oracle's on the same
    grid distribution."""
    sc, pos = bb.scenes.pcisph_1m()
    with bb.Solver(sc, pos=pos) as s:
        for _ in range(3):
            s.advance_time_step(sc["dt"])
        p, _ = s.download()
        s.upload(p)
        s.setup()
        s.update_grid_distribution()
        lv = s.lnm_boundary(sc["spacing"])
    o = O.OracleSim(sc, p)
    o.update_grid_distribution()
    want = o.lnm(sc["spacing"])
    o.close()
    assert np.array_equal(lv, want)
    assert (lv == 1).sum() > 0 and (lv == 2).sum() > 0 and (lv == 0).sum() > 0
