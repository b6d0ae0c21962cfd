"""Continuous emission: ContinuousParticleSetBuilder3::MapGrid / MapGridEmit on the device.

Pinned against the reference builder itself (tests/golden/continuous_f32.npz: MapGrid after
Setup, positions moved by hand, two MapGridEmit calls, with a capacity that holds the new
particles and one that stops the first call), and at a larger size against a numpy
restatement of MapGridEmit on the device's own grid (cells in ascending order, chain order,
float32 distances).
"""
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "continuous_f32.npz")


def same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_map_grid_emit_matches_reference(gpu):
    d = np.load(GOLDEN, allow_pickle=False)
    sc = json.loads(str(d["scene"]))
    cases = json.loads(str(d["cases"]))
    for i, (cap, dist, vel) in enumerate(cases):
        with bb.Solver(sc, pos=d["pos0"], capacity=cap) as s:
            assert s.map_grid() == len(d["pos0"])
            s.set(bb.FIELD_POSITION, d["pos1"])
            for k in range(2):
                s.map_grid_emit(dist, vel)
                p, v = s.download()
                assert same_bits(p, d["pos_%d_%d" % (i, k)]), (i, k)
                assert same_bits(v, d["vel_%d_%d" % (i, k)]), (i, k)


def map_emit_numpy(cell_of, counts, ids, p0, p1, dist, limit=100):
    """MapGridEmit restated: cells ascending, the first min(limit - held, remembered) chain
    positions of each cell with no current particle of the cell closer than dist."""
    chain = ids   # the cells' chains, concatenated in cell order
    starts = np.concatenate([[0], np.cumsum(counts.astype(np.int64))]).astype(np.int64)
    d32 = np.float32(dist)
    out = []
    for c in np.nonzero(counts)[0]:
        members = chain[starts[c]:starts[c + 1]]
        held = len(members)
        if held >= limit:
            continue
        cur = p1[members].astype(np.float32)
        for i in range(min(limit - held, held)):
            pi = p0[members[i]].astype(np.float32)
            dx = cur - pi
            l2 = dx[:, 0] * dx[:, 0] + dx[:, 1] * dx[:, 1] + dx[:, 2] * dx[:, 2]
            if not np.any(np.sqrt(l2) < d32):
                out.append(pi)
    return np.array(out, np.float32).reshape(-1, 3)


def test_map_grid_emit_larger_against_restatement(gpu):
    sc = dict(scenes.base_scene("pcisph", 0.01, (1.0, 0.8, 1.0)), dt=2e-4)
    p0 = scenes.dam_block(sc, (40, 30, 40), seed=3).astype(np.float32)
    rng = np.random.default_rng(4)
    p1 = (p0 + rng.normal(0.0, 0.006, p0.shape)).astype(np.float32)
    with bb.Solver(sc, pos=p0, capacity=3 * len(p0)) as s:
        s.map_grid()
        cell_of, counts, ids = s.dump_grid()
        s.set(bb.FIELD_POSITION, p1)
        n = s.map_grid_emit(0.004, (0.0, 1.0, 0.0))
        p, v = s.download()
    want = map_emit_numpy(cell_of, counts, ids.astype(np.int64), p0, p1, 0.004)
    assert n == len(want) > 0
    assert same_bits(p[len(p0):], want)
    assert np.all(v[len(p0):] == np.array([0.0, 1.0, 0.0], np.float32))


def test_map_grid_emit_then_step(gpu, small):
    """The refilled set steps like any other (the appended particles sort into the grid)."""
    sc, pos = small
    with bb.Solver(sc, pos=pos, capacity=4 * len(pos)) as s:
        s.map_grid()
        s.advance_time_step(sc["dt"])
        p, _ = s.download()
        s.set(bb.FIELD_POSITION, p + np.array([0.0, 0.0, 0.015], np.float32))   # the block slides
        added = s.map_grid_emit(0.5 * sc["spacing"])
        assert added > 0 and s.n == len(pos) + added
        st = s.advance_time_step(sc["dt"], stats=True)
        assert st["out_of_grid"] == 0
        p, _ = s.download()
        assert np.all(np.isfinite(p))
    with pytest.raises(bb.BbgError):
        with bb.Solver(sc, pos=pos) as t:
            t.map_grid_emit(0.01)   # no map yet
