"""Particle seeding: VolumeParticleEmitter3 (BCC lattice, jitter from the C library's
rand(), Shape::SignedDistance <= 0, max_particles) on the device.

The oracle's restatement (oracle/sph_oracle.c, orc_emit_volume) is pinned against the
particles the reference emitter itself produced (tests/golden/emit_f32.npz); the device
emitter is compared with both bit for bit.  Each emission is preceded by srand(seed), as
the reference's own rand() stream would be.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "emit_f32.npz")
LIBC = ctypes.CDLL(None)


def golden():
    d = np.load(GOLDEN, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["cases"]))


def kwargs(case):
    shape, sp, jit, vel, mx, bounds, seed = case
    return dict(jitter=jit, velocity=vel, bounds=bounds,
                max_particles=mx if mx is not None else 2**31 - 1), shape, sp, seed


def same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_oracle_emitter_is_the_reference():
    g, cases = golden()
    for i, case in enumerate(cases):
        kw, shape, sp, seed = kwargs(case)
        LIBC.srand(seed)
        p, v = O.emit_volume(shape, sp, **kw)
        assert same_bits(p, g["pos_%d" % i]) and same_bits(v, g["vel_%d" % i]), i


def test_oracle_map_grid_emit_is_the_reference():
    """The oracle's MapGrid / MapGridEmit gives the positions the reference builder added."""
    d = np.load(os.path.join(os.path.dirname(GOLDEN), "continuous_f32.npz"), allow_pickle=False)
    sc = json.loads(str(d["scene"]))
    for i, (cap, dist, _) in enumerate(json.loads(str(d["cases"]))):
        o = O.OracleSim(sc, d["pos0"])
        o.update_grid_distribution()
        o.map_grid()
        o.set(O.POSITION, d["pos1"])
        new = o.map_grid_emit(dist)
        k = min(len(new), cap - len(d["pos0"]))
        assert same_bits(new[:k], d["pos_%d_0" % i][len(d["pos0"]):])
        o.close()


@pytest.mark.gpu
def test_emit_matches_reference(gpu):
    g, cases = golden()
    sc = scenes.base_scene("pcisph", 0.02, (1.0, 1.0, 1.0))
    with bb.Solver(sc, capacity=20000) as s:
        for i, case in enumerate(cases):
            kw, shape, sp, seed = kwargs(case)
            LIBC.srand(seed)
            n = s.emit_volume(shape, sp, **kw)
            p, v = s.download()
            assert n == len(g["pos_%d" % i]) == s.n
            assert same_bits(p, g["pos_%d" % i]) and same_bits(v, g["vel_%d" % i]), i
            # the rand() stream advanced by two values per lattice point, as the oracle's
            LIBC.srand(seed)
            O.emit_volume(shape, sp, **dict(kw, max_particles=2**31 - 1))
            after_oracle = LIBC.rand()
            LIBC.srand(seed)
            s.emit_volume(shape, sp, **dict(kw, max_particles=2**31 - 1))
            assert LIBC.rand() == after_oracle


@pytest.mark.gpu
def test_emit_full_size_and_step(gpu):
    """A jittered sphere of about a million particles equals the oracle's; the emitted set
    then steps like any uploaded one."""
    sc = dict(scenes.base_scene("pcisph", 0.008, (2.0, 1.0, 1.2)), dt=2e-4)
    shape = {"type": "sphere", "radius": 0.35, "center": (0.0, 0.0, 0.0)}
    LIBC.srand(42)
    want, wv = O.emit_volume(shape, 0.008, jitter=0.2)
    assert len(want) > 600000
    with bb.Solver(sc, capacity=len(want)) as s:
        LIBC.srand(42)
        n = s.emit_volume(shape, 0.008, jitter=0.2)
        p, v = s.download()
        assert n == len(want) and same_bits(p, want) and same_bits(v, wv)
        s.setup()
        st = s.advance_time_step(sc["dt"], stats=True)
        assert st["out_of_grid"] == 0 and st["iterations"] >= 1


@pytest.mark.gpu
def test_emit_append_continues_the_set(gpu, small):
    """append=True adds the emitted particles after the existing ones (new ids at the end);
    the result equals uploading the concatenation."""
    sc, pos = small
    shape = {"type": "box", "size": (0.1, 0.08, 0.1), "center": (0.15, 0.1, 0.15)}
    LIBC.srand(9)
    extra, ev = O.emit_volume(shape, 0.02, jitter=0.1, velocity=(0.0, -1.0, 0.0))
    with bb.Solver(sc, pos=pos, capacity=len(pos) + len(extra)) as s:
        s.advance_time_step(sc["dt"])
        p0, v0 = s.download()
        LIBC.srand(9)
        n = s.emit_volume(shape, 0.02, jitter=0.1, velocity=(0.0, -1.0, 0.0), append=True)
        assert n == len(extra) and s.n == len(pos) + n
        p, v = s.download()
        assert same_bits(p[: len(pos)], p0) and same_bits(p[len(pos):], extra)
        assert same_bits(v[len(pos):], ev)
        s.advance_time_step(sc["dt"])
        pa, va = s.download()
    with bb.Solver(sc, pos=np.concatenate([p0, extra]), vel=np.concatenate([v0, ev])) as r:
        r.advance_time_step(sc["dt"])
        pb, vb = r.download()
    assert same_bits(pa, pb) and same_bits(va, vb)


@pytest.mark.gpu
def test_emit_refusals(gpu, small):
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        with pytest.raises(bb.BbgError):   # capacity
            s.emit_volume({"type": "box", "size": (0.5, 0.5, 0.5)}, 0.01)
        assert s.n == len(pos)
        with pytest.raises(bb.BbgError):
            s.emit_volume({"type": "sphere", "radius": 0.1}, 0.0)
        assert s.emit_volume({"type": "sphere", "radius": 0.1, "center": (5.0, 5.0, 5.0)}, 0.02,
                             bounds=((0, 0, 0), (0.1, 0.1, 0.1))) == 0
