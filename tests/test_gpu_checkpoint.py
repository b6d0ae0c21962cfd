"""Checkpoints: a run continued from a checkpoint in a new solver is bit-identical to the
run that wrote it (positions, velocities, every carried field, the learned warm start's
training), and bad or mismatched checkpoints are refused without touching the solver."""
import numpy as np
import pytest

import bubbles_gb300 as bb
from test_gpu_batch import small_batch

pytestmark = pytest.mark.gpu


def state(g):
    p, v = g.download()
    return p, v, g.get(bb.FIELD_PRESSURE), g.get(bb.FIELD_DENSITY), g.get(bb.FIELD_FORCE)


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def resume_pair(sc, p, v, before, after, advance=False):
    """Run `before` substeps, checkpoint, run `after` more; continue a new solver from the
    checkpoint for the same `after` substeps.  Returns both solvers."""
    dt = sc["dt"]
    a = bb.Solver(sc, pos=p, vel=v)
    for _ in range(before):
        a.advance_time_step(dt)
    data = a.checkpoint()
    b = bb.Solver(sc, capacity=len(p))
    b.restore(data)
    for g in (a, b):
        for _ in range(after):
            if advance:
                g.advance(2 * dt)   # CFL substep loop: reads the restored forces
            else:
                g.advance_time_step(dt)
    return a, b


@pytest.mark.parametrize("init", ["zero", "previous"])
def test_resume_is_bit_exact(gpu, moved, init):
    sc, p, v = moved
    sc = dict(sc, pressure_init=init)
    a, b = resume_pair(sc, p, v, before=3, after=4)
    assert same(state(a), state(b))
    a, b = resume_pair(sc, p, v, before=2, after=2, advance=True)
    assert same(state(a), state(b))


def test_resume_learned_during_and_after_training(gpu, moved):
    sc, p, v = moved
    scl = dict(sc, pressure_init="learned", mlp=dict(train_substeps=4, batch=1024))
    # checkpoint in the middle of training; the continuation trains, then uses the model
    a, b = resume_pair(scl, p, v, before=2, after=5)
    assert same(state(a), state(b))
    assert np.array_equal(a.get(bb.FIELD_DIVERGENCE), b.get(bb.FIELD_DIVERGENCE))
    assert np.array_equal(a.mlp_params(), b.mlp_params())
    sa, sb = a.mlp_status(), b.mlp_status()
    assert sa == sb and sa["trained_substeps"] == 4


def test_resume_batch(gpu):
    sc, boxes, pos = small_batch()
    a = bb.BatchSolver(sc, boxes, pos)
    for _ in range(2):
        a.advance_time_step(sc["dt"])
    data = a.checkpoint()
    b = bb.BatchSolver(sc, boxes, pos)
    b.restore(data)
    for g in (a, b):
        for _ in range(3):
            g.advance_time_step(sc["dt"])
    pa, va = a.download_scenes()
    pb, vb = b.download_scenes()
    for i in range(len(pa)):
        assert np.array_equal(pa[i], pb[i]) and np.array_equal(va[i], vb[i])
    assert np.array_equal(a.scene_stats()[0], b.scene_stats()[0])


def test_checkpoint_file_and_refusals(gpu, moved, tmp_path):
    sc, p, v = moved
    dt = sc["dt"]
    a = bb.Solver(sc, pos=p, vel=v)
    a.advance_time_step(dt)
    path = tmp_path / "state.bbg"
    a.save_checkpoint(path)
    data = a.checkpoint()
    assert path.read_bytes() == data
    b = bb.Solver(sc, capacity=len(p) + 10)
    b.load_checkpoint(path)
    assert b.n == len(p)
    assert same(state(a), state(b))

    c = bb.Solver(sc, pos=p[: len(p) // 2], capacity=len(p))
    c.advance_time_step(dt)
    before = state(c)
    for bad in (data[:100], data[: len(data) // 2], b"x" * len(data), data[:-4]):
        with pytest.raises(bb.BbgError):
            c.restore(bad)
        assert same(state(c), before)   # untouched
    with pytest.raises(bb.BbgError):
        bb.Solver(sc, capacity=len(p) - 1).restore(data)   # capacity
    with pytest.raises(bb.BbgError):
        bb.Solver(dict(sc, viscosity=0.05), capacity=len(p)).restore(data)   # description
    with pytest.raises(bb.BbgError):
        learned = dict(sc, pressure_init="learned", mlp=dict(train_substeps=4, batch=1024))
        bb.Solver(learned, capacity=len(p)).restore(data)
    with pytest.raises(bb.BbgError):
        b.load_checkpoint(tmp_path / "missing.bbg")


def test_resume_with_fields_into_a_fresh_solver(gpu, small):
    """Colliders with signed-distance fields travel in the checkpoint: a box whose field was
    generated on the device and a field-only sphere, restored into a solver with no fields
    attached, continue bit-identically; corrupt field records are refused untouched."""
    from test_gpu_sdf import attach, field_scene, golden
    gold, _ = golden()
    sc, pos = small
    scf = field_scene(sc)
    dt = sc["dt"]
    a = bb.Solver(scf, pos=pos)
    attach(a, gold)
    a.generate_sdf(0, dx=0.02, margin=0.1)
    for _ in range(5):
        a.advance_time_step(dt)
    data = a.checkpoint()
    b = bb.Solver(scf, capacity=len(pos))
    b.restore(data)
    for k in (0, 1):
        na, oa, sa, va = a.get_sdf(k)
        nb, ob, sb, vb = b.get_sdf(k)
        assert np.array_equal(na, nb) and np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    for g in (a, b):
        for _ in range(4):
            g.advance_time_step(dt)
    assert same(state(a), state(b))

    c = bb.Solver(scf, pos=pos, capacity=len(pos))
    attach(c, gold)
    c.advance_time_step(dt)
    before = state(c)
    bad = bytearray(data)
    bad[28:32] = (0).to_bytes(4, "little")   # the header's field count
    for corrupt in (bytes(bad), data[: len(data) - 4 * len(pos)]):
        with pytest.raises(bb.BbgError):
            c.restore(corrupt)
        assert same(state(c), before)
