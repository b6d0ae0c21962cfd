"""Batches of independent scenes: each scene of a batch advances like the same scene in
its own solver (same corrector iterations, positions within the rounding of the
translation into the packed domain), scenes converge independently, and the layout keeps
every scene two empty grid cells away from the next."""
import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes

pytestmark = pytest.mark.gpu


def small_batch(seed=0):
    # containers whose extents are whole grid cells (0.04) so that the single-scene grids
    # have the batch's cell length too
    sc = scenes.base_scene("pcisph", 0.02, (1.0, 1.0, 1.0))
    sc.update(dt=4e-4, max_iterations=20, max_density_error_ratio=0.01)
    specs = [((8, 6, 8), (0.48, 0.32, 0.40)), ((10, 5, 6), (0.56, 0.28, 0.24)),
             ((6, 9, 5), (0.32, 0.40, 0.20))]
    boxes, pos = [], []
    rng = np.random.default_rng(seed)
    for dims, ext in specs:
        ext = np.asarray(ext)
        lo, hi = -ext / 2, ext / 2
        boxes.append((tuple(lo), tuple(hi)))
        pos.append(scenes.dam_block({"spacing": 0.02, "domain_min": tuple(lo)}, dims, int(rng.integers(1000))))
    return sc, boxes, pos


def single(sc, box, p, v=None):
    lo, hi = box
    ext = tuple(float(b - a) for a, b in zip(lo, hi))
    center = tuple(float(a + b) / 2 for a, b in zip(lo, hi))
    one = dict(sc, domain_min=tuple(lo), domain_max=tuple(hi),
               colliders=[{"type": "box", "size": ext, "center": center, "reverse": True}])
    return bb.Solver(one, pos=p, vel=v)


def test_batch_layout_separates_scenes(gpu):
    sc, boxes, pos = small_batch()
    g = bb.BatchSolver(sc, boxes, pos)
    off = g.layout()
    cell = 0.04
    zlo = [boxes[i][0][2] + off[i, 2] for i in range(3)]
    zhi = [boxes[i][1][2] + off[i, 2] for i in range(3)]
    for i in range(2):
        assert zlo[i + 1] - zhi[i] >= 2 * cell - 1e-9
    for i in range(3):
        assert np.allclose(np.asarray(boxes[i][0])[:2] + off[i, :2], 0.0)
    p, _ = g.download_scenes()
    for a, b in zip(p, pos):
        assert np.max(np.abs(a - b)) <= 1e-6
    g.close()


def test_batch_substeps_match_single_scenes(gpu):
    sc, boxes, pos = small_batch()
    g = bb.BatchSolver(sc, boxes, pos)
    for _ in range(4):
        ps, vs = g.download_scenes()
        g.advance_time_step(sc["dt"])
        its, errs = g.scene_stats()
        nxt, _ = g.download_scenes()
        for i in range(3):
            s1 = single(sc, boxes[i], ps[i], vs[i])
            st = s1.advance_time_step(sc["dt"], stats=True)
            p1, _ = s1.download()
            s1.close()
            assert its[i] == st["iterations"]
            assert errs[i] < 0.01
            # the packed coordinates round to ~2e-7 here
            assert np.max(np.abs(nxt[i] - p1)) <= 2e-6
    g.close()


def test_batch_scenes_converge_independently(gpu):
    sc, boxes, pos = small_batch()
    g = bb.BatchSolver(sc, boxes, pos)
    for _ in range(3):
        st = g.advance_time_step(sc["dt"], stats=True)
    its, errs = g.scene_stats()
    assert st["iterations"] == its.max()
    assert np.all(errs < 0.01)
    g.close()


def test_batch_learned_warm_start_runs(gpu):
    sc, boxes, pos = small_batch()
    scl = dict(sc, pressure_init="learned", mlp={"train_substeps": 4, "batch": 1024})
    g = bb.BatchSolver(scl, boxes, pos)
    for _ in range(8):
        st = g.advance_time_step(sc["dt"], stats=True)
        assert st["max_density_error_ratio"] < 0.01
    assert g.mlp_status()["trained_substeps"] == 4
    g.close()


def test_batched_64_scenes_against_oracle(gpu):
    """Config 4 (64 dam breaks of uneven sizes in one batch): after 30 substeps, one substep
    of four scenes -- the smallest, the largest and two from the middle -- against the FP32
    oracle (the reference algorithm) run on each scene alone from the batch's state: the
    same corrector iterations, the tolerance met, and positions within 16 ulps of the packed
    coordinate plus 1e-5 x spacing.  The batch computes in the packed domain, where scenes
    stacked along z sit at |z| up to ~12 (ulp ~1e-6); relative positions there carry that
    absolute rounding, so a scene matches the same scene computed at its own origin only to
    a few ulps of its packed coordinates."""
    import os
    from oracle import oracle as O
    sc, pos = scenes.config("batched_64", seed=0)
    boxes = sc["boxes"]
    g = bb.BatchSolver(sc, boxes, pos)
    for _ in range(30):
        g.advance_time_step(sc["dt"])
    ps, vs = g.download_scenes()
    g.advance_time_step(sc["dt"])
    its, errs = g.scene_stats()
    nxt, _ = g.download_scenes()
    off = g.layout()
    g.close()
    order = np.argsort([len(p) for p in pos])
    picks = [int(order[0]), int(order[-1]), int(order[len(order) // 2]), int(order[len(order) // 3])]
    threads = os.cpu_count() or 1
    for k in picks:
        lo, hi = boxes[k]
        ext = tuple(float(b - a) for a, b in zip(lo, hi))
        center = tuple(float(a + b) / 2 for a, b in zip(lo, hi))
        one = dict(sc, domain_min=tuple(lo), domain_max=tuple(hi), batch=False,
                   colliders=[{"type": "box", "size": ext, "center": center, "reverse": True}])
        o = O.OracleSim(one, ps[k], vs[k], variant="f32", threads=threads)
        it_o, _ = o.pcisph_substep(sc["dt"], sc["max_density_error_ratio"], sc["max_iterations"],
                                   O.PCISPH_TOLERANCE)
        want = o.get(O.POSITION)
        o.close()
        assert its[k] == it_o, (k, its[k], it_o)
        assert errs[k] < sc["max_density_error_ratio"]
        packed = np.abs(want + off[k][None, :]).astype(np.float32)
        allowed = 16.0 * np.spacing(packed).astype(np.float64) + 1e-5 * sc["spacing"]
        assert np.all(np.abs(nxt[k] - want) <= allowed), (k, float(np.max(np.abs(nxt[k] - want) - allowed)))
