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


@pytest.mark.parametrize("tuning", [dict(batch_worklist=0), dict(batch_worklist=1, particles_per_thread=2),
                                    dict(batch_worklist=2, block_size=64)])
def test_batch_work_lists_do_not_change_results(gpu, tuning):
    """The corrector passes over every scene's tiles, over a work list of the tiles of the
    scenes still iterating (one block per tile, or persistent blocks taking tiles from it):
    bitwise the same substeps, per-scene iterations and errors as the default."""
    sc, boxes, pos = small_batch()
    ga = bb.BatchSolver(sc, boxes, pos)
    gb = bb.BatchSolver(sc, boxes, pos)
    gb.set_tuning(**tuning)
    for _ in range(4):
        ga.advance_time_step(sc["dt"])
        gb.advance_time_step(sc["dt"])
        ia, ea = ga.scene_stats()
        ib, eb = gb.scene_stats()
        assert np.array_equal(ia, ib) and np.array_equal(ea, eb)
    pa, va = ga.download()
    pb, vb = gb.download()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    ga.close()
    gb.close()


def test_batch_learned_warm_start_runs(gpu):
    sc, boxes, pos = small_batch()
    scl = dict(sc, pressure_init="learned", mlp={"train_substeps": 4, "batch": 1024})
    g = bb.BatchSolver(scl, boxes, pos)
    for _ in range(8):
        st = g.advance_time_step(sc["dt"], stats=True)
        assert st["max_density_error_ratio"] < 0.01
    assert g.mlp_status()["trained_substeps"] == 4
    g.close()


def packed_frame(sc, boxes):
    """The batch's packed domain and each scene's container in it, by the layout rule of
    bbg_batch_create: scenes stacked along z, each container's min corner on a cell
    boundary, two empty cells between consecutive containers (the same double arithmetic)."""
    import math
    from bubbles_gb300.solver import desc_from_scene
    d = desc_from_scene(dict(sc, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0)))
    cell = d.target_spacing * d.grid_spacing_scale
    xmax = ymax = z = 0.0
    offsets, containers = [], []
    for lo, hi in boxes:
        ext = [float(b) - float(a) for a, b in zip(lo, hi)]
        xmax, ymax = max(xmax, ext[0]), max(ymax, ext[1])
        offsets.append((-float(lo[0]), -float(lo[1]), z - float(lo[2])))
        containers.append({"type": "box", "size": tuple(ext), "reverse": True,
                           "center": (0.5 * ext[0], 0.5 * ext[1], z + 0.5 * ext[2])})
        z = math.ceil((z + ext[2]) / cell) * cell + 2.0 * cell
    dmax = (math.ceil(xmax / cell) * cell, math.ceil(ymax / cell) * cell, z - 2.0 * cell)
    return (0.0, 0.0, 0.0), dmax, np.asarray(offsets), containers


def test_batched_64_scenes_against_oracle(gpu):
    """Config 4 (64 dam breaks of uneven sizes in one batch): after 30 substeps, one substep
    of four scenes -- the smallest, the largest and two from the middle -- against the FP32
    oracle (the reference algorithm) run on each scene alone in the batch's packed frame
    (the packed domain's grid, the scene's container where the batch puts it, the scene's
    particles at their packed coordinates): the same corrector iterations, the tolerance
    met, the same maximum density error, and positions within 1e-5 x spacing or 8 ulps of
    the coordinate, the bound of the single-scene parity tests.  The frame makes the
    arithmetic the batch's own: scenes are independent, so each one is the reference step
    of that scene alone."""
    import os
    from oracle import oracle as O
    sc, pos = scenes.config("batched_64", seed=0)
    boxes = sc["boxes"]
    dmin, dmax, offsets, containers = packed_frame(sc, boxes)
    g = bb.BatchSolver(sc, boxes, pos)
    assert np.array_equal(g.layout(), offsets)
    for _ in range(30):
        g.advance_time_step(sc["dt"])
    ps, vs = bb.Solver.download(g)          # packed coordinates, scene after scene
    g.advance_time_step(sc["dt"])
    its, errs = g.scene_stats()
    nxt, _ = bb.Solver.download(g)
    g.close()
    first = np.concatenate([[0], np.cumsum([len(p) for p in pos])])
    order = np.argsort([len(p) for p in pos])
    picks = [int(order[0]), int(order[-1]), int(order[len(order) // 2]), int(order[len(order) // 3])]
    threads = os.cpu_count() or 1
    h0 = sc["spacing"]
    for k in picks:
        a, b = first[k], first[k + 1]
        one = dict(sc, domain_min=dmin, domain_max=dmax, batch=False, colliders=[containers[k]])
        o = O.OracleSim(one, ps[a:b], vs[a:b], variant="f32", threads=threads)
        it_o, err_o = o.pcisph_substep(sc["dt"], sc["max_density_error_ratio"], sc["max_iterations"],
                                       O.PCISPH_TOLERANCE)
        want = o.get(O.POSITION)
        o.close()
        assert its[k] == it_o, (k, its[k], it_o)
        assert errs[k] < sc["max_density_error_ratio"]
        assert abs(errs[k] - err_o) <= 1e-4, (k, errs[k], err_o)
        allowed = np.maximum(1e-5 * h0, 8.0 * np.spacing(np.abs(want).astype(np.float32)).astype(np.float64))
        d = np.abs(nxt[a:b].astype(np.float64) - want)
        assert np.all(d <= allowed), (k, float(np.max(d / allowed)))
