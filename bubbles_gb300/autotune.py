"""Autotuner of the solver's launch parameters and, for batches, of the grid cell size.

For one configuration it advances the scene to a representative state, then times the
same substeps (replayed as CUDA graphs from that state) for candidate settings:

  * block size of the neighbour passes (the tile of consecutive cell-sorted particles a
    block walks): 64, 128, 256;
  * members whose neighbour records a thread requests together, separately for the
    non-pressure, predicted-density and pressure-force passes: 2, 4, 8;
  * whether the density pass leaves out the neighbour cells and rows each particle's
    sphere cannot reach (bitwise the same results): 0, 1;
  * particles per thread of the predicted-density and pressure-force passes: 1, 2;
  * the order in which blocks take tiles: 0 (block b, tile b) or 1 (the blocks an SM runs
    take neighbouring tiles);
  * for batches, how the corrector passes cover the scenes: one block per tile of every
    scene (0), one block per tile of the scenes still iterating, from a work list rebuilt
    every iteration (1), or persistent blocks over that work list (2);
  * for batches only, the grid cell as a multiple of the particle spacing: 2 (the kernel
    radius), 2.5, 3 -- any cell at least the kernel radius keeps every neighbour inside
    the 27 cells, and a batch has no reference grid to match.  A single scene keeps the
    reference's grid (cell ids and permutation are part of its contract).

The search is coordinate descent (one parameter at a time, the rest at their best so
far).  Results do not depend on these settings; only time does.  The tuned values are
written to a JSON file that `bench.py` and `Solver.set_tuning` read:

    python -m bubbles_gb300.autotune --config pcisph_1m --out bubbles_gb300/tuned/pcisph_1m.json
"""
import argparse
import json
import os
import time

from . import scenes
from .solver import BatchSolver, Solver

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED_DIR = os.path.join(HERE, "tuned")
BLOCKS = (64, 128, 256)
BATCHES = (2, 4, 8)
PRUNES = (0, 1)
PPTS = (1, 2)
TILE_ORDERS = (0, 1)
WORKLISTS = (0, 1, 2)
CELL_SCALES = (2.0, 2.5, 3.0)


def tuned_path(config):
    return os.path.join(TUNED_DIR, "%s.json" % config)


def load(config):
    """Tuned settings of a configuration, or None."""
    path = tuned_path(config)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def make(scene, pos):
    if scene.get("batch"):
        return BatchSolver(scene, scene["boxes"], pos)
    return Solver(scene, pos=pos)


FIELD_PRESSURE, FIELD_DIVERGENCE = 5, 11


def restore(g, snap):
    p, v, pr, dv = snap
    g.upload(p, v)
    if pr is not None:
        g.set(FIELD_PRESSURE, pr)
    if dv is not None:
        g.set(FIELD_DIVERGENCE, dv)


def time_substeps(g, dt, snap, steps, warm):
    """Seconds for `steps` substeps from the snapshot (after two untimed ones)."""
    restore(g, snap)
    for _ in range(2):
        g.advance_time_step(dt)
    restore(g, snap)
    g.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        g.advance_time_step(dt)
    g.synchronize()
    return time.perf_counter() - t0


def tune_launches(g, dt, snap, steps, warm, log):
    best = dict(g.tuning())
    best_t = time_substeps(g, dt, snap, steps, warm)
    log.append({"tuning": dict(best), "seconds": best_t})
    knobs = [("block_size", BLOCKS), ("prune", PRUNES), ("batch_pf", BATCHES), ("batch_pd", BATCHES),
             ("batch_np", BATCHES), ("particles_per_thread", PPTS), ("tile_order", TILE_ORDERS)]
    if isinstance(g, BatchSolver):
        knobs.append(("batch_worklist", WORKLISTS))
    for key, values in knobs:
        for v in values:
            if v == best[key]:
                continue
            cand = dict(best, **{key: v})
            g.set_tuning(**cand)
            t = time_substeps(g, dt, snap, steps, warm)
            log.append({"tuning": dict(cand), "seconds": t})
            if t < best_t:
                best, best_t = cand, t
        g.set_tuning(**best)
    return best, best_t


def tune(config, prep=100, steps=20, variant="plain", seed=0):
    scene, pos = scenes.config(config, seed=seed)
    scene["pressure_init"] = {"plain": "zero", "warm": "previous", "learned": "learned"}[variant]
    if variant == "learned":
        scene["mlp"] = {"train_substeps": prep}
    warm = variant != "plain"
    dt = scene["dt"]
    log = []
    results = []
    scales = CELL_SCALES if scene.get("batch") else (scene.get("grid_spacing_scale", 2.0),)
    for scale in scales:
        sc = dict(scene, grid_spacing_scale=scale)
        g = make(sc, pos)
        for _ in range(prep):
            g.advance_time_step(dt)
        p, v = g.download()
        pr = g.get(FIELD_PRESSURE) if warm else None
        dv = g.get(FIELD_DIVERGENCE) if variant == "learned" else None
        best, t = tune_launches(g, dt, (p, v, pr, dv), steps, warm, log)
        results.append((t, scale, best))
        g.close()
    t, scale, best = min(results, key=lambda r: r[0])
    n = sum(len(x) for x in pos) if scene.get("batch") else len(pos)
    return {"config": config, "variant": variant, "particles": n, "grid_spacing_scale": scale,
            "tuning": best, "particle_updates_per_s": n * steps / t,
            "measured": "%d substeps from the state after %d substeps, wall clock around graph "
                        "launches (device-bound)" % (steps, prep),
            "candidates": log}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="pcisph_1m")
    ap.add_argument("--variant", default="plain", choices=["plain", "warm", "learned"])
    ap.add_argument("--prep", type=int, default=100)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--out", default=None)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    res = tune(args.config, args.prep, args.steps, args.variant, args.seed)
    out = args.out or tuned_path(args.config)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({k: v for k, v in res.items() if k != "candidates"}))


if __name__ == "__main__":
    main()
