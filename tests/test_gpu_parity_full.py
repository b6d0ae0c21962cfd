"""Per-particle parity on the benchmark configurations at their full sizes.

Each case runs the real scene on the GPU until it is in motion, then takes one substep
from that identical state on both sides -- the CUDA path through the C ABI and the FP32
oracle (the reference CPU path restated, all host threads) -- pass by pass:

  - grid: cell of every particle, per-cell counts, stable permutation (bit-exact);
  - neighbour sets: every particle's members, as sets (not only their number), equal to
    the oracle's buckets (src/core/grid.h:423-447);
  - density: relative 1e-5 per particle (all summands positive);
  - non-pressure force (from identical density) and pressure of one corrector pass:
    |error_i| <= 1e-5 x the sum of the magnitudes of particle i's summands -- the FP32
    error bound of a sum with cancellation, per particle;
  - pressure force (from identical p, rho*): the same with each summand's conditioned
    magnitude.  A summand c (1 - d/h)^2 is computed from a distance d that carries its own
    rounding, and 1 - d/h cancels near the kernel radius: its first-order error is
    c x (x + 2 d/h) eps <= c x (x + 2) eps with x = 1 - d/h, so the bound is
    1e-5 x sum_j c_j x_j (x_j + 2) (a few times the summand far inside the kernel; near
    the kernel radius, where (1 - d/h)^2 is tiny, the conditioning term dominates);
  - predictions, accumulation and integration with colliders: bit-exact from identical
    inputs;
  - a whole tolerance-mode substep (src/equations/pcisph_equations3.cpp:218-256): the
    same number of corrector iterations and positions within 1e-5 x spacing or 8 ulps of
    the coordinate, whichever is larger (an FP32 coordinate cannot be closer than its ulp;
    the integration x + dt (v + dt F / m) rounds on the coordinate's scale -- the report
    gives the worst particle in ulps).  A particle in contact with a collider gets 2 ulps
    of the collider frame's scale instead when that is larger: its normal coordinate can
    land within an ulp of the surface, the projection then fires on one side only, and it
    rounds every coordinate in the collider's frame (a box measures from its corner, so a
    coordinate near 0 moves by an ulp of the box's half extent).

Every case prints the per-particle relative error percentiles (p50, p99, max), and
appends them as one JSON line to $BBG_PARITY_REPORT when that is set.
"""
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-5
CHUNK = 1 << 16


def percentiles(x):
    x = np.asarray(x, np.float64)
    return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)), "max": float(x.max())}


def report(rep):
    print(json.dumps(rep))
    path = os.environ.get("BBG_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(rep) + "\n")


def bucket_rows(ids, cnt):
    """The oracle's buckets as rows of member ids other than the particle itself, -1 padded
    and sorted (so that -1 comes first), over the widest bucket."""
    w = int(cnt.max())
    rows = np.array(ids[:, :w], np.int64)
    rows[np.arange(w)[None, :] >= cnt[:, None]] = -1
    rows[rows == np.arange(len(rows))[:, None]] = -1
    rows.sort(axis=1)
    return rows


def gpu_rows(ids, cnt, w):
    rows = np.full((len(ids), w), -1, np.int64)
    k = min(w, ids.shape[1])
    rows[:, :k] = ids[:, :k]
    rows[np.arange(w)[None, :] >= cnt[:, None]] = -1
    rows.sort(axis=1)
    return rows


def pair_sum(x, rows, term):
    """sum over j in rows[i] (>= 0) of term(i_idx, j_idx, r) for every particle, in chunks;
    r = |x_j - x_i| in FP64."""
    n = len(rows)
    out = np.zeros(n)
    for a in range(0, n, CHUNK):
        b = min(n, a + CHUNK)
        j = rows[a:b]
        ok = j >= 0
        jj = np.where(ok, j, 0)
        ii = np.arange(a, b)[:, None]
        r = np.linalg.norm(x[jj] - x[ii], axis=2)
        out[a:b] = np.sum(np.where(ok, term(ii, jj, r), 0.0), axis=1)
    return out


def collider_frame(sc, *positions):
    """The largest coordinate of the colliders' frames (corner or centre + radius), and
    which particles lie within a particle radius (+ 1e-4) of a collider surface in any of
    the given position arrays."""
    r = sc["spacing"] + 1e-4
    scale, contact = 0.0, np.zeros(len(positions[0]), bool)
    for c in sc.get("colliders", []):
        t = np.asarray(c.get("center", (0.0, 0.0, 0.0)), np.float64)
        if c["type"] == "box":
            half = np.asarray(c["size"], np.float64) / 2
            scale = max(scale, float(np.max(np.abs(t) + half)))
            for x in positions:
                gap = half[None, :] - np.abs(np.asarray(x, np.float64) - t[None, :])
                contact |= gap.min(axis=1) <= r if c.get("reverse") else gap.max(axis=1) >= -r
        else:
            scale = max(scale, float(np.max(np.abs(t)) + c["radius"]))
            for x in positions:
                d = np.linalg.norm(np.asarray(x, np.float64) - t[None, :], axis=1) - c["radius"]
                contact |= np.abs(d) <= r
    return scale, contact


def moving_state(name, seed, substeps):
    sc, pos = scenes.config(name, seed=seed)
    with bb.Solver(sc, pos=pos) as g:
        for _ in range(substeps):
            g.advance_time_step(sc["dt"])
        p, v = g.download()
    return sc, p, v


@pytest.mark.parametrize("name,seed,substeps", [("pcisph_262k", 1, 120), ("pcisph_1m", 2, 120),
                                                ("pcisph_4m", 3, 60)])
def test_substep_parity_full_size(gpu, name, seed, substeps):
    sc, p, v = moving_state(name, seed, substeps)
    dt, h0, rho0 = sc["dt"], sc["spacing"], sc["target_density"]
    n = len(p)
    threads = os.cpu_count() or 1
    rep = {"config": name, "particles": n, "after_substeps": substeps, "oracle_threads": threads}
    g = bb.Solver(sc, pos=p, vel=v)
    o = O.OracleSim(sc, p, v, variant="f32", threads=threads)
    m, h = g.scalars()["mass"], g.scalars()["kernel_radius"]

    # grid: bit-exact (DistributeByParticle's stable order)
    g.update_grid_distribution()
    o.update_grid_distribution()
    cell_g, counts_g, ids_g = g.dump_grid()
    cell_o, counts_o, chains_o = o.cells()
    assert np.array_equal(cell_g, cell_o)
    assert np.array_equal(counts_g, counts_o)
    assert np.array_equal(ids_g, chains_o)

    # neighbour sets: equal as sets
    g.compute_density(1)
    o.compute_particle_interaction()
    o.compute_density(1)
    cnt_o, bids, over = o.buckets()
    assert over == 0
    cnt_g, nb_g = g.neighbor_lists(64)
    assert np.array_equal(cnt_g + 1, cnt_o)
    rows = bucket_rows(bids, cnt_o)
    del bids
    assert np.array_equal(gpu_rows(nb_g, cnt_g, rows.shape[1]), rows)
    del nb_g
    rep["neighbours"] = {"mean": float(cnt_g.mean()), "max": int(cnt_g.max()), "sets_equal": True}

    # density (positive summands): relative 1e-5 per particle
    rho_g, rho_o = g.get(bb.FIELD_DENSITY), o.get(O.DENSITY)
    rel = np.abs(rho_g - rho_o) / rho_o
    rep["density_rel"] = percentiles(rel)
    checks = {"density": rel.max() <= RTOL}
    # EOS pressure p = B ((rho / rho0)^gamma - 1): error bound 1e-5 x B ((rho / rho0)^gamma + 1)
    bmod = rho0 * sc["sound_speed"] ** 2 / sc["eos_exponent"]
    s_eos = bmod * ((rho_o / rho0) ** sc["eos_exponent"] + 1.0)
    d_eos = np.abs(g.get(bb.FIELD_PRESSURE) - o.get(O.PRESSURE)) / s_eos
    rep["eos_pressure_err_over_summands"] = percentiles(d_eos)
    checks["eos_pressure"] = d_eos.max() <= RTOL

    # non-pressure force from identical density
    o.set(O.DENSITY, rho_g)
    g.compute_non_pressure_force()
    o.compute_non_pressure_force()
    f_g, f_o = g.get(bb.FIELD_FORCE), o.get(O.FORCE)
    x = o.get(O.POSITION)
    vo = o.get(O.VELOCITY)
    kv = sc["viscosity"] * m * m * 90.0 / (np.pi * h ** 5)
    grav = np.linalg.norm(np.asarray(sc["gravity"]))
    s_np = m * grav + sc["drag_coefficient"] * np.linalg.norm(vo, axis=1) + pair_sum(
        x, rows, lambda i, j, r: kv * np.linalg.norm(vo[j] - vo[i], axis=2) * np.clip(1 - r / h, 0, None) / rho_g[j])
    df = np.linalg.norm(f_g - f_o, axis=1)
    rep["non_pressure_err_over_summands"] = percentiles(df / s_np)
    rep["non_pressure_rel"] = percentiles(df / np.maximum(np.linalg.norm(f_o, axis=1), 1e-30))
    checks["non_pressure"] = bool(np.all(df <= RTOL * s_np))

    # corrector passes from identical inputs
    o.set(O.FORCE, f_g)
    delta = g.compute_delta(dt)
    assert delta == o.compute_delta(dt)
    g.predict_velocity_and_position(dt, 1)
    o.predict_velocity_and_position(dt, 1)
    assert np.array_equal(g.get(bb.FIELD_PRED_POSITION), o.get(O.PRED_POSITION).astype(np.float32))
    g.predict_pressure(delta)
    o.predict_pressure(delta)
    rs_g, rs_o = g.get(bb.FIELD_PRED_DENSITY), o.get(O.PRED_DENSITY)
    rel = np.abs(rs_g - rs_o) / rs_o
    rep["pred_density_rel"] = percentiles(rel)
    checks["pred_density"] = rel.max() <= RTOL
    # p = delta (rho* - rho0): summands delta rho* and delta rho0
    pg, po = g.get(bb.FIELD_PRESSURE), o.get(O.PRESSURE)
    d_p = np.abs(pg - po) / (abs(delta) * (rs_o + rho0))
    rep["pressure_err_over_summands"] = percentiles(d_p)
    checks["pressure"] = d_p.max() <= RTOL
    o.set(O.PRESSURE, pg)
    o.set(O.PRED_DENSITY, rs_g)
    g.predict_pressure_force()
    o.predict_pressure_force()
    a = np.abs(pg.astype(np.float64)) / (rs_g.astype(np.float64) ** 2)
    kg = m * m * 45.0 / (np.pi * h ** 4)

    def conditioned(i, j, r):
        xk = np.clip(1 - r / h, 0, None)
        return kg * (a[i] + a[j]) * xk * (xk + 2.0)
    s_pf = pair_sum(x, rows, conditioned)
    fp_g, fp_o = g.get(bb.FIELD_PRESSURE_FORCE), o.get(O.PRESSURE_FORCE)
    dfp = np.linalg.norm(fp_g - fp_o, axis=1)
    rep["pressure_force_err_over_summands"] = percentiles(dfp / np.maximum(s_pf, 1e-30))
    rep["pressure_force_rel"] = percentiles(dfp / np.maximum(np.linalg.norm(fp_o, axis=1), 1e-30))
    checks["pressure_force"] = bool(np.all(dfp <= RTOL * s_pf))
    if not checks["pressure_force"]:
        w = int(np.argmax(dfp - RTOL * s_pf))
        rep["pressure_force_worst"] = {"particle": w, "err": float(dfp[w]), "summands": float(s_pf[w]),
                                       "gpu": fp_g[w].tolist(), "oracle": fp_o[w].tolist(),
                                       "p": float(pg[w]), "rho_star": float(rs_g[w]),
                                       "members": int(cnt_g[w]),
                                       "violations": int(np.sum(dfp > RTOL * s_pf))}
    o.set(O.PRESSURE_FORCE, fp_g)
    g.predict_velocity_and_position(dt, 0)
    o.predict_velocity_and_position(dt, 0)
    checks["prediction_bits"] = bool(np.array_equal(g.get(bb.FIELD_PRED_POSITION),
                                                    o.get(O.PRED_POSITION).astype(np.float32)))
    g.accumulate_and_integrate(dt)
    o.accumulate_and_integrate(dt)
    pg2, vg2 = g.download()
    checks["integration_bits"] = bool(np.array_equal(pg2, o.get(O.POSITION).astype(np.float32)) and
                                      np.array_equal(vg2, o.get(O.VELOCITY).astype(np.float32)))
    g.close()
    o.close()

    # a whole tolerance-mode substep from the same state
    g = bb.Solver(sc, pos=p, vel=v)
    o = O.OracleSim(sc, p, v, variant="f32", threads=threads)
    st = g.advance_time_step(dt, stats=True)
    it_o, err_o = o.pcisph_substep(dt, sc["max_density_error_ratio"], sc["max_iterations"], O.PCISPH_TOLERANCE)
    rep["substep"] = {"iterations_gpu": st["iterations"], "iterations_oracle": it_o,
                      "max_err_gpu": st["max_density_error_ratio"], "max_err_oracle": err_o}
    pg3, vg3 = g.download()
    po3 = o.get(O.POSITION)
    dxyz = np.abs(pg3.astype(np.float64) - po3)
    ulp = np.spacing(np.abs(po3).astype(np.float32)).astype(np.float64)
    allowed = np.maximum(RTOL * h0, 8.0 * ulp)
    # a particle in contact with a collider may be projected on one side only (its normal
    # coordinate lies within an ulp of the surface), and the projection rounds every
    # coordinate in the collider's frame (box.cpp:111-172 measures from a box corner)
    scale, contact = collider_frame(sc, pg3, po3)
    allowed[contact] = np.maximum(allowed[contact], 2.0 * float(np.spacing(np.float32(2.0 * scale))))
    rep["substep"]["collider_contacts"] = int(contact.sum())
    rep["substep"]["position_err_max_ulps"] = float((dxyz / ulp).max())
    dx = np.linalg.norm(pg3 - po3, axis=1) / h0
    rep["substep"]["position_err_over_spacing"] = percentiles(dx)
    rep["substep"]["position_err_over_allowed"] = percentiles((dxyz / allowed).max(axis=1))
    rep["substep"]["density_rel"] = percentiles(np.abs(g.get(bb.FIELD_DENSITY) - o.get(O.DENSITY)) / o.get(O.DENSITY))
    # the particles farthest from their bound, with the fields that decide their positions
    over = (dxyz / allowed).max(axis=1)
    worst = np.argsort(over)[-4:][::-1]
    fields = {"force": (bb.FIELD_FORCE, O.FORCE), "pressure_force": (bb.FIELD_PRESSURE_FORCE, O.PRESSURE_FORCE),
              "pressure": (bb.FIELD_PRESSURE, O.PRESSURE), "pred_density": (bb.FIELD_PRED_DENSITY, O.PRED_DENSITY)}
    got = {k: (g.get(a), o.get(b)) for k, (a, b) in fields.items()}
    vo3 = o.get(O.VELOCITY)
    rep["substep"]["worst"] = [
        {"particle": int(w), "over_allowed": float(over[w]), "start": p[w].tolist(), "start_vel": v[w].tolist(),
         "gpu": pg3[w].tolist(), "oracle": po3[w].tolist(), "gpu_vel": vg3[w].tolist(), "oracle_vel": vo3[w].tolist(),
         **{k + "_gpu": np.asarray(a[w]).tolist() for k, (a, b) in got.items()},
         **{k + "_oracle": np.asarray(b[w]).tolist() for k, (a, b) in got.items()}}
        for w in worst]
    g.close()
    o.close()
    checks["substep_iterations"] = st["iterations"] == it_o
    checks["substep_max_error"] = abs(st["max_density_error_ratio"] - err_o) <= 1e-4
    checks["substep_positions"] = bool(np.all(dxyz <= allowed))
    rep["checks"] = {k: bool(v) for k, v in checks.items()}
    report(rep)
    assert all(checks.values()), [k for k, v in checks.items() if not v]
