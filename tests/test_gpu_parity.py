"""GPU parity: the CUDA path (through the bbg C ABI) against the FP32 oracle.

Contract (per substep, from identical input state):
  - grid cell ids, per-cell counts and the cell-sorted permutation: bit-exact;
  - neighbour counts: equal to the reference bucket counts;
  - integration / prediction with colliders, given identical forces: bit-exact;
  - density, pressure, forces: relative 1e-5 in FP32.  For vector sums with
    cancellation the bound is |dF_i| <= 1e-5 * (|F_i| + max_j |F_j|).
Full-size workloads are checked through size-independent invariants.
"""
import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def pair(sc, pos, vel=None, variant="f32"):
    g = bb.Solver(sc, pos=pos, vel=vel)
    o = O.OracleSim(sc, pos, vel, variant=variant)
    return g, o


def pressure_force_scale(o, x, mass, h):
    """S_i = sum_j |m^2 (p_i / rho_i^2 + p_j / rho_j^2) grad W_spiky(x_i - x_j)| over the
    oracle's bucket of i: the magnitude of the summands of the (cancelling) pressure force."""
    counts, ids, _ = o.buckets()
    p = o.get(O.PRESSURE)
    r = o.get(O.PRED_DENSITY)
    a = np.abs(p) / (r * r)
    kg = 45.0 / (np.pi * h ** 4)
    s = np.zeros(len(x))
    for i in range(len(x)):
        js = ids[i, :counts[i]]
        js = js[js != i]
        d = np.linalg.norm(x[js] - x[i], axis=1)
        g = kg * np.clip(1.0 - d / h, 0.0, None) ** 2
        s[i] = np.sum(mass * mass * (a[i] + a[js]) * g)
    return s


def rel_close(a, b, rtol=RTOL):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim == 2:
        err = np.linalg.norm(a - b, axis=1)
        scale = np.linalg.norm(b, axis=1) + np.linalg.norm(b, axis=1).max()
    else:
        err = np.abs(a - b)
        scale = np.abs(b) + 1e-30
    worst = float(np.max(err / scale))
    return worst <= rtol, worst


def test_grid_bit_exact_initial(gpu, small):
    sc, pos = small
    g, o = pair(sc, pos)
    g.update_grid_distribution()
    cell_g, counts_g, ids_g = g.dump_grid()
    cell_o, counts_o, chains_o = o.cells()          # DistributeByParticle state
    assert np.array_equal(cell_g, cell_o)
    assert np.array_equal(counts_g, counts_o)
    assert np.array_equal(ids_g, chains_o)           # stable sort by (cell, index)
    g.close()


def test_grid_bit_exact_in_motion(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    g.update_grid_distribution()
    cell_g, counts_g, ids_g = g.dump_grid()
    cell_o, counts_o, chains_o = o.cells()
    assert np.array_equal(cell_g, cell_o)
    assert np.array_equal(counts_g, counts_o)
    assert np.array_equal(ids_g, np.lexsort((np.arange(len(p)), cell_o)).astype(np.uint32))
    assert np.array_equal(ids_g, chains_o)
    g.close()


def test_neighbor_sets_match_buckets(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    g.update_grid_distribution()
    g.compute_density(0)
    o.update_grid_distribution()
    counts_o, _, over = o.buckets()
    assert over == 0
    assert np.array_equal(g.neighbor_counts(), counts_o)
    g.close()


def test_density_and_pressure(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    g.update_grid_distribution()
    g.compute_density(1)
    o.update_grid_distribution()
    o.compute_density(1)
    ok, worst = rel_close(g.get(bb.FIELD_DENSITY), o.get(O.DENSITY))
    assert ok, worst
    # EOS pressure (FP32 powf of rho/rho0 ~ 1 to the 7th): same bound relative to rho0 c^2 / gamma
    pg, po = g.get(bb.FIELD_PRESSURE), o.get(O.PRESSURE)
    scale = 1000.0 * 100.0 ** 2 / 7.0
    assert np.max(np.abs(pg - po)) <= 1e-4 * scale
    g.close()


def test_non_pressure_force(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    g.update_grid_distribution()
    g.compute_density(0)
    o.update_grid_distribution()
    o.compute_particle_interaction()
    o.set(O.DENSITY, g.get(bb.FIELD_DENSITY))        # identical input state
    g.compute_non_pressure_force()
    o.compute_non_pressure_force()
    ok, worst = rel_close(g.get(bb.FIELD_FORCE), o.get(O.FORCE))
    assert ok, worst
    g.close()


def test_time_integration_bit_exact(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    rng = np.random.default_rng(5)
    m = g.scalars()["mass"]
    f = (rng.normal(size=p.shape) * 50 * m).astype(np.float32)   # accelerations ~50 m/s^2
    g.update_grid_distribution()
    g.set(bb.FIELD_FORCE, f)
    o.set(O.FORCE, f)
    g.time_integration(sc["dt"])
    o.time_integration(sc["dt"])
    pg, vg = g.download()
    assert np.array_equal(pg, o.get(O.POSITION).astype(np.float32))
    assert np.array_equal(vg, o.get(O.VELOCITY).astype(np.float32))
    g.close()


def test_collider_response_bit_exact(gpu, small):
    # particles driven into the walls and the sphere: push-out, restitution and clamping
    sc, pos = small
    rng = np.random.default_rng(9)
    lo, hi = np.array(sc["domain_min"]), np.array(sc["domain_max"])
    p = rng.uniform(lo - 0.01, hi + 0.01, size=(4000, 3))
    sph = sc["colliders"][1]
    p[:500] = np.array(sph["center"]) + rng.normal(size=(500, 3)) * sph["radius"] * 0.6
    v = rng.normal(size=p.shape) * 2.0
    p32, v32 = p.astype(np.float32), v.astype(np.float32)
    g, o = pair(sc, p32, v32)
    f = np.zeros_like(p32)
    g.update_grid_distribution()
    g.set(bb.FIELD_FORCE, f)
    o.set(O.FORCE, f)
    g.time_integration(1e-3)
    o.time_integration(1e-3)
    pg, vg = g.download()
    assert np.array_equal(pg, o.get(O.POSITION).astype(np.float32))
    assert np.array_equal(vg, o.get(O.VELOCITY).astype(np.float32))
    g.close()


def test_corrector_fixed_iterations(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    dt = sc["dt"]
    g.update_grid_distribution()
    g.compute_density(0)
    o.update_grid_distribution()
    o.compute_particle_interaction()
    o.set(O.DENSITY, g.get(bb.FIELD_DENSITY))
    g.compute_non_pressure_force()
    o.set(O.FORCE, g.get(bb.FIELD_FORCE))
    delta = g.compute_delta(dt)
    assert delta == o.compute_delta(dt)
    x0 = o.get(O.POSITION)
    f_np = o.get(O.FORCE)
    # tolerance 0 never converges: exactly 3 predict-correct passes on both sides
    g.compute_pressure_force_and_integrate(dt, 0.0, delta, 3)
    o.pressure_force_and_integrate(dt, 0.0, delta, 3, O.PCISPH_TOLERANCE)
    ok, worst = rel_close(g.get(bb.FIELD_PRED_DENSITY), o.get(O.PRED_DENSITY))
    assert ok, worst
    # pressure: p = sum_k delta (rho*_k - rho0) inherits the FP32 cancellation of
    # rho* - rho0, so its bound is relative to delta * rho0 per iteration
    pg_, po_ = g.get(bb.FIELD_PRESSURE), o.get(O.PRESSURE)
    assert np.max(np.abs(pg_ - po_)) <= RTOL * 3 * abs(delta) * 1000.0
    # pressure force after 3 iterations: p = sum_k delta (rho*_k - rho0) amplifies FP32
    # rounding of rho* by delta, so the bound is the FP32 envelope of the reference
    # algorithm itself, measured as the FP32-vs-FP64 oracle difference on this input
    # (each sub-pass is held to 1e-5 from identical inputs in test_corrector_sub_passes)
    o64 = O.OracleSim(sc, p, v, variant="f64")
    o64.update_grid_distribution()
    o64.compute_particle_interaction()
    o64.set(O.DENSITY, g.get(bb.FIELD_DENSITY))
    o64.set(O.FORCE, f_np)
    o64.pressure_force_and_integrate(dt, 0.0, delta, 3, O.PCISPH_TOLERANCE)
    scale = pressure_force_scale(o, x0, g.scalars()["mass"], g.scalars()["kernel_radius"])
    env = np.linalg.norm(o.get(O.PRESSURE_FORCE) - o64.get(O.PRESSURE_FORCE), axis=1)
    dfp = np.linalg.norm(g.get(bb.FIELD_PRESSURE_FORCE) - o.get(O.PRESSURE_FORCE), axis=1)
    assert np.all(dfp <= np.maximum(RTOL * scale, 2.0 * env.max())), float(np.max(dfp - 2 * env.max()))
    pg, vg = g.download()
    assert np.max(np.abs(pg - o.get(O.POSITION))) <= RTOL * sc["spacing"]
    assert np.max(np.abs(vg - o.get(O.VELOCITY))) <= RTOL * max(1.0, np.abs(vg).max())
    g.close()


def test_corrector_sub_passes(gpu, moved):
    """PredictVelocityAndPosition, PredictPressure, PredictPressureForce and
    AccumulateAndIntegrate each from identical inputs."""
    sc, p, v = moved
    g, o = pair(sc, p, v)
    dt = sc["dt"]
    g.update_grid_distribution()
    g.compute_density(0)
    o.update_grid_distribution()
    o.compute_particle_interaction()
    o.set(O.DENSITY, g.get(bb.FIELD_DENSITY))
    g.compute_non_pressure_force()
    o.set(O.FORCE, g.get(bb.FIELD_FORCE))
    delta = g.compute_delta(dt)
    # prediction (collider included): bit-exact from identical forces
    g.predict_velocity_and_position(dt, 1)
    o.predict_velocity_and_position(dt, 1)
    assert np.array_equal(g.get(bb.FIELD_PRED_POSITION), o.get(O.PRED_POSITION).astype(np.float32))
    # predicted density and pressure: 1e-5 relative (pressure relative to delta * rho0)
    g.predict_pressure(delta)
    o.predict_pressure(delta)
    ok, worst = rel_close(g.get(bb.FIELD_PRED_DENSITY), o.get(O.PRED_DENSITY))
    assert ok, worst
    assert np.max(np.abs(g.get(bb.FIELD_PRESSURE) - o.get(O.PRESSURE))) <= RTOL * abs(delta) * 1000.0
    # pressure force from identical pressure and predicted density
    o.set(O.PRESSURE, g.get(bb.FIELD_PRESSURE))
    o.set(O.PRED_DENSITY, g.get(bb.FIELD_PRED_DENSITY))
    g.predict_pressure_force()
    o.predict_pressure_force()
    x0 = o.get(O.POSITION)
    scale = pressure_force_scale(o, x0, g.scalars()["mass"], g.scalars()["kernel_radius"])
    dfp = np.linalg.norm(g.get(bb.FIELD_PRESSURE_FORCE) - o.get(O.PRESSURE_FORCE), axis=1)
    assert np.all(dfp <= RTOL * scale)
    # second prediction uses F + Fp: bit-exact from identical F and Fp
    o.set(O.PRESSURE_FORCE, g.get(bb.FIELD_PRESSURE_FORCE))
    g.predict_velocity_and_position(dt, 0)
    o.predict_velocity_and_position(dt, 0)
    assert np.array_equal(g.get(bb.FIELD_PRED_POSITION), o.get(O.PRED_POSITION).astype(np.float32))
    # accumulate + integrate: bit-exact
    g.accumulate_and_integrate(dt)
    o.accumulate_and_integrate(dt)
    pg, vg = g.download()
    assert np.array_equal(pg, o.get(O.POSITION).astype(np.float32))
    assert np.array_equal(vg, o.get(O.VELOCITY).astype(np.float32))
    g.close()


@pytest.mark.parametrize("mode", ["tolerance", "as_shipped"])
def test_full_substep(gpu, moved, mode):
    sc, p, v = moved
    sc = dict(sc, pcisph_mode=mode)
    g, o = pair(sc, p, v)
    om = O.PCISPH_TOLERANCE if mode == "tolerance" else O.PCISPH_AS_SHIPPED
    st = g.advance_time_step(sc["dt"], stats=True)
    it_o, err_o = o.pcisph_substep(sc["dt"], 0.01, sc["max_iterations"], om)
    assert st["iterations"] == it_o
    if mode == "tolerance":
        assert abs(st["max_density_error_ratio"] - err_o) <= 1e-4
    pg, vg = g.download()
    assert np.max(np.abs(pg - o.get(O.POSITION))) <= RTOL * sc["spacing"]
    ok, worst = rel_close(g.get(bb.FIELD_DENSITY), o.get(O.DENSITY))
    assert ok, worst
    g.close()


@pytest.mark.parametrize("rule,scale,mode", [("clamp_total", 1.0, O.PCISPH_WARM),
                                              ("monotone", 0.5, O.PCISPH_WARM_MONOTONE)])
def test_warm_started_substeps_match_oracle(gpu, moved, rule, scale, mode):
    """Corrector started from (a multiple of) the previous substep's pressure: each
    substep, from the GPU's own state (positions, velocities and the carried pressure),
    matches the oracle run the same way; the warm start never needs more iterations than
    the zero start."""
    sc, p, v = moved
    scw = dict(sc, pressure_init="previous", warm_rule=rule, warm_scale=scale)
    g = bb.Solver(scw, pos=p, vel=v)
    gz = bb.Solver(sc, pos=p, vel=v)
    its_w, its_z = [], []
    for _ in range(6):
        pg, vg = g.download()
        o = O.OracleSim(scw, pg, vg, variant="f32")
        if its_w:
            o.set(O.PRESSURE, np.float32(scale) * g.get(bb.FIELD_PRESSURE))
        st = g.advance_time_step(sc["dt"], stats=True)
        it_o, _ = o.pcisph_substep(sc["dt"], 0.01, sc["max_iterations"], mode)
        assert st["iterations"] == it_o
        assert st["max_density_error_ratio"] < 0.01
        pg2, _ = g.download()
        assert np.max(np.abs(pg2 - o.get(O.POSITION))) <= RTOL * sc["spacing"]
        its_w.append(st["iterations"])
        its_z.append(gz.advance_time_step(sc["dt"], stats=True)["iterations"])
        o.close()
    assert sum(its_w) <= sum(its_z)
    g.close()
    gz.close()


def test_cfl_substep_count(gpu, moved):
    sc, p, v = moved
    g, o = pair(sc, p, v)
    g.advance_time_step(sc["dt"])
    o.pcisph_substep(sc["dt"], 0.01, sc["max_iterations"], O.PCISPH_TOLERANCE)
    o.set(O.FORCE, g.get(bb.FIELD_FORCE))
    for dt in (1e-3, 5e-3, 2e-2):
        assert g.compute_number_of_time_steps(dt, 5.0) == o.number_of_time_steps(dt, 5.0)
    g.close()


def test_advance_matches_oracle_substeps(gpu, small):
    sc, pos = small
    g, o = pair(sc, pos)
    st = g.advance(2e-3)
    steps, iters = o.advance_pcisph(2e-3, 0.01, sc["max_iterations"], O.PCISPH_TOLERANCE)
    assert st["substeps"] == steps
    pg, _ = g.download()
    assert np.max(np.abs(pg - o.get(O.POSITION))) <= 1e-3 * sc["spacing"]
    g.close()


def test_sph_jacobi_substep(gpu):
    sc, pos = scenes.sph_16k(seed=2)
    g, o = pair(sc, pos)
    for _ in range(5):    # let the block start moving on the GPU
        g.advance_time_step(sc["dt"] / 7)
    p, v = g.download()
    g.close()
    g, o = pair(sc, p, v)
    g.update_grid_distribution()
    g.compute_density(1)
    o.update_grid_distribution()
    o.compute_particle_interaction()
    o.compute_density(1)
    ok, worst = rel_close(g.get(bb.FIELD_DENSITY), o.get(O.DENSITY))
    assert ok, worst
    o.set(O.DENSITY, g.get(bb.FIELD_DENSITY))
    o.set(O.PRESSURE, g.get(bb.FIELD_PRESSURE))
    g.compute_pressure_force(sc["dt"] / 7)
    o.sph_all_forces(sc["dt"] / 7, inplace=0)
    ok, worst = rel_close(g.get(bb.FIELD_FORCE), o.get(O.FORCE))
    assert ok, worst
    pg, _ = g.download()
    assert np.max(np.abs(pg - o.get(O.POSITION))) <= RTOL * sc["spacing"]
    g.close()


def test_graph_and_direct_launches_agree_bitwise(gpu, moved):
    sc, p, v = moved
    outs = []
    for graphs in (True, False):
        with bb.Solver(sc, pos=p, vel=v) as g:
            g.use_cuda_graphs(graphs)
            its = [g.advance_time_step(sc["dt"], stats=True)["iterations"] for _ in range(6)]
            outs.append((g.download(), its, g.get(bb.FIELD_PRESSURE)))
    (pa, va), ia, pra = outs[0]
    (pb, vb), ib, prb = outs[1]
    assert ia == ib
    assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(pra, prb)


def test_deterministic_bitwise(gpu, small):
    sc, pos = small
    outs = []
    for _ in range(2):
        with bb.Solver(sc, pos=pos) as g:
            for _ in range(10):
                g.advance_time_step(sc["dt"])
            outs.append(g.download())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_drift_against_fp64_reported(gpu, small):
    # reported, not gated beyond sanity: FP32 GPU vs FP64 oracle after 20 substeps
    sc, pos = small
    g, o = pair(sc, pos, variant="f64")
    for _ in range(20):
        g.advance_time_step(sc["dt"])
        o.pcisph_substep(sc["dt"], 0.01, sc["max_iterations"], O.PCISPH_TOLERANCE)
    pg, _ = g.download()
    drift = float(np.max(np.abs(pg - o.get(O.POSITION))))
    print("max position drift vs FP64 after 20 substeps: %.3e (spacing %.3g)" % (drift, sc["spacing"]))
    assert drift < 0.1 * sc["spacing"]
    g.close()


def test_empty_and_tiny_inputs(gpu, small):
    sc, pos = small
    with pytest.raises((bb.BbgError, ValueError)):
        bb.Solver(sc, pos=np.zeros((0, 3)))
    # a single particle: no neighbours but itself, falls under gravity
    one = np.array([[0.0, 0.0, 0.2]])
    with bb.Solver(sc, pos=one) as g:
        st = g.advance_time_step(sc["dt"], stats=True)
        p, v = g.download()
        assert v[0, 1] < 0 and st["out_of_grid"] == 0


def test_capacity_and_state_errors(gpu, small):
    sc, pos = small
    g = bb.Solver(sc, capacity=10)
    with pytest.raises(bb.BbgError) as e:
        g.upload(pos)
    assert e.value.status == 4
    g.upload(pos[:10])
    with pytest.raises(bb.BbgError) as e:     # no setup yet
        g.advance_time_step(1e-4)
    assert e.value.status == 5
    g.setup()
    with pytest.raises(bb.BbgError) as e:     # density needs a grid
        g.compute_density(1)
    assert e.value.status == 5
    g.close()


def test_out_of_grid_particles_are_clamped_and_counted(gpu, small):
    sc, pos = small
    p = pos.copy()
    p[0] = [5.0, 5.0, 5.0]   # far outside the domain
    with bb.Solver(sc, pos=p) as g:
        st = g.advance_time_step(sc["dt"], stats=True)
        assert st["out_of_grid"] == 1
        q, _ = g.download()
        assert np.all(np.isfinite(q))


def test_full_size_invariants_1m(gpu):
    sc, pos = scenes.pcisph_1m(seed=0)
    n = len(pos)
    with bb.Solver(sc, pos=pos) as g:
        for _ in range(3):
            st = g.advance_time_step(sc["dt"], stats=True)
        assert st["out_of_grid"] == 0 and st["neighbor_overflow"] == 0
        p, v = g.download()
        assert np.all(np.isfinite(p)) and np.all(np.isfinite(v))
        g.update_grid_distribution()
        cell, counts, ids = g.dump_grid()
        assert counts.sum() == n
        assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))   # a permutation
        sc_cells = cell[ids]
        assert np.all(np.diff(sc_cells.astype(np.int64)) >= 0)             # sorted by cell
        same = np.diff(sc_cells.astype(np.int64)) == 0
        assert np.all(np.diff(ids.astype(np.int64))[same] > 0)             # stable inside cells
        o = O.OracleSim(sc, np.zeros((1, 3)), variant="f32")
        want, _ = o.hash_points(p.astype(np.float64))                      # exact reference hash
        assert np.array_equal(cell, want)
        o.close()
        g.compute_density(0)
        rho = g.get(bb.FIELD_DENSITY)
        assert 300 < np.median(rho) < 1100


def _golden(name):
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name)
    d = np.load(path, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["scene"]))


def test_gpu_against_reference_fixtures(gpu):
    """The CUDA path on the reference's own inputs and outputs (tests/golden, produced by
    the reference's CPU path built with Float = float; FP64 gives the rounding envelope)."""
    g32, sc = _golden("pcisph_f32.npz")
    g64, _ = _golden("pcisph_f64.npz")
    dt, h0 = sc["dt"], sc["spacing"]
    shipped = dict(sc, pcisph_mode="as_shipped")
    with bb.Solver(shipped, pos=g32["pos0"]) as g:
        g.update_grid_distribution()
        cell, counts, ids = g.dump_grid()
        assert np.array_equal(cell, g32["setup_cell_of"])
        assert np.array_equal(counts, g32["setup_counts"])
        assert np.array_equal(ids, g32["setup_chains"])
        for _ in range(3):
            g.advance_time_step(dt)
        p, v = g.download()
        assert np.max(np.abs(p - g32["step3_pos"])) <= RTOL * h0
        assert np.max(np.abs(v - g32["step3_vel"])) <= RTOL * max(1.0, np.abs(g32["step3_vel"]).max())
        ok, worst = rel_close(g.get(bb.FIELD_DENSITY), g32["step3_density"])
        assert ok, worst
    # corrector from the reference's state after those substeps
    with bb.Solver(sc, pos=g32["step3_pos"], vel=g32["step3_vel"]) as g:
        g.update_grid_distribution()
        g.compute_density(1)
        g.compute_non_pressure_force()
        delta = g.compute_delta(dt)
        assert delta == float(g32["corr_delta"])
        for k in range(3):
            g.predict_velocity_and_position(dt, int(k == 0))
            g.predict_pressure(delta)
            g.predict_pressure_force()
        ok, worst = rel_close(g.get(bb.FIELD_PRED_DENSITY), g32["corr_pred_density"])
        assert ok, worst
        assert np.max(np.abs(g.get(bb.FIELD_PRESSURE) - g32["corr_pressure"])) <= RTOL * 3 * abs(delta) * 1000.0
        env = np.linalg.norm(g32["corr_pressure_force"] - g64["corr_pressure_force"], axis=1).max()
        dfp = np.linalg.norm(g.get(bb.FIELD_PRESSURE_FORCE) - g32["corr_pressure_force"], axis=1)
        assert np.all(dfp <= 2.0 * env + RTOL * np.linalg.norm(g32["corr_pressure_force"], axis=1))
        g.accumulate_and_integrate(dt)
        p, v = g.download()
        assert np.max(np.abs(p - g32["corr_pos"])) <= RTOL * h0


@pytest.mark.parametrize("tuning", [dict(block_size=64, batch_np=2, batch_pd=8, batch_pf=2, prune=0,
                                         particles_per_thread=2, tile_order=1, batch_worklist=0),
                                    dict(block_size=256, batch_np=8, batch_pd=2, batch_pf=8, prune=1,
                                         particles_per_thread=1, tile_order=1, batch_worklist=2)])
def test_launch_tuning_does_not_change_results(gpu, moved, tuning):
    """Block size, gather batches, the density pass's reach test and particles per thread
    change the launch shape, not the arithmetic: the substeps are bitwise identical to the
    default tuning."""
    sc, p, v = moved
    ga = bb.Solver(sc, pos=p, vel=v)
    gb = bb.Solver(sc, pos=p, vel=v)
    gb.set_tuning(**tuning)
    assert gb.tuning() == tuning
    for _ in range(3):
        sa = ga.advance_time_step(sc["dt"], stats=True)
        sb = gb.advance_time_step(sc["dt"], stats=True)
        assert sa["iterations"] == sb["iterations"]
    pa, va = ga.download()
    pb, vb = gb.download()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    with pytest.raises(bb.BbgError):
        gb.set_tuning(block_size=96)
    ga.close()
    gb.close()


def test_degenerate_pileup_is_bounded_and_reported(gpu, small):
    """Particles piled into one point (a blown-up state): the per-cell rank and the
    candidate search stay within their work caps, the substep ends and reports it."""
    import time
    sc, _ = small
    pos = np.tile(np.array([[0.0, -0.1, 0.0]]), (3000, 1))
    g = bb.Solver(sc, pos=pos)
    t0 = time.time()
    st = g.advance_time_step(sc["dt"], stats=True)
    assert time.time() - t0 < 60
    assert st["crowded"] > 0
    p, _ = g.download()
    assert np.all(np.isfinite(p))
    g.close()
