"""Learned warm start: the tensor-core MLP inference and the training kernels against
an FP32 reference (tests/mlp_ref.py), the per-particle features against direct
restatements, and a learned substep against the oracle started from the same pressure."""
import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes
from oracle import oracle as O

from mlp_ref import N_PARAMS, forward_bf16, loss_and_grad

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    th = rng.uniform(-0.3, 0.3, N_PARAMS).astype(np.float32) * scale
    return th


def learned_solver(sc, p, v=None, **mlp):
    return bb.Solver(dict(sc, pressure_init="learned", mlp=mlp), pos=p, vel=v)


def test_mlp_inference_matches_reference(gpu, small):
    sc, p = small
    g = learned_solver(sc, p)
    rng = np.random.default_rng(1)
    for seed in (0, 1):
        th = random_params(seed)
        g.mlp_set_params(th)
        feats = rng.normal(0.0, 2.0, (1000, 4)).astype(np.float32)
        got = g.mlp_infer(feats)
        want = forward_bf16(th, feats)
        # BF16 GELU arithmetic with the hardware tanh approximation and FP32 accumulation in
        # another order: a few 1e-2 of the output scale at worst, 5e-3 on average
        scale = max(1.0, float(np.abs(want).max()))
        assert np.max(np.abs(got - want)) <= 3e-2 * scale
        assert np.mean(np.abs(got - want)) <= 5e-3 * scale
    # ragged count (not a multiple of the 16-particle MMA tile)
    got = g.mlp_infer(feats[:37])
    assert np.allclose(got, forward_bf16(th, feats[:37]), atol=3e-2 * scale)
    g.close()


def test_mlp_params_round_trip(gpu, small):
    sc, p = small
    g = learned_solver(sc, p)
    th = random_params(7)
    g.mlp_set_params(th)
    assert np.array_equal(g.mlp_params(), th)
    g.close()


@pytest.mark.parametrize("expectile,batch", [(0.5, 1000), (0.3, 1000), (0.5, 40000)])
def test_mlp_gradient_matches_autograd(gpu, small, expectile, batch):
    """With Adam's epsilon far above |g| one step moves theta by -lr * g / eps, which
    exposes the gradient of the training kernel (plain and expectile-weighted loss; a
    batch of 40,000 makes each of the 128 training blocks sum several 128-sample tiles)."""
    sc, p = small
    mlp = dict(learning_rate=1.0, epsilon=1e3, beta1=0.0, beta2=0.0, expectile=expectile)
    g = bb.Solver(dict(sc, pressure_init="learned", mlp=mlp), pos=p, capacity=max(len(p), batch))
    th = random_params(3, 0.5)
    g.mlp_set_params(th)
    rng = np.random.default_rng(2)
    x = rng.normal(0.0, 1.0, (batch, 4)).astype(np.float32)
    t = rng.normal(0.0, 1.0, batch).astype(np.float32)
    g.mlp_train_batch(x, t)
    moved = (th.astype(np.float64) - g.mlp_params()) * 1e3   # = g / (1 + |g| / eps)
    loss, grad = loss_and_grad(th, x, t, expectile)
    want = grad / (1.0 + np.abs(grad) / 1e3)
    assert np.max(np.abs(moved - want)) <= 1e-4 * max(1.0, np.abs(want).max())
    st = g.mlp_status()
    assert st["adam_steps"] == 1
    assert abs(st["last_loss"] - loss) <= 1e-4 * loss
    g.close()


def test_mlp_training_reduces_loss(gpu, small):
    sc, p = small
    g = learned_solver(sc, p, learning_rate=3e-3)
    rng = np.random.default_rng(5)
    x = rng.normal(0.0, 1.0, (1536, 4)).astype(np.float32)   # within the 1,440-particle staging
    t = (np.tanh(x[:, 0]) + 0.5 * x[:, 3]).astype(np.float32)
    losses = []
    for _ in range(200):
        g.mlp_train_batch(x, t)
        losses.append(g.mlp_status()["last_loss"])
    assert losses[-1] < 0.1 * losses[0]
    g.close()


def test_mlp_training_is_deterministic(gpu, small):
    """Gradients and losses are summed in a fixed order: two solvers trained on the same
    batches hold bit-identical weights, moments and losses."""
    sc, p = small
    rng = np.random.default_rng(9)
    x = rng.normal(0.0, 1.0, (30000, 4)).astype(np.float32)
    t = (np.tanh(x[:, 0]) + 0.5 * x[:, 3]).astype(np.float32)
    out = []
    for _ in range(2):
        g = bb.Solver(dict(sc, pressure_init="learned", mlp=dict(learning_rate=3e-3)), pos=p, capacity=30000)
        for _ in range(5):
            g.mlp_train_batch(x, t)
        out.append((g.mlp_params(), g.mlp_status()["last_loss"]))
        g.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]


def test_features_match_definitions(gpu, moved):
    """Features of a substep: density error and neighbour count of its start state, the
    previous substep's pressure, and the velocity divergence of the previous substep's
    start state (carried, so the warm start can precede the force pass)."""
    sc, p, v = moved
    g = learned_solver(sc, p, v, train_substeps=1000)
    g.advance_time_step(sc["dt"])
    f0 = g.mlp_features()
    assert np.all(f0[:, 1] == 0.0)   # nothing carried across an upload
    assert np.all(f0[:, 3] == 0.0)
    p1, v1 = g.download()
    pr1 = g.get(bb.FIELD_PRESSURE)
    div1 = g.get(bb.FIELD_DIVERGENCE)   # computed by the first substep at (p, v)
    g.advance_time_step(sc["dt"])
    f = g.mlp_features()
    o = O.OracleSim(sc, p1, v1, variant="f64")
    o.update_grid_distribution()
    o.compute_density(0)
    rho = o.get(O.DENSITY)
    assert np.max(np.abs(f[:, 0] - 100.0 * (rho / 1000.0 - 1.0))) <= 1e-3
    counts = g.neighbor_counts()
    assert np.array_equal(f[:, 2], ((counts - 1) / 32.0).astype(np.float32))
    delta = o.compute_delta(sc["dt"])
    p_unit = np.float32(delta) * np.float32(1000.0) * np.float32(0.01)
    assert np.allclose(f[:, 3], pr1 / p_unit, rtol=1e-5, atol=1e-6)
    # velocity divergence of (p, v): brute force over the step-start neighbour sets
    h = 2.0 * sc["spacing"]
    o0 = O.OracleSim(sc, p, v, variant="f64")
    o0.update_grid_distribution()
    o0.compute_density(0)
    rho0 = o0.get(O.DENSITY)
    d = p[:, None, :] - p[None, :, :]
    r = np.sqrt((d ** 2).sum(-1))
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where((r < h) & (r > 0), (1.0 - r / h) ** 2 / r, 0.0)
    dv = ((v[None, :, :] - v[:, None, :]) * (-d)).sum(-1)
    divsum = (w * dv / rho0[None, :]).sum(1)
    assert np.max(np.abs(div1 - divsum)) <= 1e-3 * max(1.0, np.abs(divsum).max())
    m = sc["mass"]
    want = -100.0 * sc["dt"] * m * 45.0 / (np.pi * h ** 4) * divsum
    assert np.max(np.abs(f[:, 1] - want)) <= 1e-3 * max(1.0, np.abs(want).max())
    g.close()


def test_learned_substep_matches_oracle(gpu, moved):
    """A learned substep (after its training phase) against the oracle started from the
    same pressure with the warm-start corrector."""
    sc, p, v = moved
    scl = dict(sc, warm_rule="monotone", warm_scale=0.5)
    g = learned_solver(scl, p, v, train_substeps=3, batch=1024)
    for _ in range(3):
        g.advance_time_step(sc["dt"])
    assert g.mlp_status()["trained_substeps"] == 3
    pg, vg = g.download()
    pprev = g.get(bb.FIELD_PRESSURE)
    st = g.advance_time_step(sc["dt"], stats=True)
    feats = g.mlp_features()
    raw = g.mlp_infer(feats)
    o = O.OracleSim(dict(scl, pressure_init="previous"), pg, vg, variant="f32")
    o.update_grid_distribution()
    o.compute_density(0)
    delta = o.compute_delta(sc["dt"])
    p_unit = np.float32(delta) * np.float32(1000.0) * np.float32(0.01)
    start = np.float32(0.5) * p_unit * np.maximum(raw, 0).astype(np.float32)
    assert np.allclose(feats[:, 3], pprev / p_unit, rtol=1e-5, atol=1e-6)
    o2 = O.OracleSim(dict(scl, pressure_init="previous"), pg, vg, variant="f32")
    o2.set(O.PRESSURE, start)
    it_o, err_o = o2.pcisph_substep(sc["dt"], 0.01, sc["max_iterations"], O.PCISPH_WARM_MONOTONE)
    assert st["iterations"] == it_o
    assert st["max_density_error_ratio"] < 0.01
    pg2, _ = g.download()
    assert np.max(np.abs(pg2 - o2.get(O.POSITION))) <= RTOL * sc["spacing"]
    g.close()
