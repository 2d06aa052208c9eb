"""Learned warm start: GPU MLP gradients against the float64 CPU oracle, training
on GPU, and the burn-in gain of warm-started chains over cold-started ones."""
import numpy as np
import pytest

import mlp_oracle

pytestmark = pytest.mark.gpu


def test_mlp_gradients_match_cpu_oracle():
    from suqa_gb300.warmstart import WarmStartNet
    net = WarmStartNet(hidden=128, layers=3, seed=3)
    rng = np.random.default_rng(0)
    B = 64
    x = rng.uniform(0.2, 2.0, size=(B, 4)).astype(np.float32)
    t = rng.uniform(-1.5, 1.5, size=(B, 12)).astype(np.float32)
    m = (rng.random((B, 12)) < 0.8).astype(np.float32)
    g, loss = net.gradients(x, t, m)
    _, wloss, wg = mlp_oracle.forward_backward(net.params(), net.dims, x.astype(np.float64), t.astype(np.float64), m)
    rel = np.linalg.norm(g - wg) / np.linalg.norm(wg)
    cos = float(np.dot(g, wg) / (np.linalg.norm(g) * np.linalg.norm(wg)))
    assert abs(loss - wloss) <= 1e-3 * max(1.0, wloss)
    # BF16 activations: an FP32 and a float64 sum can round a hidden unit to
    # neighbouring BF16 values, so gradients agree to BF16 level, not FP32
    assert rel < 2e-2 and cos > 0.9995, (rel, cos)
    y = net.forward(x)
    wy, _, _ = mlp_oracle.forward_backward(net.params(), net.dims, x.astype(np.float64), t.astype(np.float64), m)
    assert np.max(np.abs(y - wy)) < 2e-2 * max(1.0, np.max(np.abs(wy)))


def test_training_reduces_loss():
    from suqa_gb300.warmstart import WarmStartNet
    net = WarmStartNet(seed=5)
    rng = np.random.default_rng(1)
    x = rng.uniform(0.2, 2.0, size=(512, 4)).astype(np.float32)
    target = np.tile((np.sin(x[:, 2:3]) * 0.8 - 0.3 * x[:, 3:4]), (1, 12)).astype(np.float32)
    mask = np.ones_like(target)
    losses = net.fit(x, target, mask, iters=400, batch=128, lr=2e-3)
    assert np.mean(losses[-20:]) < 0.1 * np.mean(losses[:20])


def test_energy_target_warm_start_lowers_first_sample_error():
    """With product-state energy targets, chains started from the trained
    network's product state are closer to the equilibrium energy in their first
    steps than cold-started chains (their later burn-in is not shorter: these
    chains keep memory of their start)."""
    from suqa_gb300.warmstart import burn_in_experiment
    res = burn_in_experiment()
    print(res)
    assert res["loss_last"] < res["loss_first"]
    cold = np.mean([g["cold_first_err"] for g in res["groups"]])
    warm = np.mean([g["warm_first_err"] for g in res["groups"]])
    assert warm < cold, (warm, cold)

