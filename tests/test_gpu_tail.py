"""Learned null-tail surrogate: the MLP kernels against the FP64 oracle, BF16
inference, training, and what the trained network gains over the classical
GPD fit of the same small null sample.

Gradient bar: relative (Frobenius) error <= 1e-4 per parameter tensor (FP32
kernels vs FP64 numpy); BF16 inference: relative error <= 3e-2.
"""
import os

import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30)


def test_mlp_forward_backward_vs_fp64_oracle():
    import torch
    from tfce_mediation_gb300.tail.mlp import MLP
    rng = np.random.default_rng(0)
    model = MLP((21, 128, 128, 128, 3), seed=3)
    X = rng.standard_normal((200, 21)).astype(np.float32)
    T = rng.standard_normal((200, 3)).astype(np.float32)
    w = np.array([1.0, 0.5, 2.0], np.float32)
    y = model.forward(torch.from_numpy(X).cuda())
    loss, dy = model.loss(y, torch.from_numpy(T).cuda(), w)
    grads = model.backward(dy)
    Ws = [W.cpu().numpy() for W in model.W]
    bs = [b.cpu().numpy() for b in model.b]
    l_ref, gW, gb, y_ref = mlp_oracle.loss_and_grads(Ws, bs, X, T, w)
    assert _rel(y.cpu().numpy(), y_ref) <= 1e-5
    assert abs(loss.item() - l_ref) <= 1e-5 * abs(l_ref)
    for i in range(4):
        assert _rel(grads[i].cpu().numpy(), gW[i]) <= 1e-4, ("W", i)
        assert _rel(grads[4 + i].cpu().numpy(), gb[i]) <= 1e-4, ("b", i)


def test_bf16_inference_close_to_fp32():
    from tfce_mediation_gb300.tail.mlp import MLP
    rng = np.random.default_rng(1)
    model = MLP((21, 128, 128, 128, 3), seed=4)
    X = rng.standard_normal((64, 21)).astype(np.float32)
    assert _rel(model.predict_bf16(X), model.predict(X)) <= 3e-2


def test_training_reduces_loss():
    from tfce_mediation_gb300.tail.mlp import MLP
    rng = np.random.default_rng(2)
    X = rng.standard_normal((512, 8)).astype(np.float32)
    Y = np.stack([np.sin(X[:, 0]) + X[:, 1] * X[:, 2], np.tanh(X[:, 3]), X[:, 4] ** 2 - 1], axis=1)
    model = MLP((8, 128, 128, 128, 3), seed=5)
    curve = model.fit(X, Y.astype(np.float32), epochs=150, batch=128, lr=2e-3)
    assert curve[-1] < 0.1 * curve[0], (curve[0], curve[-1])


def test_adam_step_matches_reference_formula():
    import torch
    from tfce_mediation_gb300 import _lib
    from tfce_mediation_gb300.device import ptr
    lib = _lib.load()
    rng = np.random.default_rng(3)
    p0 = rng.standard_normal(1000).astype(np.float32)
    g = rng.standard_normal(1000).astype(np.float32)
    p, gd = torch.from_numpy(p0.copy()).cuda(), torch.from_numpy(g).cuda()
    m, v = torch.zeros_like(p), torch.zeros_like(p)
    for step in (1, 2):
        _lib.check(lib.mlp_adam_step(ptr(p), ptr(gd), ptr(m), ptr(v), 1000, 1e-2, 0.9, 0.999, 1e-8, step, 0.0, None))
    mr, vr, pr = np.zeros(1000), np.zeros(1000), p0.astype(np.float64)
    for step in (1, 2):
        mr = 0.9 * mr + 0.1 * g
        vr = 0.999 * vr + 0.001 * g * g
        pr = pr - 1e-2 * (mr / (1 - 0.9 ** step)) / (np.sqrt(vr / (1 - 0.999 ** step)) + 1e-8)
    np.testing.assert_allclose(p.cpu().numpy(), pr, rtol=1e-5, atol=1e-6)


WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tfce_mediation_gb300",
                       "tail", "weights.npz")


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights")
def test_trained_network_gains_over_classical_fit():
    """Held-out settings (seeds outside training): tail p-value error of the
    network's GPD vs the maximum-likelihood GPD fit of the same 300
    permutations, against each setting's 1500-permutation null."""
    from tfce_mediation_gb300.tail import data, gpd
    from tfce_mediation_gb300.tail.surrogate import TailSurrogate
    sur = TailSurrogate()
    settings = data.sample_settings(8, seed=987, levels=(5, 6), level_p=(0.6, 0.4))
    err_mlp, err_gpd = [], []
    for s in settings:
        null, rho, V = data.null_for_setting(s, 1500)
        sub = null[:600]
        qs = np.quantile(null, 1 - np.linspace(0.002, 0.05, 25))
        ref = gpd.one_minus_p(qs, null)
        u, xi, sg = sur.tail(sub, V, rho, s["E"], s["n"], s["k"])
        err_mlp.append(np.abs(gpd.one_minus_p(qs, sub, u, xi, sg) - ref).max())
        u0, xi0, s0 = gpd.tail_params(sub)
        err_gpd.append(np.abs(gpd.one_minus_p(qs, sub, u0, xi0, s0) - ref).max())
    assert np.mean(err_mlp) < np.mean(err_gpd), (np.mean(err_mlp), np.mean(err_gpd))
