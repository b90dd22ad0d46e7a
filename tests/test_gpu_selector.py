"""The selector's CUDA kernels against the FP64 network oracle, training on
the GPU, and the committed model on held-out configurations.

Bars: forward outputs to 2e-5 relative (FP32 against FP64), loss and
gradient to 1e-4 relative per block of the parameter vector, an Adam step to
1e-6; the selected parameters (after the sampled FP64 check and its
fallback) meet the tolerance, and the selector is faster in total than the
drivers' analytic FP64 choice.
"""
import os

import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _sel():
    from fasttools2d_gb300 import selector

    return selector


def _data(seed, n):
    rng = np.random.default_rng(seed)
    p = (mlp_ref.init(seed) + 0.05 * rng.standard_normal(mlp_ref.NPARAMS)).astype(np.float32)
    X = rng.standard_normal((n, 8)).astype(np.float32)
    T = rng.standard_normal((n, 4)).astype(np.float32)
    w = (rng.random(n) + 0.5).astype(np.float32)
    return p, X, T, w


@pytest.mark.parametrize("n", [1, 37, 1000])
def test_forward_matches_oracle(gpu_ctx, n):
    sel = _sel()
    p, X, _, _ = _data(n, n)
    y = sel.mlp_forward(p, X)
    ref = mlp_ref.forward(p.astype(np.float64), X.astype(np.float64))
    assert np.max(np.abs(y - ref)) <= 2e-5 * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("n,weighted", [(5, False), (300, True), (2000, True)])
def test_loss_gradient_matches_oracle(gpu_ctx, n, weighted):
    sel = _sel()
    p, X, T, w = _data(100 + n, n)
    loss, g = sel.mlp_loss_grad(p, X, T, w if weighted else None)
    rl, rg = mlp_ref.loss_grad(p.astype(np.float64), X.astype(np.float64), T.astype(np.float64),
                               w.astype(np.float64) if weighted else None)
    assert abs(loss - rl) <= 1e-5 * abs(rl)
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in mlp_ref.SHAPES])
    for (name, _), a, b in zip(mlp_ref.SHAPES, offs[:-1], offs[1:]):
        err = np.max(np.abs(g[a:b] - rg[a:b])) / max(np.max(np.abs(rg[a:b])), 1e-30)
        assert err <= 1e-4, (name, err)


def test_adam_step_matches_oracle(gpu_ctx):
    import ctypes as C

    import torch

    sel = _sel()
    from fasttools2d_gb300 import _check, lib

    rng = np.random.default_rng(7)
    P = mlp_ref.NPARAMS
    p, g = rng.standard_normal(P), rng.standard_normal(P)
    m, v = 0.1 * rng.standard_normal(P), rng.random(P)
    t = [torch.tensor(a.astype(np.float32), device="cuda") for a in (p, g, m, v)]
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _check(lib().fte_mlp_adam(sel._ptr(t[0]), sel._ptr(t[1]), sel._ptr(t[2]), sel._ptr(t[3]), 3, 1e-3, 0.9, 0.999,
                              1e-8, st))
    rp, rm, rv = mlp_ref.adam(p.astype(np.float32).astype(np.float64), g.astype(np.float32).astype(np.float64),
                              m.astype(np.float32).astype(np.float64), v.astype(np.float32).astype(np.float64), 3)
    assert np.max(np.abs(t[0].cpu().numpy() - rp)) <= 1e-6
    assert np.max(np.abs(t[2].cpu().numpy() - rm)) <= 1e-6
    assert np.max(np.abs(t[3].cpu().numpy() - rv)) <= 1e-6


@pytest.mark.parametrize("layout", ["uniform", "clustered", "narrow"])
def test_nn_sample_matches_brute_force(gpu_ctx, layout):
    """fte_nn_sample (device cell list, ring search) against a brute-force
    minimum-image search of the same sampled sources."""
    import fasttools2d_gb300 as ft

    rng = np.random.default_rng(7)
    n, Lx, Ly = 30000, 1.0, 1.0
    if layout == "uniform":
        x, y = rng.random(n) - 0.5, rng.random(n) - 0.5
    elif layout == "clustered":
        c = rng.integers(0, 5, n)
        x = (rng.random(5) - 0.5)[c] + 0.01 * rng.standard_normal(n)
        y = (rng.random(5) - 0.5)[c] + 0.01 * rng.standard_normal(n)
    else:
        n, Lx, Ly = 4000, 7.3, 0.05
        x, y = (rng.random(n) - 0.5) * Lx, (rng.random(n) - 0.5) * Ly
    d = ft.nn_sample(x, y, Lx, Ly, nsample=500, ctx=gpu_ctx)
    stride = max(1, n // 500)
    idx = np.arange(0, n, stride)[:len(d)]
    wx = np.mod(x + Lx / 2, Lx) - Lx / 2
    wy = np.mod(y + Ly / 2, Ly) - Ly / 2
    dx = wx[idx, None] - wx[None, :]
    dy = wy[idx, None] - wy[None, :]
    dx -= Lx * np.round(dx / Lx)
    dy -= Ly * np.round(dy / Ly)
    dd = np.hypot(dx, dy)
    dd[np.arange(len(idx)), idx] = np.inf
    ref = dd.min(1)
    assert len(d) == len(idx) == 500
    assert np.allclose(d, ref, rtol=1e-12, atol=1e-15)


def test_training_fits_a_smooth_map(gpu_ctx):
    sel = _sel()
    rng = np.random.default_rng(11)
    X = rng.uniform(-1, 1, (1500, 8))
    Y = np.stack([np.sin(X[:, 0]) + X[:, 1] ** 2, X[:, 2] * X[:, 3], np.tanh(X[:, 4] - X[:, 5]), X[:, 6] + X[:, 7]], 1)
    res = sel.train(X, Y, steps=1500, lr=3e-3, seed=1)
    xn = (X - res["xmean"]) / res["xstd"]
    pred = sel.mlp_forward(res["params"], xn) * res["yscale"]
    rms = np.sqrt(np.mean((pred - Y) ** 2, 0)) / np.std(Y, 0)
    assert np.all(rms < 0.15), rms
    h = res["history"]
    assert h[-1, 1] < 0.1 * h[0, 1]


def test_committed_selector_meets_tolerance_and_beats_analytic(gpu_ctx):
    sel = _sel()
    if not os.path.exists(sel.MODEL_PATH):
        pytest.skip("no trained selector model in this checkout")
    s = sel.Selector(ctx=gpu_ctx)
    gpu_ctx.set_timing(True)
    rng = np.random.default_rng(2024)
    cfgs = [sel.random_config(rng, nmin=2e4, nmax=1e5) for _ in range(6)]
    rows = sel.evaluate_heldout(s, cfgs, gpu_ctx)
    gpu_ctx.set_timing(False)
    for r in rows:
        assert r["err_selected"] <= r["tol"], r
    t_an = sum(r["t_analytic_ms"] for r in rows)
    t_sel = sum(r["t_selected_ms"] for r in rows)
    assert t_sel < t_an / 1.5, (t_sel, t_an)


def test_committed_selector_gains_over_tuned_choice(gpu_ctx):
    """What the trained network adds to the method without it: on
    configurations of 1e4 to 1e5 points (uniform or half on ellipses), the
    evaluations with the learned parameters (and their fallback evaluations,
    if any) take less GPU time in total than with the tuned analytic choice.
    The 500-configuration held-out evaluation of this build measured 12 % less
    on this class; the bar is any gain."""
    sel = _sel()
    if not os.path.exists(sel.MODEL_PATH):
        pytest.skip("no trained selector model in this checkout")
    s = sel.Selector(ctx=gpu_ctx)
    gpu_ctx.set_timing(True)
    rng = np.random.default_rng(77)
    cfgs = [sel.random_config(rng, nmin=1e4, nmax=1e5) for _ in range(24)]
    rows = sel.evaluate_heldout(s, cfgs, gpu_ctx)
    gpu_ctx.set_timing(False)
    t_tuned = sum(r["t_tuned_ms"] for r in rows)
    t_sel = sum(r["t_selected_ms"] for r in rows)
    assert t_sel < t_tuned, (t_sel, t_tuned)
