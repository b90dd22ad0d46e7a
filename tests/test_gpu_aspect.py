"""Boxes whose aspect ratio is not a small rational (the improved parameter
choice of the mixed form).

The reference's drivers need Lx / Ly = A / B with small A and B: they take
[A, B] = rat(Lx / Ly), make A B cells per unit cell count and the grid
(A M) x (B M) (PeriodicEwald/src/matlab/StokesSLP_ewald_2p.m:85-101), so
1 x sqrt(2) (rat: 985 / 1393) gives a grid of billions of nodes.  The mixed
form's tuned choice gives such boxes nearly square cells (cutoff = the
shorter side) and a grid step per axis, Mx and My each a cheap even size
resolving the same wave number, with one Gaussian window shape.  Checked
against the converged FP64 Ewald sum at sampled targets: max |u - u_truth| /
max |u_truth| <= tol; the drivers' (plain) form rejects these boxes.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _case(n, Lx, Ly, seed, clustered=False):
    rng = np.random.default_rng(seed)
    if clustered:
        # half the points on a few ellipses, half uniform
        m = n // 2
        k = 8
        th = 2 * np.pi * rng.random(m)
        c = rng.integers(0, k, m)
        cx, cy = (rng.random(k) - 0.5) * Lx * 0.8, (rng.random(k) - 0.5) * Ly * 0.8
        a, b = 0.03 + 0.05 * rng.random(k), 0.03 + 0.05 * rng.random(k)
        xs = np.concatenate([cx[c] + a[c] * np.cos(th), (rng.random(n - m) - 0.5) * Lx])
        ys = np.concatenate([cy[c] + b[c] * np.sin(th), (rng.random(n - m) - 0.5) * Ly])
    else:
        xs, ys = (rng.random(n) - 0.5) * Lx, (rng.random(n) - 0.5) * Ly
    xt, yt = (rng.random(n) - 0.5) * Lx, (rng.random(n) - 0.5) * Ly
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    f1 -= f1.mean()
    f2 -= f2.mean()
    t = rng.random(n) * 2 * np.pi
    return xs, ys, xt, yt, f1, f2, np.cos(t), np.sin(t)


_TRUTH = {}


def _truth(kind, geom, xs, ys, xt, yt, f1, f2, n1, n2, idx):
    key = (kind, geom)
    if key not in _TRUTH:
        n, Lx, Ly, seed, clustered = geom
        if kind == "slp":
            _TRUTH[key] = po.ewald_truth(po.KIND_SLP, xs, ys, xt[idx], yt[idx], f1, f2, Lx, Ly)
        else:
            _TRUTH[key] = po.ewald_truth(po.KIND_DLP, xs, ys, xt[idx], yt[idx], f1, f2, Lx, Ly, n1=n1, n2=n2)
    return _TRUTH[key]


@pytest.mark.parametrize("tol", [1e-6, 1e-8, 1e-10])
@pytest.mark.parametrize("geom", [(16000, 1.0, np.sqrt(2.0), 41, False), (16000, 1.0, 3.7, 42, False),
                                  (20000, np.pi, 1.0, 43, False), (16000, np.sqrt(2.0), 1.0, 44, True)])
def test_irrational_box_meets_tolerance(gpu_ctx, tol, geom):
    import fasttools2d_gb300 as ft

    n, Lx, Ly, seed, clustered = geom
    xs, ys, xt, yt, f1, f2, n1, n2 = _case(n, Lx, Ly, seed, clustered)
    idx = np.arange(0, n, 50)
    aniso = False
    for kind in ("slp", "dlp"):
        if kind == "slp":
            out, info = ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1, f2, Lx, Ly, tol=tol, form=ft.FORM_MIXED,
                                              ctx=gpu_ctx, return_info=True)
        else:
            out, info = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, tol=tol, form=ft.FORM_MIXED,
                                              ctx=gpu_ctx, return_info=True)
        truth = _truth(kind, geom, xs, ys, xt, yt, f1, f2, n1, n2, idx)
        p = info.params
        hx, hy = Lx / p.Mx, Ly / p.My
        aniso = aniso or abs(hx - hy) > 1e-12 * max(hx, hy)
        assert p.nside_x * p.nside_y < 10 * n  # no rat()-sized cell list
        u = np.stack([out[0][idx], out[1][idx]], 1)
        err = np.max(np.abs(u - truth)) / np.max(np.abs(truth))
        assert err <= tol, (kind, err, p.as_dict())
    assert aniso  # the per-axis grid steps were exercised


def test_forced_kspace_arithmetic_on_irrational_box(gpu_ctx):
    """FP64, FP32, float-float and FP32-product k-space on the same
    unequal-step grid agree (the FP32 forms to their own floor)."""
    import fasttools2d_gb300 as ft

    n, Lx, Ly = 12000, 1.0, np.sqrt(2.0)
    xs, ys, xt, yt, f1, f2, n1, n2 = _case(n, Lx, Ly, 45)
    res = {}
    over = {}
    for ks in (ft.KSPACE_FP64, ft.KSPACE_FF, ft.KSPACE_FP32, ft.KSPACE_FF32):
        # the same parameters for every arithmetic (those of the first call)
        out, info = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, tol=1e-6, form=ft.FORM_MIXED,
                                          kspace=ks, near=ft.NEAR_FP64, ctx=gpu_ctx, return_info=True, **over)
        res[ks] = np.stack([out[0], out[1]], 1)
        p = info.params
        if not over:
            over = dict(P=p.P, xi=p.xi, Mx=p.Mx, My=p.My, nside_x=p.nside_x, nside_y=p.nside_y)
        assert (p.P, p.Mx, p.My, p.nside_x, p.nside_y) == (over["P"], over["Mx"], over["My"], over["nside_x"],
                                                           over["nside_y"])
    assert abs(Lx / p.Mx - Ly / p.My) > 1e-6 * (Lx / p.Mx)
    scale = np.abs(res[ft.KSPACE_FP64]).max()
    assert np.abs(res[ft.KSPACE_FF] - res[ft.KSPACE_FP64]).max() <= 1e-11 * scale
    assert np.abs(res[ft.KSPACE_FP32] - res[ft.KSPACE_FP64]).max() <= 1e-6 * scale
    assert np.abs(res[ft.KSPACE_FF32] - res[ft.KSPACE_FP64]).max() <= 1e-6 * scale


def test_plans_on_irrational_box(gpu_ctx):
    """Plans (the batched form's building block) take the same geometry."""
    import fasttools2d_gb300 as ft

    n, Lx, Ly = 10000, 1.0, 3.7
    xs, ys, xt, yt, f1, f2, n1, n2 = _case(n, Lx, Ly, 46)
    fv1 = np.stack([f1, np.roll(f1, 1)])
    fv2 = np.stack([f2, np.roll(f2, 7)])
    p = ft.Plan(ft.KIND_DLP, xs, ys, xt, yt, f1, f2, Lx, Ly, n1=n1, n2=n2, tol=1e-8, form=ft.FORM_MIXED, nvmax=2,
                ctx=gpu_ctx)
    u1, u2 = p.execute(fv1, fv2)
    p.close()
    idx = np.arange(0, n, 40)
    for v in range(2):
        truth = po.ewald_truth(po.KIND_DLP, xs, ys, xt[idx], yt[idx], fv1[v], fv2[v], Lx, Ly, n1=n1, n2=n2)
        u = np.stack([u1[v][idx], u2[v][idx]], 1)
        assert np.max(np.abs(u - truth)) / np.max(np.abs(truth)) <= 1e-8


def test_drivers_form_rejects_irrational_box(gpu_ctx):
    import fasttools2d_gb300 as ft

    xs, ys, xt, yt, f1, f2, n1, n2 = _case(2000, 1.0, np.sqrt(2.0), 47)
    with pytest.raises(ft.FteError) as e:
        ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1, f2, 1.0, np.sqrt(2.0), tol=1e-10, ctx=gpu_ctx)
    assert e.value.code in (ft.FTE_ERR_UNSUPPORTED, ft.FTE_ERR_ALLOC)
