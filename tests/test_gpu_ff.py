"""Float-float k-space (FTE_FORM_FF): spread and gather in pairs of FP32
numbers, FP64 transforms and filter.

* against the FP64 k-space on the same parameters: the k-space parts agree to
  ~1e-13 of their maximum (the pairs carry ~48 bits);
* the tuned choice picks it between the FP32 floor and 1e-11 and meets the
  tolerance against converged FP64 Ewald sums;
* plans (tile bins and window records built once, tuned tiles) give the
  driver's result.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _ft():
    import fasttools2d_gb300 as ft

    return ft


def _case(seed, n, Lx, Ly):
    rng = np.random.default_rng(seed)
    xs, ys = (rng.random(n) - 0.5) * Lx, (rng.random(n) - 0.5) * Ly
    xt, yt = (rng.random(n) - 0.5) * Lx, (rng.random(n) - 0.5) * Ly
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    f1 -= f1.mean()
    f2 -= f2.mean()
    th = rng.random(n) * 2 * np.pi
    return xs, ys, xt, yt, f1, f2, np.cos(th), np.sin(th)


def _run(ft, ctx, kind, d, Lx, Ly, **kw):
    xs, ys, xt, yt, f1, f2, n1, n2 = d
    if kind == "slp":
        return ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1, f2, Lx, Ly, form=ft.FORM_MIXED, ctx=ctx, return_info=True,
                                     **kw)
    return ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, form=ft.FORM_MIXED, ctx=ctx,
                                 return_info=True, **kw)


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("geom", [(20000, 1.0, 1.0, 41), (12000, 2.0, 1.0, 42), (9000, 1.0, 2.75, 43)])
def test_ff_kspace_matches_fp64(gpu_ctx, kind, geom):
    ft = _ft()
    n, Lx, Ly, seed = geom
    d = _case(seed, n, Lx, Ly)
    out_f, info_f = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FF)
    p = info_f.params
    assert p.form == ft.FORM_FF
    same = dict(P=p.P, xi=p.xi, Mx=p.Mx, My=p.My, nside_x=p.nside_x, nside_y=p.nside_y)
    out_d, info_d = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FP64, **same)
    q = info_d.params
    assert q.form == ft.FORM_PLAIN
    assert (q.P, q.Mx, q.My, q.nside_x, q.xi) == (p.P, p.Mx, p.My, p.nside_x, p.xi)
    uk_f, uk_d = out_f[3], out_d[3]
    rel = np.max(np.abs(uk_f - uk_d)) / np.max(np.abs(uk_d))
    assert rel <= 2e-12, rel
    # the real-space parts are the same kernel on the same parameters; the
    # cell lists' order within a box may differ between calls, which moves
    # the FP32 pair class's rounding (well below the tolerance)
    assert np.max(np.abs(out_f[2] - out_d[2])) <= 1e-10 * np.max(np.abs(out_d[2]))


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("P", [12, 16, 24, 32, 48])
def test_ff_gather_supports(gpu_ctx, kind, P):
    """Window supports on either side of the gather's register bounds (16, 24
    and 32 nodes) and beyond them (the shared-memory form; 49 nodes: the
    spread's rows in two blocks of 32)."""
    ft = _ft()
    Lx, Ly = 1.0, 1.5
    d = _case(60 + P, 6000, Lx, Ly)
    out_f, info_f = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FF, P=P)
    p = info_f.params
    assert p.form == ft.FORM_FF and p.P == P
    same = dict(P=p.P, xi=p.xi, Mx=p.Mx, My=p.My, nside_x=p.nside_x, nside_y=p.nside_y)
    out_d, _ = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FP64, **same)
    rel = np.max(np.abs(out_f[3] - out_d[3])) / np.max(np.abs(out_d[3]))
    assert rel <= 2e-12, rel


@pytest.mark.parametrize("tol", [1e-9, 1e-11])
@pytest.mark.parametrize("geom", [(20000, 1.0, 1.0, 51), (12000, 3.75, 1.0, 52)])
def test_ff_chosen_and_meets_tolerance(gpu_ctx, tol, geom):
    ft = _ft()
    n, Lx, Ly, seed = geom
    d = _case(seed, n, Lx, Ly)
    xs, ys, xt, yt, f1, f2, n1, n2 = d
    idx = np.arange(0, n, 40)
    for kind in ("slp", "dlp"):
        out, info = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=tol)
        assert info.params.form == ft.FORM_FF, info.params.as_dict()
        if kind == "slp":
            truth = po.ewald_truth(po.KIND_SLP, xs, ys, xt[idx], yt[idx], f1, f2, Lx, Ly)
        else:
            truth = po.ewald_truth(po.KIND_DLP, xs, ys, xt[idx], yt[idx], f1, f2, Lx, Ly, n1=n1, n2=n2)
        u = np.stack([out[0][idx], out[1][idx]], 1)
        err = np.max(np.abs(u - truth)) / np.max(np.abs(truth))
        assert err <= tol, (kind, err, info.params.as_dict())


def test_ff_on_ellipses(gpu_ctx):
    """Clustered boundary points with self-coincident targets, FF forced at
    tol 1e-10, against the reference's own SE output (absolute criterion, as
    for the other forms)."""
    ft = _ft()
    g = load_golden("config2_mini")
    for kind in ("slp", "dlp"):
        d = (g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["f1"], g["f2"], g["n1"], g["n2"])
        out, info = _run(ft, gpu_ctx, kind, d, 2.0, 1.0, tol=1e-10, kspace=ft.KSPACE_FF)
        assert info.params.form == ft.FORM_FF
        ref = g[kind + "_u"]
        u = np.stack([out[0], out[1]], 1)
        assert np.max(np.abs(u - ref)) <= 1e-10 * max(1.0, np.max(np.abs(ref))), kind


@pytest.mark.parametrize("tune", [False, True])
def test_ff_plan_matches_driver(gpu_ctx, tune):
    ft = _ft()
    n, Lx, Ly = 15000, 2.0, 1.0
    xs, ys, xt, yt, f1, f2, n1, n2 = _case(61, n, Lx, Ly)
    rng = np.random.default_rng(62)
    fs1, fs2 = rng.standard_normal((3, n)), rng.standard_normal((3, n))
    for kind in (ft.KIND_SLP, ft.KIND_DLP):
        plan = ft.Plan(kind, xs, ys, xt, yt, f1, f2, Lx, Ly, n1=n1, n2=n2, tol=1e-10, form=ft.FORM_MIXED,
                       kspace=ft.KSPACE_FF, nvmax=3, tune=tune, ctx=gpu_ctx)
        p = plan.params
        assert p.form == ft.FORM_FF
        u1s, u2s = plan.execute(fs1, fs2)
        for v in range(3):
            kw = dict(tol=1e-10, form=ft.FORM_MIXED, kspace=ft.KSPACE_FF, P=p.P, xi=p.xi, Mx=p.Mx, My=p.My,
                      nside_x=p.nside_x, nside_y=p.nside_y, ctx=gpu_ctx)
            if kind == ft.KIND_SLP:
                o = ft.StokesSLP_ewald_2p(xs, ys, xt, yt, fs1[v], fs2[v], Lx, Ly, **kw)
            else:
                o = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, fs1[v], fs2[v], Lx, Ly, **kw)
            ref = np.stack([o[0], o[1]], 1)
            got = np.stack([np.asarray(u1s[v]), np.asarray(u2s[v])], 1)
            assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), (kind, v)


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("geom", [(20000, 1.0, 1.0, 71), (12000, 2.0, 1.0, 72), (9000, 1.0, 2.75, 73)])
def test_ff_near_matches_fp64(gpu_ctx, kind, geom):
    """Float-float pairs against FP64 pairs on the same parameters, without
    the FP32 class: real-space parts within 1e-12 of their maximum."""
    ft = _ft()
    n, Lx, Ly, seed = geom
    d = _case(seed, n, Lx, Ly)
    out_f, info = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FP64, near=ft.NEAR_FF)
    p = info.params
    same = dict(P=p.P, xi=p.xi, Mx=p.Mx, My=p.My, nside_x=p.nside_x, nside_y=p.nside_y)
    out_d, _ = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FP64, near=ft.NEAR_FP64, **same)
    ur_f, ur_d = out_f[2], out_d[2]
    rel = np.max(np.abs(ur_f - ur_d)) / np.max(np.abs(ur_d))
    assert rel <= 1e-12, rel


def test_ff_near_two_vectors(gpu_ctx):
    """Plans with two density vectors (two targets in flight per warp) take
    the float-float class too; compared with FP64 pairs."""
    ft = _ft()
    n, Lx, Ly = 15000, 1.0, 1.0
    xs, ys, xt, yt, f1, f2, n1, n2 = _case(81, n, Lx, Ly)
    rng = np.random.default_rng(82)
    fs1, fs2 = rng.standard_normal((2, n)), rng.standard_normal((2, n))
    for kind in (ft.KIND_SLP, ft.KIND_DLP):
        res = []
        for near in (ft.NEAR_FF, ft.NEAR_FP64):
            plan = ft.Plan(kind, xs, ys, xt, yt, f1, f2, Lx, Ly, n1=n1, n2=n2, tol=1e-10, form=ft.FORM_MIXED,
                           kspace=ft.KSPACE_FP64, near=near, nvmax=2, ctx=gpu_ctx, nside_x=60, nside_y=60)
            u1s, u2s = plan.execute(fs1, fs2)
            res.append(np.stack([np.asarray(u1s), np.asarray(u2s)], -1))
        rel = np.max(np.abs(res[0] - res[1])) / np.max(np.abs(res[1]))
        assert rel <= 1e-12, (kind, rel)


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("grid", [(218, 218, 1.0, 1.0), (436, 218, 2.0, 1.0)])
def test_ff_transforms_bluestein_and_odd_radices(gpu_ctx, kind, grid):
    """Grids whose lines need Bluestein (218 = 2 * 109, 436 = 4 * 109) in the
    float-float transforms: k-space parts against the FP64 transforms on the
    same parameters."""
    ft = _ft()
    Mx, My, Lx, Ly = grid
    d = _case(91, 6000, Lx, Ly)
    kw = dict(tol=1e-10, Mx=Mx, My=My, nside_x=int(12 * Lx), nside_y=int(12 * Ly), P=16)
    out_f, info = _run(ft, gpu_ctx, kind, d, Lx, Ly, kspace=ft.KSPACE_FF, **kw)
    assert info.params.form == ft.FORM_FF and info.params.Mx == Mx
    out_d, _ = _run(ft, gpu_ctx, kind, d, Lx, Ly, kspace=ft.KSPACE_FP64, xi=info.params.xi, **kw)
    rel = np.max(np.abs(out_f[3] - out_d[3])) / np.max(np.abs(out_d[3]))
    assert rel <= 2e-12, rel


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_ff_transforms_smooth_radices(gpu_ctx, kind):
    """7-smooth grids with radices 3, 5 and 7 (210 = 2 3 5 7, 252 = 4 9 7)."""
    ft = _ft()
    d = _case(92, 6000, 1.0, 1.2)
    kw = dict(tol=1e-10, Mx=210, My=252, nside_x=12, nside_y=14, P=16)
    out_f, info = _run(ft, gpu_ctx, kind, d, 1.0, 1.2, kspace=ft.KSPACE_FF, **kw)
    assert info.params.form == ft.FORM_FF
    out_d, _ = _run(ft, gpu_ctx, kind, d, 1.0, 1.2, kspace=ft.KSPACE_FP64, xi=info.params.xi, **kw)
    rel = np.max(np.abs(out_f[3] - out_d[3])) / np.max(np.abs(out_d[3]))
    assert rel <= 2e-12, rel


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_ff_spread_gather_around_long_transforms(gpu_ctx, kind):
    """Lines beyond one block (8000 x 32 grid of a 250 x 1 box): the
    float-float spread and gather run around the FP64 long transforms and the
    FP64 multiplier, the stresslet on its three symmetric grids; k-space parts
    against the FP64 k-space on the same parameters."""
    ft = _ft()
    Lx, Ly = 250.0, 1.0
    d = _case(77, 3000, Lx, Ly)
    same = dict(P=16, xi=10.0, Mx=8000, My=32, nside_x=500, nside_y=2)
    out_f, info_f = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FF, **same)
    assert info_f.params.form == ft.FORM_FF
    out_d, info_d = _run(ft, gpu_ctx, kind, d, Lx, Ly, tol=1e-10, kspace=ft.KSPACE_FP64, **same)
    assert info_d.params.form == ft.FORM_PLAIN
    rel = np.max(np.abs(out_f[3] - out_d[3])) / np.max(np.abs(out_d[3]))
    assert rel <= 2e-12, rel
