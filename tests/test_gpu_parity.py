"""GPU parity: the CUDA path through the C ABI against the reference's own
outputs (golden fixtures from its compiled gateways) and against the CPU
oracle on seeded inputs.

Tolerance: the plain form computes in FP64 and reorders sums (cell-sorted
near field, atomics in the spread, a different FFT), so agreement is to
rounding: max |u_gpu - u_ref| <= 1e-12 max |u_ref| (written per test).
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_max
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
SE_CASES = [n for n in golden_names() if not n.startswith("mex_")]
MEX_CASES = golden_names("mex_")


def _ft():
    import fasttools2d_gb300 as ft

    return ft


def _run_driver(ft, ctx, kind, g, **kw):
    args = dict(P=int(g["P"]), Nb=float(g["Nb"]) or None, tol=float(g["tol"]), ctx=ctx)
    args.update(kw)
    if kind == "slp":
        return ft.StokesSLP_ewald_2p(g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["f1"], g["f2"], float(g["Lx"]),
                                     float(g["Ly"]), **args)
    return ft.StokesDLP_ewald_2p(g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["n1"], g["n2"], g["f1"], g["f2"],
                                 float(g["Lx"]), float(g["Ly"]), **args)


@pytest.mark.parametrize("name", SE_CASES)
def test_driver_matches_reference_fixture(gpu_ctx, name):
    ft = _ft()
    g = load_golden(name)
    for kind in ("slp", "dlp"):
        if kind + "_u" not in g:
            continue
        u1, u2, ur, uk, xi = _run_driver(ft, gpu_ctx, kind, g)
        assert abs(xi - float(g[kind + "_prm_xi"])) <= 1e-13 * xi
        scale = np.max(np.abs(g[kind + "_u"]))
        assert np.max(np.abs(ur - g[kind + "_ur"])) <= TOL_FP64 * scale, (kind, "real")
        assert np.max(np.abs(uk - g[kind + "_uk"])) <= TOL_FP64 * scale, (kind, "kspace")
        assert np.max(np.abs(np.stack([u1, u2], 1) - g[kind + "_u"])) <= TOL_FP64 * scale, (kind, "total")


@pytest.mark.parametrize("name", MEX_CASES)
def test_gateways_match_reference_fixture(gpu_ctx, name):
    ft = _ft()
    g = load_golden(name)
    args = [g[f"arg{i}"] for i in range(int(g["nargs"]))]
    args = [float(a) if a.ndim == 0 else a for a in args]
    gw = str(g["gateway"])
    if gw == "slp_real":
        ps, pt, f, xi, nx, ny, Lx, Ly = args
        out = ft.mex_stokes_slp_real(ps, pt, f, xi, int(nx), int(ny), Lx, Ly, ctx=gpu_ctx)
    elif gw == "dlp_real":
        ps, pt, f, n, xi, nx, ny, Lx, Ly = args
        out = ft.mex_stokes_dlp_real(ps, pt, f, n, xi, int(nx), int(ny), Lx, Ly, ctx=gpu_ctx)
    elif gw == "slp_kspace":
        ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P = args
        out = ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, int(Mx), int(My), Lx, Ly, w, int(P), ctx=gpu_ctx)
    else:
        ps, pt, xi, eta, f, n, Mx, My, Lx, Ly, w, P = args
        out = ft.mex_stokes_dlp_kspace(ps, pt, xi, eta, f, n, int(Mx), int(My), Lx, Ly, w, int(P), ctx=gpu_ctx)
    assert rel_max(out, g["out"]) <= TOL_FP64


RANDOM_CASES = [
    # (nsrc, ntar, Lx, Ly, tol, seed)
    (3000, 2000, 1.0, 1.0, 1e-10, 11),
    (2500, 2500, 2.0, 1.0, 1e-8, 12),
    (4000, 1000, 1.0, 2.0, 1e-12, 13),
    (1500, 3000, 1.5, 1.0, 1e-6, 14),
    (50, 70, 1.0, 1.0, 1e-14, 15),
]


@pytest.mark.parametrize("case", RANDOM_CASES)
def test_driver_matches_oracle(gpu_ctx, case):
    ft = _ft()
    ns, nt, Lx, Ly, tol, seed = case
    rng = np.random.default_rng(seed)
    xs, ys = rng.random(ns) * Lx, rng.random(ns) * Ly
    xt, yt = rng.random(nt) * Lx, rng.random(nt) * Ly
    f1, f2 = rng.standard_normal(ns), rng.standard_normal(ns)
    th = rng.random(ns) * 2 * np.pi
    n1, n2 = np.cos(th), np.sin(th)
    o = po.stokes_slp_ewald_2p(xs, ys, xt, yt, f1, f2, Lx, Ly, tol=tol)
    g = ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1, f2, Lx, Ly, tol=tol, ctx=gpu_ctx)
    scale = max(np.max(np.abs(o[0])), np.max(np.abs(o[1])))
    assert np.max(np.abs(g[2] - o[2])) <= TOL_FP64 * scale
    assert np.max(np.abs(g[3] - o[3])) <= TOL_FP64 * scale
    o = po.stokes_dlp_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, tol=tol)
    g = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, tol=tol, ctx=gpu_ctx)
    scale = max(np.max(np.abs(o[0])), np.max(np.abs(o[1])))
    assert np.max(np.abs(g[2] - o[2])) <= TOL_FP64 * scale
    assert np.max(np.abs(g[3] - o[3])) <= TOL_FP64 * scale


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_kspace_gateway_points_outside_box(gpu_ctx, kind):
    """Gateway-level callers may pass points outside [-L/2, L/2) (the drivers
    wrap, the gateways do not): windows then leave their tile's region."""
    ft = _ft()
    rng = np.random.default_rng(21)
    ns, nt = 3000, 2000
    ps = (rng.random((ns, 2)) - 0.5) * 1.8
    pt = (rng.random((nt, 2)) - 0.5) * 1.8
    f = rng.standard_normal((ns, 2))
    th = rng.random(ns) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], 1)
    Mx = My = 96
    P, xi = 24, 30.0
    w = P * (1.0 / Mx) / 2
    eta = (2 * xi * w / (0.95 * np.sqrt(np.pi * P))) ** 2
    if kind == "slp":
        ref = po.slp_kspace(ps, pt, xi, eta, f, Mx, My, 1.0, 1.0, w, P)
        out = ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, 1.0, 1.0, w, P, ctx=gpu_ctx)
    else:
        ref = po.dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, 1.0, 1.0, w, P)
        out = ft.mex_stokes_dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, 1.0, 1.0, w, P, ctx=gpu_ctx)
    assert rel_max(out, ref) <= TOL_FP64


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("P", [32, 40, 48, 64])
def test_kspace_gateway_wide_windows(gpu_ctx, kind, P):
    """Window supports of 33 to 65 nodes (the gateways accept P up to 64):
    the tiled spread covers a window's rows in blocks of 32 lanes."""
    ft = _ft()
    rng = np.random.default_rng(22 + P)
    ns, nt = 1500, 800
    ps = rng.random((ns, 2)) - 0.5
    pt = rng.random((nt, 2)) - 0.5
    f = rng.standard_normal((ns, 2))
    th = rng.random(ns) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], 1)
    Mx = My = 128
    xi = 30.0
    w = P * (1.0 / Mx) / 2
    eta = (2 * xi * w / (0.95 * np.sqrt(np.pi * P))) ** 2
    if kind == "slp":
        ref = po.slp_kspace(ps, pt, xi, eta, f, Mx, My, 1.0, 1.0, w, P)
        out = ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, 1.0, 1.0, w, P, ctx=gpu_ctx)
    else:
        ref = po.dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, 1.0, 1.0, w, P)
        out = ft.mex_stokes_dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, 1.0, 1.0, w, P, ctx=gpu_ctx)
    assert rel_max(out, ref) <= TOL_FP64


def test_device_pointers_match_host(gpu_ctx):
    import torch

    ft = _ft()
    g = load_golden("config1_n1000")
    host = _run_driver(ft, gpu_ctx, "dlp", g)
    dev = {k: torch.tensor(g[k], device="cuda") for k in ("xsrc", "ysrc", "xtar", "ytar", "f1", "f2", "n1", "n2")}
    out = ft.StokesDLP_ewald_2p(dev["xsrc"], dev["ysrc"], dev["xtar"], dev["ytar"], dev["n1"], dev["n2"], dev["f1"],
                                dev["f2"], 1.0, 1.0, tol=float(g["tol"]), ctx=gpu_ctx)
    assert out[0].is_cuda
    assert rel_max(out[0].cpu().numpy(), host[0]) <= 1e-13
    assert rel_max(out[3].cpu().numpy(), host[3]) <= 1e-13


def test_weights_option_equals_prescaled_density(gpu_ctx):
    ft = _ft()
    g = load_golden("config2_mini")
    rng = np.random.default_rng(3)
    w = rng.random(len(g["xsrc"])) + 0.5
    a = ft.StokesSLP_ewald_2p(g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["f1"], g["f2"], 2.0, 1.0, tol=1e-10,
                              weights=w, ctx=gpu_ctx)
    b = ft.StokesSLP_ewald_2p(g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["f1"] * w, g["f2"] * w, 2.0, 1.0,
                              tol=1e-10, ctx=gpu_ctx)
    assert rel_max(a[0], b[0]) <= 1e-13 and rel_max(a[1], b[1]) <= 1e-13


def test_empty_sources_and_targets(gpu_ctx):
    ft = _ft()
    rng = np.random.default_rng(4)
    xt, yt = rng.random(10) - 0.5, rng.random(10) - 0.5
    out = ft.mex_stokes_slp_real(np.zeros((0, 2)), np.stack([xt, yt], 1), np.zeros((0, 2)), 10.0, 3, 3, 1.0, 1.0,
                                 ctx=gpu_ctx)
    assert out.shape == (10, 2) and np.all(out == 0)
    out = ft.mex_stokes_slp_kspace(np.zeros((0, 2)), np.stack([xt, yt], 1), 10.0, 0.8, np.zeros((0, 2)), 48, 48, 1.0,
                                   1.0, 24 / 48 / 2, 24, ctx=gpu_ctx)
    assert out.shape == (10, 2) and np.all(out == 0)
    xs, ys = rng.random(5) - 0.5, rng.random(5) - 0.5
    res = ft.StokesSLP_ewald_2p(xs, ys, np.zeros(0), np.zeros(0), np.ones(5), np.ones(5), 1.0, 1.0, tol=1e-8,
                                ctx=gpu_ctx)
    assert res[0].shape == (0,)


def test_invalid_arguments_are_rejected(gpu_ctx):
    ft = _ft()
    ps = np.zeros((4, 2))
    f = np.ones((4, 2))
    bad = [
        lambda: ft.mex_stokes_slp_kspace(ps, ps, 10.0, 0.8, f, 47, 48, 1.0, 1.0, 0.25, 24, ctx=gpu_ctx),  # odd M
        lambda: ft.mex_stokes_slp_kspace(ps, ps, 10.0, 0.8, f, 48, 48, 1.0, 1.0, 0.25, 23, ctx=gpu_ctx),  # odd P
        lambda: ft.mex_stokes_slp_kspace(ps, ps, 10.0, 0.8, f, 48, 64, 1.0, 1.0, 0.25, 24, ctx=gpu_ctx),  # hx != hy
        lambda: ft.mex_stokes_slp_real(ps, ps, f, -1.0, 3, 3, 1.0, 1.0, ctx=gpu_ctx),  # xi <= 0
        lambda: ft.mex_stokes_slp_real(ps, ps, f, 10.0, 0, 3, 1.0, 1.0, ctx=gpu_ctx),  # no cells
        lambda: ft.mex_stokes_dlp_real(ps, ps, f, f, 10.0, 3, 3, 0.0, 1.0, ctx=gpu_ctx),  # L <= 0
    ]
    for fn in bad:
        with pytest.raises(ft.FteError) as e:
            fn()
        assert e.value.code == ft.FTE_ERR_INVALID
    with pytest.raises(ValueError):
        ft.mex_stokes_slp_real(ps, ps, np.ones((3, 2)), 10.0, 3, 3, 1.0, 1.0, ctx=gpu_ctx)
    # the context stays usable after rejected calls
    out = ft.mex_stokes_slp_real(ps + 0.1, ps, f, 10.0, 3, 3, 1.0, 1.0, ctx=gpu_ctx)
    assert np.all(np.isfinite(out))


def test_kernel_counter_moves(gpu_ctx):
    ft = _ft()
    g = load_golden("tiny_n3")
    k0 = gpu_ctx.kernel_count
    _run_driver(ft, gpu_ctx, "slp", g)
    assert gpu_ctx.kernel_count - k0 >= 8
