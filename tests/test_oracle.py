"""The CPU oracle pinned against the reference's own outputs (golden fixtures),
against the reference tests' direct sums, and against numpy/scipy.

The fixtures in tests/golden were produced by the reference's own compiled
gateways (tests/golden/gen_golden.py); the oracle is the C restatement in
oracle/or_ewald.c.  These tests run on the CPU only.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_max
from oracle import pyoracle as po

SE_CASES = [n for n in golden_names() if not n.startswith("mex_")]
MEX_CASES = golden_names("mex_")


def _driver(kind, g):
    args = dict(P=int(g["P"]), Nb=float(g["Nb"]), tol=float(g["tol"]))
    if kind == "slp":
        return po.stokes_slp_ewald_2p(g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["f1"], g["f2"], float(g["Lx"]),
                                      float(g["Ly"]), **args)
    return po.stokes_dlp_ewald_2p(g["xsrc"], g["ysrc"], g["xtar"], g["ytar"], g["n1"], g["n2"], g["f1"], g["f2"],
                                  float(g["Lx"]), float(g["Ly"]), **args)


@pytest.mark.parametrize("name", SE_CASES)
def test_oracle_matches_reference_fixture(name):
    g = load_golden(name)
    for kind in ("slp", "dlp"):
        if kind + "_u" not in g:
            continue
        u1, u2, ur, uk, prm = _driver(kind, g)
        # parameter choice is identical (integers exactly, reals to rounding)
        for key in ("nside_x", "nside_y", "Mx", "My", "kinf", "A", "B"):
            assert getattr(prm, key) == int(g[f"{kind}_prm_{key}"]), (kind, key)
        for key in ("xi", "eta", "w", "rc"):
            assert abs(getattr(prm, key) - float(g[f"{kind}_prm_{key}"])) <= 1e-13 * abs(float(g[f"{kind}_prm_{key}"]))
        scale = np.max(np.abs(g[kind + "_u"]))
        assert np.max(np.abs(ur - g[kind + "_ur"])) <= 1e-13 * scale
        assert np.max(np.abs(uk - g[kind + "_uk"])) <= 1e-13 * scale
        assert np.max(np.abs(np.stack([u1, u2], 1) - g[kind + "_u"])) <= 1e-13 * scale


@pytest.mark.parametrize("name", MEX_CASES)
def test_oracle_gateways_match_reference_fixture(name):
    g = load_golden(name)
    args = [g[f"arg{i}"] for i in range(int(g["nargs"]))]
    args = [float(a) if a.ndim == 0 else a for a in args]
    gw = str(g["gateway"])
    fn = {"slp_real": po.slp_real, "dlp_real": po.dlp_real, "slp_kspace": po.slp_kspace,
          "dlp_kspace": po.dlp_kspace}[gw]
    if gw == "slp_real":
        ps, pt, f, xi, nx, ny, Lx, Ly = args
        out = fn(ps, pt, f, xi, int(nx), int(ny), Lx, Ly)
    elif gw == "dlp_real":
        ps, pt, f, n, xi, nx, ny, Lx, Ly = args
        out = fn(ps, pt, f, n, xi, int(nx), int(ny), Lx, Ly)
    elif gw == "slp_kspace":
        ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P = args
        out = fn(ps, pt, xi, eta, f, int(Mx), int(My), Lx, Ly, w, int(P))
    else:
        ps, pt, xi, eta, f, n, Mx, My, Lx, Ly, w, P = args
        out = fn(ps, pt, xi, eta, f, n, int(Mx), int(My), Lx, Ly, w, int(P))
    assert rel_max(out, g["out"]) <= 1e-13


def test_reference_fixture_matches_direct_sums():
    """PeriodicEwald/tests/direct_sums/direct_sums_velocity_test.m restated with
    thresholds: SE real/k parts vs the direct real sum (3x3 images) and the
    direct Fourier sum (kinf = 70)."""
    g = load_golden("direct_sums_n20")
    for kind in ("slp", "dlp"):
        scale = np.max(np.abs(g[kind + "_u"]))
        assert np.max(np.abs(g[kind + "_ur"] - g[kind + "_ur_ds"])) <= 1e-14 * scale
        assert np.max(np.abs(g[kind + "_uk"] - g[kind + "_uk_ds"])) <= 1e-13 * scale


def test_oracle_direct_sums_reproduce_fixture():
    g = load_golden("direct_sums_n20")
    wx = po.matlab_wrap(g["xsrc"], 1.0)
    wy = po.matlab_wrap(g["ysrc"], 1.0)
    tx = po.matlab_wrap(g["xtar"], 1.0)
    ty = po.matlab_wrap(g["ytar"], 1.0)
    xi = float(g["slp_prm_xi"])
    ur = po.slp_real_ds(wx, wy, tx, ty, g["f1"], g["f2"], 1.0, 1.0, xi)
    assert rel_max(ur, g["slp_ur_ds"]) <= 1e-14


def test_e1_against_scipy():
    special = pytest.importorskip("scipy.special")
    xs = np.concatenate([np.logspace(-12, 0, 120), np.linspace(1, 60, 300), np.logspace(1.8, 2.8, 40)])
    e = np.array([po.expint_e1(x) for x in xs])
    assert np.max(np.abs(e - special.exp1(xs)) / special.exp1(xs)) <= 1e-14


@pytest.mark.parametrize("shape", [(48, 48), (30, 18), (766, 1532), (64, 1001), (58, 986)])
def test_oracle_fft2_against_numpy(shape):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape)
    F = po.fft2(a)
    Fn = np.fft.fft2(a)
    assert np.max(np.abs(F - Fn)) <= 1e-14 * np.max(np.abs(Fn))
    back = po.fft2(F.real, F.imag, inverse=True)
    assert np.max(np.abs(back - a)) <= 1e-13


def test_matlab_rat():
    assert po.rat(2.0) == (2, 1)
    assert po.rat(0.5) == (1, 2)
    assert po.rat(1.0) == (1, 1)
    assert po.rat(0.75) == (3, 4)
    assert po.rat(1.25) == (5, 4)
    assert po.rat(np.pi) == (355, 113)


def test_chooser_reproduces_config_table():
    """Parameters of the configurations (ξ, M, cells, η) as chosen by the
    reference drivers' analytic estimates, P = 24."""
    rng = np.random.default_rng(1)
    N = 1000
    f1, f2 = rng.standard_normal(N), rng.standard_normal(N)
    f1 -= f1.mean()
    f2 -= f2.mean()
    p = po.choose_params(po.KIND_SLP, f1, f2, N, N, 1.0, 1.0, 24, 0, 1e-10)
    assert (p.nside_x, p.nside_y, p.Mx, p.My) == (3, 3, 48, 48)
    assert abs(p.xi - 15.04) < 0.05 and abs(p.eta - 0.83) < 0.01
    N = 10 ** 6
    f1, f2 = rng.standard_normal(N), rng.standard_normal(N)
    for kind, tol, M, xi in [(po.KIND_SLP, 1e-6, 710, 264.3), (po.KIND_DLP, 1e-6, 986, 301.8),
                             (po.KIND_SLP, 1e-10, 1072, 324.9), (po.KIND_DLP, 1e-10, 1360, 357.8)]:
        p = po.choose_params(kind, f1, f2, N, N, 1.0, 1.0, 24, 0, tol)
        assert (p.nside_x, p.nside_y) == (63, 63)
        assert (p.Mx, p.My) == (M, M), (kind, tol, p.Mx)
        assert abs(p.xi - xi) < 0.2
