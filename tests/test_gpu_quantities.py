"""GPU gateways of the other spectral Ewald quantities (pressure, pressure
gradient, velocity gradient, stress, vorticity; Stokeslet and stresslet)
against the reference's own gateways (golden vectors) and against the oracle
on random inputs, to 1e-12 relative (max |a - b| / max |b|)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_max
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL = 1e-12
NAMES = [n for n in golden_names("quant_") if not n.startswith("quant_drv_")]


def _ft():
    import fasttools2d_gb300 as ft

    return ft


@pytest.mark.parametrize("name", NAMES)
def test_quantity_gateways_match_reference(gpu_ctx, name):
    ft = _ft()
    g = load_golden(name)
    kind, q = int(g["kind"]), int(g["quantity"])
    n = g["n"] if kind == ft.KIND_DLP else None
    ur = ft.q_real(kind, q, g["psrc"], g["ptar"], g["f"], n, float(g["xi"]), int(g["nside_x"]), int(g["nside_y"]),
                   float(g["Lx"]), float(g["Ly"]), ctx=gpu_ctx)
    uk = ft.q_kspace(kind, q, g["psrc"], g["ptar"], g["f"], n, float(g["xi"]), float(g["eta"]), int(g["Mx"]),
                     int(g["My"]), float(g["Lx"]), float(g["Ly"]), float(g["w"]), int(g["P"]), ctx=gpu_ctx)
    assert rel_max(ur, g["real"]) <= TOL, (name, "real")
    assert rel_max(uk, g["kspace"]) <= TOL, (name, "kspace")


def _case(seed, Lx, Ly, ns, nt, Mx, P=16, xi=10.0):
    rng = np.random.default_rng(seed)
    ps = np.stack([(rng.random(ns) - 0.5) * Lx, (rng.random(ns) - 0.5) * Ly], 1)
    pt = np.concatenate([np.stack([(rng.random(nt) - 0.5) * Lx, (rng.random(nt) - 0.5) * Ly], 1), ps[:16]])
    f = rng.standard_normal((ns, 2))
    th = rng.random(ns) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], 1)
    My = int(round(Mx * Ly / Lx))
    w = P * (Lx / Mx) / 2
    eta = (2 * xi * w / (0.95 * np.sqrt(np.pi * P))) ** 2
    return ps, pt, f, n, xi, P, Mx, My, w, eta


@pytest.mark.parametrize("q", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("geom", [(1.0, 1.0, 900, 600, 96), (1.0, 2.5, 700, 500, 40)])
def test_quantities_match_oracle(gpu_ctx, kind, q, geom):
    ft = _ft()
    Lx, Ly, ns, nt, Mx = geom
    ps, pt, f, n, xi, P, Mx, My, w, eta = _case(7 * q + kind, Lx, Ly, ns, nt, Mx)
    nsx, nsy = int(4 * Lx), int(round(4 * Ly))
    nn = n if kind == ft.KIND_DLP else None
    ur = ft.q_real(kind, q, ps, pt, f, nn, xi, nsx, nsy, Lx, Ly, ctx=gpu_ctx)
    ref_r = po.q_real(kind, q, ps, pt, f, nn, xi, nsx, nsy, Lx, Ly)
    assert rel_max(ur, ref_r) <= TOL, ("real", kind, q, geom)
    uk = ft.q_kspace(kind, q, ps, pt, f, nn, xi, eta, Mx, My, Lx, Ly, w, P, ctx=gpu_ctx)
    ref_k = po.q_kspace(kind, q, ps, pt, f, nn, xi, eta, Mx, My, Lx, Ly, w, P)
    assert rel_max(uk, ref_k) <= TOL, ("kspace", kind, q, geom)


def test_quantity_long_grid_matches_oracle(gpu_ctx):
    """An 8000 x 32 grid: the k-space of a quantity through the long transform."""
    ft = _ft()
    ps, pt, f, n, xi, P, Mx, My, w, eta = _case(99, 250.0, 1.0, 300, 200, 8000)
    for kind, q in ((0, 3), (1, 4), (1, 2)):
        nn = n if kind == 1 else None
        uk = ft.q_kspace(kind, q, ps, pt, f, nn, xi, eta, Mx, My, 250.0, 1.0, w, P, ctx=gpu_ctx)
        ref = po.q_kspace(kind, q, ps, pt, f, nn, xi, eta, Mx, My, 250.0, 1.0, w, P)
        assert rel_max(uk, ref) <= TOL, (kind, q)


def test_named_gateways_and_device_pointers(gpu_ctx):
    torch = pytest.importorskip("torch")
    ft = _ft()
    g = load_golden("quant_dlp_vorticity")
    t = {k: torch.tensor(g[k], device="cuda") for k in ("psrc", "ptar", "f", "n")}
    uk = ft.mex_stokes_dlp_vorticity_kspace(t["psrc"], t["ptar"], t["f"], t["n"], float(g["xi"]), float(g["eta"]),
                                            int(g["Mx"]), int(g["My"]), float(g["Lx"]), float(g["Ly"]),
                                            float(g["w"]), int(g["P"]), ctx=gpu_ctx)
    assert rel_max(uk.cpu().numpy(), g["kspace"]) <= TOL
    g = load_golden("quant_slp_gradient")
    ur = ft.mex_stokes_slp_gradient_real(g["psrc"], g["ptar"], g["f"], float(g["xi"]), int(g["nside_x"]),
                                         int(g["nside_y"]), float(g["Lx"]), float(g["Ly"]), ctx=gpu_ctx)
    assert rel_max(ur, g["real"]) <= TOL
    uk = ft.mex_stokes_slp_gradient_kspace(g["psrc"], g["ptar"], float(g["xi"]), float(g["eta"]), g["f"],
                                           int(g["Mx"]), int(g["My"]), float(g["Lx"]), float(g["Ly"]), float(g["w"]),
                                           int(g["P"]), ctx=gpu_ctx)
    assert rel_max(uk, g["kspace"]) <= TOL


def test_unknown_quantity_is_rejected(gpu_ctx):
    ft = _ft()
    ps = np.zeros((4, 2))
    with pytest.raises(ft.FteError):
        ft.q_real(0, 9, ps, ps, ps, None, 10.0, 2, 2, 1.0, 1.0, ctx=gpu_ctx)


DRV = golden_names("quant_drv_")


@pytest.mark.parametrize("name", DRV)
def test_quantity_drivers_match_reference(gpu_ctx, name):
    """StokesSLP/DLP_<q>_ewald_2p on the GPU against the drivers built on the
    reference's gateways: targets equal to the sources (self terms) and
    separate targets."""
    ft = _ft()
    g = load_golden(name)
    kind, q = int(g["kind"]), int(g["quantity"])
    for i in (0, 1):
        d = {k[3:]: g[k] for k in g if k.startswith(f"c{i}_")}
        (o, r, k, xi), info = ft.q_ewald_2p(kind, q, d["xsrc"], d["ysrc"], d["xtar"], d["ytar"], d["f1"], d["f2"],
                                            float(d["Lx"]), float(d["Ly"]), n1=d["n1"], n2=d["n2"], b1=d["b1"],
                                            b2=d["b2"], tol=float(d["tol"]), ctx=gpu_ctx, return_info=True)
        assert xi == pytest.approx(float(d["xi"]), rel=1e-14) and info.params.Mx == int(d["Mx"])
        assert rel_max(o, d["out"]) <= TOL, (name, i)
        assert rel_max(r, d["out_real"]) <= TOL and rel_max(k, d["out_k"]) <= TOL, (name, i)


def test_named_quantity_drivers(gpu_ctx):
    ft = _ft()
    g = load_golden("quant_drv_dlp_stress")
    d = {k[3:]: g[k] for k in g if k.startswith("c0_")}
    s1, s2, sr, sk, xi = ft.StokesDLP_stress_ewald_2p(d["xsrc"], d["ysrc"], d["xtar"], d["ytar"], d["n1"], d["n2"],
                                                      d["f1"], d["f2"], d["b1"], d["b2"], float(d["Lx"]),
                                                      float(d["Ly"]), tol=float(d["tol"]), ctx=gpu_ctx)
    assert rel_max(np.stack([s1, s2], 1), d["out"]) <= TOL
    g = load_golden("quant_drv_slp_pressure")
    d = {k[3:]: g[k] for k in g if k.startswith("c1_")}
    p, pr, pk, xi = ft.StokesSLP_pressure_ewald_2p(d["xsrc"], d["ysrc"], d["xtar"], d["ytar"], d["f1"], d["f2"],
                                                   float(d["Lx"]), float(d["Ly"]), tol=float(d["tol"]), ctx=gpu_ctx)
    assert rel_max(p, d["out"]) <= TOL
