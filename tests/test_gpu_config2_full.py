"""Config 2 at its full size: box 2 x 1, 40 ellipses x 256 boundary points
(10,240 sources with trapezoidal weights and outward normals), 534,528
targets (a 1024 x 512 grid plus every boundary point), tolerance 1e-10.

* plain form (FP64): the near-field and k-space parts at 2,000 sampled
  targets against the oracle's gateways on the same parameters, to 1e-12 of
  the parts' maxima (same arithmetic, different summation order);
* plain and mixed forms: the velocities at 300 sampled targets against the
  converged FP64 Ewald sum (own xi, truncations below e^-40, the stresslet's
  zero mode included as the drivers add it): max error at most the
  tolerance times the maximum velocity.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


@pytest.fixture(scope="module")
def cfg2():
    from fasttools2d_gb300 import workloads as wl

    c = wl.config2()
    assert len(c["xsrc"]) == 10240 and len(c["xtar"]) == 534528
    rng = np.random.default_rng(22)
    c["sub"] = np.sort(rng.choice(len(c["xtar"]), size=2000, replace=False))
    c["sub_truth"] = c["sub"][::7][:300]
    return c


def _run(ft, ctx, kind, c, **kw):
    a = (c["xsrc"], c["ysrc"], c["xtar"], c["ytar"])
    if kind == "slp":
        return ft.StokesSLP_ewald_2p(*a, c["f1"], c["f2"], c["Lx"], c["Ly"], tol=c["tol"], weights=c["weights"],
                                     ctx=ctx, return_info=True, **kw)
    return ft.StokesDLP_ewald_2p(*a, c["n1"], c["n2"], c["f1"], c["f2"], c["Lx"], c["Ly"], tol=c["tol"],
                                 weights=c["weights"], ctx=ctx, return_info=True, **kw)


def _wrapped(c, idx):
    Lx, Ly = c["Lx"], c["Ly"]
    ps = np.stack([po.matlab_wrap(c["xsrc"], Lx), po.matlab_wrap(c["ysrc"], Ly)], 1)
    pt = np.stack([po.matlab_wrap(c["xtar"][idx], Lx), po.matlab_wrap(c["ytar"][idx], Ly)], 1)
    return ps, pt


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_config2_full_parts_match_oracle(gpu_ctx, cfg2, kind):
    import fasttools2d_gb300 as ft

    c = cfg2
    (u1, u2, ur, uk, xi), info = _run(ft, gpu_ctx, kind, c)
    p = info.params
    assert ur.shape == (534528, 2) and uk.shape == (534528, 2)
    ps, pt = _wrapped(c, c["sub"])
    w = c["weights"]
    f = np.stack([c["f1"] * w, c["f2"] * w], 1)
    n = np.stack([c["n1"], c["n2"]], 1)
    if kind == "slp":
        our = po.slp_real(ps, pt, f, p.xi, p.nside_x, p.nside_y, c["Lx"], c["Ly"])
        ouk = po.slp_kspace(ps, pt, p.xi, p.eta, f, p.Mx, p.My, c["Lx"], c["Ly"], p.w, p.P)
    else:
        our = po.dlp_real(ps, pt, f, n, p.xi, p.nside_x, p.nside_y, c["Lx"], c["Ly"])
        ouk = po.dlp_kspace(ps, pt, p.xi, p.eta, f, n, p.Mx, p.My, c["Lx"], c["Ly"], p.w, p.P)
        # the drivers' zero mode (StokesDLP_ewald_2p.m:149-151) is part of uk:
        # sum over sources of (f . n) times the wrapped position, over Lx Ly
        fn = f[:, 0] * n[:, 0] + f[:, 1] * n[:, 1]
        ouk = ouk + (fn[:, None] * ps).sum(0) / (c["Lx"] * c["Ly"])
    assert np.max(np.abs(ur[c["sub"]] - our)) <= TOL_FP64 * np.max(np.abs(our))
    assert np.max(np.abs(uk[c["sub"]] - ouk)) <= TOL_FP64 * np.max(np.abs(ouk))


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_config2_full_meets_tolerance(gpu_ctx, cfg2, kind, form):
    import fasttools2d_gb300 as ft

    c = cfg2
    fm = ft.FORM_PLAIN if form == "plain" else ft.FORM_MIXED
    (u1, u2, _, _, _), _ = _run(ft, gpu_ctx, kind, c, form=fm, parts=False)
    idx = c["sub_truth"]
    ps, pt = _wrapped(c, idx)
    w = c["weights"]
    n1, n2 = (c["n1"], c["n2"]) if kind == "dlp" else (None, None)
    t = po.ewald_truth(0 if kind == "slp" else 1, ps[:, 0], ps[:, 1], pt[:, 0], pt[:, 1], c["f1"] * w,
                       c["f2"] * w, c["Lx"], c["Ly"], n1, n2)
    u = np.stack([np.asarray(u1)[idx], np.asarray(u2)[idx]], 1)
    err = np.max(np.abs(u - t)) / np.max(np.abs(t))
    assert err <= c["tol"], err

