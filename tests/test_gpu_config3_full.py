"""The headline workload at its full size: 10^6 sources and 10^6 targets
uniform in the unit box, zero-mean N(0,1) densities, unit normals at random
angles (fasttools2d_gb300.workloads.config3), Stokeslet and stresslet.

* plain form (FP64, the drivers' parameters), tol 1e-10: the near-field and
  k-space parts at 2,000 sampled targets against the oracle's gateways on
  the same parameters, to 1e-12 of the parts' maxima (same arithmetic,
  different summation order);
* plain and mixed forms at tol 1e-6 and 1e-10: the velocities at the 10,000
  sampled targets of tests/golden/truth_config3.npz (converged FP64 Ewald
  sums, own xi, truncations below e^-40) within the tolerance:
  max |u - u_truth| / max |u_truth| <= tol.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


@pytest.fixture(scope="module")
def cfg3():
    from fasttools2d_gb300 import workloads as wl

    c = wl.config3()
    truth = load_golden("truth_config3")
    keys = ("xsrc", "ysrc", "xtar", "ytar", "f1", "f2", "n1", "n2")
    ck = wl.checksum(*(c[k] for k in keys))
    assert abs(ck - float(truth["checksum"])) <= 1e-9 * abs(float(truth["checksum"])), "inputs differ from the truth's"
    c["truth"] = truth
    rng = np.random.default_rng(33)
    c["sub"] = np.sort(rng.choice(len(c["xtar"]), size=2000, replace=False))
    return c


def _run(ft, ctx, kind, c, **kw):
    a = (c["xsrc"], c["ysrc"], c["xtar"], c["ytar"])
    if kind == "slp":
        return ft.StokesSLP_ewald_2p(*a, c["f1"], c["f2"], 1.0, 1.0, ctx=ctx, return_info=True, **kw)
    return ft.StokesDLP_ewald_2p(*a, c["n1"], c["n2"], c["f1"], c["f2"], 1.0, 1.0, ctx=ctx, return_info=True, **kw)


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_config3_plain_parts_match_oracle(gpu_ctx, cfg3, kind):
    import fasttools2d_gb300 as ft

    c = cfg3
    (u1, u2, ur, uk, xi), info = _run(ft, gpu_ctx, kind, c, tol=1e-10)
    p = info.params
    assert (p.Mx, p.My) == ((1072, 1072) if kind == "slp" else (1360, 1360))  # the drivers' grids at 1e6, 1e-10
    idx = c["sub"]
    ps = np.stack([po.matlab_wrap(c["xsrc"], 1.0), po.matlab_wrap(c["ysrc"], 1.0)], 1)
    pt = np.stack([po.matlab_wrap(c["xtar"][idx], 1.0), po.matlab_wrap(c["ytar"][idx], 1.0)], 1)
    f = np.stack([c["f1"], c["f2"]], 1)
    n = np.stack([c["n1"], c["n2"]], 1)
    if kind == "slp":
        our = po.slp_real(ps, pt, f, p.xi, p.nside_x, p.nside_y, 1.0, 1.0)
        ouk = po.slp_kspace(ps, pt, p.xi, p.eta, f, p.Mx, p.My, 1.0, 1.0, p.w, p.P)
    else:
        our = po.dlp_real(ps, pt, f, n, p.xi, p.nside_x, p.nside_y, 1.0, 1.0)
        ouk = po.dlp_kspace(ps, pt, p.xi, p.eta, f, n, p.Mx, p.My, 1.0, 1.0, p.w, p.P)
        fn = f[:, 0] * n[:, 0] + f[:, 1] * n[:, 1]
        ouk = ouk + (fn[:, None] * ps).sum(0)  # the drivers' zero mode (Lx Ly = 1)
    assert np.max(np.abs(ur[idx] - our)) <= TOL_FP64 * np.max(np.abs(our))
    assert np.max(np.abs(uk[idx] - ouk)) <= TOL_FP64 * np.max(np.abs(ouk))


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_config3_meets_tolerance(gpu_ctx, cfg3, form, tol):
    import fasttools2d_gb300 as ft

    c = cfg3
    t = c["truth"]
    fm = ft.FORM_PLAIN if form == "plain" else ft.FORM_MIXED
    for kind in ("slp", "dlp"):
        (u1, u2, _, _, _), info = _run(ft, gpu_ctx, kind, c, tol=tol, form=fm, parts=False)
        u = np.stack([np.asarray(u1)[t["idx"]], np.asarray(u2)[t["idx"]]], 1)
        err = np.max(np.abs(u - t[kind])) / np.max(np.abs(t[kind]))
        assert err <= tol, (kind, form, tol, err, info.params.as_dict())
