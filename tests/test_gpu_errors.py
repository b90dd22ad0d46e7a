"""Error paths of the C ABI, made on the host: no kernel faults, traps or hangs.

* Non-finite inputs (NaN or Inf in a coordinate, a density, a normal or a
  weight) are rejected with FTE_ERR_INVALID before any compute kernel runs,
  by every entry that takes them (gateways, drivers, quantities, plans).  The
  reference checks shapes only (PeriodicEwald/src/mex/StokesDLP/
  mex_stokes_dlp_kspace.cpp:12-26) and would return NaNs; the message names
  the entry and the count.
* A device allocation that fails (forced on the host by
  fte_debug_fail_alloc, the test hook of include/fasttools2d_debug.h) makes
  the entry return FTE_ERR_ALLOC, and the same context then evaluates the
  next call correctly.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu


def _case(n=600, seed=5):
    rng = np.random.default_rng(seed)
    xs, ys, xt, yt = (rng.random(n) for _ in range(4))
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    th = rng.random(n) * 2 * np.pi
    return dict(xs=xs, ys=ys, xt=xt, yt=yt, f1=f1, f2=f2, n1=np.cos(th), n2=np.sin(th), w=np.full(n, 0.5))


def _spoil(c, key, value, at=17):
    d = {k: v.copy() for k, v in c.items()}
    d[key][at] = value
    return d


def _slp(ft, ctx, c, **kw):
    return ft.StokesSLP_ewald_2p(c["xs"], c["ys"], c["xt"], c["yt"], c["f1"], c["f2"], 1.0, 1.0, tol=1e-8, ctx=ctx,
                                 **kw)


def _dlp(ft, ctx, c, **kw):
    return ft.StokesDLP_ewald_2p(c["xs"], c["ys"], c["xt"], c["yt"], c["n1"], c["n2"], c["f1"], c["f2"], 1.0, 1.0,
                                 tol=1e-8, ctx=ctx, **kw)


@pytest.mark.parametrize("key", ["xs", "yt", "f1", "f2", "n1", "n2", "w"])
@pytest.mark.parametrize("value", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_drivers_reject_non_finite_inputs(gpu_ctx, key, value, form):
    import fasttools2d_gb300 as ft

    fm = ft.FORM_PLAIN if form == "plain" else ft.FORM_MIXED
    c = _case()
    bad = _spoil(c, key, value)
    calls = [lambda d: _dlp(ft, gpu_ctx, d, weights=d["w"], form=fm)]
    if key not in ("n1", "n2"):
        calls.append(lambda d: _slp(ft, gpu_ctx, d, weights=d["w"], form=fm))
    for call in calls:
        with pytest.raises(ft.FteError) as e:
            call(bad)
        assert e.value.code == ft.FTE_ERR_INVALID
        assert "non-finite" in str(e.value)
    # the context is unharmed: the clean input still matches a fresh context's
    # evaluation (to rounding in the FP64 form; the mixed form's FP32 and
    # float-float sums may differ in their last bits between runs, so to
    # within its tolerance)
    u = _dlp(ft, gpu_ctx, c, weights=c["w"], form=fm)
    ref = _dlp(ft, ft.Context(0), c, weights=c["w"], form=fm)
    assert rel_max(np.stack(u[:2]), np.stack(ref[:2])) <= (1e-13 if form == "plain" else 1e-8)


def test_gateways_reject_non_finite_inputs(gpu_ctx):
    import fasttools2d_gb300 as ft

    c = _case()
    ps = np.stack([c["xs"] - 0.5, c["ys"] - 0.5], 1)
    pt = np.stack([c["xt"] - 0.5, c["yt"] - 0.5], 1)
    f = np.stack([c["f1"], c["f2"]], 1)
    n = np.stack([c["n1"], c["n2"]], 1)
    prm = ft.choose_params(ft.KIND_SLP, c["f1"], c["f2"], len(pt), 1.0, 1.0, P=24, tol=1e-8)
    xi, nx, ny, eta, Mx, My, w, P = prm.xi, prm.nside_x, prm.nside_y, prm.eta, prm.Mx, prm.My, prm.w, prm.P
    for arr in ("ps", "pt", "f", "n"):
        a = {"ps": ps.copy(), "pt": pt.copy(), "f": f.copy(), "n": n.copy()}
        a[arr][3, 1] = np.nan
        calls = [lambda: ft.mex_stokes_dlp_real(a["ps"], a["pt"], a["f"], a["n"], xi, nx, ny, 1.0, 1.0, ctx=gpu_ctx),
                 lambda: ft.mex_stokes_dlp_kspace(a["ps"], a["pt"], xi, eta, a["f"], a["n"], Mx, My, 1.0, 1.0, w, P,
                                                  ctx=gpu_ctx)]
        if arr != "n":
            calls += [lambda: ft.mex_stokes_slp_real(a["ps"], a["pt"], a["f"], xi, nx, ny, 1.0, 1.0, ctx=gpu_ctx),
                      lambda: ft.mex_stokes_slp_kspace(a["ps"], a["pt"], xi, eta, a["f"], Mx, My, 1.0, 1.0, w, P,
                                                       ctx=gpu_ctx)]
        for call in calls:
            with pytest.raises(ft.FteError) as e:
                call()
            assert e.value.code == ft.FTE_ERR_INVALID and "non-finite" in str(e.value)
    # quantity gateways and plans take the same path
    bad_f = f.copy()
    bad_f[0, 0] = np.inf
    with pytest.raises(ft.FteError) as e:
        ft.mex_stokes_slp_pressure_real(ps, pt, bad_f, xi, nx, ny, 1.0, 1.0, ctx=gpu_ctx)
    assert e.value.code == ft.FTE_ERR_INVALID
    bad = _spoil(c, "xt", np.nan)
    with pytest.raises(ft.FteError) as e:
        ft.Plan(ft.KIND_SLP, bad["xs"], bad["ys"], bad["xt"], bad["yt"], bad["f1"], bad["f2"], 1.0, 1.0, tol=1e-8,
                ctx=gpu_ctx)
    assert e.value.code == ft.FTE_ERR_INVALID
    # and the context still works
    u = ft.mex_stokes_slp_real(ps, pt, f, xi, nx, ny, 1.0, 1.0, ctx=gpu_ctx)
    assert np.all(np.isfinite(u))


def _fail_alloc(ft, after):
    fn = ft.lib().fte_debug_fail_alloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int]
    assert fn(after) == ft.FTE_OK


@pytest.mark.parametrize("after", [1, 2])
def test_allocation_failure_is_reported_and_recovered(after):
    """A fresh context has no workspace yet: its first driver call allocates
    the staging workspace (allocation 1) and then the grid workspace
    (allocation 2).  Either failing gives FTE_ERR_ALLOC; the next call on the
    same context allocates again and returns the right velocities."""
    import fasttools2d_gb300 as ft

    c = _case(n=800, seed=9)
    ctx = ft.Context(0)
    _fail_alloc(ft, after)
    try:
        with pytest.raises(ft.FteError) as e:
            _dlp(ft, ctx, c)
        assert e.value.code == ft.FTE_ERR_ALLOC
        assert "could not be allocated" in str(e.value)
    finally:
        _fail_alloc(ft, 0)
    u = _dlp(ft, ctx, c)
    ref = _dlp(ft, ft.Context(0), c)
    assert rel_max(np.stack(u[:2]), np.stack(ref[:2])) <= 1e-13


def test_plan_allocation_failure_is_reported(gpu_ctx):
    import fasttools2d_gb300 as ft

    c = _case(n=700, seed=11)
    # warm the context so that the plan's own memory is the next allocation
    _slp(ft, gpu_ctx, c)
    _fail_alloc(ft, 1)
    try:
        with pytest.raises(ft.FteError) as e:
            ft.Plan(ft.KIND_SLP, c["xs"], c["ys"], c["xt"], c["yt"], c["f1"], c["f2"], 1.0, 1.0, tol=1e-8,
                    ctx=gpu_ctx)
        assert e.value.code == ft.FTE_ERR_ALLOC
    finally:
        _fail_alloc(ft, 0)
    p = ft.Plan(ft.KIND_SLP, c["xs"], c["ys"], c["xt"], c["yt"], c["f1"], c["f2"], 1.0, 1.0, tol=1e-8, ctx=gpu_ctx)
    u = p.execute(c["f1"][None], c["f2"][None])
    ref = _slp(ft, gpu_ctx, c)
    assert rel_max(np.stack([u[0][0], u[1][0]]), np.stack(ref[:2])) <= 1e-12
    p.close()
