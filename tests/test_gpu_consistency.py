"""The reference's consistency tests, restated with thresholds, on the GPU
library.

* Cell-count (Nb) invariance: Nb in {3, 9, 27} changes the cutoff, xi and
  the grid, but not the velocities
  (PeriodicEwald/tests/consistency_checks/consistency_test_velocity.m:54-76,
  130-152).
* Periodic replicate: doubling Lx with the sources duplicated at x + Lx gives
  the same velocities; for the stresslet after subtracting each evaluation's
  k = 0 mode, sum((f.n) x_wrapped) / (Lx Ly), which depends on where the
  sources are (:78-94, :154-194, zero mode :162-169, 184-191).
* Stresslet identity: 256 trapezoidal points on the unit circle in a 4 x 4
  box with f = h e_i (the quadrature weight folded into the density): the
  velocity is e_i at 16 targets on r = 0.5 and 0 at 16 targets on r = 1.5
  (PeriodicEwald/tests/stresslet_identity_test.m:23-78).

Setup as the reference: N = 10^4 sources and targets in the Lx = 1, Ly = 2
box, f = 10 rand, n1 = rand, n2 = sqrt(1 - n1^2), the drivers' default
tolerance 1e-16 (plain FP64 form); the mixed form is held to its tolerance.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

NB = (3, 9, 27)


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(20260101)
    N, Lx, Ly = 10000, 1.0, 2.0
    n1 = rng.random(N)
    return dict(N=N, Lx=Lx, Ly=Ly, xs=Lx * rng.random(N), ys=Ly * rng.random(N), xt=Lx * rng.random(N),
                yt=Ly * rng.random(N), f1=10 * rng.random(N), f2=10 * rng.random(N), n1=n1, n2=np.sqrt(1 - n1 ** 2))


def _eval(ft, ctx, kind, d, xs, ys, f1, f2, n1, n2, Lx, **kw):
    if kind == "slp":
        u = ft.StokesSLP_ewald_2p(xs, ys, d["xt"], d["yt"], f1, f2, Lx, d["Ly"], ctx=ctx, parts=False, **kw)
    else:
        u = ft.StokesDLP_ewald_2p(xs, ys, d["xt"], d["yt"], n1, n2, f1, f2, Lx, d["Ly"], ctx=ctx, parts=False, **kw)
    return np.stack([np.asarray(u[0]), np.asarray(u[1])], 1)


def _zero_mode(xs, ys, f1, f2, n1, n2, Lx, Ly):
    fn = f1 * n1 + f2 * n2
    return np.array([np.sum(fn * po.matlab_wrap(xs, Lx)), np.sum(fn * po.matlab_wrap(ys, Ly))]) / (Lx * Ly)


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_nb_invariance(gpu_ctx, data, kind):
    import fasttools2d_gb300 as ft

    d = data
    us = [_eval(ft, gpu_ctx, kind, d, d["xs"], d["ys"], d["f1"], d["f2"], d["n1"], d["n2"], d["Lx"], Nb=nb)
          for nb in NB]
    scale = max(np.abs(u).max() for u in us)
    worst = max(np.abs(a - b).max() for a in us for b in us)
    assert worst <= 1e-11 * scale, worst / scale


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("form,tol,bound", [("plain", 1e-16, 1e-11), ("mixed", 1e-10, 4e-10)])
def test_periodic_replicate(gpu_ctx, data, kind, form, tol, bound):
    import fasttools2d_gb300 as ft

    d = data
    fm = ft.FORM_PLAIN if form == "plain" else ft.FORM_MIXED
    Lx, Ly = d["Lx"], d["Ly"]
    u1 = _eval(ft, gpu_ctx, kind, d, d["xs"], d["ys"], d["f1"], d["f2"], d["n1"], d["n2"], Lx, tol=tol, form=fm)
    xs2 = np.concatenate([d["xs"], d["xs"] + Lx])
    ys2 = np.concatenate([d["ys"], d["ys"]])
    f1, f2, n1, n2 = (np.concatenate([d[k], d[k]]) for k in ("f1", "f2", "n1", "n2"))
    u2 = _eval(ft, gpu_ctx, kind, d, xs2, ys2, f1, f2, n1, n2, 2 * Lx, tol=tol, form=fm)
    if kind == "dlp":
        u1 = u1 - _zero_mode(d["xs"], d["ys"], d["f1"], d["f2"], d["n1"], d["n2"], Lx, Ly)
        u2 = u2 - _zero_mode(xs2, ys2, f1, f2, n1, n2, 2 * Lx, Ly)
    err = np.abs(u1 - u2).max() / np.abs(u1).max()
    assert err <= bound, err


@pytest.mark.parametrize("comp", [0, 1])
@pytest.mark.parametrize("form,tol,bound", [("plain", 1e-16, 1e-13), ("mixed", 1e-10, 2e-10)])
def test_stresslet_identity(gpu_ctx, comp, form, tol, bound):
    import fasttools2d_gb300 as ft

    r, Nsrc, Ntar = 1.0, 256, 16
    h = 2 * np.pi / Nsrc
    th = h * np.arange(1, Nsrc + 1)
    xs, ys = r * np.cos(th), r * np.sin(th)
    f = [np.zeros(Nsrc), np.zeros(Nsrc)]
    f[comp] = h * np.ones(Nsrc)
    tt = 2 * np.pi / Ntar * np.arange(1, Ntar + 1)
    xt = np.concatenate([0.5 * r * np.cos(tt), 1.5 * r * np.cos(tt)])
    yt = np.concatenate([0.5 * r * np.sin(tt), 1.5 * r * np.sin(tt)])
    fm = ft.FORM_PLAIN if form == "plain" else ft.FORM_MIXED
    u1, u2 = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, np.cos(th), np.sin(th), f[0], f[1], 4 * r, 4 * r, tol=tol,
                                   form=fm, ctx=gpu_ctx, parts=False)[:2]
    u = np.stack([np.asarray(u1), np.asarray(u2)], 1)
    e = np.zeros(2)
    e[comp] = 1.0
    assert np.abs(u[:Ntar] - e).max() <= bound
    assert np.abs(u[Ntar:]).max() <= bound
