"""The reference's consistency tests, restated with thresholds, on the CPU
oracle (the C restatement of the reference's path, pinned to the reference's
own gateways by tests/test_oracle.py).  The same checks run on the GPU
library at the reference's sizes in tests/test_gpu_consistency.py.

* Nb invariance (PeriodicEwald/tests/consistency_checks/consistency_test_velocity.m:54-76,130-152)
* periodic replicate with the stresslet's zero mode subtracted (:78-94, :154-194)
* stresslet identity (PeriodicEwald/tests/stresslet_identity_test.m:23-78)

Sizes here are small enough for the CPU (600 points, tol 1e-12).
"""
import numpy as np
import pytest

from oracle import pyoracle as po


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(77)
    N, Lx, Ly = 600, 1.0, 2.0
    n1 = rng.random(N)
    return dict(Lx=Lx, Ly=Ly, xs=Lx * rng.random(N), ys=Ly * rng.random(N), xt=Lx * rng.random(N),
                yt=Ly * rng.random(N), f1=10 * rng.random(N), f2=10 * rng.random(N), n1=n1, n2=np.sqrt(1 - n1 ** 2))


def _eval(kind, d, xs, ys, f1, f2, n1, n2, Lx, **kw):
    if kind == "slp":
        u = po.stokes_slp_ewald_2p(xs, ys, d["xt"], d["yt"], f1, f2, Lx, d["Ly"], **kw)
    else:
        u = po.stokes_dlp_ewald_2p(xs, ys, d["xt"], d["yt"], n1, n2, f1, f2, Lx, d["Ly"], **kw)
    return np.stack([u[0], u[1]], 1)


def _zero_mode(xs, ys, f1, f2, n1, n2, Lx, Ly):
    fn = f1 * n1 + f2 * n2
    return np.array([np.sum(fn * po.matlab_wrap(xs, Lx)), np.sum(fn * po.matlab_wrap(ys, Ly))]) / (Lx * Ly)


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_oracle_nb_invariance(data, kind):
    d = data
    us = [_eval(kind, d, d["xs"], d["ys"], d["f1"], d["f2"], d["n1"], d["n2"], d["Lx"], Nb=nb, tol=1e-12)
          for nb in (3, 9, 27)]
    scale = max(np.abs(u).max() for u in us)
    assert max(np.abs(a - b).max() for a in us for b in us) <= 3e-12 * scale


@pytest.mark.parametrize("kind", ["slp", "dlp"])
def test_oracle_periodic_replicate(data, kind):
    d = data
    Lx, Ly = d["Lx"], d["Ly"]
    u1 = _eval(kind, d, d["xs"], d["ys"], d["f1"], d["f2"], d["n1"], d["n2"], Lx, tol=1e-12)
    xs2 = np.concatenate([d["xs"], d["xs"] + Lx])
    ys2 = np.concatenate([d["ys"], d["ys"]])
    f1, f2, n1, n2 = (np.concatenate([d[k], d[k]]) for k in ("f1", "f2", "n1", "n2"))
    u2 = _eval(kind, d, xs2, ys2, f1, f2, n1, n2, 2 * Lx, tol=1e-12)
    if kind == "dlp":
        u1 = u1 - _zero_mode(d["xs"], d["ys"], d["f1"], d["f2"], d["n1"], d["n2"], Lx, Ly)
        u2 = u2 - _zero_mode(xs2, ys2, f1, f2, n1, n2, 2 * Lx, Ly)
    assert np.abs(u1 - u2).max() <= 3e-12 * np.abs(u1).max()


@pytest.mark.parametrize("comp", [0, 1])
def test_oracle_stresslet_identity(comp):
    r, Nsrc, Ntar = 1.0, 256, 16
    h = 2 * np.pi / Nsrc
    th = h * np.arange(1, Nsrc + 1)
    f = [np.zeros(Nsrc), np.zeros(Nsrc)]
    f[comp] = h * np.ones(Nsrc)
    tt = 2 * np.pi / Ntar * np.arange(1, Ntar + 1)
    xt = np.concatenate([0.5 * np.cos(tt), 1.5 * np.cos(tt)])
    yt = np.concatenate([0.5 * np.sin(tt), 1.5 * np.sin(tt)])
    u1, u2 = po.stokes_dlp_ewald_2p(r * np.cos(th), r * np.sin(th), xt, yt, np.cos(th), np.sin(th), f[0], f[1],
                                    4 * r, 4 * r)[:2]
    u = np.stack([u1, u2], 1)
    e = np.zeros(2)
    e[comp] = 1.0
    assert np.abs(u[:Ntar] - e).max() <= 1e-13
    assert np.abs(u[Ntar:]).max() <= 1e-13


@pytest.mark.parametrize("comp", [0, 1])
def test_reference_fixture_satisfies_stresslet_identity(comp):
    """The reference's own output (the compiled gateways, stored in
    tests/golden) meets the identity's analytic answer."""
    from conftest import load_golden

    g = load_golden(f"stresslet_identity_e{comp + 1}")
    u = g["dlp_u"]
    n = len(u) // 2
    e = np.zeros(2)
    e[comp] = 1.0
    assert np.abs(u[:n] - e).max() <= 1e-13
    assert np.abs(u[n:]).max() <= 1e-13
