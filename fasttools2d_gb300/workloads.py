"""Seeded synthetic inputs of the benchmark configurations.

All generators use numpy's PCG64 (``np.random.default_rng(seed)``) so the
same arrays are produced on every machine.

* ``config1``: Stokeslet, [0,1]^2, 1000 sources / 1000 separate targets,
  i.i.d. uniform; f ~ N(0,1)^2 with the mean removed; tol 1e-10.
* ``config2``: box 2 x 1, 40 non-overlapping ellipses (semi-axes U[0.02,0.06],
  random orientation), 256 equispaced-theta points each with outward unit
  normals and trapezoid weights; densities N(0,1) 2-vectors (weights folded
  in by the caller); targets = 1024 x 512 cell-centred grid plus every
  boundary point; tol 1e-10.
* ``config3``: 10^6 sources / 10^6 targets uniform in [0,1]^2, zero-mean
  N(0,1) densities, unit normals at uniform random angles; tol 1e-6 and 1e-10.
* ``config4``: batched configurations, N log-uniform in [2e3, 2e5], aspect
  ratio p/4 in [1, 4], half uniform points and half on ellipses; 4 density
  vectors each; tol 1e-8.
"""
from __future__ import annotations

import numpy as np


def _zero_mean(a):
    return a - a.mean()


def config1(seed: int = 1):
    rng = np.random.default_rng(seed)
    N = 1000
    xs, ys, xt, yt = (rng.random(N) for _ in range(4))
    f1 = _zero_mean(rng.standard_normal(N))
    f2 = _zero_mean(rng.standard_normal(N))
    th = rng.random(N) * 2 * np.pi
    return dict(xsrc=xs, ysrc=ys, xtar=xt, ytar=yt, f1=f1, f2=f2, n1=np.cos(th), n2=np.sin(th), Lx=1.0, Ly=1.0,
                tol=1e-10)


def ellipses(rng, n_ell, n_per, Lx, Ly, amin, amax, margin=0.01, max_tries=100000):
    """Non-overlapping ellipses (minimum-image centre distance > a1 + a2 +
    margin) discretised at equispaced theta; returns x, y, n1, n2, weights."""
    cs, axes = [], []
    tries = 0
    while len(cs) < n_ell and tries < max_tries:
        tries += 1
        c = np.array([(rng.random() - 0.5) * Lx, (rng.random() - 0.5) * Ly])
        a = rng.uniform(amin, amax, size=2)
        ok = True
        for c2, a2 in zip(cs, axes):
            d = c - c2
            d[0] -= Lx * np.round(d[0] / Lx)
            d[1] -= Ly * np.round(d[1] / Ly)
            if np.hypot(*d) <= a.max() + a2.max() + margin:
                ok = False
                break
        if ok:
            cs.append(c)
            axes.append(a)
    th = 2 * np.pi * np.arange(n_per) / n_per
    X, Y, N1, N2, W = [], [], [], [], []
    for c, a in zip(cs, axes):
        rot = rng.uniform(0, np.pi)
        cr, sr = np.cos(rot), np.sin(rot)
        ex, ey = a[0] * np.cos(th), a[1] * np.sin(th)
        dx, dy = -a[0] * np.sin(th), a[1] * np.cos(th)
        X.append(c[0] + cr * ex - sr * ey)
        Y.append(c[1] + sr * ex + cr * ey)
        tx, ty = cr * dx - sr * dy, sr * dx + cr * dy
        sp = np.hypot(tx, ty)
        N1.append(ty / sp)
        N2.append(-tx / sp)
        W.append(2 * np.pi / n_per * sp)
    return (np.concatenate(X), np.concatenate(Y), np.concatenate(N1), np.concatenate(N2), np.concatenate(W))


def config2(seed: int = 2, n_ell: int = 40, n_per: int = 256, grid=(1024, 512)):
    rng = np.random.default_rng(seed)
    Lx, Ly = 2.0, 1.0
    X, Y, N1, N2, W = ellipses(rng, n_ell, n_per, Lx, Ly, 0.02, 0.06)
    f1 = rng.standard_normal(len(X))
    f2 = rng.standard_normal(len(X))
    gx, gy = np.meshgrid((np.arange(grid[0]) + 0.5) / grid[0] * Lx - Lx / 2,
                         (np.arange(grid[1]) + 0.5) / grid[1] * Ly - Ly / 2, indexing="ij")
    xt = np.concatenate([gx.ravel(), X])
    yt = np.concatenate([gy.ravel(), Y])
    return dict(xsrc=X, ysrc=Y, xtar=xt, ytar=yt, f1=f1, f2=f2, n1=N1, n2=N2, weights=W, Lx=Lx, Ly=Ly, tol=1e-10)


def config3(seed: int = 3, n: int = 1_000_000):
    rng = np.random.default_rng(seed)
    xs, ys, xt, yt = (rng.random(n) for _ in range(4))
    f1 = _zero_mean(rng.standard_normal(n))
    f2 = _zero_mean(rng.standard_normal(n))
    th = rng.random(n) * 2 * np.pi
    return dict(xsrc=xs, ysrc=ys, xtar=xt, ytar=yt, f1=f1, f2=f2, n1=np.cos(th), n2=np.sin(th), Lx=1.0, Ly=1.0)


def config3_sample(n: int = 1_000_000, count: int = 10_000, seed: int = 33):
    """Indices of the targets on which config 3's errors are measured."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=count, replace=False))


def ellipse_field(rng, n_ell, n_per, Lx, Ly, amin, amax, margin=0.01):
    """Like ``ellipses`` (same geometry rules), with a vectorised overlap test
    and at most 50 placement attempts per ellipse, so that a crowded box
    returns fewer ellipses instead of searching for long."""
    cs = np.zeros((0, 2))
    rad = np.zeros(0)
    axes = []
    for _ in range(50 * n_ell):
        if len(axes) == n_ell:
            break
        c = np.array([(rng.random() - 0.5) * Lx, (rng.random() - 0.5) * Ly])
        a = rng.uniform(amin, amax, size=2)
        d = cs - c
        d[:, 0] -= Lx * np.round(d[:, 0] / Lx)
        d[:, 1] -= Ly * np.round(d[:, 1] / Ly)
        if np.all(np.hypot(d[:, 0], d[:, 1]) > a.max() + rad + margin):
            cs = np.vstack([cs, c])
            rad = np.append(rad, a.max())
            axes.append(a)
    th = 2 * np.pi * np.arange(n_per) / n_per
    X, Y, N1, N2, W = [], [], [], [], []
    for c, a in zip(cs, axes):
        rot = rng.uniform(0, np.pi)
        cr, sr = np.cos(rot), np.sin(rot)
        ex, ey = a[0] * np.cos(th), a[1] * np.sin(th)
        dx, dy = -a[0] * np.sin(th), a[1] * np.cos(th)
        X.append(c[0] + cr * ex - sr * ey)
        Y.append(c[1] + sr * ex + cr * ey)
        tx, ty = cr * dx - sr * dy, sr * dx + cr * dy
        sp = np.hypot(tx, ty)
        N1.append(ty / sp)
        N2.append(-tx / sp)
        W.append(2 * np.pi / n_per * sp)
    return (np.concatenate(X), np.concatenate(Y), np.concatenate(N1), np.concatenate(N2), np.concatenate(W))


def config4(seed: int = 4, count: int = 64, nvec: int = 4):
    """Batched workload: ``count`` independent configurations, N log-uniform
    in [2e3, 2e5], box aspect p/4 (p = 4..16, so rat(Lx/Ly) stays small),
    half the points uniform and half on non-overlapping ellipses (semi-axes
    U[0.02, 0.06]; about 256 points per ellipse, fewer ellipses with more
    points each where the box is crowded), ``nvec`` zero-mean N(0,1) density
    vectors, tolerance 1e-8; targets are the source points."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        N = int(round(np.exp(rng.uniform(np.log(2e3), np.log(2e5)))))
        p = int(rng.integers(4, 17))  # aspect ratio p/4 in [1, 4]
        Lx, Ly = p / 4.0, 1.0
        nu = N // 2
        xs = list((rng.random(nu) - 0.5) * Lx)
        ys = list((rng.random(nu) - 0.5) * Ly)
        cap = max(1, int(30 * Lx * Ly))  # ellipses that fit without a long search
        n_ell = max(1, min((N - nu) // 256, cap))
        X, Y, N1, N2, W = ellipse_field(rng, n_ell, max(16, (N - nu) // n_ell), Lx, Ly, 0.02, 0.06)
        xs = np.concatenate([xs, X])
        ys = np.concatenate([ys, Y])
        n = len(xs)
        # uniform points: random unit normals; boundary points: outward normals
        th = rng.random(nu) * 2 * np.pi
        n1 = np.concatenate([np.cos(th), N1])
        n2 = np.concatenate([np.sin(th), N2])
        f = [(_zero_mean(rng.standard_normal(n)), _zero_mean(rng.standard_normal(n))) for _ in range(nvec)]
        out.append(dict(xsrc=xs, ysrc=ys, xtar=xs.copy(), ytar=ys.copy(), n1=n1, n2=n2, f=f, Lx=Lx,
                        Ly=Ly, tol=1e-8))
    return out


def checksum(*arrays) -> float:
    """Order-sensitive checksum used to confirm that regenerated inputs match."""
    s = 0.0
    for k, a in enumerate(arrays):
        a = np.asarray(a, dtype=np.float64)
        w = np.arange(1, a.size + 1, dtype=np.float64) % 97 + 1
        s += (k + 1) * float(np.dot(a.ravel()[:100000], w[:100000]))
    return s
