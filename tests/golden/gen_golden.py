"""Generate the golden fixtures in tests/golden/*.npz.

Each fixture stores seeded inputs, the parameters the MATLAB drivers choose
for them, and the outputs of the reference's OWN compiled gateways
(PeriodicEwald/src/mex/{StokesSLP,StokesDLP}/mex_stokes_{slp,dlp}_{real,kspace}.cpp,
built unmodified under oracle/_ref by ``make -C oracle ref`` against the MEX
stand-in).  The drivers' MATLAB glue (wrapping, parameter choice, zero mode)
is the restatement in oracle/pyoracle.py.  Where the reference tests compare
against direct sums, the direct sums (restated from
PeriodicEwald/tests/direct_sums/matlab_sums/*_ds.m) are stored as well.

Run from the repository root on an x86-64 machine that has the reference
checkout:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def ellipses(rng, n_ell, n_per, Lx, Ly, amin, amax, margin=0.01, max_tries=20000):
    """Non-overlapping ellipses in an Lx x Ly box (minimum-image centre
    distance > a1 + a2 + margin); equispaced-theta points, outward unit
    normals and trapezoid weights (2 pi / n) |x'(theta)|."""
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


def run_case(name, xs, ys, xt, yt, f1, f2, n1, n2, Lx, Ly, tol, P=24, Nb=0.0, ds_kinf=None, kinds=("slp", "dlp")):
    rec = dict(xsrc=xs, ysrc=ys, xtar=xt, ytar=yt, f1=f1, f2=f2, n1=n1, n2=n2, Lx=Lx, Ly=Ly, tol=tol, P=P, Nb=Nb)
    for kind in kinds:
        if kind == "slp":
            u1, u2, ur, uk, prm = po.ref_stokes_slp_ewald_2p(xs, ys, xt, yt, f1, f2, Lx, Ly, P, Nb, tol)
        else:
            u1, u2, ur, uk, prm = po.ref_stokes_dlp_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, P, Nb, tol)
        rec[f"{kind}_u"] = np.stack([u1, u2], axis=1)
        rec[f"{kind}_ur"] = ur
        rec[f"{kind}_uk"] = uk
        for k, v in prm.as_dict().items():
            rec[f"{kind}_prm_{k}"] = v
        if ds_kinf is not None:
            wx, wy = po.matlab_wrap(xs, Lx), po.matlab_wrap(ys, Ly)
            tx, ty = po.matlab_wrap(xt, Lx), po.matlab_wrap(yt, Ly)
            if kind == "slp":
                rec["slp_ur_ds"] = po.slp_real_ds(wx, wy, tx, ty, f1, f2, Lx, Ly, prm.xi)
                rec["slp_uk_ds"] = po.slp_kspace_ds(wx, wy, tx, ty, f1, f2, Lx, Ly, prm.xi, ds_kinf)
            else:
                rec["dlp_ur_ds"] = po.dlp_real_ds(wx, wy, tx, ty, n1, n2, f1, f2, Lx, Ly, prm.xi)
                rec["dlp_uk_ds"] = po.dlp_kspace_ds(wx, wy, tx, ty, n1, n2, f1, f2, Lx, Ly, prm.xi, ds_kinf)
            rec["ds_kinf"] = ds_kinf
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **rec)
    print("wrote", name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in rec.items() if k.endswith("_u")})


def run_mex_case(name, gateway, args, n_out, **meta):
    """A direct gateway call with explicit parameters."""
    out = po.ref_call(gateway, args, n_out)
    rec = {f"arg{i}": np.asarray(a, dtype=np.float64) for i, a in enumerate(args)}
    rec["nargs"] = len(args)
    rec["gateway"] = gateway
    rec["out"] = out
    rec.update(meta)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **rec)
    print("wrote", name, gateway, out.shape)


def main():
    if not po.ref_available("O3"):
        if not po.build_reference(os.environ.get("FTE_REF_ROOT", "/root/reference")):
            raise SystemExit("reference gateways unavailable: run `make -C oracle ref REF_ROOT=<checkout>`")

    # 1. The reference's direct-sum test setup
    #    (PeriodicEwald/tests/direct_sums/direct_sums_velocity_test.m:13-44):
    #    20 sources / 20 targets, L = 1, f = 10 rand, n1 = rand, n2 = sqrt(1 - n1^2),
    #    tol 1e-16, direct k-sum truncated at kinf = 70.
    rng = np.random.default_rng(20240101)
    Ns = Nt = 20
    f1, f2 = 10 * rng.random(Ns), 10 * rng.random(Ns)
    n1 = rng.random(Ns)
    n2 = np.sqrt(1 - n1 ** 2)
    xs, ys, xt, yt = rng.random(Ns), rng.random(Ns), rng.random(Nt), rng.random(Nt)
    xs, ys, xt, yt = (po.matlab_wrap(v, 1.0) for v in (xs, ys, xt, yt))
    run_case("direct_sums_n20", xs, ys, xt, yt, f1, f2, n1, n2, 1.0, 1.0, 1e-16, ds_kinf=70)

    # 2. Config 1: SLP, [0,1]^2, 1000 sources / 1000 separate targets, zero-mean
    #    N(0,1) densities, tol 1e-10 (DLP with unit normals recorded alongside).
    rng = np.random.default_rng(1)
    N = 1000
    xs, ys, xt, yt = (rng.random(N) for _ in range(4))
    f1, f2 = rng.standard_normal(N), rng.standard_normal(N)
    f1 -= f1.mean()
    f2 -= f2.mean()
    th = rng.random(N) * 2 * np.pi
    run_case("config1_n1000", xs, ys, xt, yt, f1, f2, np.cos(th), np.sin(th), 1.0, 1.0, 1e-10)

    # 3. Config 2 in miniature: box 2 x 1, 10 ellipses x 64 points, densities
    #    N(0,1) x trapezoid weights, targets = 64 x 32 cell-centred grid plus
    #    every boundary point (self-coincident targets), tol 1e-10.
    rng = np.random.default_rng(2)
    X, Y, N1, N2, W = ellipses(rng, 10, 64, 2.0, 1.0, 0.02, 0.06)
    f1 = rng.standard_normal(len(X)) * W
    f2 = rng.standard_normal(len(X)) * W
    gx, gy = np.meshgrid((np.arange(64) + 0.5) / 64 * 2.0 - 1.0, (np.arange(32) + 0.5) / 32 - 0.5, indexing="ij")
    xt = np.concatenate([gx.ravel(), X])
    yt = np.concatenate([gy.ravel(), Y])
    run_case("config2_mini", X, Y, xt, yt, f1, f2, N1, N2, 2.0, 1.0, 1e-10)

    # 4. Stresslet identity (PeriodicEwald/tests/stresslet_identity_test.m:17-66):
    #    circle r = 1 in a 4 x 4 box, 256 trapezoid points, f = h e_1, targets on
    #    circles of radius 0.5 and 1.5 (16 each).
    Nsrc, Ntar = 256, 16
    h = 2 * np.pi / Nsrc
    th = h * np.arange(1, Nsrc + 1)
    xs, ys = np.cos(th), np.sin(th)
    tt = 2 * np.pi / Ntar * np.arange(1, Ntar + 1)
    xt = np.concatenate([0.5 * np.cos(tt), 1.5 * np.cos(tt)])
    yt = np.concatenate([0.5 * np.sin(tt), 1.5 * np.sin(tt)])
    run_case("stresslet_identity_e1", xs, ys, xt, yt, h * np.ones(Nsrc), np.zeros(Nsrc), np.cos(th), np.sin(th),
             4.0, 4.0, 1e-16, kinds=("dlp",))
    run_case("stresslet_identity_e2", xs, ys, xt, yt, np.zeros(Nsrc), h * np.ones(Nsrc), np.cos(th), np.sin(th),
             4.0, 4.0, 1e-16, kinds=("dlp",))

    # 5. Aspect ratio 1 x 2 as in the consistency and timing tests
    #    (consistency_test_velocity.m:13-16), f = 10 rand, 2000 points, tol 1e-12,
    #    with self-coincident targets (targets = sources) to exercise the SLP self
    #    term and the DLP r = 0 skip.
    rng = np.random.default_rng(5)
    N = 2000
    xs, ys = rng.random(N), 2 * rng.random(N)
    f1, f2 = 10 * rng.random(N), 10 * rng.random(N)
    n1 = rng.random(N)
    n2 = np.sqrt(1 - n1 ** 2)
    run_case("aspect_1x2_self", xs, ys, xs.copy(), ys.copy(), f1, f2, n1, n2, 1.0, 2.0, 1e-12)

    # 6. Tiny problems: nside = 1 (all 8 neighbours are images of the own box),
    #    one source / one target, and points exactly on grid nodes and on cell
    #    boundaries (window tie-break in FindClosestNode).
    rng = np.random.default_rng(6)
    xs, ys = rng.random(3) - 0.5, rng.random(3) - 0.5
    xt, yt = rng.random(2) - 0.5, rng.random(2) - 0.5
    f1, f2 = rng.standard_normal(3), rng.standard_normal(3)
    th = rng.random(3) * 2 * np.pi
    run_case("tiny_n3", xs, ys, xt, yt, f1, f2, np.cos(th), np.sin(th), 1.0, 1.0, 1e-10, Nb=10.0)
    run_case("single_pair", np.array([0.1]), np.array([-0.2]), np.array([0.3]), np.array([0.25]), np.array([1.0]),
             np.array([-0.5]), np.array([0.6]), np.array([0.8]), 1.0, 1.0, 1e-10)
    M = 48
    hgrid = 1.0 / M
    node = -0.5 + hgrid * np.array([0, 1, 7, 24, 47, 13, 30, 5])
    xs = np.concatenate([node, [-0.5, 0.0, 1.0 / 3 - 0.5, 2.0 / 3 - 0.5]])
    ys = np.concatenate([node[::-1], [0.0, -0.5, 1.0 / 3 - 0.5, 0.1]])
    rng = np.random.default_rng(7)
    f1, f2 = rng.standard_normal(len(xs)), rng.standard_normal(len(xs))
    th = rng.random(len(xs)) * 2 * np.pi
    xt = np.concatenate([xs, rng.random(20) - 0.5])
    yt = np.concatenate([ys, rng.random(20) - 0.5])
    run_case("grid_nodes", xs, ys, xt, yt, f1, f2, np.cos(th), np.sin(th), 1.0, 1.0, 1e-10, Nb=4.0)

    # 7. Direct gateway calls with explicit, non-driver parameters: P = 16,
    #    unequal and non-smooth grids (986 = 2*17*29 has prime factors no
    #    small-radix FFT covers), window width w != P h / 2.
    rng = np.random.default_rng(8)
    Ns, Nt = 700, 500
    ps = np.stack([rng.random(Ns) - 0.5, rng.random(Ns) - 0.5], axis=1)
    pt = np.stack([rng.random(Nt) - 0.5, rng.random(Nt) - 0.5], axis=1)
    f = rng.standard_normal((Ns, 2))
    th = rng.random(Ns) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], axis=1)
    run_mex_case("mex_slp_real_explicit", "slp_real", [ps, pt, f, 21.0, 5, 5, 1.0, 1.0], Nt)
    run_mex_case("mex_dlp_real_explicit", "dlp_real", [ps, pt, f, n, 23.5, 4, 4, 1.0, 1.0], Nt)
    Mx, My, P = 174, 174, 16
    h = 1.0 / Mx
    w = P * h / 2
    eta = (2 * 21.0 * w / (0.95 * np.sqrt(np.pi * P))) ** 2
    run_mex_case("mex_slp_kspace_p16", "slp_kspace", [ps, pt, 21.0, eta, f, Mx, My, 1.0, 1.0, w, P], Nt)
    run_mex_case("mex_dlp_kspace_p16", "dlp_kspace", [ps, pt, 21.0, eta, f, n, Mx, My, 1.0, 1.0, w, P], Nt)
    Mx, My, P = 986, 116, 24
    ps2 = np.stack([(rng.random(Ns) - 0.5) * 1.0, (rng.random(Ns) - 0.5) * (116 / 986)], axis=1)
    pt2 = np.stack([(rng.random(Nt) - 0.5) * 1.0, (rng.random(Nt) - 0.5) * (116 / 986)], axis=1)
    h = 1.0 / Mx
    w = 0.9 * P * h / 2
    eta = (2 * 300.0 * w / (0.95 * np.sqrt(np.pi * P))) ** 2
    Ly = 116 / 986
    run_mex_case("mex_slp_kspace_rect986", "slp_kspace", [ps2, pt2, 300.0, eta, f, Mx, My, 1.0, Ly, w, P], Nt)
    run_mex_case("mex_dlp_kspace_rect986", "dlp_kspace", [ps2, pt2, 300.0, eta, f, n, Mx, My, 1.0, Ly, w, P], Nt)


if __name__ == "__main__":
    main()
