#!/usr/bin/env python
"""Golden vectors of the other spectral Ewald quantities, from the
reference's own MEX gateways (and of their MATLAB drivers, restated around
those gateways in oracle/pyoracle.py:ref_q_ewald_2p).

Runs the unmodified gateways mex_stokes_{slp,dlp}_{pressure,pressure_grad,
gradient,stress,vorticity}_{real,kspace}.cpp (PeriodicEwald/src/mex/Stokes{SLP,DLP}/),
compiled by ``make -C oracle ref`` from the reference checkout against the
MEX stand-in in oracle/mexshim, on one seeded case per quantity and kernel,
and writes tests/golden/quant_<kind>_<quantity>.npz with the inputs and both
outputs; tests/golden/quant_drv_<kind>_<quantity>.npz hold two driver cases
(targets equal to the sources, and separate targets) at tol 1e-10.  The case: a 2 x 1 box, 300 sources, 220 targets of which 20
coincide with sources (the own-box skip), P = 16, a 128 x 64 grid.

Usage (x86-64 host with the reference checkout; `make -C oracle ref` first):
    python tests/golden/gen_golden_quant.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402


def case(seed=11):
    rng = np.random.default_rng(seed)
    Lx, Ly = 2.0, 1.0
    ns, nt = 300, 200
    ps = np.stack([(rng.random(ns) - 0.5) * Lx, (rng.random(ns) - 0.5) * Ly], 1)
    pt = np.concatenate([np.stack([(rng.random(nt) - 0.5) * Lx, (rng.random(nt) - 0.5) * Ly], 1), ps[:20]])
    f = rng.standard_normal((ns, 2))
    th = rng.random(ns) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], 1)
    xi, nsx, nsy = 12.0, 8, 4
    P, Mx, My = 16, 128, 64
    h = Lx / Mx
    w = P * h / 2
    eta = (2 * xi * w / (0.95 * np.sqrt(np.pi * P))) ** 2
    return dict(psrc=ps, ptar=pt, f=f, n=n, xi=xi, nside_x=nsx, nside_y=nsy, Lx=Lx, Ly=Ly, P=P, Mx=Mx, My=My, w=w,
                eta=eta)


def driver_cases(seed=23):
    """Driver inputs: case 0 has the targets equal to the sources (the drivers'
    self terms), case 1 separate targets; a 1 x 1.5 box, tol 1e-10."""
    rng = np.random.default_rng(seed)
    Lx, Ly = 1.0, 1.5
    out = []
    for sep in (False, True):
        ns = 500
        xs, ys = (rng.random(ns) - 0.5) * Lx, (rng.random(ns) - 0.5) * Ly
        if sep:
            nt = 350
            xt, yt = (rng.random(nt) - 0.5) * Lx * 1.2, (rng.random(nt) - 0.5) * Ly
        else:
            xt, yt = xs.copy(), ys.copy()
        th = rng.random(ns) * 2 * np.pi
        out.append(dict(xsrc=xs, ysrc=ys, xtar=xt, ytar=yt, f1=rng.standard_normal(ns), f2=rng.standard_normal(ns),
                        n1=np.cos(th), n2=np.sin(th), b1=rng.standard_normal(len(xt)), b2=rng.standard_normal(len(xt)),
                        Lx=Lx, Ly=Ly, tol=1e-10))
    return out


def main():
    if not po.ref_available("O3"):
        raise SystemExit("reference gateways not built: run `make -C oracle ref` on x86-64")
    for kind, kn in ((po.KIND_SLP, "slp"), (po.KIND_DLP, "dlp")):
        for q, qn in po.Q_NAMES.items():
            arrays = {}
            for i, d in enumerate(driver_cases()):
                o, r, k, prm = po.ref_q_ewald_2p(kind, q, d["xsrc"], d["ysrc"], d["xtar"], d["ytar"], d["f1"], d["f2"],
                                                 d["Lx"], d["Ly"], d["n1"], d["n2"], d["b1"], d["b2"], tol=d["tol"])
                arrays.update({f"c{i}_{key}": np.asarray(v) for key, v in d.items()})
                arrays.update({f"c{i}_out": o, f"c{i}_out_real": r, f"c{i}_out_k": k, f"c{i}_xi": prm.xi,
                               f"c{i}_Mx": prm.Mx, f"c{i}_nside_x": prm.nside_x})
            path = os.path.join(HERE, f"quant_drv_{kn}_{qn}.npz")
            np.savez_compressed(path, kind=kind, quantity=q, **arrays)
            print(path)
    c = case()
    for kind, kn in ((po.KIND_SLP, "slp"), (po.KIND_DLP, "dlp")):
        for q, qn in po.Q_NAMES.items():
            ur = po.ref_q_real(kind, q, c["psrc"], c["ptar"], c["f"], c["n"], c["xi"], c["nside_x"], c["nside_y"],
                               c["Lx"], c["Ly"])
            uk = po.ref_q_kspace(kind, q, c["psrc"], c["ptar"], c["f"], c["n"], c["xi"], c["eta"], c["Mx"], c["My"],
                                 c["Lx"], c["Ly"], c["w"], c["P"])
            path = os.path.join(HERE, f"quant_{kn}_{qn}.npz")
            np.savez_compressed(path, kind=kind, quantity=q, real=ur, kspace=uk,
                                **{k: np.asarray(v) for k, v in c.items()})
            print(path, ur.shape, float(np.abs(ur).max()), float(np.abs(uk).max()))


if __name__ == "__main__":
    main()
