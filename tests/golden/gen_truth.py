"""Generate tests/golden/truth_config3.npz: converged FP64 Ewald sums of the
1,000,000-point configuration (fasttools2d_gb300.workloads.config3) at the
10,000 sampled targets (workloads.config3_sample), for the Stokeslet and the
stresslet.

The values come from the oracle's truth sum (oracle/or_ewald.c,
or_ewald_truth): an Ewald split with its own xi_o, a real-space cutoff with
exp(-xi_o^2 r^2) < e^-40 over periodic images, and every Fourier mode with
exp(-k^2/(4 xi_o^2)) > e^-40 -- the reference tests' direct sums
(PeriodicEwald/tests/direct_sums/matlab_sums/*_ds.m) made convergent.  The
file also stores checksums of the regenerated inputs so that users can
confirm they rebuilt the same arrays.

Run from the repository root:  python tests/golden/gen_truth.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from fasttools2d_gb300 import workloads as wl  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

XI_O = 22.0


def main():
    cfg = wl.config3()
    idx = wl.config3_sample()
    Lx, Ly = cfg["Lx"], cfg["Ly"]
    xs, ys = po.matlab_wrap(cfg["xsrc"], Lx), po.matlab_wrap(cfg["ysrc"], Ly)
    xt, yt = po.matlab_wrap(cfg["xtar"][idx], Lx), po.matlab_wrap(cfg["ytar"][idx], Ly)
    xi, rcut, kinf = po.truth_params(Lx, Ly, xi=XI_O)
    out = dict(idx=idx, xi_o=xi, rcut=rcut, kinf=kinf,
               checksum=wl.checksum(cfg["xsrc"], cfg["ysrc"], cfg["xtar"], cfg["ytar"], cfg["f1"], cfg["f2"],
                                    cfg["n1"], cfg["n2"]))
    for kind, name in ((po.KIND_SLP, "slp"), (po.KIND_DLP, "dlp")):
        t = time.time()
        out[name] = po.ewald_truth(kind, xs, ys, xt, yt, cfg["f1"], cfg["f2"], Lx, Ly, n1=cfg["n1"], n2=cfg["n2"],
                                   xi=xi, rcut=rcut, kinf=kinf)
        print(name, "done in", round(time.time() - t, 1), "s", flush=True)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "truth_config3.npz"), **out)
    print("wrote truth_config3.npz")


if __name__ == "__main__":
    main()
