"""Cost-model calibration of the tuned parameter choice on the present GPU.

Sweeps the cell-list size of the mixed form at 1e6 uniform points (every
other choice left to the chooser), prints the stage times of each point as
JSON lines, and fits the near-field cost model

    near ~ a N_trg + b pairs + c boxes,   pairs = N_src N_trg pi rc^2 / (Lx Ly) * 1.03

per kernel and tolerance, the form of ``kCostTarget`` / ``kCostPair`` /
``kCostBox`` in ``csrc/api.cu``.  The spread/gather and transform unit costs
follow from the same lines (stage time over window nodes x grids, and over
``fft_work``).

    python -m fasttools2d_gb300.calibrate --tol 1e-10 1e-8 1e-6
"""
import argparse
import json
import math

import numpy as np


def sweep(tols, nsides, n=1_000_000, seed=3, reps=3):
    import fasttools2d_gb300 as ft

    rng = np.random.default_rng(seed)
    xs, ys, xt, yt = [rng.random(n) - 0.5 for _ in range(4)]
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    th = rng.random(n) * 2 * np.pi
    n1, n2 = np.cos(th), np.sin(th)
    ctx = ft.Context(0)
    ctx.set_timing(True)
    rows = []
    for tol in tols:
        for kind in ("slp", "dlp"):
            for ns in nsides:
                ts = []
                for _ in range(reps):
                    kw = dict(tol=tol, form=ft.FORM_MIXED, ctx=ctx, return_info=True, parts=False, nside_x=ns,
                              nside_y=ns)
                    if kind == "slp":
                        _, info = ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1, f2, 1.0, 1.0, **kw)
                    else:
                        _, info = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, 1.0, 1.0, **kw)
                    ts.append((info.ms_total, info.ms_near, info.ms_spread, info.ms_fft, info.ms_gather))
                t = sorted(ts)[len(ts) // 2]
                p = info.params
                row = {"tol": tol, "kind": kind, "ns": ns, "n": n, "xi": round(p.xi, 1), "Mx": p.Mx, "My": p.My,
                       "P": p.P, "form": p.form, "total": round(t[0], 3), "near": round(t[1], 3),
                       "spread": round(t[2], 3), "fft": round(t[3], 3), "gather": round(t[4], 3)}
                print(json.dumps(row), flush=True)
                rows.append(row)
    return rows


def fit_near(rows):
    """Least-squares (a, b, c) of near = a N_trg + b pairs + c boxes per (tol, kind)."""
    out = {}
    for key in sorted({(r["tol"], r["kind"]) for r in rows}):
        R = [r for r in rows if (r["tol"], r["kind"]) == key]
        ns = np.array([r["ns"] for r in R], float)
        n = float(R[0]["n"])
        near = np.array([r["near"] for r in R]) * 1e-3
        pairs = n * n * math.pi / ns ** 2 * 1.03
        A = np.stack([np.full_like(ns, n), pairs, ns ** 2], 1)
        c, *_ = np.linalg.lstsq(A, near, rcond=None)
        best = min(R, key=lambda r: r["total"])
        out[f"{key[1]}@{key[0]:g}"] = {"per_target_ns": c[0] * 1e9, "per_pair_ps": c[1] * 1e12,
                                       "per_box_ns": c[2] * 1e9, "best_nside": best["ns"], "best_ms": best["total"]}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--tol", type=float, nargs="+", default=[1e-10])
    ap.add_argument("--nside", type=int, nargs="+", default=[100, 115, 130, 149, 165, 180, 200, 225])
    a = ap.parse_args(argv)
    rows = sweep(a.tol, a.nside)
    print(json.dumps({"fit": fit_near(rows)}), flush=True)


if __name__ == "__main__":
    main()
