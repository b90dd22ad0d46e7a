#!/usr/bin/env python
"""Benchmark of the doubly-periodic spectral Ewald Stokeslet + stresslet on GB300.

Metric: targets/s at 1M points (10^6 sources, 10^6 targets uniform in [0,1]^2,
zero-mean N(0,1) densities, unit normals at random angles), one step = one
Stokeslet (SLP) plus one stresslet (DLP) evaluation of all targets, parameter
selection included.  Reported per tolerance (1e-10 headline, 1e-6 alongside)
with max and RMS relative error against the converged FP64 Ewald sums of
10,000 sampled targets (tests/golden/truth_config3.npz).

Arms:
  default            the GPU library through its public API (C ABI, ctypes)
  --impl reference   the reference's CPU spectral Ewald path on this host's
                     cores at the same N: the reference's own gateways
                     (oracle/_ref, compiled on this host from the checkout or
                     its staged copy) where built, else the oracle's C
                     restatement (oracle/or_ewald.c); OpenMP over all cores.

Multi-GPU (torchrun): replicas only -- every rank evaluates the same
configuration on its own GPU, no collective on the data path; value = total
targets of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "targets/s at 1M pts, tol 1e-6 & 1e-10: chosen vs plain GPU form; max rel err"
UNIT = "targets/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000, help="sources = targets")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="headline only (for profiling runs)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 64-configuration section")
    ap.add_argument("--profile", choices=["plain", "mixed", "batched"], default=None,
                    help="time only this form at tol 1e-10, or only the batched form's graph step (for profiler "
                         "launch lists); no other sections")
    ap.add_argument("--profile-tol", type=float, default=1e-10,
                    help="the tolerance of --profile plain|mixed (default 1e-10)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the timed region is short (~0.2 s): begin it only once the sampler
        # is writing, so that its samples fall inside the region
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        import numpy as np

        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# reference arm: CPU
# ---------------------------------------------------------------------------
def _ref_impl():
    """(kind, runner) of the reference CPU path on this host: the reference's
    own gateways compiled here (oracle/_ref, O3) where they were built, else
    the oracle's C restatement."""
    from oracle import pyoracle as po

    if not os.path.exists(po.LIB_PATH):
        po.build()
    use_ref = po.ref_available("O3")

    def run(cfg, tol, flavour="O3"):
        a = [cfg[k] for k in ("xsrc", "ysrc", "xtar", "ytar")]
        if use_ref:
            po.ref_stokes_slp_ewald_2p(*a, cfg["f1"], cfg["f2"], 1.0, 1.0, tol=tol, flavour=flavour)
            po.ref_stokes_dlp_ewald_2p(*a, cfg["n1"], cfg["n2"], cfg["f1"], cfg["f2"], 1.0, 1.0, tol=tol,
                                       flavour=flavour)
        else:
            po.stokes_slp_ewald_2p(*a, cfg["f1"], cfg["f2"], 1.0, 1.0, tol=tol)
            po.stokes_dlp_ewald_2p(*a, cfg["n1"], cfg["n2"], cfg["f1"], cfg["f2"], 1.0, 1.0, tol=tol)

    return ("reference" if use_ref else "port"), run


def _ref_fixture_check():
    """Max relative difference of the reference gateways built on this host
    from the committed fixtures (made by the same sources on x86-64)."""
    import numpy as np

    from oracle import pyoracle as po

    gold = os.path.join(ROOT, "tests", "golden")
    worst = 0.0
    for f in sorted(os.listdir(gold)):
        if not f.startswith("mex_"):
            continue
        with np.load(os.path.join(gold, f)) as z:
            g = {k: z[k] for k in z.files}
        args = [g[f"arg{i}"] for i in range(int(g["nargs"]))]
        args = [float(a) if a.ndim == 0 else a for a in args]
        out = po.ref_call(str(g["gateway"]), args, g["out"].shape[0], "O3")
        worst = max(worst, float(np.abs(out - g["out"]).max() / np.abs(g["out"]).max()))
    return worst


def reference_arm(args):
    """The reference's CPU spectral Ewald path on this host's cores, on the
    same workload as the GPU arm: config 3 at N = args.n (default 10^6), one
    SLP + one DLP evaluation at tol 1e-10 per step, the drivers' analytic
    parameters (P = 24), OpenMP over every host core.  The gateways are the
    reference's own, compiled here with -O3 (the flags it ships, -O0, are
    timed once beside them)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    from fasttools2d_gb300 import workloads as wl
    from oracle import pyoracle as po

    kind, run = _ref_impl()
    cfg = wl.config3(n=args.n)
    for _ in range(args.warmup):
        run(cfg, 1e-10)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run(cfg, 1e-10)
    dt = (time.perf_counter() - t0) / args.steps
    value = args.n / dt
    extra = {}
    if kind == "reference":
        extra["fixture_max_rel"] = _ref_fixture_check()
        if po.ref_available("O0") and not args.quick:
            t = time.perf_counter()
            run(cfg, 1e-10, "O0")
            extra["as_shipped_O0_ms_per_step"] = (time.perf_counter() - t) * 1e3
    sample = (f"config-3 workload at full size, N = {args.n} sources and {args.n} targets (uniform [0,1]^2, "
              f"zero-mean N(0,1) densities), one SLP + one DLP evaluation at tol 1e-10 per step, P = 24, the "
              f"drivers' analytic parameters; " +
              ("the reference's own gateways (oracle/_ref, -O3)" if kind == "reference"
               else "the oracle's C restatement"))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"config3: SLP+DLP spectral Ewald, {args.n} sources / {args.n} targets, unit box, "
                               f"tol 1e-10", "sample_n": args.n, "same_config": True, "l2": "n/a (CPU)",
                   "host": platform.machine(), **extra},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": po.num_threads(), "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(n_full):
    """The reference CPU path (its own gateways where built here) on one
    SLP + DLP evaluation of the full workload (about 10 s on 16 cores)."""
    from fasttools2d_gb300 import workloads as wl
    from oracle import pyoracle as po

    kind, run = _ref_impl()
    cfg = wl.config3(n=n_full)
    t = time.perf_counter()
    run(cfg, 1e-10)
    dt = time.perf_counter() - t
    return {"value": n_full / dt, "unit": UNIT, "cores": po.num_threads(), "kind": kind,
            "sample": f"one SLP + one DLP evaluation of the config-3 workload at N = {n_full}, tol 1e-10, "
                      f"{dt:.1f} s"}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def config4_device(ft, wl, nv):
    """The 64-configuration workload on the device (positions, normals, nv
    density vectors per configuration)."""
    import numpy as np
    import torch

    dev = []
    for c in wl.config4():
        d = {k: torch.tensor(c[k], dtype=torch.float64, device="cuda") for k in ("xsrc", "ysrc", "n1", "n2")}
        d["f1"] = torch.tensor(np.stack([f[0] for f in c["f"][:nv]]), dtype=torch.float64, device="cuda")
        d["f2"] = torch.tensor(np.stack([f[1] for f in c["f"][:nv]]), dtype=torch.float64, device="cuda")
        d["Lx"], d["Ly"] = c["Lx"], c["Ly"]
        dev.append(d)
    return dev


def batched_profile(ft, wl, ctx, stream, steps, warmup, flush):
    """The batched form's graph step alone (plans with autotuned tiles, one
    batch, `warmup` untimed replays, then `steps` timed ones): for launch
    lists of the batch's kernels."""
    import torch

    nv, tol = 4, 1e-8
    kinds = (ft.KIND_SLP, ft.KIND_DLP)
    dev = config4_device(ft, wl, nv)
    plans = [ft.Plan(kind, d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["f1"][0], d["f2"][0], d["Lx"], d["Ly"],
                     n1=d["n1"], n2=d["n2"], tol=tol, form=ft.FORM_MIXED, nvmax=nv, tune=True, ctx=ctx)
             for d in dev for kind in kinds]
    batch = ft.Batch(plans, nv, ctx=ctx)
    for i in range(len(plans)):
        d = dev[i // len(kinds)]
        batch.set_density(i, d["f1"], d["f2"])
    k0 = ctx.kernel_count
    batch.launch(False)  # one step outside the graph: its launches are counted
    launches = ctx.kernel_count - k0
    for _ in range(max(warmup, 1)):
        batch.launch(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        batch.launch(True)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    npts = sum(int(d["xsrc"].numel()) for d in dev)
    return {"metric": "targets/s, 64-configuration batch (config 4), tol 1e-8", "profile": "batched",
            "ms_per_step": ms, "value": npts * nv * len(kinds) / (ms / 1e3), "unit": "targets/s",
            "gpu_launches_per_step": launches}


def batched_section(ft, wl, ctx, stream, steps, warmup, flush):
    """Batched form on the 64-configuration workload (config 4): every
    configuration evaluated with the Stokeslet and the stresslet for 4
    density vectors, at tolerance 1e-8.

    ours:     one plan per (configuration, kernel) with the tuned parameter
              choice and autotuned spread/gather tiles, all bound into one
              batch (every stage one launch over all plans, with the work
              lists' own tile sizes); a step is one replay of its CUDA graph.
    baseline: the untuned plain per-instance loop -- one FP64 driver call per
              (configuration, kernel, vector) with the analytic parameters.
    ablations, to separate what each part adds:
      mixed_loop     the mixed form's driver called per (configuration,
                     kernel, vector) with the batch's parameters (same
                     arithmetic and parameters; no plans, batch or graph)
      plans_loop     the batch's plans executed one after another (geometry
                     reused, all vectors per call; no batch or graph)
      plans_loop_untuned  the same, plans with the default tile sizes (what
                     the autotuner adds to plans executed alone)
    All with inputs resident on the GPU; L2 flushed before every step."""
    import numpy as np
    import torch

    cfgs = wl.config4()
    nv, tol = 4, 1e-8
    kinds = (ft.KIND_SLP, ft.KIND_DLP)
    dev = config4_device(ft, wl, nv)
    npts = sum(len(c["xsrc"]) for c in cfgs)
    targets_per_step = npts * nv * len(kinds)

    def events(n):
        return [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]

    # ---- baseline: plain per-instance loop
    loop_out = [[(torch.empty_like(d["f1"]), torch.empty_like(d["f1"])) for _ in kinds] for d in dev]

    def loop_step():
        for d, outs in zip(dev, loop_out):
            for kind, (u1, u2) in zip(kinds, outs):
                for v in range(nv):
                    if kind == ft.KIND_SLP:
                        ft.StokesSLP_ewald_2p(d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["f1"][v], d["f2"][v],
                                              d["Lx"], d["Ly"], tol=tol, ctx=ctx, out=(u1[v], u2[v]), parts=False)
                    else:
                        ft.StokesDLP_ewald_2p(d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["n1"], d["n2"],
                                              d["f1"][v], d["f2"][v], d["Lx"], d["Ly"], tol=tol, ctx=ctx,
                                              out=(u1[v], u2[v]), parts=False)

    loop_step()
    lsteps = 1
    ev = events(lsteps)
    torch.cuda.synchronize()
    for i in range(lsteps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        loop_step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    loop_ms = sum(a.elapsed_time(b) for a, b in ev) / lsteps

    # ---- ours: plans + batch + graph
    t0 = time.perf_counter()
    plans = []
    for d in dev:
        for kind in kinds:
            plans.append(ft.Plan(kind, d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["f1"][0], d["f2"][0], d["Lx"],
                                 d["Ly"], n1=d["n1"], n2=d["n2"], tol=tol, form=ft.FORM_MIXED, nvmax=nv, tune=True,
                                 ctx=ctx))
    batch = ft.Batch(plans, nv, ctx=ctx)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    for i, p in enumerate(plans):
        d = dev[i // len(kinds)]
        batch.set_density(i, d["f1"], d["f2"])
    k0 = ctx.kernel_count
    batch.launch(False)
    launches = ctx.kernel_count - k0
    for _ in range(warmup):
        batch.launch(True)
    bsteps = max(3, min(steps, 10))
    ev = events(bsteps)
    torch.cuda.synchronize()
    for i in range(bsteps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        batch.launch(True)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    graph_ms = sum(a.elapsed_time(b) for a, b in ev) / bsteps

    def device_ms(fn, reps):
        ev = events(reps)
        torch.cuda.synchronize()
        for i in range(reps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            fn()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / reps

    # ablation 1: the mixed form's driver per instance with the batch's parameters
    ov = []
    for p in plans:
        q = p.params
        ov.append(dict(P=q.P, xi=q.xi, Mx=q.Mx, My=q.My, nside_x=q.nside_x, nside_y=q.nside_y))
    mix_out = [(torch.empty_like(dev[i // len(kinds)]["f1"][0]), torch.empty_like(dev[i // len(kinds)]["f1"][0]))
               for i in range(len(plans))]

    def mixed_loop():
        for i, p in enumerate(plans):
            d = dev[i // len(kinds)]
            u1, u2 = mix_out[i]
            for v in range(nv):
                if p.kind == ft.KIND_SLP:
                    ft.StokesSLP_ewald_2p(d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["f1"][v], d["f2"][v],
                                          d["Lx"], d["Ly"], tol=tol, form=ft.FORM_MIXED, ctx=ctx, out=(u1, u2),
                                          parts=False, **ov[i])
                else:
                    ft.StokesDLP_ewald_2p(d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["n1"], d["n2"], d["f1"][v],
                                          d["f2"][v], d["Lx"], d["Ly"], tol=tol, form=ft.FORM_MIXED, ctx=ctx,
                                          out=(u1, u2), parts=False, **ov[i])

    mixed_loop()
    mixed_loop_ms = device_ms(mixed_loop, 2)

    # ablation 2: the plans one after another (no batch, no graph)
    def plans_loop():
        for i, p in enumerate(plans):
            d = dev[i // len(kinds)]
            p.execute(d["f1"], d["f2"])

    plans_loop()
    plans_loop_ms = device_ms(plans_loop, 2)

    # ablation 3: the plans one after another with the default tiles (what
    # the autotuner adds to plans executed alone; a batch's work lists use
    # their own tile sizes either way)
    plans_u = []
    for d in dev:
        for kind in kinds:
            plans_u.append(ft.Plan(kind, d["xsrc"], d["ysrc"], d["xsrc"], d["ysrc"], d["f1"][0], d["f2"][0], d["Lx"],
                                   d["Ly"], n1=d["n1"], n2=d["n2"], tol=tol, form=ft.FORM_MIXED, nvmax=nv, tune=False,
                                   ctx=ctx))

    def plans_loop_untuned():
        for i, p in enumerate(plans_u):
            d = dev[i // len(kinds)]
            p.execute(d["f1"], d["f2"])

    plans_loop_untuned()
    untuned_ms = device_ms(plans_loop_untuned, 2)
    for p in plans_u:
        p.close()

    # agreement with the FP64 plain loop (both at tolerance 1e-8)
    worst = 0.0
    for i, p in enumerate(plans):
        b1, b2 = batch.velocity(i)
        u1, u2 = loop_out[i // len(kinds)][i % len(kinds)]
        ref = np.stack([u1.cpu().numpy(), u2.cpu().numpy()])
        worst = max(worst, float(np.abs(np.stack([b1, b2]) - ref).max() / np.abs(ref).max()))

    # end to end through the public API: densities from pinned host memory in,
    # velocities out to pinned host memory, every step
    hf = [(dev[i // len(kinds)]["f1"].cpu().pin_memory(), dev[i // len(kinds)]["f2"].cpu().pin_memory())
          for i in range(len(plans))]
    hu = [torch.empty((nv, p.ntar), dtype=torch.float64).pin_memory() for p in plans]
    hu2 = [torch.empty((nv, p.ntar), dtype=torch.float64).pin_memory() for p in plans]
    import ctypes as C

    lib = ft.lib()

    def e2e_step():
        # pinned host buffers: the copies are queued without a synchronisation
        # each; the step ends when the stream has delivered every velocity
        for i in range(len(plans)):
            batch.set_density(i, hf[i][0].numpy(), hf[i][1].numpy(), pinned_async=True)
        batch.launch(True)
        for i in range(len(plans)):
            ft._check(lib.fte_batch_get_velocity(batch.h, i, C.c_void_p(hu[i].data_ptr()),
                                                 C.c_void_p(hu2[i].data_ptr()), ft.FTE_HOST_ASYNC))
        stream.synchronize()

    e2e_step()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(bsteps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t1) / bsteps * 1e3
    h2d = sum(2 * 8 * nv * p.nsrc for p in plans)
    d2h = sum(2 * 8 * nv * p.ntar for p in plans)

    tiles = {}
    forms = {}
    for p in plans:
        q = p.params
        key = f"{q.ts_spread}/{q.ts_gather}"
        tiles[key] = tiles.get(key, 0) + 1
        forms[q.form] = forms.get(q.form, 0) + 1
    batch.close()
    for p in plans:
        p.close()
    return {
        "workload": f"config4: {len(cfgs)} configurations, {npts} points in total (N log-uniform in [2e3, 2e5]), "
                    f"aspect p/4 in [1, 4], half uniform / half on ellipses, SLP and DLP, {nv} density vectors, "
                    f"tol {tol:g}",
        "targets_per_s": targets_per_step / (graph_ms / 1e3), "ms_per_step": graph_ms,
        "plain_loop": {"targets_per_s": targets_per_step / (loop_ms / 1e3), "ms_per_step": loop_ms,
                       "calls_per_step": len(cfgs) * len(kinds) * nv},
        "speedup_vs_plain_loop": loop_ms / graph_ms,
        "ablation_ms_per_step": {"mixed_loop": mixed_loop_ms, "plans_loop": plans_loop_ms,
                                 "plans_loop_untuned": untuned_ms, "batch_tuned_graph": graph_ms},
        "setup_s": setup_s, "gpu_launches_per_step": launches,
        "max_rel_diff_vs_plain_loop": worst,
        "distinct_tile_pairs": len(tiles),
        "kspace_forms": {{ft.FORM_MIXED: "fp32", ft.FORM_FF: "float-float", ft.FORM_FF32: "float-float/fp32"}.get(k, "fp64"): v
                         for k, v in forms.items()},
        "e2e": {"targets_per_s": targets_per_step / (e2e_ms / 1e3), "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "l2": "flushed before every step",
    }


def main():
    args = parse_args()
    if args.impl == "reference":
        reference_arm(args)
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    import numpy as np
    import torch

    import fasttools2d_gb300 as ft
    from fasttools2d_gb300 import workloads as wl

    from fasttools2d_gb300.replicas import Replicas

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    reps = Replicas()
    world, rank, local_rank = reps.world, reps.rank, reps.local_rank
    barrier = reps.barrier
    max_over_ranks = reps.max

    if not os.path.exists(ft.LIB_PATH):
        ft.build()
    ctx = ft.Context(local_rank)
    # one non-default stream shared by torch (L2 flush, events) and the library
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    cfg = wl.config3(n=args.n)
    N = args.n
    keys = ("xsrc", "ysrc", "xtar", "ytar", "f1", "f2", "n1", "n2")
    dev = {k: torch.tensor(cfg[k], dtype=torch.float64, device="cuda") for k in keys}
    outs = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(4)]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    if args.profile == "batched":
        line = batched_profile(ft, wl, ctx, stream, args.steps, args.warmup, flush)
        if rank == 0:
            print(json.dumps(line), flush=True)
        reps.close()
        return

    def step(tol, form, arrays=None, out=None):
        a = arrays or dev
        o = out or outs
        ft.StokesSLP_ewald_2p(a["xsrc"], a["ysrc"], a["xtar"], a["ytar"], a["f1"], a["f2"], 1.0, 1.0, tol=tol,
                              form=form, ctx=ctx, out=(o[0], o[1]), parts=False)
        ft.StokesDLP_ewald_2p(a["xsrc"], a["ysrc"], a["xtar"], a["ytar"], a["n1"], a["n2"], a["f1"], a["f2"], 1.0,
                              1.0, tol=tol, form=form, ctx=ctx, out=(o[2], o[3]), parts=False)

    def timed(tol, form, steps, arrays=None, out=None, flush_l2=True):
        """Mean device time per step (CUDA events on the library's stream),
        L2 flushed before every step outside the timed events."""
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        k0 = ctx.kernel_count
        barrier()
        torch.cuda.synchronize()
        for i in range(steps):
            if flush_l2:
                flush.fill_(float(i))
            ev[i][0].record(stream)
            step(tol, form, arrays, out)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        return max_over_ranks(ms), ctx.kernel_count - k0

    forms = {"plain": ft.FORM_PLAIN}
    try:
        # the mixed-precision form is reported when this build provides it
        ft.StokesSLP_ewald_2p(cfg["xsrc"][:64], cfg["ysrc"][:64], cfg["xtar"][:64], cfg["ytar"][:64],
                              cfg["f1"][:64], cfg["f2"][:64], 1.0, 1.0, tol=1e-6, form=ft.FORM_MIXED, ctx=ctx)
        forms["mixed"] = ft.FORM_MIXED
    except ft.FteError:
        pass

    truth = None
    tpath = os.path.join(ROOT, "tests", "golden", "truth_config3.npz")
    if N == 1_000_000 and os.path.exists(tpath):
        z = np.load(tpath)
        truth = {k: z[k] for k in z.files}
        ck = wl.checksum(*(cfg[k] for k in keys))
        if abs(ck - float(truth["checksum"])) > 1e-9 * abs(float(truth["checksum"])):
            truth = None  # regenerated inputs differ: no error figures
    idx_t = torch.tensor(truth["idx"], device="cuda") if truth is not None else None

    def errors():
        if truth is None:
            return None
        res = {}
        for name, (a, b) in (("slp", (outs[0], outs[1])), ("dlp", (outs[2], outs[3]))):
            u = torch.stack([a[idx_t], b[idx_t]], 1).cpu().numpy()
            t = truth[name]
            d = np.abs(u - t)
            res[name] = {"max_rel": float(d.max() / np.abs(t).max()),
                         "rms_rel": float(np.sqrt((d ** 2).sum() / (t ** 2).sum()))}
        return res

    if args.profile:
        forms = {args.profile: forms[args.profile]}
    results = {}
    tols = [args.profile_tol] if args.profile else ([1e-10] if args.quick else [1e-10, 1e-6])
    # warm up every variant (plans, workspaces)
    for form in forms.values():
        for tol in tols:
            for _ in range(args.warmup):
                step(tol, form)
    torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    headline_form = args.profile or ("mixed" if "mixed" in forms else "plain")
    for fname, form in forms.items():
        for tol in tols:
            is_head = (fname == headline_form and tol == tols[0])
            if is_head:
                clocks.start()
            ms, launches = timed(tol, form, args.steps)
            clk = clocks.stop() if is_head else None
            err = errors()
            results[(fname, tol)] = {"ms": ms, "launches": launches, "targets_per_s": world * N / (ms / 1e3),
                                     "err": err, "clocks": clk}

    if args.profile:
        r = results[(args.profile, args.profile_tol)]
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": r["targets_per_s"], "unit": UNIT, "ms_per_step": r["ms"],
                              "profile": args.profile, "gpu_launches": r["launches"], "err": r["err"]}), flush=True)
        reps.close()
        return

    # per-stage timings of the headline form (separate pass, events inside the library)
    ctx.set_timing(True)
    stage = {"near": [], "spread": [], "fft": [], "gather": [], "cells": [], "total": []}
    info_params = {}
    for _ in range(max(3, min(args.steps, 5))):
        for kind in (ft.KIND_SLP, ft.KIND_DLP):
            fn = ft.StokesSLP_ewald_2p if kind == ft.KIND_SLP else ft.StokesDLP_ewald_2p
            a = dev
            extra = (a["n1"], a["n2"]) if kind == ft.KIND_DLP else ()
            (_, info) = fn(a["xsrc"], a["ysrc"], a["xtar"], a["ytar"], *extra, a["f1"], a["f2"], 1.0, 1.0, tol=1e-10,
                           form=forms[headline_form], ctx=ctx, out=(outs[0], outs[1]), parts=False,
                           return_info=True)
            key = "slp" if kind == ft.KIND_SLP else "dlp"
            info_params[key] = info.params.as_dict()
            for s, v in (("near", info.ms_near), ("spread", info.ms_spread), ("fft", info.ms_fft),
                         ("gather", info.ms_gather), ("cells", info.ms_cells), ("total", info.ms_total)):
                stage[s].append((key, v))
    ctx.set_timing(False)

    def mean_stage(s, key):
        v = [x for k, x in stage[s] if k == key]
        return float(np.mean(v)) if v else 0.0

    # e2e: the same public API on pinned host buffers (H2D of inputs and D2H of
    # the velocities inside the timed region)
    pin = {k: torch.from_numpy(cfg[k]).pin_memory() for k in keys}
    hin = {k: v.numpy() for k, v in pin.items()}
    hout = [torch.empty(N, dtype=torch.float64).pin_memory().numpy() for _ in range(4)]
    for _ in range(2):
        step(1e-10, forms[headline_form], hin, hout)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(1e-10, forms[headline_form], hin, hout)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) / args.steps * 1e3)
    h2d = 8 * N * (6 + 8)  # SLP: xs, ys, xt, yt, f1, f2 ; DLP: + n1, n2
    d2h = 8 * N * 4

    head = results[(headline_form, 1e-10)]
    # roofline of the dominant kernel (the real-space sum): algorithmic bytes
    # per launch = sorted sources (position + densities) and targets (position,
    # index, output) read/written once.  The kernel is bound by instruction
    # issue on the FP32 pipe (float-float pairs), so its pair rate is reported
    # beside the HBM fraction: expected pairs within the cutoff N^2 pi rc^2 / area
    # (uniform points) per second of the launch.
    near_ms = {k: mean_stage("near", k) for k in ("slp", "dlp")}
    bytes_near = {"slp": N * (16 + 16) + N * (16 + 4 + 16), "dlp": N * (16 + 24) + N * (16 + 4 + 16)}
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        hbm_peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    dom = "dlp" if near_ms["dlp"] > near_ms["slp"] else "slp"
    achieved = bytes_near[dom] / (near_ms[dom] / 1e3) / 1e9 if near_ms[dom] > 0 else 0.0
    rc = float(info_params.get(dom, {}).get("rc", 0.0))
    pairs = float(N) * float(N) * np.pi * rc * rc
    pair_rate = pairs / (near_ms[dom] / 1e3) if near_ms[dom] > 0 else 0.0
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tr_path):
        traffic = json.load(open(tr_path)).get(f"near_{dom}_bytes_per_launch_1M")

    keep = ("nside_x", "xi", "Mx", "My", "P", "form")
    line = {
        "metric": METRIC, "value": head["targets_per_s"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if headline_form == "plain" else "f64/f32", "data": "synthetic",
        "config": {"workload": f"config3: SLP+DLP spectral Ewald, {N} sources / {N} targets uniform in [0,1]^2, "
                               f"zero-mean N(0,1) densities, random unit normals, tol 1e-10, {headline_form} form",
                   "l2": "flushed before every step (256 MB write, outside the timed events)",
                   "parallelism": f"replicas x{world}",
                   "params": {k: {q: v[q] for q in keep if q in v} for k, v in info_params.items()}},
        "stages_ms": {k: {s: round(mean_stage(s, k), 4) for s in stage} for k in ("slp", "dlp")},
    }
    if not (args.quick or args.no_batch):
        line["batched"] = batched_section(ft, wl, ctx, stream, args.steps, args.warmup, flush)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(N)
    # the figures a reader checks first go last, where a truncated log keeps them
    line["roofline"] = {"bound": "hbm", "kernel": f"k_near<{dom.upper()}>", "achieved": achieved,
                        "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                        "peak_source": peak_src, "pairs_per_s": pair_rate,
                        "note": "issue-bound kernel (FP32 pipe in the mixed form, FP64 pipe in the plain form); "
                                "pipe figures in profiles/"}
    line["clocks"] = head["clocks"]
    line["gpu_launches"] = head["launches"]
    line["e2e"] = {"value": world * N / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    line["forms"] = {f"{f}@{t:g}": {"targets_per_s": r["targets_per_s"], "ms_per_step": r["ms"], "err": r["err"]}
                     for (f, t), r in results.items()}
    if "plain" in forms and "mixed" in forms:
        line["mixed_over_plain"] = {f"{t:g}": results[("plain", t)]["ms"] / results[("mixed", t)]["ms"]
                                    for t in tols}
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()


if __name__ == "__main__":
    main()
