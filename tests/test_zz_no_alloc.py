"""The allocation-free Stokeslet k-space entry, fte_slp_kspace_noalloc.

It exists for callers that may not allocate device memory (an application
that gives all GPU memory to its own pool, a real-time loop that must not
allocate after start-up, a plugin host that forbids allocation outside its
initialisation).  Such a caller passes device inputs and outputs and a stream;
the entry takes its scratch from a fixed device array inside the library.

Here it is called through the C ABI on device pointers and must return what
the allocating entry fte_slp_kspace returns for the same inputs, within the
FP64 tolerance used by the other GPU tests, on consecutive calls of different
sizes (the calls share the array, which keeps the previous call's contents).
This file is collected last so that a failure here cannot hide the others.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _entry():
    import fasttools2d_gb300 as ft

    fn = ft.lib().fte_slp_kspace_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p, C.c_int,
                   C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
    return ft, fn


def _cases():
    """(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P) of two different problems."""
    g = load_golden("config1_n1000")
    ps = np.stack([g["xsrc"] - 0.5, g["ysrc"] - 0.5], 1)
    pt = np.stack([g["xtar"] - 0.5, g["ytar"] - 0.5], 1)
    f = np.stack([g["f1"], g["f2"]], 1)
    first = (ps, pt, float(g["slp_prm_xi"]), float(g["slp_prm_eta"]), f, int(g["slp_prm_Mx"]),
             int(g["slp_prm_My"]), 1.0, 1.0, float(g["slp_prm_w"]), int(g["slp_prm_P"]))
    h = load_golden("mex_slp_kspace_p16")
    a = [h[f"arg{i}"] for i in range(int(h["nargs"]))]
    second = (a[0], a[1], float(a[2]), float(a[3]), a[4], int(a[5]), int(a[6]), float(a[7]), float(a[8]), float(a[9]),
              int(a[10]))
    return first, second


def _call_noalloc(fn, case, stream):
    import torch

    ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P = case
    dps = torch.tensor(ps, dtype=torch.float64, device="cuda").reshape(-1, 2)
    dpt = torch.tensor(pt, dtype=torch.float64, device="cuda")
    df = torch.tensor(f, dtype=torch.float64, device="cuda").reshape(-1, 2)
    out = torch.full((len(pt), 2), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = fn(dps.data_ptr(), len(dps), dpt.data_ptr(), len(pt), xi, eta, df.data_ptr(), Mx, My, Lx, Ly, w, P,
            out.data_ptr(), stream)
    torch.cuda.synchronize()
    return st, out.cpu().numpy()


def test_noalloc_matches_allocating_entry(gpu_ctx):
    import torch

    ft, fn = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    first, second = _cases()
    # two different problems back to back, then the first again
    for case in (first, second, first):
        st, out = _call_noalloc(fn, case, stream)
        assert st == ft.FTE_OK, ft.lib().fte_last_error()
        ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P = case
        ref = ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P, ctx=gpu_ctx)
        assert np.all(np.isfinite(out))
        assert rel_max(out, ref) <= TOL_FP64


def test_noalloc_matches_reference_fixture(gpu_ctx):
    """The p16 case (P = 16, a window half-width the drivers would not pick)
    against the reference gateway's own output stored in the fixture."""
    import torch

    ft, fn = _entry()
    case = _cases()[1]
    st, out = _call_noalloc(fn, case, torch.cuda.current_stream().cuda_stream)
    assert st == ft.FTE_OK, ft.lib().fte_last_error()
    assert rel_max(out, load_golden("mex_slp_kspace_p16")["out"]) <= TOL_FP64


def test_noalloc_on_a_new_stream_and_without_sources(gpu_ctx):
    """A call on a freshly created stream (the grid clear, the transforms and
    the gather are ordered on that stream), then a call with no sources after
    it: the shared array still holds the previous grids, which the entry must
    clear, so the result is exactly zero."""
    import torch

    ft, fn = _entry()
    first = _cases()[0]
    s = torch.cuda.Stream()
    st, out = _call_noalloc(fn, first, s.cuda_stream)
    assert st == ft.FTE_OK, ft.lib().fte_last_error()
    ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P = first
    ref = ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P, ctx=gpu_ctx)
    assert rel_max(out, ref) <= TOL_FP64
    empty = (np.zeros((0, 2)), pt, xi, eta, np.zeros((0, 2)), Mx, My, Lx, Ly, w, P)
    st, out = _call_noalloc(fn, empty, s.cuda_stream)
    assert st == ft.FTE_OK, ft.lib().fte_last_error()
    assert np.array_equal(out, np.zeros_like(out))


def test_noalloc_rejects_grids_beyond_its_scratch(gpu_ctx):
    import torch

    ft, fn = _entry()
    ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P = _cases()[0]
    big = (ps, pt, xi, eta, f, 1024, 1024, 1.0, 1.0, 24 / 1024 / 2, 24)
    st, _ = _call_noalloc(fn, big, torch.cuda.current_stream().cuda_stream)
    assert st == ft.FTE_ERR_UNSUPPORTED
    assert b"exceeds the fixed scratch" in ft.lib().fte_last_error()
