"""GB300 spectral Ewald summation for the doubly-periodic 2-D Stokeslet and stresslet.

Python mirror of annabroms/FastTools2D's spectral Ewald interface, backed by
the CUDA library ``_build/libfte_gb300.so`` (C ABI in ``include/fasttools2d.h``):

* ``StokesSLP_ewald_2p`` / ``StokesDLP_ewald_2p`` mirror the MATLAB drivers
  (PeriodicEwald/src/matlab/StokesSLP_ewald_2p.m:1-2, StokesDLP_ewald_2p.m:1-2):
  same positional arguments, the options ``P``, ``Nb``, ``tol``, ``verbose``,
  and the outputs ``(u1, u2, ur, uk, xi)``.
* ``mex_stokes_slp_real``, ``mex_stokes_slp_kspace``, ``mex_stokes_dlp_real``,
  ``mex_stokes_dlp_kspace`` mirror the four MEX gateways (argument order of
  PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:65-83, ..._kspace.cpp:19-45,
  PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:36-52, ..._kspace.cpp:239-264);
  2 x N arrays are given as (N, 2) arrays (x/y interleaved, the same memory).

Arrays may be numpy arrays (host memory; copied to the GPU inside the call) or
CUDA torch tensors (used in place).  There is no CPU fallback: if the library
is missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfte_gb300.so")

FTE_OK = 0
FTE_ERR_INVALID = 1
FTE_ERR_CUDA = 2
FTE_ERR_ALLOC = 3
FTE_ERR_UNSUPPORTED = 4
FTE_ERR_DEVICE = 5
FTE_DEVICE_POINTERS = 1
FTE_HOST_ASYNC = 2
FORM_PLAIN = 0
FORM_MIXED = 1
FORM_FF = 2  # fte_params.form only: float-float spread and gather
FORM_FF32 = 3  # fte_params.form only: float-float transforms, FP32 spread and gather products
KSPACE_AUTO, KSPACE_FP64, KSPACE_FP32, KSPACE_FF, KSPACE_FF32 = 0, 1, 2, 3, 4
NEAR_AUTO, NEAR_FP64, NEAR_FF = 0, 1, 2
KIND_SLP = 0
KIND_DLP = 1
Q_VELOCITY = 0
Q_PRESSURE = 1
Q_PRESSURE_GRAD = 2
Q_GRADIENT = 3
Q_STRESS = 4
Q_VORTICITY = 5
Q_NCOMP = {Q_VELOCITY: 2, Q_PRESSURE: 1, Q_PRESSURE_GRAD: 2, Q_GRADIENT: 4, Q_STRESS: 4, Q_VORTICITY: 1}


class FteError(RuntimeError):
    """A call into the GPU library failed; ``code`` is the FTE_ERR_* status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[fte status {code}] {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("P", C.c_int), ("Nb", C.c_double), ("tol", C.c_double), ("Q", C.c_double),
                ("A", C.c_int), ("B", C.c_int), ("nside_x", C.c_int), ("nside_y", C.c_int),
                ("rc", C.c_double), ("xi", C.c_double), ("kinf", C.c_int), ("Mx", C.c_int), ("My", C.c_int),
                ("w", C.c_double), ("eta", C.c_double), ("form", C.c_int), ("ts_spread", C.c_int),
                ("ts_gather", C.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Options(C.Structure):
    _fields_ = [("P", C.c_int), ("Nb", C.c_double), ("tol", C.c_double), ("xi", C.c_double),
                ("Mx", C.c_int), ("My", C.c_int), ("nside_x", C.c_int), ("nside_y", C.c_int),
                ("weights", C.c_void_p), ("form", C.c_int), ("tune", C.c_int), ("slack", C.c_double),
                ("kspace", C.c_int), ("near", C.c_int)]


class Info(C.Structure):
    _fields_ = [("params", Params), ("ms_total", C.c_double), ("ms_cells", C.c_double), ("ms_near", C.c_double),
                ("ms_spread", C.c_double), ("ms_fft", C.c_double), ("ms_gather", C.c_double),
                ("near_pairs", C.c_longlong), ("kernels_launched", C.c_int)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "params"}
        d["params"] = self.params.as_dict()
        return d


_lock = threading.Lock()
_lib = None
_default_ctx = None

_vp = C.c_void_p
_i64 = C.c_int64
_d = C.c_double
_i = C.c_int
_u = C.c_uint

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "fte_last_error": (C.c_char_p, []),
    "fte_version": (_i, []),
    "fte_create": (_i, [C.POINTER(_vp), _i]),
    "fte_destroy": (_i, [_vp]),
    "fte_set_stream": (_i, [_vp, _vp]),
    "fte_set_timing": (_i, [_vp, _i]),
    "fte_kernel_count": (C.c_longlong, [_vp]),
    "fte_slp_real": (_i, [_vp, _vp, _i64, _vp, _i64, _vp, _d, _i, _i, _d, _d, _vp, _u]),
    "fte_dlp_real": (_i, [_vp, _vp, _i64, _vp, _i64, _vp, _vp, _d, _i, _i, _d, _d, _vp, _u]),
    "fte_slp_kspace": (_i, [_vp, _vp, _i64, _vp, _i64, _d, _d, _vp, _i, _i, _d, _d, _d, _i, _vp, _u]),
    "fte_dlp_kspace": (_i, [_vp, _vp, _i64, _vp, _i64, _d, _d, _vp, _vp, _i, _i, _d, _d, _d, _i, _vp, _u]),
    "fte_stokes_slp_ewald_2p": (_i, [_vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _d, _d, C.POINTER(Options),
                                     _vp, _vp, _vp, _vp, C.POINTER(Info), _u]),
    "fte_stokes_dlp_ewald_2p": (_i, [_vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _d, _d,
                                     C.POINTER(Options), _vp, _vp, _vp, _vp, C.POINTER(Info), _u]),
    "fte_choose_params": (_i, [_i, _i64, _i64, _vp, _vp, _d, _d, C.POINTER(Options), C.POINTER(Params)]),
    "fte_plan_create": (_i, [_vp, _i, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _d, _d,
                             C.POINTER(Options), _i, C.POINTER(_vp), _u]),
    "fte_plan_params": (_i, [_vp, C.POINTER(Params)]),
    "fte_plan_execute": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _u]),
    "fte_plan_destroy": (_i, [_vp]),
    "fte_batch_create": (_i, [_vp, C.POINTER(_vp), _i, _i, C.POINTER(_vp)]),
    "fte_batch_launch": (_i, [_vp, _i]),
    "fte_batch_destroy": (_i, [_vp]),
    "fte_batch_set_density": (_i, [_vp, _i, _vp, _vp, _u]),
    "fte_batch_get_velocity": (_i, [_vp, _i, _vp, _vp, _u]),
    "fte_q_ncomp": (_i, [_i]),
    "fte_q_real": (_i, [_vp, _i, _i, _vp, _i64, _vp, _i64, _vp, _vp, _d, _i, _i, _d, _d, _vp, _u]),
    "fte_q_kspace": (_i, [_vp, _i, _i, _vp, _i64, _vp, _i64, _vp, _vp, _d, _d, _i, _i, _d, _d, _d, _i, _vp, _u]),
    "fte_stokes_q_ewald_2p": (_i, [_vp, _i, _i, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d,
                                   C.POINTER(Options), _vp, _vp, _vp, C.POINTER(Info), _u]),
    "fte_nn_sample": (_i, [_vp, _vp, _vp, _i64, _d, _d, _i, _vp, _u]),
    "fte_mlp_param_count": (_i, []),
    "fte_mlp_scratch_floats": (C.c_size_t, [_i]),
    "fte_mlp_forward": (_i, [_vp, _vp, _i, _vp, _vp]),
    "fte_mlp_loss_grad": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "fte_mlp_adam": (_i, [_vp, _vp, _vp, _vp, _i, C.c_float, C.c_float, C.c_float, C.c_float, _vp]),
}


def build(verbose: bool = False) -> str:
    """Compile the CUDA library for sm_103a (see buildlib.py)."""
    from . import buildlib

    return buildlib.build(verbose=verbose)


def lib():
    """Load the GPU library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise FteError(FTE_ERR_UNSUPPORTED,
                               f"GPU library not built: {LIB_PATH} is missing (run fasttools2d_gb300.build())")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _check(status: int):
    if status != FTE_OK:
        msg = lib().fte_last_error()
        raise FteError(status, msg.decode() if msg else "")


class Context:
    """Owns a CUDA stream and the device workspace of the library."""

    def __init__(self, device: int = 0):
        h = _vp()
        _check(lib().fte_create(C.byref(h), int(device)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            lib().fte_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        _check(lib().fte_set_stream(self.h, _vp(stream_handle) if stream_handle else None))

    def set_timing(self, on: bool):
        _check(lib().fte_set_timing(self.h, 1 if on else 0))

    @property
    def kernel_count(self) -> int:
        return lib().fte_kernel_count(self.h)


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---- argument marshalling ----------------------------------------------------

def _is_cuda_tensor(a) -> bool:
    return hasattr(a, "is_cuda") and getattr(a, "is_cuda")


class _Args:
    """Collects pointers for one call; all arrays must be on the same side."""

    def __init__(self):
        self.keep = []
        self.device = None

    def arr(self, a, ncomp: int, n: int | None = None):
        if a is None:
            return None, 0
        if _is_cuda_tensor(a):
            import torch

            t = a.to(torch.float64).contiguous()
            if self.device is False:
                raise ValueError("mixing host and device arrays in one call")
            self.device = True
            self.keep.append(t)
            cnt = t.numel() // ncomp
            return t.data_ptr(), cnt
        x = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        if ncomp == 2 and x.ndim == 2 and x.shape[1] != 2 and x.shape[0] == 2:
            x = np.ascontiguousarray(x.T)  # accept MATLAB-shaped 2 x N
        if self.device is True:
            raise ValueError("mixing host and device arrays in one call")
        self.device = False
        self.keep.append(x)
        return x.ctypes.data, x.size // ncomp

    def out(self, shape, given=None):
        if given is not None:
            if _is_cuda_tensor(given) != bool(self.device):
                raise ValueError("output buffer on the wrong side")
            if tuple(given.shape) != tuple(shape):
                raise ValueError(f"output buffer has shape {tuple(given.shape)}, expected {tuple(shape)}")
            if _is_cuda_tensor(given):
                import torch

                if given.dtype != torch.float64 or not given.is_contiguous():
                    raise ValueError("output buffer must be contiguous float64")
                return given, given.data_ptr()
            if given.dtype != np.float64 or not given.flags["C_CONTIGUOUS"]:
                raise ValueError("output buffer must be contiguous float64")
            return given, given.ctypes.data
        if self.device:
            import torch

            t = torch.empty(shape, dtype=torch.float64, device="cuda")
            self.keep.append(t)
            return t, t.data_ptr()
        x = np.empty(shape, dtype=np.float64)
        self.keep.append(x)
        return x, x.ctypes.data

    @property
    def flags(self) -> int:
        return FTE_DEVICE_POINTERS if self.device else 0


# ---- MEX-shaped entries --------------------------------------------------------

def mex_stokes_slp_real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly, ctx: Context | None = None):
    ctx = ctx or default_context()
    A = _Args()
    ps, ns = A.arr(psrc, 2)
    pt, nt = A.arr(ptar, 2)
    pf, nf = A.arr(f, 2)
    if nf != ns:
        raise ValueError("psrc and f must be the same size.")
    out, po = A.out((nt, 2))
    _check(lib().fte_slp_real(ctx.h, ps, ns, pt, nt, pf, float(xi), int(nside_x), int(nside_y), float(Lx), float(Ly),
                              po, A.flags))
    return out


def mex_stokes_dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly, ctx: Context | None = None):
    ctx = ctx or default_context()
    A = _Args()
    ps, ns = A.arr(psrc, 2)
    pt, nt = A.arr(ptar, 2)
    pf, nf = A.arr(f, 2)
    pn, nn = A.arr(n, 2)
    if nf != ns:
        raise ValueError("psrc and f must be the same size.")
    if nn != ns:
        raise ValueError("psrc and n must be the same size.")
    out, po = A.out((nt, 2))
    _check(lib().fte_dlp_real(ctx.h, ps, ns, pt, nt, pf, pn, float(xi), int(nside_x), int(nside_y), float(Lx),
                              float(Ly), po, A.flags))
    return out


def mex_stokes_slp_kspace(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P, ctx: Context | None = None):
    ctx = ctx or default_context()
    A = _Args()
    ps, ns = A.arr(psrc, 2)
    pt, nt = A.arr(ptar, 2)
    pf, nf = A.arr(f, 2)
    if nf != ns:
        raise ValueError("psrc and f must be the same size.")
    out, po = A.out((nt, 2))
    _check(lib().fte_slp_kspace(ctx.h, ps, ns, pt, nt, float(xi), float(eta), pf, int(Mx), int(My), float(Lx),
                                float(Ly), float(w), int(P), po, A.flags))
    return out


def mex_stokes_dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P, ctx: Context | None = None):
    ctx = ctx or default_context()
    A = _Args()
    ps, ns = A.arr(psrc, 2)
    pt, nt = A.arr(ptar, 2)
    pf, nf = A.arr(f, 2)
    pn, nn = A.arr(n, 2)
    if nf != ns:
        raise ValueError("psrc and f must be the same size.")
    if nn != ns:
        raise ValueError("psrc and n must be the same size.")
    out, po = A.out((nt, 2))
    _check(lib().fte_dlp_kspace(ctx.h, ps, ns, pt, nt, float(xi), float(eta), pf, pn, int(Mx), int(My), float(Lx),
                                float(Ly), float(w), int(P), po, A.flags))
    return out


# ---- driver-shaped entries -----------------------------------------------------

def _options(P=None, Nb=None, tol=1e-16, xi=None, Mx=None, My=None, nside_x=None, nside_y=None, weights_ptr=None,
             form=FORM_PLAIN, tune=False, slack=None, kspace=KSPACE_AUTO, near=NEAR_AUTO) -> Options:
    o = Options()
    o.P = int(P or 0)
    o.Nb = float(Nb) if Nb else 0.0
    o.tol = float(tol) if tol else 0.0
    o.xi = float(xi) if xi else 0.0
    o.Mx = int(Mx or 0)
    o.My = int(My or 0)
    o.nside_x = int(nside_x or 0)
    o.nside_y = int(nside_y or 0)
    o.weights = weights_ptr
    o.form = int(form)
    o.tune = 1 if tune else 0
    o.slack = float(slack) if slack else 0.0
    o.kspace = int(kspace or 0)
    o.near = int(near or 0)
    return o


def _print_verbose(kind: str, ns: int, nt: int, info: Info):
    p = info.params
    print("*********************************************************")
    print(f"SPECTRAL EWALD FOR THE STOKES {kind} POTENTIAL (GB300)\n")
    print(f"NUMBER OF SOURCES: {ns}\nNUMBER OF TARGETS: {nt}\nTOLERANCE: {p.tol:.3e}\nP: {p.P}\n"
          f"Points per box: {p.Nb:g}")
    print(f"\nPARAMETER INFORMATION:\n\txi: {p.xi:.3f}\n\trc: {p.rc:.3f}\n\tkinf: {p.kinf}\n\tMx: {p.Mx}\n"
          f"\tMy: {p.My}\n\tw: {p.w:.3f}\n\teta: {p.eta:.3f}")
    print(f"TIME: total {info.ms_total:.3f} ms (near {info.ms_near:.3f}, spread {info.ms_spread:.3f}, "
          f"fft+filter {info.ms_fft:.3f}, gather {info.ms_gather:.3f})")
    print("*********************************************************\n")


def _ewald(kind, xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, P, Nb, tol, verbose, weights, xi, Mx, My,
           nside_x, nside_y, form, ctx, return_info, out, parts, slack=None, kspace=KSPACE_AUTO, near=NEAR_AUTO):
    ctx = ctx or default_context()
    A = _Args()
    pxs, ns = A.arr(xsrc, 1)
    pys, _ = A.arr(ysrc, 1)
    pxt, nt = A.arr(xtar, 1)
    pyt, _ = A.arr(ytar, 1)
    pn1, _ = A.arr(n1, 1)
    pn2, _ = A.arr(n2, 1)
    pf1, _ = A.arr(f1, 1)
    pf2, _ = A.arr(f2, 1)
    pw, _ = A.arr(weights, 1)
    u1, pu1 = A.out((nt,), out[0] if out is not None else None)
    u2, pu2 = A.out((nt,), out[1] if out is not None else None)
    ur = uk = None
    pur = puk = None
    if parts:
        ur, pur = A.out((nt, 2))
        uk, puk = A.out((nt, 2))
    opt = _options(P, Nb, tol, xi, Mx, My, nside_x, nside_y, pw, form, slack=slack, kspace=kspace, near=near)
    info = Info()
    if verbose:
        ctx.set_timing(True)
    if kind == KIND_SLP:
        st = lib().fte_stokes_slp_ewald_2p(ctx.h, pxs, pys, ns, pxt, pyt, nt, pf1, pf2, float(Lx), float(Ly),
                                           C.byref(opt), pu1, pu2, pur, puk, C.byref(info), A.flags)
    else:
        st = lib().fte_stokes_dlp_ewald_2p(ctx.h, pxs, pys, ns, pxt, pyt, nt, pn1, pn2, pf1, pf2, float(Lx),
                                           float(Ly), C.byref(opt), pu1, pu2, pur, puk, C.byref(info), A.flags)
    _check(st)
    if verbose:
        _print_verbose("SINGLE-LAYER" if kind == KIND_SLP else "DOUBLE-LAYER", ns, nt, info)
    res = (u1, u2, ur, uk, info.params.xi)
    return (res, info) if return_info else res


def StokesSLP_ewald_2p(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, P=None, Nb=None, tol=1e-16, verbose=0,
                       weights=None, xi=None, Mx=None, My=None, nside_x=None, nside_y=None, form=FORM_PLAIN,
                       ctx: Context | None = None, return_info: bool = False, out=None, parts: bool = True,
                       slack=None, kspace=KSPACE_AUTO, near=NEAR_AUTO):
    """Spectral Ewald evaluation of the doubly-periodic Stokeslet.

    Returns (u1, u2, ur, uk, xi) like the MATLAB driver; ur and uk are
    (Ntar, 2) (None when parts=False).  ``out=(u1, u2)`` supplies the output
    buffers (same side as the inputs).  ``form=FORM_MIXED`` takes the tuned
    parameter choice with FP32 pairs where the tolerance allows; ``kspace``
    (KSPACE_*) then forces its k-space arithmetic and ``near`` (NEAR_*) the
    arithmetic of the real-space pairs.
    """
    return _ewald(KIND_SLP, xsrc, ysrc, xtar, ytar, None, None, f1, f2, Lx, Ly, P, Nb, tol, verbose, weights, xi, Mx,
                  My, nside_x, nside_y, form, ctx, return_info, out, parts, slack, kspace, near)


def StokesDLP_ewald_2p(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, P=None, Nb=None, tol=1e-16, verbose=0,
                       weights=None, xi=None, Mx=None, My=None, nside_x=None, nside_y=None, form=FORM_PLAIN,
                       ctx: Context | None = None, return_info: bool = False, out=None, parts: bool = True,
                       slack=None, kspace=KSPACE_AUTO, near=NEAR_AUTO):
    """Spectral Ewald evaluation of the doubly-periodic stresslet (double layer).

    Returns (u1, u2, ur, uk, xi); uk includes the k = 0 mode like the MATLAB
    driver.  Options as for StokesSLP_ewald_2p.
    """
    return _ewald(KIND_DLP, xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, P, Nb, tol, verbose, weights, xi, Mx,
                  My, nside_x, nside_y, form, ctx, return_info, out, parts, slack, kspace, near)


def choose_params(kind, f1, f2, ntar, Lx, Ly, P=None, Nb=None, tol=1e-16, **kw) -> Params:
    """The drivers' analytic parameter choice (host only, no GPU needed)."""
    f1 = np.ascontiguousarray(f1, dtype=np.float64)
    f2 = np.ascontiguousarray(f2, dtype=np.float64)
    opt = _options(P, Nb, tol, **kw)
    prm = Params()
    _check(lib().fte_choose_params(int(kind), len(f1), int(ntar), f1.ctypes.data, f2.ctypes.data, float(Lx),
                                   float(Ly), C.byref(opt), C.byref(prm)))
    return prm


def nn_sample(xsrc, ysrc, Lx, Ly, nsample=2048, ctx: Context | None = None):
    """Distances from a deterministic sample of the sources (every stride-th,
    stride = max(1, N // nsample)) to their nearest other source in the
    periodic box, computed on the GPU from a device cell list
    (``fte_nn_sample``).  Host or CUDA arrays; returns a numpy array."""
    ctx = ctx or default_context()
    A = _Args()
    px, n = A.arr(xsrc, 1)
    py, _ = A.arr(ysrc, 1)
    stride = max(1, n // nsample)
    ns = min(nsample, (n + stride - 1) // stride)
    out, po = A.out((ns,))
    _check(lib().fte_nn_sample(ctx.h, px, py, n, float(Lx), float(Ly), int(nsample), po, A.flags))
    return out.cpu().numpy() if hasattr(out, "cpu") else out


# ---- plans and batches -----------------------------------------------------------

class Plan:
    """Geometry of one SE evaluation reused across density vectors (a GMRES
    loop): parameters, cell list, tile bins and scratch are set up once.

    ``execute(f1s, f2s)`` takes arrays of shape (nv, nsrc) (numpy or CUDA
    tensors) and returns velocities of shape (nv, ntar)."""

    def __init__(self, kind, xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, n1=None, n2=None, P=None, Nb=None,
                 tol=1e-16, form=FORM_PLAIN, weights=None, nvmax=4, ctx: Context | None = None, **kw):
        self.ctx = ctx or default_context()
        A = _Args()
        pxs, ns = A.arr(xsrc, 1)
        pys, _ = A.arr(ysrc, 1)
        pxt, nt = A.arr(xtar, 1)
        pyt, _ = A.arr(ytar, 1)
        pn1, _ = A.arr(n1, 1)
        pn2, _ = A.arr(n2, 1)
        pf1, _ = A.arr(f1, 1)
        pf2, _ = A.arr(f2, 1)
        pw, _ = A.arr(weights, 1)
        opt = _options(P, Nb, tol, weights_ptr=pw, form=form, **kw)
        h = _vp()
        _check(lib().fte_plan_create(self.ctx.h, int(kind), pxs, pys, ns, pxt, pyt, nt, pn1, pn2, pf1, pf2,
                                     float(Lx), float(Ly), C.byref(opt), int(nvmax), C.byref(h), A.flags))
        self.h = h
        self.kind, self.nsrc, self.ntar, self.nvmax = int(kind), ns, nt, int(nvmax)

    @property
    def params(self) -> Params:
        p = Params()
        _check(lib().fte_plan_params(self.h, C.byref(p)))
        return p

    def execute(self, f1s, f2s):
        A = _Args()
        pf1, n1 = A.arr(f1s, 1)
        pf2, _ = A.arr(f2s, 1)
        nv = n1 // max(self.nsrc, 1) if self.nsrc else 1
        u1, pu1 = A.out((nv, self.ntar))
        u2, pu2 = A.out((nv, self.ntar))
        _check(lib().fte_plan_execute(self.h, nv, pf1, pf2, pu1, pu2, A.flags))
        return u1, u2

    def close(self):
        if getattr(self, "h", None):
            lib().fte_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many plans evaluated by one launch (a replayed CUDA graph)."""

    def __init__(self, plans, nv: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.plans = list(plans)
        self.nv = int(nv)
        arr = (_vp * len(self.plans))(*[p.h for p in self.plans])
        h = _vp()
        _check(lib().fte_batch_create(self.ctx.h, arr, len(self.plans), self.nv, C.byref(h)))
        self.h = h

    def set_density(self, i, f1s, f2s, pinned_async=False):
        """Copy plan i's density vectors in.  pinned_async: f1s, f2s are
        page-locked host arrays; the copy is queued without synchronising
        (synchronise the context's stream before reusing them)."""
        if pinned_async and not _is_cuda_tensor(f1s):
            # the copy outlives the call: no temporary conversions allowed
            for a in (f1s, f2s):
                if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                    raise ValueError("pinned_async needs contiguous float64 numpy arrays (page-locked)")
        A = _Args()
        pf1, _ = A.arr(f1s, 1)
        pf2, _ = A.arr(f2s, 1)
        flags = A.flags | (FTE_HOST_ASYNC if pinned_async and not (A.flags & FTE_DEVICE_POINTERS) else 0)
        _check(lib().fte_batch_set_density(self.h, int(i), pf1, pf2, flags))

    def launch(self, use_graph: bool = True):
        _check(lib().fte_batch_launch(self.h, 1 if use_graph else 0))

    def velocity(self, i):
        p = self.plans[i]
        u1 = np.empty((self.nv, p.ntar))
        u2 = np.empty((self.nv, p.ntar))
        _check(lib().fte_batch_get_velocity(self.h, int(i), u1.ctypes.data, u2.ctypes.data, 0))
        return u1, u2

    def close(self):
        if getattr(self, "h", None):
            lib().fte_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- other quantities: gateway level ------------------------------------------------

def q_real(kind, q, psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly, ctx: Context | None = None):
    """Real-space sum of quantity q (``Q_PRESSURE`` .. ``Q_VORTICITY``): (Ntar, ncomp)."""
    ctx = ctx or default_context()
    A = _Args()
    ps, ns = A.arr(psrc, 2)
    pt, nt = A.arr(ptar, 2)
    pf, nf = A.arr(f, 2)
    pn, nn = A.arr(n, 2) if kind == KIND_DLP else (None, ns)
    if nf != ns or nn != ns:
        raise ValueError("psrc, f (and n) must be the same size.")
    out, po = A.out((nt, Q_NCOMP.get(q, 1)))  # an unknown q is rejected by the library
    _check(lib().fte_q_real(ctx.h, int(kind), int(q), ps, ns, pt, nt, pf, pn, float(xi), int(nside_x), int(nside_y),
                            float(Lx), float(Ly), po, A.flags))
    return out


def q_kspace(kind, q, psrc, ptar, f, n, xi, eta, Mx, My, Lx, Ly, w, P, ctx: Context | None = None):
    """k-space sum of quantity q: (Ntar, ncomp)."""
    ctx = ctx or default_context()
    A = _Args()
    ps, ns = A.arr(psrc, 2)
    pt, nt = A.arr(ptar, 2)
    pf, nf = A.arr(f, 2)
    pn, nn = A.arr(n, 2) if kind == KIND_DLP else (None, ns)
    if nf != ns or nn != ns:
        raise ValueError("psrc, f (and n) must be the same size.")
    out, po = A.out((nt, Q_NCOMP.get(q, 1)))  # an unknown q is rejected by the library
    _check(lib().fte_q_kspace(ctx.h, int(kind), int(q), ps, ns, pt, nt, pf, pn, float(xi), float(eta), int(Mx),
                              int(My), float(Lx), float(Ly), float(w), int(P), po, A.flags))
    return out


def _make_q_gateways():
    """mex_stokes_{slp,dlp}_<q>_{real,kspace} with each gateway's own argument
    order (PeriodicEwald/src/mex/Stokes{SLP,DLP}/mex_stokes_*_{real,kspace}.cpp):
    real (psrc, ptar, f, [n,] xi, nside_x, nside_y, Lx, Ly); k-space either
    (psrc, ptar, xi, eta, f, [n,] Mx, My, Lx, Ly, w, P) or, for the pressure, the
    pressure gradient and the stresslet vorticity, (psrc, ptar, f, [n,] xi, eta,
    Mx, My, Lx, Ly, w, P)."""
    names = {Q_PRESSURE: "pressure", Q_PRESSURE_GRAD: "pressure_grad", Q_GRADIENT: "gradient", Q_STRESS: "stress",
             Q_VORTICITY: "vorticity"}
    f_first = {(KIND_SLP, Q_PRESSURE), (KIND_SLP, Q_PRESSURE_GRAD), (KIND_DLP, Q_PRESSURE),
               (KIND_DLP, Q_PRESSURE_GRAD), (KIND_DLP, Q_VORTICITY)}
    g = globals()
    for kind, kn in ((KIND_SLP, "slp"), (KIND_DLP, "dlp")):
        for q, qn in names.items():
            if kind == KIND_SLP:
                def real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly, ctx=None, _q=q):
                    return q_real(KIND_SLP, _q, psrc, ptar, f, None, xi, nside_x, nside_y, Lx, Ly, ctx)
                if (kind, q) in f_first:
                    def ksp(psrc, ptar, f, xi, eta, Mx, My, Lx, Ly, w, P, ctx=None, _q=q):
                        return q_kspace(KIND_SLP, _q, psrc, ptar, f, None, xi, eta, Mx, My, Lx, Ly, w, P, ctx)
                else:
                    def ksp(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P, ctx=None, _q=q):
                        return q_kspace(KIND_SLP, _q, psrc, ptar, f, None, xi, eta, Mx, My, Lx, Ly, w, P, ctx)
            else:
                def real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly, ctx=None, _q=q):
                    return q_real(KIND_DLP, _q, psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly, ctx)
                if (kind, q) in f_first:
                    def ksp(psrc, ptar, f, n, xi, eta, Mx, My, Lx, Ly, w, P, ctx=None, _q=q):
                        return q_kspace(KIND_DLP, _q, psrc, ptar, f, n, xi, eta, Mx, My, Lx, Ly, w, P, ctx)
                else:
                    def ksp(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P, ctx=None, _q=q):
                        return q_kspace(KIND_DLP, _q, psrc, ptar, f, n, xi, eta, Mx, My, Lx, Ly, w, P, ctx)
            real.__name__ = f"mex_stokes_{kn}_{qn}_real"
            ksp.__name__ = f"mex_stokes_{kn}_{qn}_kspace"
            g[real.__name__] = real
            g[ksp.__name__] = ksp


_make_q_gateways()


# ---- other quantities: driver level -------------------------------------------------

def q_ewald_2p(kind, q, xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, n1=None, n2=None, b1=None, b2=None, P=None, Nb=None,
               tol=1e-16, xi=None, Mx=None, My=None, nside_x=None, nside_y=None, ctx: Context | None = None,
               return_info=False):
    """The quantity drivers (StokesSLP/DLP_<q>_ewald_2p): returns (out, out_real, out_k, xi) with out of
    shape (Ntar,) for the pressure and the vorticity and (Ntar, 2) otherwise."""
    ctx = ctx or default_context()
    A = _Args()
    pxs, ns = A.arr(xsrc, 1)
    pys, _ = A.arr(ysrc, 1)
    pxt, nt = A.arr(xtar, 1)
    pyt, _ = A.arr(ytar, 1)
    pn1, _ = A.arr(n1, 1)
    pn2, _ = A.arr(n2, 1)
    pf1, _ = A.arr(f1, 1)
    pf2, _ = A.arr(f2, 1)
    pb1, _ = A.arr(b1, 1)
    pb2, _ = A.arr(b2, 1)
    shape = (nt,) if q in (Q_PRESSURE, Q_VORTICITY) else (nt, 2)
    out, po = A.out(shape)
    outr, por = A.out(shape)
    outk, pok = A.out(shape)
    opt = _options(P, Nb, tol, xi, Mx, My, nside_x, nside_y)
    info = Info()
    _check(lib().fte_stokes_q_ewald_2p(ctx.h, int(kind), int(q), pxs, pys, ns, pxt, pyt, nt, pn1, pn2, pf1, pf2, pb1,
                                       pb2, float(Lx), float(Ly), C.byref(opt), po, por, pok, C.byref(info),
                                       A.flags))
    res = (out, outr, outk, info.params.xi)
    return (res, info) if return_info else res


def _make_q_drivers():
    """StokesSLP_<q>_ewald_2p / StokesDLP_<q>_ewald_2p with the MATLAB drivers'
    positional arguments and outputs (PeriodicEwald/src/matlab/):
      pressure, pressure_grad, vorticity: (..., [n1, n2,] f1, f2, Lx, Ly) -> (p, pr, pk, xi)
      gradient, stress: (..., [n1, n2,] f1, f2, b1, b2, Lx, Ly) -> (out1, out2, out_r, out_k, xi)"""
    names = {Q_PRESSURE: "pressure", Q_PRESSURE_GRAD: "pressure_grad", Q_GRADIENT: "gradient", Q_STRESS: "stress",
             Q_VORTICITY: "vorticity"}
    g = globals()
    for kind, kn in ((KIND_SLP, "SLP"), (KIND_DLP, "DLP")):
        for q, qn in names.items():
            with_b = q in (Q_GRADIENT, Q_STRESS)

            def drv(*args, _k=kind, _q=q, _b=with_b, **kw):
                a = list(args)
                xs, ys, xt, yt = a[:4]
                rest = a[4:]
                n1 = n2 = None
                if _k == KIND_DLP:
                    n1, n2, rest = rest[0], rest[1], rest[2:]
                f1, f2, rest = rest[0], rest[1], rest[2:]
                b1 = b2 = None
                if _b:
                    b1, b2, rest = rest[0], rest[1], rest[2:]
                Lx, Ly = rest[0], rest[1]
                out, outr, outk, xi = q_ewald_2p(_k, _q, xs, ys, xt, yt, f1, f2, Lx, Ly, n1=n1, n2=n2, b1=b1, b2=b2,
                                                 **kw)
                if _b:
                    return out[:, 0], out[:, 1], outr, outk, xi
                return out, outr, outk, xi

            drv.__name__ = f"Stokes{kn}_{qn}_ewald_2p"
            g[drv.__name__] = drv


_make_q_drivers()
