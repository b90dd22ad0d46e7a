"""ctypes access to the CPU oracle and to the compiled reference gateways.

TEST INFRASTRUCTURE ONLY.  Tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use this module as the checker; the GPU library
never imports it.

* ``liboracle`` -- ``oracle/_build/libfte_oracle.so``: the C restatement of the
  reference spectral Ewald path (or_ewald.c) plus the reference tests' direct
  sums.
* ``ref_call`` -- the reference's own MEX gateways
  (PeriodicEwald/src/mex/{StokesSLP,StokesDLP}/mex_stokes_*.cpp), compiled
  unmodified under ``oracle/_ref`` against the MEX stand-in in ``mexshim/``.
  They are built where the reference checkout is available and, on hosts
  without it (the aarch64 GPU hosts), from the verbatim copies of the
  velocity path's sources that the build with the checkout staged under
  ``oracle/_ref/src`` (checked against ``oracle/ref_sources.sha256``).

Point/density arrays are numpy float64 arrays of shape (N, 2) in C order, i.e.
the reference's 2 x N column-major layout with x/y interleaved.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfte_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

KIND_SLP = 0
KIND_DLP = 1

_lock = threading.Lock()
_lib = None
_ref = {}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Params(C.Structure):
    """Mirror of ``or_params`` (parameters chosen by the MATLAB drivers)."""

    _fields_ = [
        ("P", C.c_int), ("Nb", C.c_double), ("tol", C.c_double), ("Q", C.c_double),
        ("A", C.c_int), ("B", C.c_int), ("a", C.c_int), ("nside_x", C.c_int), ("nside_y", C.c_int),
        ("rc", C.c_double), ("xi", C.c_double), ("kinf", C.c_int), ("Mx", C.c_int), ("My", C.c_int),
        ("w", C.c_double), ("eta", C.c_double), ("m", C.c_double), ("xi_iters", C.c_int), ("k_iters", C.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def build(quiet: bool = True) -> str:
    """Compile the oracle library with the committed Makefile."""
    out = subprocess.run(["make", "-C", HERE, "oracle"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def staged_reference() -> bool:
    """True where the verbatim copies of the reference's velocity sources
    (staged under oracle/_ref/src by ``make ref`` on a host with the checkout)
    are present."""
    return os.path.exists(os.path.join(REF_DIR, "src", "common", "ewald_tools.cpp"))


def build_reference(ref_root: str | None = None, portable: bool = False) -> bool:
    """Compile the reference gateways into oracle/_ref with oracle/Makefile.

    ref_root: the reference checkout (all gateways; also stages the velocity
    path's sources); None: the staged copy (the four velocity gateways).
    portable: also the x86 flavour built on the portable SSE header (P3)."""
    cmd = ["make", "-C", HERE, f"-j{min(16, os.cpu_count() or 1)}", "ref"]
    if portable:
        cmd.append("ref-portable")
    cmd.append(f"REF_ROOT={ref_root or ''}")
    out = subprocess.run(cmd, capture_output=True, text=True)
    return out.returncode == 0


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            L = C.CDLL(LIB_PATH)
            L.or_expint_e1.restype = C.c_double
            L.or_expint_e1.argtypes = [C.c_double]
            L.or_rat.restype = C.c_double
            L.or_rat.argtypes = [C.c_double, _ip, _ip]
            L.or_num_threads.restype = C.c_int
            L.or_choose_params.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_int,
                                           C.c_double, C.c_double, C.POINTER(Params)]
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def expint_e1(x: float) -> float:
    return lib().or_expint_e1(float(x))


def rat(x: float):
    n, d = C.c_int(), C.c_int()
    lib().or_rat(float(x), C.byref(n), C.byref(d))
    return n.value, d.value


def num_threads() -> int:
    return lib().or_num_threads()


def choose_params(kind, f1, f2, nsrc, ntar, Lx, Ly, P=24, Nb=0.0, tol=1e-16) -> Params:
    prm = Params()
    f1 = _c(f1)
    f2 = _c(f2)
    lib().or_choose_params(kind, int(nsrc), int(ntar), _p(f1), _p(f2), float(Lx), float(Ly), int(P), float(Nb),
                           float(tol), C.byref(prm))
    return prm


# ---- MEX-shaped entries (interleaved 2 x N arrays) -------------------------

def slp_real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly):
    psrc, ptar, f = _c(psrc), _c(ptar), _c(f)
    out = np.zeros((ptar.shape[0], 2))
    rc = lib().or_slp_real(_p(psrc), C.c_int(psrc.shape[0]), _p(ptar), C.c_int(ptar.shape[0]), _p(f),
                           C.c_double(xi), C.c_int(nside_x), C.c_int(nside_y), C.c_double(Lx), C.c_double(Ly),
                           _p(out))
    assert rc == 0
    return out


def dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly):
    psrc, ptar, f, n = _c(psrc), _c(ptar), _c(f), _c(n)
    out = np.zeros((ptar.shape[0], 2))
    rc = lib().or_dlp_real(_p(psrc), C.c_int(psrc.shape[0]), _p(ptar), C.c_int(ptar.shape[0]), _p(f), _p(n),
                           C.c_double(xi), C.c_int(nside_x), C.c_int(nside_y), C.c_double(Lx), C.c_double(Ly),
                           _p(out))
    assert rc == 0
    return out


def slp_kspace(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P):
    psrc, ptar, f = _c(psrc), _c(ptar), _c(f)
    out = np.zeros((ptar.shape[0], 2))
    rc = lib().or_slp_kspace(_p(psrc), C.c_int(psrc.shape[0]), _p(ptar), C.c_int(ptar.shape[0]), C.c_double(xi),
                             C.c_double(eta), _p(f), C.c_int(Mx), C.c_int(My), C.c_double(Lx), C.c_double(Ly),
                             C.c_double(w), C.c_int(P), _p(out))
    assert rc == 0
    return out


def dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P):
    psrc, ptar, f, n = _c(psrc), _c(ptar), _c(f), _c(n)
    out = np.zeros((ptar.shape[0], 2))
    rc = lib().or_dlp_kspace(_p(psrc), C.c_int(psrc.shape[0]), _p(ptar), C.c_int(ptar.shape[0]), C.c_double(xi),
                             C.c_double(eta), _p(f), _p(n), C.c_int(Mx), C.c_int(My), C.c_double(Lx),
                             C.c_double(Ly), C.c_double(w), C.c_int(P), _p(out))
    assert rc == 0
    return out


def fft2(re, im=None, inverse=False):
    """MATLAB fft2/ifft2 of a (My, Mx)-shaped numpy array indexed [y, x]."""
    re = np.asarray(re, dtype=np.float64)
    My, Mx = re.shape
    r = np.ascontiguousarray(re.T).copy()  # column-major storage = x-major rows
    i = np.zeros_like(r) if im is None else np.ascontiguousarray(np.asarray(im, dtype=np.float64).T).copy()
    rc = lib().or_fft2(C.c_int(My), C.c_int(Mx), _p(r), _p(i), C.c_int(1 if inverse else 0))
    assert rc == 0
    return (r + 1j * i).T


def fft1(x, inverse=False):
    x = np.asarray(x, dtype=np.complex128)
    r = np.ascontiguousarray(x.real).copy()
    i = np.ascontiguousarray(x.imag).copy()
    rc = lib().or_fft1(C.c_int(len(x)), _p(r), _p(i), C.c_int(1 if inverse else 0))
    assert rc == 0
    return r + 1j * i


# ---- MATLAB-driver-shaped entries (separate x/y vectors) -------------------

def stokes_slp_ewald_2p(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, P=24, Nb=0.0, tol=1e-16):
    xsrc, ysrc, xtar, ytar, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, f1, f2))
    Ns, Nt = len(xsrc), len(xtar)
    u1, u2 = np.zeros(Nt), np.zeros(Nt)
    ur, uk = np.zeros((Nt, 2)), np.zeros((Nt, 2))
    prm = Params()
    rc = lib().or_stokes_slp_ewald_2p(_p(xsrc), _p(ysrc), C.c_int(Ns), _p(xtar), _p(ytar), C.c_int(Nt), _p(f1),
                                      _p(f2), C.c_double(Lx), C.c_double(Ly), C.c_int(P), C.c_double(Nb),
                                      C.c_double(tol), _p(u1), _p(u2), _p(ur), _p(uk), C.byref(prm))
    assert rc == 0
    return u1, u2, ur, uk, prm


def stokes_dlp_ewald_2p(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, P=24, Nb=0.0, tol=1e-16):
    xsrc, ysrc, xtar, ytar, n1, n2, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, n1, n2, f1, f2))
    Ns, Nt = len(xsrc), len(xtar)
    u1, u2 = np.zeros(Nt), np.zeros(Nt)
    ur, uk = np.zeros((Nt, 2)), np.zeros((Nt, 2))
    prm = Params()
    rc = lib().or_stokes_dlp_ewald_2p(_p(xsrc), _p(ysrc), C.c_int(Ns), _p(xtar), _p(ytar), C.c_int(Nt), _p(n1),
                                      _p(n2), _p(f1), _p(f2), C.c_double(Lx), C.c_double(Ly), C.c_int(P),
                                      C.c_double(Nb), C.c_double(tol), _p(u1), _p(u2), _p(ur), _p(uk),
                                      C.byref(prm))
    assert rc == 0
    return u1, u2, ur, uk, prm


def slp_real_ds(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, xi):
    xsrc, ysrc, xtar, ytar, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, f1, f2))
    u = np.zeros((len(xtar), 2))
    lib().or_slp_real_ds(_p(xsrc), _p(ysrc), C.c_int(len(xsrc)), _p(xtar), _p(ytar), C.c_int(len(xtar)), _p(f1),
                         _p(f2), C.c_double(Lx), C.c_double(Ly), C.c_double(xi), _p(u))
    return u


def dlp_real_ds(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, xi):
    xsrc, ysrc, xtar, ytar, n1, n2, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, n1, n2, f1, f2))
    u = np.zeros((len(xtar), 2))
    lib().or_dlp_real_ds(_p(xsrc), _p(ysrc), C.c_int(len(xsrc)), _p(xtar), _p(ytar), C.c_int(len(xtar)), _p(n1),
                         _p(n2), _p(f1), _p(f2), C.c_double(Lx), C.c_double(Ly), C.c_double(xi), _p(u))
    return u


def slp_kspace_ds(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, xi, kinf):
    xsrc, ysrc, xtar, ytar, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, f1, f2))
    u = np.zeros((len(xtar), 2))
    lib().or_slp_kspace_ds(_p(xsrc), _p(ysrc), C.c_int(len(xsrc)), _p(xtar), _p(ytar), C.c_int(len(xtar)),
                           _p(f1), _p(f2), C.c_double(Lx), C.c_double(Ly), C.c_double(xi), C.c_int(kinf), _p(u))
    return u


def dlp_kspace_ds(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, xi, kinf):
    xsrc, ysrc, xtar, ytar, n1, n2, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, n1, n2, f1, f2))
    u = np.zeros((len(xtar), 2))
    lib().or_dlp_kspace_ds(_p(xsrc), _p(ysrc), C.c_int(len(xsrc)), _p(xtar), _p(ytar), C.c_int(len(xtar)),
                           _p(n1), _p(n2), _p(f1), _p(f2), C.c_double(Lx), C.c_double(Ly), C.c_double(xi),
                           C.c_int(kinf), _p(u))
    return u


def truth_params(Lx, Ly, eps_exp=40.0, xi=None, rcut_cells=None):
    """xi_o, rcut, kinf for the converged truth sum: exp(-xi^2 rcut^2) and
    exp(-k^2/(4 xi^2)) at the truncation both below exp(-eps_exp)."""
    L = min(Lx, Ly)
    if xi is None:
        xi = 7.0 / L
    rcut = np.sqrt(eps_exp) / xi
    kmax = 2.0 * xi * np.sqrt(eps_exp)
    kinf = int(np.ceil(kmax * max(Lx, Ly) / (2 * np.pi))) + 1
    return float(xi), float(rcut), kinf


def ewald_truth(kind, xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, n1=None, n2=None, xi=None, rcut=None, kinf=None):
    """Converged direct Ewald sum (own xi); points must be wrapped into [-L/2, L/2)."""
    xo, ro, ko = truth_params(Lx, Ly, xi=xi)
    xi = xo if xi is None else xi
    rcut = ro if rcut is None else rcut
    kinf = ko if kinf is None else kinf
    if n1 is None:
        n1 = np.zeros_like(np.asarray(f1, dtype=np.float64))
        n2 = n1
    xsrc, ysrc, xtar, ytar, n1, n2, f1, f2 = map(_c, (xsrc, ysrc, xtar, ytar, n1, n2, f1, f2))
    u = np.zeros((len(xtar), 2))
    lib().or_ewald_truth(C.c_int(kind), _p(xsrc), _p(ysrc), C.c_int(len(xsrc)), _p(xtar), _p(ytar),
                         C.c_int(len(xtar)), _p(n1), _p(n2), _p(f1), _p(f2), C.c_double(Lx), C.c_double(Ly),
                         C.c_double(xi), C.c_double(rcut), C.c_int(kinf), _p(u))
    return u


def matlab_wrap(x, L):
    """MATLAB mod(x + L/2, L) - L/2 as the drivers apply it (with mod's
    round-off compensation)."""
    x = np.asarray(x, dtype=np.float64)
    a = x + L / 2
    q = a / L
    r = a - np.floor(q) * L
    r = np.where(np.abs(q - np.round(q)) <= np.finfo(float).eps * np.abs(q), 0.0, r)
    return r - L / 2


# ---- the reference's own gateways ------------------------------------------

def ref_available(flavour: str = "O3") -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, flavour, f"libref_{g}.so"))
               for g in ("slp_real", "slp_kspace", "dlp_real", "dlp_kspace"))


def _ref_lib(gateway: str, flavour: str):
    key = (gateway, flavour)
    with _lock:
        if key not in _ref:
            path = os.path.join(REF_DIR, flavour, f"libref_{gateway}.so")
            L = C.CDLL(path, mode=C.RTLD_LOCAL)
            L.ref_call.restype = C.c_int
            L.ref_call.argtypes = [C.c_int, C.POINTER(_dp), C.POINTER(C.c_long), C.POINTER(C.c_long), _dp,
                                   C.c_long, C.c_char_p, C.c_int]
            _ref[key] = L
    return _ref[key]


def ref_call(gateway: str, args, n_out: int, flavour: str = "O3", ncomp: int = 2):
    """Call a reference gateway.  Matrix args are (N, 2) arrays (passed as
    2 x N); scalars are passed as 1 x 1.  Returns the (n_out, ncomp) output."""
    L = _ref_lib(gateway, flavour)
    mats = []
    ms, ns = [], []
    for a in args:
        if np.isscalar(a):
            arr = np.array([float(a)])
            ms.append(1)
            ns.append(1)
        else:
            arr = _c(a)
            ms.append(2)
            ns.append(arr.shape[0])
        mats.append(arr)
    ptrs = (_dp * len(mats))(*[_p(m) for m in mats])
    out = np.zeros((n_out, ncomp))
    err = C.create_string_buffer(512)
    rc = L.ref_call(len(mats), ptrs, (C.c_long * len(ms))(*ms), (C.c_long * len(ns))(*ns), _p(out),
                    C.c_long(ncomp * n_out), err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return out


def ref_stokes_slp_ewald_2p(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, P=24, Nb=0.0, tol=1e-16, flavour="O3"):
    """The MATLAB driver StokesSLP_ewald_2p restated around the reference gateways."""
    prm = choose_params(KIND_SLP, f1, f2, len(xsrc), len(xtar), Lx, Ly, P, Nb, tol)
    ps = np.stack([matlab_wrap(xsrc, Lx), matlab_wrap(ysrc, Ly)], axis=1)
    pt = np.stack([matlab_wrap(xtar, Lx), matlab_wrap(ytar, Ly)], axis=1)
    f = np.stack([f1, f2], axis=1)
    ur = ref_call("slp_real", [ps, pt, f, prm.xi, prm.nside_x, prm.nside_y, Lx, Ly], len(xtar), flavour)
    uk = ref_call("slp_kspace", [ps, pt, prm.xi, prm.eta, f, prm.Mx, prm.My, Lx, Ly, prm.w, prm.P], len(xtar),
                  flavour)
    u = ur + uk
    return u[:, 0], u[:, 1], ur, uk, prm


def ref_stokes_dlp_ewald_2p(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, P=24, Nb=0.0, tol=1e-16,
                            flavour="O3"):
    """The MATLAB driver StokesDLP_ewald_2p restated around the reference gateways."""
    prm = choose_params(KIND_DLP, f1, f2, len(xsrc), len(xtar), Lx, Ly, P, Nb, tol)
    xs, ys = matlab_wrap(xsrc, Lx), matlab_wrap(ysrc, Ly)
    ps = np.stack([xs, ys], axis=1)
    pt = np.stack([matlab_wrap(xtar, Lx), matlab_wrap(ytar, Ly)], axis=1)
    f = np.stack([f1, f2], axis=1)
    n = np.stack([n1, n2], axis=1)
    ur = ref_call("dlp_real", [ps, pt, f, n, prm.xi, prm.nside_x, prm.nside_y, Lx, Ly], len(xtar), flavour)
    uk = ref_call("dlp_kspace", [ps, pt, prm.xi, prm.eta, f, n, prm.Mx, prm.My, Lx, Ly, prm.w, prm.P],
                  len(xtar), flavour)
    fn = np.asarray(f1) * np.asarray(n1) + np.asarray(f2) * np.asarray(n2)
    uk[:, 0] += np.sum(fn * xs) / (Lx * Ly)
    uk[:, 1] += np.sum(fn * ys) / (Lx * Ly)
    u = ur + uk
    return u[:, 0], u[:, 1], ur, uk, prm


# ---- other SE quantities (or_quant.c) ------------------------------------------
Q_PRESSURE, Q_PRESSURE_GRAD, Q_GRADIENT, Q_STRESS, Q_VORTICITY = 1, 2, 3, 4, 5
Q_NAMES = {Q_PRESSURE: "pressure", Q_PRESSURE_GRAD: "pressure_grad", Q_GRADIENT: "gradient", Q_STRESS: "stress",
           Q_VORTICITY: "vorticity"}
Q_NCOMP = {Q_PRESSURE: 1, Q_PRESSURE_GRAD: 2, Q_GRADIENT: 4, Q_STRESS: 4, Q_VORTICITY: 1}


def q_real(kind, q, psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly):
    """Real-space sum of quantity q: (Ntar, ncomp)."""
    psrc, ptar, f = _c(psrc), _c(ptar), _c(f)
    nn = _c(n) if n is not None else None
    out = np.zeros((ptar.shape[0], Q_NCOMP[q]))
    L = lib()
    L.or_q_real.restype = C.c_int
    rc = L.or_q_real(C.c_int(kind), C.c_int(q), _p(psrc), C.c_int(psrc.shape[0]), _p(ptar), C.c_int(ptar.shape[0]),
                     _p(f), _p(nn) if nn is not None else None, C.c_double(xi), C.c_int(nside_x), C.c_int(nside_y),
                     C.c_double(Lx), C.c_double(Ly), _p(out))
    assert rc == 0
    return out


def q_kspace(kind, q, psrc, ptar, f, n, xi, eta, Mx, My, Lx, Ly, w, P):
    """k-space sum of quantity q: (Ntar, ncomp)."""
    psrc, ptar, f = _c(psrc), _c(ptar), _c(f)
    nn = _c(n) if n is not None else None
    out = np.zeros((ptar.shape[0], Q_NCOMP[q]))
    L = lib()
    L.or_q_kspace.restype = C.c_int
    rc = L.or_q_kspace(C.c_int(kind), C.c_int(q), _p(psrc), C.c_int(psrc.shape[0]), _p(ptar), C.c_int(ptar.shape[0]),
                       _p(f), _p(nn) if nn is not None else None, C.c_double(xi), C.c_double(eta), C.c_int(Mx),
                       C.c_int(My), C.c_double(Lx), C.c_double(Ly), C.c_double(w), C.c_int(P), _p(out))
    assert rc == 0
    return out


# argument order of each reference quantity gateway (PeriodicEwald/src/mex/Stokes*/mex_stokes_*_{real,kspace}.cpp)
_KSPACE_F_FIRST = {("slp", Q_PRESSURE), ("slp", Q_PRESSURE_GRAD), ("dlp", Q_PRESSURE), ("dlp", Q_PRESSURE_GRAD),
                   ("dlp", Q_VORTICITY)}


def ref_q_real(kind, q, psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly, flavour="O3"):
    k = "slp" if kind == KIND_SLP else "dlp"
    args = [psrc, ptar, f] + ([n] if kind == KIND_DLP else []) + [xi, nside_x, nside_y, Lx, Ly]
    return ref_call(f"{k}_{Q_NAMES[q]}_real", args, len(ptar), flavour, Q_NCOMP[q])


def ref_q_kspace(kind, q, psrc, ptar, f, n, xi, eta, Mx, My, Lx, Ly, w, P, flavour="O3"):
    k = "slp" if kind == KIND_SLP else "dlp"
    dens = [f] + ([n] if kind == KIND_DLP else [])
    if (k, q) in _KSPACE_F_FIRST:
        args = [psrc, ptar] + dens + [xi, eta, Mx, My, Lx, Ly, w, P]
    else:
        args = [psrc, ptar, xi, eta] + dens + [Mx, My, Lx, Ly, w, P]
    return ref_call(f"{k}_{Q_NAMES[q]}_kspace", args, len(ptar), flavour, Q_NCOMP[q])


def ref_q_ewald_2p(kind, q, xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, n1=None, n2=None, b1=None, b2=None, P=24, Nb=0.0,
                   tol=1e-16, gateways="ref", flavour="O3"):
    """The MATLAB drivers StokesSLP_<q>_ewald_2p / StokesDLP_<q>_ewald_2p
    (PeriodicEwald/src/matlab/) restated around the gateways: the reference's
    own compiled gateways (gateways="ref") or the oracle's (gateways="oracle").
    Returns (out, out_real, out_k, params) with out of shape (Ntar,) for the
    pressure and the vorticity and (Ntar, 2) otherwise."""
    xsrc, ysrc, xtar, ytar = (np.asarray(a, dtype=np.float64) for a in (xsrc, ysrc, xtar, ytar))
    f1, f2 = np.asarray(f1, dtype=np.float64), np.asarray(f2, dtype=np.float64)
    nt = len(xtar)
    # sources that coincide with a target, before wrapping (ismember(zsrc, ztar))
    equal = np.nonzero(np.isin(xsrc + 1j * ysrc, xtar + 1j * ytar))[0]
    est_kind = KIND_SLP if (kind == KIND_DLP and q == Q_VORTICITY) else kind
    prm = choose_params(est_kind, f1, f2, len(xsrc), nt, Lx, Ly, P, Nb, tol)
    xs, ys = matlab_wrap(xsrc, Lx), matlab_wrap(ysrc, Ly)
    ps = np.stack([xs, ys], 1)
    pt = np.stack([matlab_wrap(xtar, Lx), matlab_wrap(ytar, Ly)], 1)
    f = np.stack([f1, f2], 1)
    n = np.stack([np.asarray(n1, dtype=np.float64), np.asarray(n2, dtype=np.float64)], 1) if kind == KIND_DLP else None
    if gateways == "ref":
        R = ref_q_real(kind, q, ps, pt, f, n, prm.xi, prm.nside_x, prm.nside_y, Lx, Ly, flavour)
        K = ref_q_kspace(kind, q, ps, pt, f, n, prm.xi, prm.eta, prm.Mx, prm.My, Lx, Ly, prm.w, prm.P, flavour)
    else:
        R = q_real(kind, q, ps, pt, f, n, prm.xi, prm.nside_x, prm.nside_y, Lx, Ly)
        K = q_kspace(kind, q, ps, pt, f, n, prm.xi, prm.eta, prm.Mx, prm.My, Lx, Ly, prm.w, prm.P)
    xi = prm.xi
    area2 = 2 * Lx * Ly

    def per_target(v):
        """the drivers' elementwise (or scalar-broadcast) addition of self terms"""
        if len(equal) == nt or len(equal) == 1:
            return v if len(equal) == nt else np.broadcast_to(v, (nt,) + np.shape(v)[1:])
        raise ValueError("self terms need one coincident source per target")

    has_eq = len(equal) > 0
    if q == Q_PRESSURE:
        r, k = R[:, 0], K[:, 0]
        if kind == KIND_SLP:
            k = k + -np.sum(f1 * xs + f2 * ys) / area2
            return r + k, r, k, prm
        k = k + -(np.sum(n[:, 0] * f1 + n[:, 1] * f2) / area2)
        pself = 0.0
        if has_eq:
            q_ = f1[equal] + 1j * f2[equal]
            m_ = n[equal, 0] + 1j * n[equal, 1]
            pself = per_target(xi ** 2 * np.real(q_ * np.conj(m_)) / (2 * np.pi))
        return r + k + pself, r, k, prm
    if q == Q_PRESSURE_GRAD:
        if kind == KIND_SLP:
            pself = 0.0
            if has_eq:
                pself = per_target(xi ** 2 * f[equal] / (2 * np.pi))
            return -(R + K + pself), R, K, prm
        return -2 * (R + K), R, K, prm
    if q in (Q_GRADIENT, Q_STRESS):
        b1, b2 = np.asarray(b1, dtype=np.float64), np.asarray(b2, dtype=np.float64)
        if kind == KIND_DLP and q == Q_STRESS:
            rr = np.stack([R[:, 0] * b1 + R[:, 1] * b2, R[:, 2] * b1 + R[:, 3] * b2], 1)
        else:
            rr = np.stack([R[:, 0] * b1 + R[:, 2] * b2, R[:, 1] * b1 + R[:, 3] * b2], 1)
        kk = np.stack([K[:, 0] * b1 + K[:, 2] * b2, K[:, 1] * b1 + K[:, 3] * b2], 1)
        if q == Q_STRESS and kind == KIND_SLP:
            u = rr + kk + np.sum(f1 * xs + f2 * ys) / area2
            return u, rr, kk, prm
        if q == Q_STRESS:
            kk = kk + np.sum(n[:, 0] * f1 + n[:, 1] * f2) / area2
        u = rr + kk
        if kind == KIND_DLP and has_eq:
            q_ = f1[equal] + 1j * f2[equal]
            m_ = n[equal, 0] + 1j * n[equal, 1]
            b_ = b1 + 1j * b2
            us = xi ** 2 * (q_ * np.real(b_ * np.conj(m_)) + m_ * np.real(q_ * np.conj(b_)) +
                            b_ * np.real(q_ * np.conj(m_))) / (2 * np.pi)
            us = per_target(us)
            if q == Q_GRADIENT:
                u = u + np.stack([np.real(us), np.imag(us)], 1)
            else:
                pself = xi ** 2 * b_ * np.real(q_ * np.conj(m_)) / (2 * np.pi)
                pself = per_target(pself)
                # the driver's first component is complex there; its real part
                u = u + np.stack([-np.real(pself) + 2 * np.real(us), 2 * np.imag(us)], 1)
        return u, rr, kk, prm
    r, k = R[:, 0], K[:, 0]
    v = r + k
    if kind == KIND_SLP:
        v = v - np.sum(f1 * ys - f2 * xs) / area2
    return v, r, k, prm
