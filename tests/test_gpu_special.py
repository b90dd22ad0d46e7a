"""Device special functions of the real-space kernels against CUDA's own exp
and division (computed by torch on the same GPU) and against scipy's E1."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _probe(which, x):
    import torch

    import fasttools2d_gb300 as ft

    fn = ft.lib().fte_debug_special
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    out = torch.empty_like(xd)
    assert fn(which, xd.data_ptr(), out.data_ptr(), len(x)) == 0
    return out.cpu().numpy(), xd


def _xs():
    rng = np.random.default_rng(0)
    return np.concatenate([np.logspace(-12, 0, 2000), 1 + rng.random(4000) * 60, rng.random(2000) * 700,
                           np.array([1.0, 2.0, 4.0, 1023.0, 0.5, 1e-15])])


def test_exp_matches_cuda_exp(gpu_ctx):
    import torch

    x = _xs()
    mine, xd = _probe(1, x)
    ref = torch.exp(-xd).cpu().numpy()
    nz = ref > 1e-300
    assert np.max(np.abs(mine[nz] - ref[nz]) / ref[nz]) <= 4e-16


def test_reciprocal_matches_division(gpu_ctx):
    import torch

    x = _xs()
    mine, xd = _probe(3, x)
    ref = (1.0 / xd).cpu().numpy()
    assert np.max(np.abs(mine - ref) / ref) <= 2.3e-16


def test_e1_and_stokeslet_weight_against_scipy(gpu_ctx):
    special = pytest.importorskip("scipy.special")
    x = _xs()
    x = x[x < 690]
    e1, _ = _probe(0, x)
    ref = special.exp1(x)
    assert np.max(np.abs(e1 - ref) / ref) <= 2e-15
    w, _ = _probe(2, x)
    refw = 0.5 * ref - np.exp(-x)
    # absolute accuracy relative to the larger of the two terms
    scale = np.maximum(0.5 * ref, np.exp(-x))
    assert np.max(np.abs(w - refw) / scale) <= 2e-15
