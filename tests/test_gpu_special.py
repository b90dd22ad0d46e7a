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


@pytest.mark.parametrize("which,L", [(4, 1.0), (5, 2.75)])
def test_coordinate_wrap_is_the_drivers_formula_bit_for_bit(gpu_ctx, which, L):
    """The device wrap (with its shortcut for points inside the box) equals
    MATLAB's mod(x + L/2, L) - L/2 with mod's round-off compensation, as the
    oracle restates it, bit for bit: random points in and around the box,
    the box edges and their neighbouring doubles, multiples of L, and points
    whose shifted coordinate lies just below L."""
    from oracle import pyoracle as po

    rng = np.random.default_rng(11)
    edges = np.array([-L / 2, L / 2, 0.0, L, -L, 2.5 * L, -3.5 * L, 1e-300, -1e-300])
    near = np.concatenate([np.nextafter(edges, np.inf), np.nextafter(edges, -np.inf)])
    below = L / 2 - L * np.array([1e-16, 2e-16, 5e-16, 1e-15, 2e-15, 1e-14])
    x = np.concatenate([(rng.random(20000) - 0.5) * L, (rng.random(20000) - 0.5) * 7 * L, edges, near, below,
                        np.nextafter(below, np.inf), np.nextafter(below, -np.inf)])
    mine, _ = _probe(which, x)
    ref = po.matlab_wrap(x, L)
    assert np.array_equal(mine.view(np.int64), ref.view(np.int64))
