"""FP64 k-space sums on grids whose lines do not fit one block's shared memory.

The drivers' analytic grid is (A M, B M) with M up to 10000 and A/B = rat(Lx/Ly),
so lines longer than a block transform (about 7000 FP64 values) occur for
elongated boxes.  Those lines run through the long transform (four-step, or
Bluestein in global memory over a factorable length); the MEX-shaped k-space
entries must still match the oracle to 1e-12 relative:

  * x lines of 8000 = 2^6 5^3         four-step 100 x 80
  * x lines of 11490 = 2 3 5 383      four-step 383 x 30 (in-block Bluestein for 383)
  * x lines of 7666 = 2 3833          Bluestein over 15360 = 128 x 120
  * y lines of 8000                   staged rows, four-step
"""
import numpy as np
import pytest

from conftest import rel_max
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _ft():
    import fasttools2d_gb300 as ft

    return ft


CASES = [  # (Mx, My, Lx, Ly)
    (8000, 32, 250.0, 1.0),
    (11490, 30, 383.0, 1.0),
    (7666, 32, 7666 / 32, 1.0),
    (32, 8000, 1.0, 250.0),
]


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}x{c[1]}" for c in CASES])
def test_long_lines_match_oracle(gpu_ctx, kind, case):
    ft = _ft()
    Mx, My, Lx, Ly = case
    assert abs(Lx / Mx - Ly / My) < 1e-12 * Lx / Mx
    rng = np.random.default_rng(Mx + My)
    ns, nt = 300, 200
    ps = np.stack([(rng.random(ns) - 0.5) * Lx, (rng.random(ns) - 0.5) * Ly], 1)
    pt = np.stack([(rng.random(nt) - 0.5) * Lx, (rng.random(nt) - 0.5) * Ly], 1)
    f = rng.standard_normal((ns, 2))
    P = 16
    h = Lx / Mx
    xi = 10.0
    w = P * h / 2
    m = 0.95 * np.sqrt(np.pi * P)
    eta = (2 * xi * w / m) ** 2
    if kind == "slp":
        ref = po.slp_kspace(ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P)
        out = ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P, ctx=gpu_ctx)
    else:
        th = rng.random(ns) * 2 * np.pi
        n = np.stack([np.cos(th), np.sin(th)], 1)
        ref = po.dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, Lx, Ly, w, P)
        out = ft.mex_stokes_dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, Lx, Ly, w, P, ctx=gpu_ctx)
    assert np.max(np.abs(ref)) > 0
    assert rel_max(out, ref) <= 1e-12, (kind, case)
