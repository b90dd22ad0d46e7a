"""The C-ABI library: it loads without a GPU, exports every symbol the public
headers declare, and its host-side parameter chooser equals the oracle's."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import pyoracle as po


def _lib():
    import fasttools2d_gb300 as ft

    if not os.path.exists(ft.LIB_PATH):
        ft.build()
    return ft, ft.lib()


def _declared_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(fte_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return syms


def test_library_exports_declared_symbols():
    ft, L = _lib()
    syms = _declared_symbols()
    assert "fte_stokes_slp_ewald_2p" in syms and "fte_dlp_kspace" in syms
    for s in sorted(syms):
        assert hasattr(L, s), s
    assert L.fte_version() >= 100


def test_python_constants_match_header():
    """Every status, flag, form, arithmetic and kind code of the public header
    has the same value in the Python mirror (FTE_FORM_FF -> FORM_FF, ...)."""
    import fasttools2d_gb300 as ft

    text = open(os.path.join(ROOT, "include", "fasttools2d.h")).read()
    defs = dict(re.findall(r"^#define (FTE_[A-Z0-9_]+) (\d+)u?\b", text, flags=re.M))
    checked = 0
    for name, val in defs.items():
        short = name[4:]
        if short.startswith(("OK", "ERR_", "DEVICE_POINTERS", "HOST_ASYNC")):
            assert getattr(ft, name) == int(val), name  # status codes and flags keep the prefix
        elif short.startswith(("FORM_", "KSPACE_", "NEAR_", "KIND_")):
            assert getattr(ft, short) == int(val), name
        else:
            continue
        checked += 1
    assert checked >= 20


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("case", [(1000, 1000, 1.0, 1.0, 1e-10), (20, 20, 1.0, 1.0, 1e-16), (500, 300, 2.0, 1.0, 1e-8),
                                  (2000, 2000, 1.0, 2.0, 1e-12), (10240, 534528, 2.0, 1.0, 1e-10),
                                  (1, 1, 1.0, 1.0, 1e-10)])
def test_chooser_matches_oracle(kind, case):
    ft, L = _lib()
    ns, nt, Lx, Ly, tol = case
    rng = np.random.default_rng(ns + nt)
    f1, f2 = rng.standard_normal(ns), rng.standard_normal(ns)
    a = ft.choose_params(kind, f1, f2, nt, Lx, Ly, P=24, tol=tol)
    b = po.choose_params(kind, f1, f2, ns, nt, Lx, Ly, 24, 0, tol)
    for key in ("nside_x", "nside_y", "Mx", "My", "kinf", "A", "B", "P"):
        assert getattr(a, key) == getattr(b, key), key
    for key in ("xi", "eta", "w", "rc", "Nb"):
        assert abs(getattr(a, key) - getattr(b, key)) <= 1e-12 * abs(getattr(b, key)), key


def test_chooser_rejects_bad_box():
    ft, L = _lib()
    with pytest.raises(ft.FteError) as e:
        ft.choose_params(0, np.ones(3), np.ones(3), 3, -1.0, 1.0)
    assert e.value.code == ft.FTE_ERR_INVALID


def test_no_gpu_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ft, L = _lib()
    with pytest.raises(ft.FteError) as e:
        ft.Context(0)
    assert e.value.code in (ft.FTE_ERR_CUDA, ft.FTE_ERR_INVALID)
