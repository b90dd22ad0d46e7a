"""The quantity oracle (oracle/or_quant.c) against the reference's own
gateways: golden vectors produced by the compiled, unmodified
mex_stokes_{slp,dlp}_<quantity>_{real,kspace}.cpp (tests/golden/gen_golden_quant.py)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_max
from oracle import pyoracle as po

NAMES = golden_names("quant_")


@pytest.fixture(scope="module", autouse=True)
def _built():
    po.build()


def test_all_quantity_fixtures_present():
    assert len(NAMES) == 10


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_gateways(name):
    g = load_golden(name)
    kind, q = int(g["kind"]), int(g["quantity"])
    n = g["n"] if kind == po.KIND_DLP else None
    ur = po.q_real(kind, q, g["psrc"], g["ptar"], g["f"], n, float(g["xi"]), int(g["nside_x"]), int(g["nside_y"]),
                   float(g["Lx"]), float(g["Ly"]))
    uk = po.q_kspace(kind, q, g["psrc"], g["ptar"], g["f"], n, float(g["xi"]), float(g["eta"]), int(g["Mx"]),
                     int(g["My"]), float(g["Lx"]), float(g["Ly"]), float(g["w"]), int(g["P"]))
    assert ur.shape == g["real"].shape and uk.shape == g["kspace"].shape
    assert rel_max(ur, g["real"]) <= 1e-13, name
    assert rel_max(uk, g["kspace"]) <= 1e-13, name
