"""The quantity oracle (oracle/or_quant.c) against the reference's own
gateways: golden vectors produced by the compiled, unmodified
mex_stokes_{slp,dlp}_<quantity>_{real,kspace}.cpp (tests/golden/gen_golden_quant.py)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_max
from oracle import pyoracle as po

NAMES = [n for n in golden_names("quant_") if not n.startswith("quant_drv_")]


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


DRV = golden_names("quant_drv_")


@pytest.mark.parametrize("name", DRV)
def test_driver_restatement_on_oracle_gateways(name):
    """The drivers' glue around the oracle's gateways reproduces the golden
    drivers built around the reference's own gateways."""
    g = load_golden(name)
    kind, q = int(g["kind"]), int(g["quantity"])
    for i in (0, 1):
        d = {k[3:]: g[k] for k in g if k.startswith(f"c{i}_")}
        o, r, k, prm = po.ref_q_ewald_2p(kind, q, d["xsrc"], d["ysrc"], d["xtar"], d["ytar"], d["f1"], d["f2"],
                                         float(d["Lx"]), float(d["Ly"]), d["n1"], d["n2"], d["b1"], d["b2"],
                                         tol=float(d["tol"]), gateways="oracle")
        assert prm.xi == pytest.approx(float(d["xi"])) and prm.Mx == int(d["Mx"])
        assert rel_max(o, d["out"]) <= 1e-13, (name, i)
        assert rel_max(r, d["out_real"]) <= 1e-13 and rel_max(k, d["out_k"]) <= 1e-13, (name, i)
