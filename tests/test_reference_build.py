"""The reference's own gateways as built here: sources byte-for-byte the
reference's, and the portable SSE header (oracle/mexshim/portable/pmmintrin.h,
used on the aarch64 GPU hosts) changing no result.

The reference's real-space gateways include <pmmintrin.h>
(PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:4,
PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:4).  On x86-64 the
oracle's Makefile also builds a flavour P3 on the portable header; its
outputs must equal, bit for bit, those of the O3 flavour built on the
compiler's header, on every gateway fixture.  CPU only.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_max
from oracle import pyoracle as po

MANIFEST = os.path.join(os.path.dirname(po.HERE), "oracle", "ref_sources.sha256")
MEX_CASES = golden_names("mex_")


def _fixture_args(g):
    args = [g[f"arg{i}"] for i in range(int(g["nargs"]))]
    return [float(a) if a.ndim == 0 else a for a in args], str(g["gateway"])


def test_manifest_lists_the_velocity_path_sources():
    names = sorted(line.split()[1] for line in open(MANIFEST) if line.strip())
    assert names == sorted([
        "StokesSLP/mex_stokes_slp_real.cpp", "StokesSLP/mex_stokes_slp_kspace.cpp",
        "StokesDLP/mex_stokes_dlp_real.cpp", "StokesDLP/mex_stokes_dlp_kspace.cpp",
        "common/ewald_tools.cpp", "common/ewald_tools.h", "common/mm_mxmalloc.h"])


def test_staged_sources_are_unmodified():
    if not po.staged_reference():
        pytest.skip("no staged reference sources on this host")
    src = os.path.join(po.REF_DIR, "src")
    for line in open(MANIFEST):
        digest, name = line.split()
        with open(os.path.join(src, name), "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == digest, name


@pytest.mark.parametrize("name", MEX_CASES)
def test_reference_gateways_reproduce_fixture(name):
    """The gateways built on this host give the committed fixture outputs
    (made by the same sources) to rounding, in both flavours."""
    if not po.ref_available("O3"):
        pytest.skip("reference gateways not built on this host")
    g = load_golden(name)
    args, gw = _fixture_args(g)
    for flavour in ("O3", "O0"):
        if not po.ref_available(flavour):
            continue
        out = po.ref_call(gw, args, g["out"].shape[0], flavour)
        assert rel_max(out, g["out"]) <= 1e-13, flavour


_BITWISE = r"""
import json, sys
sys.path[:0] = [ROOT, ROOT + "/tests"]
import numpy as np
from conftest import golden_names, load_golden
from oracle import pyoracle as po
res = {}
for name in golden_names("mex_"):
    g = load_golden(name)
    args = [g[f"arg{i}"] for i in range(int(g["nargs"]))]
    args = [float(a) if a.ndim == 0 else a for a in args]
    n = g["out"].shape[0]
    a = po.ref_call(str(g["gateway"]), args, n, "O3")
    b = po.ref_call(str(g["gateway"]), args, n, "P3")
    res[name] = bool(np.array_equal(a, b))
print(json.dumps(res))
"""


def test_portable_sse_header_is_bitwise_neutral():
    """One OpenMP thread (the reference's Spread accumulates grid columns
    under locks in thread order, so with several threads its k-space sums
    differ run to run in the last bits): every gateway fixture gives
    identical bits through the compiler's SSE header and the portable one."""
    if not (po.ref_available("O3") and po.ref_available("P3")):
        pytest.skip("the portable-header flavour is built on x86-64 with the checkout only")
    import json
    import subprocess
    import sys

    root = os.path.dirname(po.HERE)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {root!r}\n" + _BITWISE], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert set(res) == set(MEX_CASES)
    assert all(res.values()), res
