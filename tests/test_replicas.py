"""The multi-GPU benchmark path is replicas only: ranks synchronise around the
timed region and reduce their times with a max; no collective touches the
data.  Exercised here with two gloo ranks on the CPU, plus the reference arm's
rule that ranks other than 0 exit without work."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    from fasttools2d_gb300.replicas import Replicas

    r = Replicas(backend="gloo")
    r.barrier()
    seconds = 1.0 + rank  # rank 1 is the slow one
    out[rank] = (r.max(seconds), r.throughput(1000.0, seconds), r.world, r.rank)
    r.barrier()
    r.close()


def test_two_gloo_ranks_reduce_with_max():
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        mx, thr, world, rk = out[rank]
        assert world == 2 and rk == rank
        assert mx == 2.0
        assert thr == pytest.approx(2 * 1000.0 / 2.0)


def test_single_process_without_env():
    sys.path.insert(0, ROOT)
    from fasttools2d_gb300.replicas import Replicas

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        r = Replicas()
        assert r.world == 1 and r.max(3.5) == 3.5 and r.throughput(10.0, 2.0) == 5.0
    finally:
        os.environ.update(env)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], env=env, capture_output=True, text=True, timeout=120)
    assert res.returncode == 0
    assert res.stdout.strip() == ""


def test_reference_arm_prints_one_line():
    """Rank 0 of the reference arm times the CPU path on a bounded sample."""
    env = dict(os.environ, OMP_NUM_THREADS="4")
    env.pop("WORLD_SIZE", None)
    env.pop("RANK", None)
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", "--n", "4000"], env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"]["h2d_bytes_per_step"] == 0
