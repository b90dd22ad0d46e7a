"""Replica bookkeeping for multi-GPU benchmark runs.

The spectral Ewald evaluations of the benchmark are independent problems, so
N GPUs run N replicas with no data-path collective: every rank evaluates the
configuration on its own device; the host only synchronises ranks around the
timed region and reduces the per-rank time with a max.  Whole-job throughput
is (units of all ranks) / (slowest rank's time).
"""
from __future__ import annotations

import os


class Replicas:
    """Ranks from the torchrun environment (RANK, WORLD_SIZE, LOCAL_RANK,
    MASTER_ADDR/PORT); a single process when WORLD_SIZE is unset or 1."""

    def __init__(self, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist

            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend)
            self.dist = dist
            if backend == "nccl":
                self.device = "cuda"

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """Maximum of a per-rank float over all ranks."""
        if self.dist is None:
            return float(x)
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds: float) -> float:
        """Whole-job rate: all ranks' units over the slowest rank's time."""
        return self.world * units_per_rank / self.max(seconds)

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
