"""Replica jobs on several GPUs of one node (the multi-GPU mode of the evaluation path).

Every (theta, window) rollout is independent and an identification job has no exchange
with another, so N GPUs run N independent jobs -- one process per GPU, launched by torchrun
-- and nothing crosses GPUs on the data path. The only collectives are host bookkeeping: a
barrier around the timed region and the maximum of the ranks' times, from which the
whole-job rate is the units all ranks processed divided by the slowest rank's time.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Ranks:
    dist: object          # torch.distributed, or None for a single process
    rank: int
    world: int
    local: int

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max_over_ranks(self, x: float, device=None) -> float:
        """The largest x over all ranks (every rank gets it)."""
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def whole_job_rate(self, units_per_rank: float, local_ms: float, device=None) -> tuple[float, float]:
        """(units of all ranks per second over the slowest rank's time, that time in ms)."""
        ms = self.max_over_ranks(local_ms, device)
        return self.world * units_per_rank / (ms * 1e-3), ms

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()


def init(backend: str | None = None) -> Ranks:
    """Join the process group torchrun describes (WORLD_SIZE, RANK, LOCAL_RANK, MASTER_*).

    backend: "nccl" on GPUs (the default when CUDA is available), "gloo" for CPU tests. With
    WORLD_SIZE unset or 1 nothing is initialised."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return Ranks(None, 0, 1, 0)
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return Ranks(dist, dist.get_rank(), world, local)
