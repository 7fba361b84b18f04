"""Bookkeeping of multi-GPU runs as replicas: one process per GPU, each
solving its own copy of the workload, with no collective on the data path
(the stair-step path shards by independent units: right-hand sides, bodies,
frames).  The ranks only meet at barriers around the timed region and in one
max-reduction of the time; the job's throughput is the units of all ranks
over the slowest rank's time."""
from __future__ import annotations

import os


class Replicas:
    """world / rank from the launcher's environment (torchrun sets WORLD_SIZE,
    RANK, LOCAL_RANK, MASTER_ADDR, MASTER_PORT); a gloo group when world > 1."""

    def __init__(self, world: int | None = None, rank: int | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1")) if world is None else world
        self.rank = int(os.environ.get("RANK", "0")) if rank is None else rank
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """The maximum of x over the ranks (x itself on one rank)."""
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds: float) -> tuple[float, float]:
        """(job throughput, job time): world x units over the slowest rank's time."""
        t = self.max(seconds)
        return self.world * units_per_rank / t, t

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
