"""Process-group plumbing for multi-GPU runs of the hot path.

The force hot path has no exchange step: independent simulations (replicas of
one workload, or the instances of an ensemble) are the units, each rank owns a
disjoint share of them, and ranks only meet at the timing barrier and the
max-over-ranks reduction of elapsed time.  One process per GPU; rendezvous from
the torchrun environment (RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR/PORT).
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Dist:
    rank: int = 0
    world: int = 1
    local_rank: int = 0
    backend: str = ""

    @property
    def active(self) -> bool:
        return self.world > 1


def init(backend: str | None = None) -> Dist:
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return Dist(rank=0, world=1, local_rank=0, backend="")
    import torch
    import torch.distributed as td

    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if not td.is_initialized():
        td.init_process_group(backend=backend, rank=rank, world_size=world)
    if backend == "nccl":
        torch.cuda.set_device(local)
    return Dist(rank=rank, world=world, local_rank=local, backend=backend)


def shard(n_units: int, d: Dist) -> range:
    """Contiguous share of n_units for this rank (sizes differ by at most one)."""
    lo = n_units * d.rank // d.world
    hi = n_units * (d.rank + 1) // d.world
    return range(lo, hi)


def _reduce(x: float, d: Dist, op: str) -> float:
    if not d.active:
        return float(x)
    import torch
    import torch.distributed as td

    dev = torch.device("cuda", d.local_rank) if d.backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.MAX if op == "max" else td.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(x: float, d: Dist) -> float:
    return _reduce(x, d, "max")


def sum_over_ranks(x: float, d: Dist) -> float:
    return _reduce(x, d, "sum")


def barrier(d: Dist) -> None:
    if d.active:
        import torch.distributed as td

        if d.backend == "nccl":
            import torch

            td.barrier(device_ids=[d.local_rank])
            torch.cuda.synchronize()
        else:
            td.barrier()


def finalize(d: Dist) -> None:
    if d.active:
        import torch.distributed as td

        if td.is_initialized():
            td.destroy_process_group()
