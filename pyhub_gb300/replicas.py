"""Replicas across GPUs: one process per GPU, no collective on the data path.

A single Hubbard or Heisenberg sector does not shard without an all-to-all
transpose of the vector per H*v (the down hops mix rows, the up hops mix
columns), so single-sector workloads run as independent replicas.  Batched
Green's-function sweeps shard by cluster: clusters are independent, each
rank sweeps its own share.  The collectives are host bookkeeping -- barriers
around a timed region, the maximum time over ranks, the sum of the units
processed -- and, after a sweep, one gather of every rank's results to rank
0, outside the data path.

The launch follows torchrun's environment (WORLD_SIZE, RANK, LOCAL_RANK,
MASTER_ADDR, MASTER_PORT); the rendezvous address defaults to 127.0.0.1.
"""
from __future__ import annotations

import os


def world():
    """(world_size, rank, local_rank) from the launcher's environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return ws, rank, local


def init(backend: str = "nccl"):
    """Join the process group when there is more than one rank ("nccl" for
    GPU ranks, "gloo" for host-only ranks).  Returns world()."""
    ws, rank, local = world()
    if ws > 1:
        import torch.distributed as D
        if not D.is_initialized():
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            D.init_process_group(backend, rank=rank, world_size=ws)
    return ws, rank, local


def finish():
    import torch.distributed as D
    if D.is_available() and D.is_initialized():
        D.destroy_process_group()


def shard(items, rank: int, ws: int):
    """The rank's share of independent work items: every ws-th item from its
    rank (disjoint across ranks, together exactly the item list)."""
    return list(items)[rank::ws]


def _device():
    import torch
    import torch.distributed as D
    if D.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier(sync_cuda: bool = True):
    """Barrier over ranks (if any) and a device synchronize."""
    import torch
    import torch.distributed as D
    if D.is_available() and D.is_initialized():
        D.barrier()
    if sync_cuda and torch.cuda.is_available():
        torch.cuda.synchronize()


def _reduce(value: float, op: str) -> float:
    import torch
    import torch.distributed as D
    if not (D.is_available() and D.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device())
    D.all_reduce(t, op=D.ReduceOp.MAX if op == "max" else D.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(value: float) -> float:
    return _reduce(value, "max")


def sum_over_ranks(value: float) -> float:
    return _reduce(value, "sum")


def aggregate_rate(units: float, seconds: float) -> tuple[float, float, float]:
    """Whole-job rate: the units all ranks processed over the slowest rank's
    time.  Returns (rate, total units, max seconds)."""
    total = sum_over_ranks(units)
    tmax = max_over_ranks(seconds)
    return (total / tmax if tmax > 0 else float("inf")), total, tmax


def gather_to_root(obj):
    """Every rank's obj, in rank order, as a list on rank 0 (None on the other
    ranks); [obj] without a process group."""
    import torch.distributed as D
    if not (D.is_available() and D.is_initialized()) or D.get_world_size() == 1:
        return [obj]
    rank = D.get_rank()
    out = [None] * D.get_world_size() if rank == 0 else None
    D.gather_object(obj, out, dst=0)
    return out
