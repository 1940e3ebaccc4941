"""Catalog work-lists across GPUs: one process per GPU, no data-path collective.

Catalogs (mocks, lines of sight, folds) are independent, so N GPUs split the
list and each runs its share through ``Grid.power_batch_f32``; the only
exchange is the gather of the per-catalog bin tables (a few KB each) at rank 0
over ``torch.distributed`` (NCCL between GPUs, gloo on CPU).  A single catalog
is never split across GPUs: the largest grid (Ng = 2048, two 34 GB FP32 grids)
fits one GB300.
"""
from __future__ import annotations


def shard(n: int, rank: int, world: int) -> list[int]:
    """Catalog indices of ``rank``: round robin, so uneven catalog sizes spread."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    return list(range(rank, n, world))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(x: float) -> float:
    """The largest ``x`` over all ranks (the whole job's time); ``x`` alone
    without an initialised process group."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(x)
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_tables(local: dict, n: int):
    """Merge {catalog index: result} of every rank into a list of n results on
    rank 0 (None on the other ranks).  Every index must come from one rank."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        parts = [local]
        rank = 0
    else:
        rank = dist.get_rank()
        parts = [None] * dist.get_world_size() if rank == 0 else None
        dist.gather_object(local, parts, dst=0)
    if rank != 0:
        return None
    out = [None] * n
    for part in parts:
        for i, res in part.items():
            if out[i] is not None:
                raise RuntimeError(f"catalog {i} measured twice")
            out[i] = res
    missing = [i for i, r in enumerate(out) if r is None]
    if missing:
        raise RuntimeError(f"catalogs {missing[:8]} were not measured")
    return out


def power_worklist(grid, catalogs, V, los, dK: float, Nmu: int = 3, rank: int = 0, world: int = 1):
    """P_l and wedges of every (x, y, z) host catalog of the list, this rank's
    share computed with fftgal_power_batch_f32 (uploads overlapped), the bin
    tables gathered on rank 0 (returned there in catalog order; None elsewhere).
    V: one volume for all catalogs or one per catalog."""
    n = len(catalogs)
    mine = shard(n, rank, world)
    Vs = [V] * n if not hasattr(V, "__len__") else list(V)
    local = {}
    if mine:
        res = grid.power_batch_f32([catalogs[i] for i in mine], [Vs[i] for i in mine], los, dK, Nmu=Nmu)
        local = dict(zip(mine, res))
    return gather_tables(local, n)
