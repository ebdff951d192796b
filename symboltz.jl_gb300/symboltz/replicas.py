"""Replica runs: one process per GPU, each solving its own modes or cosmologies.

The perturbation path has no exchange step: every k-mode of every cosmology integrates
independently (src/solve.jl:543-568 spawns one independent task per mode),
and the line-of-sight integral and C_l of a cosmology need only that cosmology's sources.  So a
multi-process run splits whole cosmologies (or the modes of one cosmology) over the ranks with no
collective on the data path; the collectives here are only the barrier that opens a timed region,
the max over ranks of its duration, and an optional gather of per-rank results for the caller.

Rank and world size come from the torchrun environment (RANK, WORLD_SIZE, LOCAL_RANK).  The same
functions run over `gloo` on CPU processes and over `nccl` on GPUs.
"""
from __future__ import annotations

import os

import numpy as np


def rank_world():
    """(rank, world_size) from the launcher's environment; (0, 1) for a plain process."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def init(backend=None):
    """Join the process group when launched with more than one rank; returns (rank, world).

    backend defaults to nccl when CUDA is available and gloo otherwise; under nccl the process
    binds LOCAL_RANK's device first."""
    rank, world = rank_world()
    if world <= 1:
        return rank, world
    import torch
    import torch.distributed as dist
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist.get_rank(), dist.get_world_size()


def _active():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1 else None


def finalize():
    dist = _active()
    if dist is not None:
        dist.destroy_process_group()


def shard(n, rank, world):
    """[lo, hi) of this rank in a contiguous split of n items; sizes differ by at most one and
    the ranks' ranges tile [0, n) in rank order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, extra = divmod(int(n), world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_by_cost(costs, rank, world):
    """Indices of this rank when items of the given costs (e.g. k-modes per cosmology) are split
    greedily, largest first, onto the least-loaded rank; every item goes to exactly one rank and
    the split is the same on every rank (ties break by item index, then rank)."""
    costs = np.asarray(costs, dtype=np.float64)
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in np.lexsort((np.arange(len(costs)), -costs)):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return np.flatnonzero(owner == rank)


def barrier():
    dist = _active()
    if dist is not None:
        dist.barrier()


def _device():
    dist = _active()
    if dist is not None and dist.get_backend() == "nccl":
        import torch
        return torch.device("cuda", torch.cuda.current_device())
    return "cpu"


def reduce_over_ranks(values, op="max"):
    """Elementwise max (or sum) of a list of floats over the ranks; the input unchanged for one rank."""
    dist = _active()
    vals = [float(v) for v in values]
    if dist is None:
        return vals
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=_device())
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[op])
    return t.cpu().tolist()


def gather_rows(local, order):
    """Concatenate every rank's rows (a numpy array, first axis = this rank's items) and return them
    in item order: `order` is this rank's item indices (as from shard/shard_by_cost)."""
    dist = _active()
    local = np.asarray(local)
    if dist is None:
        out = np.empty_like(local)
        out[np.asarray(order)] = local
        return out
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, (np.asarray(order, dtype=np.int64), local))
    n = sum(len(o) for o, _ in parts)
    out = np.empty((n,) + local.shape[1:], dtype=local.dtype)
    for o, rows in parts:
        out[o] = rows
    return out


def throughput(units_per_rank, seconds_per_rank):
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    units = reduce_over_ranks([units_per_rank], op="sum")[0]
    t = reduce_over_ranks([seconds_per_rank], op="max")[0]
    return units / t, units, t
