"""Replicated interpolants across ranks (one process per GPU).

Queries are independent and a field fits one GPU, so the multi-GPU form of
the path is a replica per rank: every rank builds the same interpolant from
the same field, evaluates its own contiguous range of the query rows, and
the ranges are concatenated on the host.  There is no collective on the data
path; `torch.distributed` is used only to agree on timings and, when asked,
to assemble the full result on every rank.  (Fields beyond one GPU's HBM
would need a slab decomposition along the slowest axis with a 3-plane halo;
every box here has one GPU, so that form is not built.)
"""
from __future__ import annotations

import numpy as np
import torch
import torch.distributed as dist


def shard_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous rows [start, stop) of n rows for `rank` of `world`; the
    first n % world ranks take one extra row."""
    if world <= 0 or not 0 <= rank < world or n < 0:
        raise ValueError("need 0 <= rank < world and n >= 0")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, group=None) -> float:
    """Largest `value` over the ranks (the whole-job time of a timed region)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return float(value)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def query_sharded(evaluate, queries, group=None, gather=True):
    """Evaluate this rank's contiguous share of `queries` with
    `evaluate(rows) -> tuple of per-row arrays` (e.g. an interpolant's
    Query); with `gather`, return the outputs for all rows, concatenated in
    rank order on every rank (host arrays), else this rank's share."""
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    start, stop = shard_range(len(queries), world, rank)
    local = evaluate(queries[start:stop])
    local = local if isinstance(local, tuple) else (local,)
    local = tuple(x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x) for x in local)
    if not gather or world == 1:
        return local
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(len(local)))
