"""Batch sharding across ranks (one process per GPU) with a host-side gather.

Instances are independent, so several GPUs shard a batch with no collective on the data
path; the only exchange is the gather of the per-instance results, the analogue of the
MPI_Allgather in SQUANDER's optimization_problem_batched
(src-cpp/decomposition/Optimization_Interface.cpp:962-1006).  Unlike the reference, uneven
batches are allowed: rank r takes a contiguous block whose size differs by at most one.
"""
import numpy as np


def shard_range(batch, rank, world):
    """[start, stop) of rank's contiguous share of `batch` instances."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(int(batch), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def sharded_batch(evaluate, params, group=None):
    """Evaluates `params` (B, P) across the ranks of `group` (torch.distributed): each rank
    calls evaluate(local_params) -> (local_costs (b,), local_grads (b, P) or None) on its
    share, then every rank receives the full (costs, grads) in instance order."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    B = params.shape[0]
    a, b = shard_range(B, rank, world)
    costs, grads = evaluate(params[a:b])
    costs = np.asarray(costs, dtype=np.float64).reshape(-1)
    parts = [None] * world
    payload = (a, costs, None if grads is None else np.asarray(grads, dtype=np.float64))
    dist.all_gather_object(parts, payload, group=group)
    out_c = np.empty(B, dtype=np.float64)
    out_g = None if grads is None else np.empty((B, params.shape[1]), dtype=np.float64)
    for start, c, g in parts:
        out_c[start:start + c.size] = c
        if out_g is not None:
            out_g[start:start + c.size] = g
    return out_c, out_g
