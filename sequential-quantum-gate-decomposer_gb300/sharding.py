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


# The decomposition kernel draws restart perturbation i of instance b from the counter
# seed * _MUL + b * _STEP (+ i); the oracle uses the same counters.  _MUL is odd, hence
# invertible modulo 2^64.
_MUL = 0x2545F4914F6CDD1D
_STEP = 0x9E3779B97F4A7C15
_MASK = (1 << 64) - 1


def shard_seed(seed, start):
    """Seed under which a shard starting at global instance `start` draws exactly the restart
    perturbations its instances get in the unsharded batch: s' * _MUL = seed * _MUL + start *
    _STEP (mod 2^64)."""
    return ((int(seed) * _MUL + int(start) * _STEP) * pow(_MUL, -1, 1 << 64)) & _MASK


def distributed(group=None):
    """(rank, world) of torch.distributed when it is initialised with more than one rank,
    else None."""
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover
        return None
    if not (dist.is_available() and dist.is_initialized()):
        return None
    world = dist.get_world_size(group)
    return (dist.get_rank(group), world) if world > 1 else None


def sharded_decompose(run, targets, x0, seed=0, group=None):
    """Batched decompositions sharded across the ranks of `group`: rank r decomposes its
    contiguous share of the instances with run(local_targets, local_x0, local_seed) ->
    (x, cost, calls) (host arrays), seeded so that every instance draws what it would in the
    unsharded batch, and every rank receives the full (x, cost, calls) in instance order."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    B = targets.shape[0]
    a, b = shard_range(B, rank, world)
    x, cost, calls = run(targets[a:b], x0[a:b], shard_seed(seed, a))
    parts = [None] * world
    dist.all_gather_object(parts, (a, np.asarray(x), np.asarray(cost), np.asarray(calls)), group=group)
    out_x = np.empty((B, x0.shape[1]), dtype=np.float64)
    out_c = np.empty(B, dtype=np.float64)
    out_n = np.empty(B, dtype=np.int64)
    for start, xs, cs, ns in parts:
        out_x[start:start + cs.size] = xs
        out_c[start:start + cs.size] = cs
        out_n[start:start + cs.size] = ns
    return out_x, out_c, out_n
