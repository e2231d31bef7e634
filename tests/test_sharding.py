"""Multi-rank batch sharding with gloo on CPU (world size 2 and 3).  The per-rank evaluation
is the oracle here (the GPU evaluator on a GPU machine); the test covers the split, the gather
and the ordering, which are the same either way."""
import importlib
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, REPO)
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sh = importlib.import_module("sequential-quantum-gate-decomposer_gb300.sharding")
    rng = np.random.default_rng(5)
    recs = np.array([[7, 0, -1, 0], [5, 1, 0, 3], [7, 1, -1, 3], [14, 0, 1, 6]], dtype=np.int32)
    P = 7
    target = np.ascontiguousarray(O.get_matrix(2, recs, rng.uniform(0, 2 * np.pi, P)).conj().T)
    params = rng.uniform(0, 2 * np.pi, (11, P))

    def evaluate(local):
        if local.shape[0] == 0:
            return np.zeros(0), np.zeros((0, P))
        return O.batch(2, recs, local, target, with_grad=True, nthreads=1)

    c, g = sh.sharded_batch(evaluate, params)
    rc, rg = O.batch(2, recs, params, target, with_grad=True, nthreads=1)
    ok = np.allclose(c, rc, atol=0, rtol=0) and np.allclose(g, rg, atol=0, rtol=0)
    q.put((rank, ok))
    dist.destroy_process_group()


def test_shard_range_covers_batch():
    sh = importlib.import_module("sequential-quantum-gate-decomposer_gb300.sharding")
    for B in (0, 1, 7, 64, 1000):
        for world in (1, 2, 3, 8):
            spans = [sh.shard_range(B, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == B
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_sharded_batch_matches_single_process(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + world * 7 + os.getpid() % 500
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    assert sorted(results) == [(r, True) for r in range(world)]


def _worker_api(rank, world, port, q):
    """The public APIs that shard: BatchedDecomposer.run_sharded (through
    sharding.sharded_decompose, with the oracle standing in for the device run on CPU) and
    N_Qubit_Decomposition_custom.Optimization_Problem_Batch (its evaluator replaced by the
    oracle)."""
    import sys

    sys.path.insert(0, REPO)
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pkg = importlib.import_module("sequential-quantum-gate-decomposer_gb300")
    sh = importlib.import_module("sequential-quantum-gate-decomposer_gb300.sharding")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    rng = np.random.default_rng(8)
    c = wl.cnot_u3_ansatz(2, 3)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    targets = np.stack([np.ascontiguousarray(O.get_matrix(2, recs, rng.uniform(0, 2 * np.pi, P)).conj().T)
                        for _ in range(7)])
    x0 = rng.uniform(0, 2 * np.pi, (7, P))

    def run(t, x, s):
        if t.shape[0] == 0:
            return np.zeros((0, P)), np.zeros(0), np.zeros(0, dtype=np.int64)
        return O.decompose(2, recs, t, x, max_inner=40, max_outer=3, seed=s, nthreads=1)

    xs, cs, ns = sh.sharded_decompose(run, targets, x0, seed=11)
    xr, cr, nr = O.decompose(2, recs, targets, x0, max_inner=40, max_outer=3, seed=11, nthreads=1)
    ok = np.array_equal(xs, xr) and np.array_equal(cs, cr) and np.array_equal(ns, nr)
    # Optimization_Problem_Batch of the drop-in class gathers across the ranks
    d = pkg.N_Qubit_Decomposition_custom(np.ascontiguousarray(targets[0]))
    d.set_Gate_Structure(c)

    class OracleEvaluator:
        def cost_grad(self, theta, with_grad=True):
            import torch

            th = theta.numpy()
            return torch.from_numpy(O.batch(2, recs, th.reshape(-1, P), targets[0], nthreads=1)), None

    d._evaluator = OracleEvaluator()
    pkg_dev = importlib.import_module("sequential-quantum-gate-decomposer_gb300._device")
    pkg_dev.to_device_real = lambda a, device="cuda": __import__("torch").from_numpy(np.asarray(a, dtype=np.float64))
    params = rng.uniform(0, 2 * np.pi, (5, P))
    got = d.Optimization_Problem_Batch(params)
    ok = ok and got.shape == (5, 1) and np.array_equal(got.reshape(-1), O.batch(2, recs, params, targets[0], nthreads=1))
    q.put((rank, bool(ok)))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_sharded_public_apis_match_single_process(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29900 + world * 7 + os.getpid() % 500
    procs = [ctx.Process(target=_worker_api, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    assert sorted(results) == [(r, True) for r in range(world)]


def test_shard_seed_reproduces_the_unsharded_counters():
    sh = importlib.import_module("sequential-quantum-gate-decomposer_gb300.sharding")
    for seed in (0, 7, 2 ** 40 + 3):
        for start in (0, 1, 1000, 4095):
            s2 = sh.shard_seed(seed, start)
            for b in (0, 3):
                lhs = (s2 * sh._MUL + b * sh._STEP) & sh._MASK
                rhs = (seed * sh._MUL + (start + b) * sh._STEP) & sh._MASK
                assert lhs == rhs
