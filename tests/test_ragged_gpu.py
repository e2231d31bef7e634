"""Ragged batches (instances with different qubit counts in one persistent launch) against
the oracle, with tile-width overrides, CUDA-graph replay and the autotuner."""
import importlib

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def mods():
    rg = importlib.import_module("sequential-quantum-gate-decomposer_gb300.ragged")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    return rg, wl


def make_instances(wl, rng, ns):
    circs, targets = [], []
    for n in ns:
        c = wl.random_gate_circuit(n, 12 + 4 * n, rng) if n > 1 else wl.cnot_u3_ansatz(1, 0)
        N = 1 << n
        cols = int(rng.integers(1, N + 1)) if n % 2 else N
        U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
        circs.append(c)
        targets.append(np.ascontiguousarray(U[:cols, :].conj().T))
    return circs, targets


@pytest.mark.parametrize("variant", [0, 3, 9])
def test_ragged_matches_oracle(mods, variant):
    rg, wl = mods
    rng = np.random.default_rng(90 + variant)
    circs, targets = make_instances(wl, rng, [3, 2, 5, 4, 6, 3, 7, 2])
    rb = rg.RaggedBatch(circs, targets)
    thetas = [rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()) for c in circs]
    cost, grad = rb.cost_grad(rb.pack(thetas), variant=variant)
    torch.cuda.synchronize()
    cost = cost.cpu().numpy()
    grads = [g.cpu().numpy() for g in rb.split(grad)]
    for i, c in enumerate(circs):
        rc, rgd = O.cost_grad(c.qbit_num, c.gate_records(), thetas[i], targets[i], variant=variant)
        assert abs(cost[i] - rc) <= 1e-12 * max(1.0, abs(rc))
        assert np.max(np.abs(grads[i] - rgd)) <= 1e-12 * max(1.0, np.max(np.abs(rgd)))
    cost_only, none = rb.cost_grad(rb.pack(thetas), variant=variant, with_grad=False)
    assert none is None
    torch.cuda.synchronize()
    assert np.allclose(cost_only.cpu().numpy(), cost, atol=1e-13)


def test_ragged_large_instances_match_oracle(mods):
    """Instances of 8, 9 and 10 qubits beside small ones in one launch (the uneven batches span
    3 to 10 qubits): cost and gradient against the oracle at 1e-12."""
    rg, wl = mods
    rng = np.random.default_rng(97)
    circs, targets = make_instances(wl, rng, [8, 3, 10, 9])
    rb = rg.RaggedBatch(circs, targets)
    thetas = [rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()) for c in circs]
    cost, grad = rb.cost_grad(rb.pack(thetas))
    torch.cuda.synchronize()
    cost = cost.cpu().numpy()
    grads = [g.cpu().numpy() for g in rb.split(grad)]
    for i, c in enumerate(circs):
        rc, rgd = O.cost_grad(c.qbit_num, c.gate_records(), thetas[i], targets[i])
        assert abs(cost[i] - rc) <= 1e-12 * max(1.0, abs(rc))
        assert np.max(np.abs(grads[i] - rgd)) <= 1e-12 * max(1.0, np.max(np.abs(rgd)))


def test_tile_override_and_graph_replay(mods):
    rg, wl = mods
    rng = np.random.default_rng(95)
    circs, targets = make_instances(wl, rng, [4, 6, 5, 3])
    thetas = [rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()) for c in circs]
    base = rg.RaggedBatch(circs, targets)
    c0, g0 = base.cost_grad(base.pack(thetas))
    c0, g0 = c0.clone(), g0.clone()
    alt = rg.RaggedBatch(circs, targets, tile_cols=[1, 2, 4, 1])
    c1, g1 = alt.cost_grad(alt.pack(thetas))
    torch.cuda.synchronize()
    assert torch.allclose(c1, c0, atol=1e-13, rtol=0) and torch.allclose(g1, g0, atol=1e-13, rtol=0)
    alt.capture()
    thetas2 = [rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()) for c in circs]
    alt.theta_static.copy_(alt.pack(thetas2))
    cg, gg = alt.replay()
    torch.cuda.synchronize()
    cg, gg = cg.clone(), gg.clone()
    c2, g2 = base.cost_grad(base.pack(thetas2))
    torch.cuda.synchronize()
    assert torch.allclose(cg, c2, atol=1e-13, rtol=0) and torch.allclose(gg, g2, atol=1e-13, rtol=0)


def test_autotuner_returns_valid_tiles(mods):
    rg, wl = mods
    rng = np.random.default_rng(96)
    circs, targets = make_instances(wl, rng, [3, 3, 5, 5])
    choice, report = rg.autotune_tile_cols(circs, targets, candidates=(1, 2, 4, 8), reps=1)
    assert set(report) == {3, 5}
    assert all(c in (1, 2, 4, 8) for c in choice)
