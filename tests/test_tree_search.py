"""Structure search (tree_search.py): candidate enumeration and structure construction of
N_Qubit_Decomposition_Tree_Search (CPU), and on the GPU the many-structure decomposition
(sqg_decompose_structures) against one-structure batches and a search that recovers a known
CNOT structure."""
import importlib
import itertools

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def ts():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.tree_search")


@pytest.mark.parametrize("n,topology", [(3, None), (4, None), (4, [(0, 1), (1, 2), (2, 3)]), (5, [(0, 4), (1, 3)])])
def test_level_codes_equal_the_filtered_enumeration(ts, n, topology):
    """level_codes = every sequence over the allowed pairs that passes is_unique_structure
    (at most three equal CNOTs in a row, canonical order of commuting CNOTs), in order."""
    topo = ts.normalize_topology(topology, n)
    for level in range(5):
        brute = [list(c) for c in itertools.product(range(len(topo)), repeat=level)
                 if ts.is_unique_structure(list(c), topo)]
        assert ts.level_codes(level, topo).tolist() == brute


def test_uniqueness_rules(ts):
    topo = ts.normalize_topology(None, 4)  # (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)
    assert ts.canonical_prefix_ok([0, 5], topo) == -1   # (0,1) then (2,3): canonical
    assert ts.canonical_prefix_ok([5, 0], topo) == 0    # commuting pair out of order
    assert not ts.is_unique_structure([5, 0], topo)
    assert ts.is_unique_structure([1, 1, 1], topo)
    assert not ts.is_unique_structure([1, 1, 1, 1], topo)
    assert ts.normalize_topology([(2, 0)], 3) == [(0, 2)]
    for bad in ([(0, 0)], [(0, 3)], [(0, 1, 2)]):
        with pytest.raises(ValueError):
            ts.normalize_topology(bad, 3)


def test_structure_records_match_the_circuit(ts):
    topo = ts.normalize_topology(None, 4)
    rng = np.random.default_rng(3)
    codes = rng.integers(0, len(topo), (5, 4))
    recs = ts.structure_records(codes, topo, 4)
    for k in range(5):
        c = ts.structure_circuit(codes[k], topo, 4)
        assert np.array_equal(c.gate_records(), recs[k])
        assert c.get_Parameter_Num() == 6 * 4 + 3 * 4
        assert len(c.get_Gates()) == 5  # four two-qubit blocks and the final layer


@pytest.mark.gpu
def test_structures_equal_one_structure_batches(sqg, ts):
    """Instance k of one many-structure launch gives bit for bit what a batch of structure k
    alone gives for the same instance index, start point, target and seed."""
    torch = pytest.importorskip("torch")
    topo = ts.normalize_topology(None, 3)
    codes = ts.level_codes(3, topo)[[0, 4, 9, 13, 20, 26]]
    B = codes.shape[0]
    rng = np.random.default_rng(8)
    U = O.get_matrix(3, ts.structure_circuit(codes[2], topo, 3).gate_records(), rng.uniform(0, 2 * np.pi, 27))
    T = np.ascontiguousarray(U.conj().T)
    x0 = rng.uniform(0, 2 * np.pi, (B, 27))
    lib = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    nc = ts.structure_circuit(codes[0], topo, 3).native()
    recs = np.ascontiguousarray(ts.structure_records(codes, topo, 3))
    t = torch.from_numpy(T).cuda()
    x = torch.from_numpy(x0.copy()).cuda()
    cost = torch.empty(B, dtype=torch.float64, device="cuda")
    calls = torch.empty(B, dtype=torch.int32, device="cuda")
    iters = torch.empty(B, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.lib().sqg_decompose_structures_workspace_bytes(nc.handle, B, 8), dtype=torch.uint8,
                     device="cuda")
    lib.check(lib.lib().sqg_decompose_structures(nc.handle, recs.ctypes.data, t.data_ptr(), 0, 8, B, 0, 0,
                                                 x.data_ptr(), cost.data_ptr(), calls.data_ptr(), iters.data_ptr(),
                                                 1e-8, 10000, 4, 1, 1, 77, ws.data_ptr(), ws.numel(),
                                                 torch.cuda.current_stream().cuda_stream), "structures")
    torch.cuda.synchronize()
    for k in range(B):
        dec = sqg.BatchedDecomposer(ts.structure_circuit(codes[k], topo, 3), tolerance=1e-8, max_calls=10000,
                                    max_outer=4, iteration_loops=1, stop_at_tolerance=True)
        xk, ck, nk = dec.run(np.stack([T] * B), x0, seed=77)
        torch.cuda.synchronize()
        assert float(ck[k]) == float(cost[k]) and int(nk[k]) == int(calls[k])
        assert torch.equal(xk[k], x[k])
    assert float(cost[2]) < 1e-8  # the structure the target was made from
    bad = recs.copy()
    bad[1, 0, 0] = 8  # RY where the circuit has U3
    with pytest.raises(lib.SQGError, match="differs"):
        lib.check(lib.lib().sqg_decompose_structures(nc.handle, bad.ctypes.data, t.data_ptr(), 0, 8, B, 0, 0,
                                                     x.data_ptr(), cost.data_ptr(), calls.data_ptr(), None, 1e-8,
                                                     10, 1, 1, 1, 0, ws.data_ptr(), ws.numel(),
                                                     torch.cuda.current_stream().cuda_stream), "structures")
    bad = recs.copy()
    bad[0, 2, 2] = bad[0, 2, 1]  # CNOT with control == target
    with pytest.raises(lib.SQGError, match="out of range"):
        lib.check(lib.lib().sqg_decompose_structures(nc.handle, bad.ctypes.data, t.data_ptr(), 0, 8, B, 0, 0,
                                                     x.data_ptr(), cost.data_ptr(), calls.data_ptr(), None, 1e-8,
                                                     10, 1, 1, 1, 0, ws.data_ptr(), ws.numel(),
                                                     torch.cuda.current_stream().cuda_stream), "structures")


@pytest.mark.gpu
@pytest.mark.parametrize("n,seq", [(3, [(0, 1), (1, 2)]), (4, [(0, 1), (2, 3), (1, 2)]), (2, [(0, 1)])])
def test_tree_search_recovers_a_known_structure(sqg, ts, n, seq):
    topo = ts.normalize_topology(None, n)
    code = [topo.index(p) for p in seq]
    c = ts.structure_circuit(code, topo, n)
    rng = np.random.default_rng(len(seq) + n)
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    dec = sqg.N_Qubit_Decomposition_Tree_Search(np.ascontiguousarray(U.conj().T),
                                                config={"optimization_tolerance": 1e-8, "random_seed": 1})
    dec.Start_Decomposition()
    assert dec.get_Decomposition_Error() < 1e-8
    assert len(dec.best_cnot_sequence) <= len(seq)
    assert dec.levels_done == len(dec.best_cnot_sequence) + 1
    x = dec.get_Optimized_Parameters()
    assert abs(O.cost(n, dec.get_Circuit().gate_records(), x, dec.get_Unitary())) < 1e-8


def test_tabu_helpers(ts):
    best = []
    ts.insert_into_best_solution(best, (1,), 0.5)
    ts.insert_into_best_solution(best, (2,), 0.2)
    ts.insert_into_best_solution(best, (3,), 0.9)  # larger than every entry: not added
    assert best == [((2,), 0.2), ((1,), 0.5)]
    for k in range(50):
        ts.insert_into_best_solution(best, (k, k), 0.1 - k * 1e-3)
    assert len(best) == 40 and best[0][1] == min(m for _, m in best)
    tested = {(0, 1)}
    mut = ts.determine_mutated_structures((0, 1), 3, 14, tested)
    assert (0, 1) not in mut and (2, 1) in mut and (1,) in mut and (0, 1, 2) in mut
    assert len(mut) == 4 + 2 + 3  # changes, removals, extensions
    assert all(len(c) <= 2 for c in ts.determine_mutated_structures((0, 1), 3, 2, tested))
    rng = np.random.default_rng(0)
    codes = [(0,), (1,), (2,)]  # equal lengths: all weights 0, the first is drawn
    assert ts.draw_gate_structure_from_list(codes, rng) == (0,) and len(codes) == 2
    codes = [(0, 1), (1,), (0, 1, 2)]  # weights 0, 4, -4: r = 0 < 4 picks the removal
    assert ts.draw_gate_structure_from_list(codes, rng) == (1,)
    codes = [(0,), (0, 1), (0, 2)]  # weights 0, -4, -4: negative sum, the first is drawn
    assert ts.draw_gate_structure_from_list(codes, rng) == (0,)
    draws = set()
    for seed in range(20):
        codes = [(0, 1), (1,), (0,), (2, 2)]  # weights 0, 4, 4, 0
        draws.add(ts.draw_gate_structure_from_list(codes, np.random.default_rng(seed)))
    assert draws <= {(1,), (0,), (0, 1)} and (1,) in draws and (0,) in draws


@pytest.mark.gpu
def test_tabu_search_reaches_tolerance(sqg, ts):
    n, seq = 3, [(0, 1), (1, 2)]
    topo = ts.normalize_topology(None, n)
    c = ts.structure_circuit([topo.index(p) for p in seq], topo, n)
    rng = np.random.default_rng(12)
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    dec = sqg.N_Qubit_Decomposition_Tabu_Search(np.ascontiguousarray(U.conj().T),
                                                config={"optimization_tolerance": 1e-8, "random_seed": 4,
                                                        "tree_level_max": 4})
    dec.Start_Decomposition()
    assert dec.get_Decomposition_Error() < 1e-8
    assert dec.structures_tested >= 2
    x = dec.get_Optimized_Parameters()
    assert abs(O.cost(n, dec.get_Circuit().gate_records(), x, dec.get_Unitary())) < 1e-8


@pytest.mark.gpu
def test_structures_with_per_instance_targets(sqg, ts):
    """target_stride > 0: instance k decomposes its own target; equal to a one-structure batch."""
    torch = pytest.importorskip("torch")
    lib = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    topo = ts.normalize_topology(None, 3)
    codes = ts.level_codes(2, topo)[[0, 3, 7]]
    B = codes.shape[0]
    rng = np.random.default_rng(12)
    xs = rng.uniform(0, 2 * np.pi, (B, 21))
    T = np.stack([np.ascontiguousarray(O.get_matrix(3, ts.structure_circuit(codes[k], topo, 3).gate_records(),
                                                     xs[k]).conj().T) for k in range(B)])
    x0 = xs + 0.1 * rng.standard_normal(xs.shape)
    nc = ts.structure_circuit(codes[0], topo, 3).native()
    recs = np.ascontiguousarray(ts.structure_records(codes, topo, 3))
    t = torch.from_numpy(T).cuda()
    x = torch.from_numpy(x0.copy()).cuda()
    cost = torch.empty(B, dtype=torch.float64, device="cuda")
    calls = torch.empty(B, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.lib().sqg_decompose_structures_workspace_bytes(nc.handle, B, 8), dtype=torch.uint8,
                     device="cuda")
    lib.check(lib.lib().sqg_decompose_structures(nc.handle, recs.ctypes.data, t.data_ptr(), 64, 8, B, 0, 0,
                                                 x.data_ptr(), cost.data_ptr(), calls.data_ptr(), None, 1e-8, 1000,
                                                 4, 1, 1, 5, ws.data_ptr(), ws.numel(),
                                                 torch.cuda.current_stream().cuda_stream), "structures")
    torch.cuda.synchronize()
    assert np.all(cost.cpu().numpy() < 1e-8)
    for k in range(B):
        dec = sqg.BatchedDecomposer(ts.structure_circuit(codes[k], topo, 3), tolerance=1e-8, max_calls=1000,
                                    max_outer=4)
        xk, ck, nk = dec.run(T, x0, seed=5)
        torch.cuda.synchronize()
        assert float(ck[k]) == float(cost[k]) and torch.equal(xk[k], x[k])
    with pytest.raises(lib.SQGError, match="target stride"):
        lib.check(lib.lib().sqg_decompose_structures(nc.handle, recs.ctypes.data, t.data_ptr(), 10, 8, B, 0, 0,
                                                     x.data_ptr(), cost.data_ptr(), calls.data_ptr(), None, 1e-8,
                                                     10, 1, 1, 1, 0, ws.data_ptr(), ws.numel(),
                                                     torch.cuda.current_stream().cuda_stream), "structures")


@pytest.mark.gpu
def test_structures_adam_equal_single_structure_runs(sqg, ts):
    """Six-qubit structures with SQUANDER's ADAM engine in one launch (the optimizer the
    structure searches use above five qubits), one CTA per structure: every instance equals,
    bit for bit, a batched ADAM run of its own structure (same CTA index, so the same random
    stream seed + 7919 b)."""
    torch = pytest.importorskip("torch")
    lib = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    n = 6
    topo = ts.normalize_topology(None, n)
    codes = ts.level_codes(1, topo)[:5]
    B = codes.shape[0]
    rng = np.random.default_rng(8)
    circs = [ts.structure_circuit(codes[k], topo, n) for k in range(B)]
    P = circs[0].get_Parameter_Num()
    T = np.stack([np.ascontiguousarray(O.get_matrix(n, circs[k].gate_records(),
                                                    rng.uniform(0, 2 * np.pi, P)).conj().T) for k in range(B)])
    x0 = rng.uniform(0, 2 * np.pi, (B, P))
    nc = circs[0].native()
    recs = np.ascontiguousarray(ts.structure_records(codes, topo, n))
    t = torch.from_numpy(T).cuda()
    x = torch.from_numpy(x0.copy()).cuda()
    cost = torch.empty(B, dtype=torch.float64, device="cuda")
    evals = torch.empty(B, dtype=torch.int32, device="cuda")
    shifts = torch.empty(B, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.lib().sqg_decompose_structures_adam_workspace_bytes(nc.handle, B), dtype=torch.uint8,
                     device="cuda")
    lib.check(lib.lib().sqg_decompose_structures_adam(
        nc.handle, recs.ctypes.data, t.data_ptr(), 64 * 64, 64, B, 0, 0, x.data_ptr(), cost.data_ptr(),
        evals.data_ptr(), shifts.data_ptr(), 1e-8, 40, 1e-3, 1, 5, 2500000, 1, 5, ws.data_ptr(), ws.numel(),
        torch.cuda.current_stream().cuda_stream), "structures_adam")
    torch.cuda.synchronize()
    assert np.all(evals.cpu().numpy() == 40)
    for k in range(B):
        dec = sqg.BatchedDecomposer(circs[k], tolerance=1e-8, max_calls=40, max_outer=1, optimizer="ADAM", eta=1e-3,
                                    random_shift_count_max=5)
        xk, ck, ek = dec.run(T, x0, seed=5)
        torch.cuda.synchronize()
        assert float(ck[k]) == float(cost[k]) and torch.equal(xk[k], x[k]) and int(ek[k]) == int(evals[k])
    bad = recs.copy()
    bad[0, -1, 1] = n
    assert lib.lib().sqg_decompose_structures_adam(
        nc.handle, bad.ctypes.data, t.data_ptr(), 64 * 64, 64, B, 0, 0, x.data_ptr(), cost.data_ptr(),
        evals.data_ptr(), None, 1e-8, 40, 1e-3, 1, 5, 2500000, 1, 5, ws.data_ptr(), ws.numel(),
        torch.cuda.current_stream().cuda_stream) == 1
    assert lib.lib().sqg_decompose_structures_adam(
        nc.handle, recs.ctypes.data, t.data_ptr(), 64 * 64, 64, B, 0, 0, x.data_ptr(), cost.data_ptr(),
        evals.data_ptr(), None, 1e-8, 40, 1e-3, 1, 5, 2500000, 1, 5, ws.data_ptr(), 64,
        torch.cuda.current_stream().cuda_stream) == 3
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_six_qubit_level_runs_as_one_adam_structure_batch(sqg, ts, monkeypatch):
    """A six-qubit level of five candidates goes through one sqg_decompose_structures_adam
    launch (budget shrunk from the reference's P / 852 * 1e7 for the test); a single candidate
    goes through the graph-driven ADAM loop."""
    torch = pytest.importorskip("torch")
    n = 6
    topo = ts.normalize_topology(None, n)
    codes = ts.level_codes(1, topo)[:5]
    rng = np.random.default_rng(9)
    c = ts.structure_circuit(codes[2], topo, n)
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    dec = sqg.N_Qubit_Decomposition_Tree_Search(np.ascontiguousarray(U.conj().T),
                                                config={"optimization_tolerance": 1e-8, "random_seed": 4})
    monkeypatch.setattr(ts.N_Qubit_Decomposition_Tree_Search, "_adam_budget", staticmethod(lambda P: 30))
    target = dec.evaluator().target
    f, k, x, evals = dec._decompose_level_large(codes, 1e-8, target)
    torch.cuda.synchronize()
    assert 0 <= k < 5 and np.isfinite(f) and x.shape == (c.get_Parameter_Num(),)
    assert evals == 5 * 30  # none reaches 1e-8 in 30 ADAM steps: every candidate runs its budget
    assert abs(O.cost(n, ts.structure_circuit(codes[k], topo, n).gate_records(), x,
                      np.ascontiguousarray(U.conj().T)) - f) < 1e-10
    f1, k1, x1, ev1 = dec._decompose_level_large(codes[:1], 1e-8, target)
    assert k1 == 0 and ev1 == 30 and np.isfinite(f1)


@pytest.mark.gpu
def test_tree_search_on_a_linear_topology(sqg, ts):
    """Four qubits on a line (0-1, 1-2, 2-3): commuting CNOTs on disjoint pairs are enumerated
    once; a target from two such CNOTs is found at level 2."""
    topo = ts.normalize_topology([(0, 1), (1, 2), (2, 3)], 4)
    code = [0, 2]  # (0,1) then (2,3): canonical
    c = ts.structure_circuit(code, topo, 4)
    rng = np.random.default_rng(3)
    U = O.get_matrix(4, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    dec = sqg.N_Qubit_Decomposition_Tree_Search(np.ascontiguousarray(U.conj().T), topology=[(0, 1), (1, 2), (2, 3)],
                                                config={"optimization_tolerance": 1e-8, "random_seed": 2})
    dec.Start_Decomposition()
    assert dec.get_Decomposition_Error() < 1e-8
    assert len(dec.best_cnot_sequence) <= 2
    assert all(p in topo for p in dec.best_cnot_sequence)


def test_adam_budget_above_five_qubits_follows_the_reference(ts):
    """The ADAM budget per candidate is SQUANDER's static_cast<int>(P / 852 * 1e7)
    (N_Qubit_Decomposition_Tree_Search.cpp:1487-1495), at least one evaluation."""
    cls = ts.N_Qubit_Decomposition_Tree_Search
    assert cls._adam_budget(852) == 10000000
    assert cls._adam_budget(36) == int(36 / 852 * 10000000.0) == 422535
    assert cls._adam_budget(0) == 1


@pytest.mark.gpu
def test_tree_search_finds_what_the_reference_finds(sqg):
    """Targets made from random 1..4-CNOT structures at 2..4 qubits, and the reference's own
    4-qubit test target data/Umtx.mat: the structure search finds a
    decomposition with as many CNOTs as the reference's own search in its default mode found
    (tests/golden/tree_search_ref.npz, made by running SQUANDER's N_Qubit_Decomposition_Tree_Search
    built from its sources), within the tolerance.  The reference's exhaustive level search, the
    mode this package restates, missed one of those minima (a 4-CNOT target solved with 5: its
    one random start per candidate structure failed at level 4); the counts here may therefore be
    lower than the reference's level-search counts, never higher than its default mode's."""
    import os

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tree_search_ref.npz"))
    found = []
    for idx in range(d["targets"].shape[0]):
        n = int(d["qbit_num"][idx])
        N = 1 << n
        T = np.ascontiguousarray(d["targets"][idx, :N, :N])
        dec = sqg.N_Qubit_Decomposition_Tree_Search(T, config={"optimization_tolerance": 1e-8, "random_seed": 1,
                                                               "tree_level_max": 8})
        dec.Start_Decomposition()
        assert dec.get_Decomposition_Error() < 1e-8
        found.append(len(dec.best_cnot_sequence))
    found = np.array(found)
    assert np.all(found <= d["default_cnots"]), (found, d["default_cnots"])
    assert np.all(found <= d["level_cnots"]), (found, d["level_cnots"])
    assert np.array_equal(found, d["default_cnots"]), (found, d["default_cnots"])
