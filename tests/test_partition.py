"""Kahn partitioner and FLOP model (partitioning.py) against the reference's own partitioner
(fixture made by tests/golden/make_partition_golden.py from squander/partitioning/kahn.py and
tools.py) and against the reference's partitioning tests (tests/partitioning/test_partition.py:
empty circuit, single gate, gate count, qubit limit, whole-register partition, and the
partitioned circuit computing the same operator)."""
import importlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def part():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.partitioning")


def _build(sqg, n, gates):
    c = sqg.Circuit(n)
    for kind, t, ctl in gates:
        if ctl >= 0:
            getattr(c, "add_" + kind)(t, ctl)
        else:
            getattr(c, "add_" + kind)(t)
    return c


def test_kahn_matches_reference_partitioner(sqg, part):
    with open(os.path.join(HERE, "golden", "partition_kahn.json")) as f:
        cases = json.load(f)["cases"]
    assert len(cases) == 32
    for case in cases:
        c = _build(sqg, case["qbit_num"], case["gates"])
        top, order, parts = part.kahn_partition(c, case["max_qubit"])
        assert [list(p) for p in parts] == case["parts"]
        assert [list(t) for t in order] == case["param_order"]
        assert [len(b._gates) for b in top.get_Gates()] == case["block_sizes"]
        gates = c.get_Gates()
        g2q = {i: set(g.get_Involved_Qbits()) for i, g in enumerate(gates)}
        g2t = {i: g.get_Target_Qbit() for i, g in enumerate(gates)}
        assert part.total_float_ops(case["qbit_num"], case["max_qubit"], g2q, None, parts) == case["float_ops"]
        assert part.total_float_ops(case["qbit_num"], case["max_qubit"], g2q, g2t, parts) == case["float_ops_ctrl"]


@pytest.mark.parametrize("max_qubits", [3, 4, 5])
def test_reference_partition_cases(sqg, part, max_qubits):
    empty = sqg.Circuit(5)
    top, order, _ = part.kahn_partition(empty, max_qubits)
    assert len(top.get_Gates()) == 1 and len(order) == 0  # one (empty) partition, as the reference
    single = sqg.Circuit(5)
    single.add_CNOT(0, 1)
    top, order, _ = part.kahn_partition(single, max_qubits)
    assert len(top.get_Gates()) == 1 and len(order) == 1
    chain = sqg.Circuit(5)
    chain.add_CNOT(0, 1)
    chain.add_CNOT(1, 2)
    chain.add_CNOT(2, 3)
    top, _, _ = part.kahn_partition(chain, max_qubits)
    assert sum(len(p.get_Gates()) for p in top.get_Gates()) == 3
    for p in top.get_Gates():
        assert len(set.union(*(part.get_qubits(g) for g in p.get_Gates()))) <= max_qubits
    whole = sqg.Circuit(max_qubits)
    whole.add_CNOT(0, 1)
    whole.add_CNOT(1, 2)
    whole.add_CRY(1, 2)
    whole.add_U3(0)
    whole.add_CZ(2, 0)
    top, _, _ = part.kahn_partition(whole, max_qubits)
    assert len(top.get_Gates()) == 1


@pytest.mark.parametrize("n,count,mq", [(6, 60, 3), (7, 80, 4), (5, 40, 2)])
def test_partitioned_circuit_computes_the_same_operator(sqg, part, n, count, mq):
    rng = np.random.default_rng(n * 100 + count)
    c = sqg.Circuit(n)
    for _ in range(count):
        k = rng.integers(7)
        t = int(rng.integers(n))
        ctl = int((t + 1 + rng.integers(n - 1)) % n)
        [lambda: c.add_U3(t), lambda: c.add_RX(t), lambda: c.add_RY(t), lambda: c.add_RZ(t),
         lambda: c.add_CNOT(t, ctl), lambda: c.add_CZ(t, ctl), lambda: c.add_CRY(t, ctl)][k]()
    theta = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    pc, ptheta, parts = part.PartitionCircuit(c, theta, mq)
    assert pc.get_Parameter_Num() == c.get_Parameter_Num()
    assert len(pc.get_Gates()) == len(parts)
    assert pc.block_ends()[-1] == c.get_Gate_Num()
    U = O.get_matrix(n, c.gate_records(), theta)
    Up = O.get_matrix(n, pc.gate_records(), ptheta)
    assert np.allclose(U, Up, atol=1e-12)


def test_partition_strategies_and_flop_model(sqg, part):
    c = sqg.Circuit(3)
    c.add_CNOT(0, 1)
    for strategy in ("ilp", "ilp-fusion", "ilp-fusion-ca"):
        pc, _, parts = part.PartitionCircuit(c, np.zeros(0), 2, strategy=strategy)
        assert parts == [[0]]
    with pytest.raises(NotImplementedError, match="Qiskit"):
        part.PartitionCircuit(c, np.zeros(0), 2, strategy="qiskit")
    # unknown names fall back to kahn, as in the reference
    pc, _, parts = part.PartitionCircuit(c, np.zeros(0), 2, strategy="no-such-strategy")
    assert parts == [[0]]
    # 2^n amplitudes x (6 g + 2 (g - 1) + 48) with g = 2^(gate qubits - controls)
    assert part.get_float_ops(3, 1, 0) == 8 * (12 + 2 + 48)
    assert part.get_float_ops(4, 2, 1, is_pure=True) == 8 * (12 + 2 + 48)
    assert part.get_float_ops(2, 2, 0) == 4 * (24 + 6 + 48)
