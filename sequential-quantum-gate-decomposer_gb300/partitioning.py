"""Circuit partitioning: the step before the fused gate passes (squander/partitioning).

Restates SQUANDER's greedy Kahn partitioner and its FLOP model:
  build_dependency            squander/partitioning/tools.py:135-164
  kahn_partition              squander/partitioning/kahn.py:7-78
  kahn_partition_preparts     squander/partitioning/kahn.py:81-165
  split_partition             squander/partitioning/kahn.py:168-198
  get_float_ops               squander/partitioning/tools.py:26-45
  parts_to_float_ops          squander/partitioning/tools.py:48-81
  total_float_ops             squander/partitioning/tools.py:84-108
  translate_param_order       squander/partitioning/tools.py:111-132
  PartitionCircuit            squander/partitioning/partition.py:50-91

The Kahn partitioner keeps the reference's data structures where they decide the result:
the ready list is a binary heap of (sorted qubit tuple, gate index) that is scanned in its
array order for the first gate that fits, entries are deleted by position and the heap is
pushed to afterwards, and successor sets are iterated as Python sets.  The same input
therefore gives the same partitions and parameter order as the reference.

The ILP strategies ("ilp", "ilp-fusion", "ilp-fusion-ca") need the PuLP modelling package with
the CBC or Gurobi solvers, and the "qiskit*" / "bqskit*" strategies need those frameworks; none
of them is in this image, so PartitionCircuit raises NotImplementedError for them.

A partitioned circuit (a Circuit of sub-circuits) hands its block boundaries to the engine:
the state-vector plan then starts fused passes only at partition boundaries, merging
consecutive partitions while they fit one shared-memory chunk (Circuit.native).
"""
import heapq
from itertools import dropwhile

import numpy as np

from .circuit import Circuit


def get_qubits(gate):
    """Set of qubit indices a gate (or sub-circuit) acts on."""
    return set(gate.get_Involved_Qbits())


def build_dependency(c):
    """(gate dict, successor sets, predecessor sets, qubit sets, start set) of the top-level
    items of circuit c."""
    gate_dict = {i: gate for i, gate in enumerate(c.get_Gates())}
    gate_to_qubit = {i: get_qubits(g) for i, g in gate_dict.items()}
    g, rg = {i: set() for i in gate_dict}, {i: set() for i in gate_dict}
    for gate in gate_dict:
        for child in c.get_Children(gate_dict[gate]):
            g[gate].add(child)
            rg[child].add(gate)
    S = {m for m in rg if len(rg[m]) == 0}
    return gate_dict, g, rg, gate_to_qubit, S


def _kahn_walk(c, max_qubit, preparts, on_gate, on_close):
    """The partitioner's topological walk: takes, from the ready heap in its array order,
    the first gate that fits the open partition (at most max_qubit qubits, or membership in
    the next predefined partition) and closes the partition when none fits.  on_gate(n,
    gate) is called for every gate taken, on_close() when a partition is closed (also for
    the last one).  Returns the list of partitions (lists of gate indices)."""
    gate_dict, g, rg, gate_to_qubit, S = build_dependency(c)
    S = [(tuple(sorted(gate_to_qubit[x])), x) for x in S]
    heapq.heapify(S)
    parts = [[]]
    curr_partition = set()

    if preparts is None:
        def partition_condition(idx):
            return len(gate_to_qubit[S[idx][1]] | curr_partition) > max_qubit
    else:
        def partition_condition(idx):
            return S[idx][1] not in preparts[len(parts) - 1]

    total = 0
    while S:
        idx = next(dropwhile(partition_condition, range(len(S))), None)
        if idx is None:  # the open partition cannot grow
            on_close()
            total += len(parts[-1])
            curr_partition = set()
            parts.append([])
            idx = next(dropwhile(partition_condition, range(len(S))), None)
            if idx is None:
                raise ValueError("a gate acts on more than max_partition_size qubits")
        n = S[idx][1]
        parts[-1].append(n)
        curr_partition |= gate_to_qubit[n]
        on_gate(n, gate_dict[n])
        del S[idx]
        for child in set(g[n]):
            g[n].remove(child)
            rg[child].remove(n)
            if not rg[child]:
                heapq.heappush(S, (tuple(sorted(gate_to_qubit[child])), child))
    on_close()
    total += len(parts[-1])
    if total != len(gate_dict):
        raise RuntimeError("partitioning lost gates")
    return parts


def kahn_partition(c, max_qubit, preparts=None):
    """Greedy Kahn partitioning of circuit c into partitions of at most max_qubit qubits.
    Returns (partitioned circuit, parameter order [(source index, destination index,
    count)], partitions [[gate index]])."""
    parts = _kahn_walk(c, max_qubit, preparts, lambda n, gate: None, lambda: None)
    return kahn_partition_preparts(c, max_qubit, preparts=parts)


def kahn_partition_preparts(c, max_qubit, preparts):
    """The partitioned circuit of c for the predefined partitions preparts (each split into
    its connected components first)."""
    _, g, rg, _, _ = build_dependency(c)
    preparts = split_partition(preparts, g, rg)
    top = Circuit(c.get_Qbit_Num())
    state = {"sub": Circuit(c.get_Qbit_Num()), "idx": 0}
    param_order = []

    def on_gate(n, gate):
        state["sub"].add_Gate(gate)
        param_order.append((gate.get_Parameter_Start_Index(), state["idx"], gate.get_Parameter_Num()))
        state["idx"] += gate.get_Parameter_Num()

    def on_close():
        top.add_Circuit(state["sub"])
        state["sub"] = Circuit(c.get_Qbit_Num())

    parts = _kahn_walk(c, max_qubit, preparts, on_gate, on_close)
    return top, param_order, parts


def split_partition(preparts, g, rg):
    """Splits every partition into its connected components of the dependency graph, each
    kept in the partition's order."""
    L = []
    for part in preparts:
        V = set(part)
        while V:
            S = [next(iter(V))]
            L.append(set())
            while S:
                node = S.pop()
                if node not in V:
                    continue
                V.remove(node)
                L[-1].add(node)
                S.extend(rg[node])
                S.extend(g[node])
    ord_dict = {x: i for i, part in enumerate(preparts) for x in part}
    return [list(sorted(x, key=ord_dict.get)) for x in L]


def translate_param_order(params, param_order):
    """Parameters of the original circuit rearranged for the partitioned circuit."""
    params = np.asarray(params)
    reordered = np.empty_like(params)
    for s_idx, n_idx, n_params in param_order:
        reordered[n_idx:n_idx + n_params] = params[s_idx:s_idx + n_params]
    return reordered


def get_float_ops(num_qubit, gate_qubits, control_qubits, is_pure=False, io_penalty=48):
    """FLOPs of applying a gate on gate_qubits qubits (control_qubits of them controls) to a
    num_qubit state: 2^num_qubit amplitudes (2^(num_qubit - controls) for a pure controlled
    gate), each a complex dot product of the gate's row (6 flops per complex multiply, 2 per
    add) plus an io_penalty per amplitude."""
    g_size = 2 ** (gate_qubits - control_qubits)
    return 2 ** (num_qubit - (control_qubits if is_pure else 0)) * (g_size * (4 + 2) + 2 * (g_size - 1) + io_penalty)


def parts_to_float_ops(num_qubit, gate_to_qubit, gate_to_tqubit, allparts):
    """FLOPs of every partition applied as one fused gate on num_qubit qubits; with
    gate_to_tqubit the non-target qubits count as controls, and a partition whose gates all
    share one control set is a pure controlled gate."""
    weights = []
    for part in allparts:
        qubits = set.union(*(gate_to_qubit[x] for x in part))
        if gate_to_tqubit is not None:
            tqubits = {gate_to_tqubit[x] for x in part}
            is_pure = len({frozenset(gate_to_qubit[x] - {gate_to_tqubit[x]}) for x in part}) == 1
            weights.append(get_float_ops(num_qubit, len(qubits), len(qubits) - len(tqubits), is_pure))
        else:
            weights.append(get_float_ops(num_qubit, len(qubits), 0, False))
    return weights


def total_float_ops(num_qubit, max_qubits_per_partition, gate_to_qubit, gate_to_tqubit, allparts):
    """FLOPs of the whole partitioned circuit: the per-partition figures on
    max_qubits_per_partition qubits scaled by 2^(num_qubit - max_qubits_per_partition)."""
    weights = parts_to_float_ops(max_qubits_per_partition, gate_to_qubit, gate_to_tqubit, allparts)
    return 2 ** (num_qubit - max_qubits_per_partition) * sum(weights)


_UNAVAILABLE = {
    "ilp": "the PuLP modelling package with the CBC or Gurobi MILP solvers",
    "ilp-fusion": "the PuLP modelling package with the CBC or Gurobi MILP solvers",
    "ilp-fusion-ca": "the PuLP modelling package with the CBC or Gurobi MILP solvers",
    "qiskit": "Qiskit", "qiskit-fusion": "Qiskit",
    "bqskit-Quick": "BQSKit", "bqskit-Scan": "BQSKit", "bqskit-Greedy": "BQSKit", "bqskit-Cluster": "BQSKit",
}


def PartitionCircuit(circ, parameters, max_partition_size, strategy="kahn", filename=None):
    """Partitions circ into sub-circuits of at most max_partition_size qubits.  Returns
    (partitioned circuit, its parameters, partitions).  Unknown strategy names use "kahn", as
    in the reference."""
    if strategy in _UNAVAILABLE:
        raise NotImplementedError("partitioning strategy %r needs %s, which this package does not include; use "
                                  "'kahn'" % (strategy, _UNAVAILABLE[strategy]))
    if strategy in ("tdag", "gtqcp"):
        raise NotImplementedError("partitioning strategy %r is not restated; use 'kahn'" % strategy)
    partitioned, param_order, parts = kahn_partition(circ, max_partition_size)
    return partitioned, translate_param_order(parameters, param_order), parts
