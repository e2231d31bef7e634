"""Circuit partitioning: the step before the fused gate passes (squander.partitioning).

Public functions and the reference functions whose results they reproduce:
  kahn_partition              squander/partitioning/kahn.py:7-78
  kahn_partition_preparts     squander/partitioning/kahn.py:81-165
  get_float_ops               squander/partitioning/tools.py:26-45
  parts_to_float_ops          squander/partitioning/tools.py:48-81
  total_float_ops             squander/partitioning/tools.py:84-108
  translate_param_order       squander/partitioning/tools.py:111-132
  PartitionCircuit            squander/partitioning/partition.py:50-91
  (the optimal strategies: partitioning_ilp.max_partitions, squander/partitioning/ilp.py)

How the greedy partitioner decides, stated as the rules this module implements:

1. The circuit's top-level items form a dependency graph (an item's successors are what
   ``Circuit.get_Children`` returns).  Items whose predecessors have all been placed are
   "ready".
2. The ready items live in a binary min-heap (Python's heapq layout) keyed by (sorted tuple
   of the item's qubits, item index).  The heap is not popped at its minimum: the
   partitioner scans the heap's array from the front and takes the first item that the open
   block admits, removing that array slot in place; items that become ready are then pushed
   with heappush.  The heap's array order therefore decides ties, and this module keeps the
   same array operations for that reason.
3. The initial heap is built (heapify) from the sources listed in the iteration order of a
   Python set of their indices; the items that become ready after an item is placed are
   visited in the iteration order of a fresh Python set of its successors.
4. A block admits an item while the union of their qubits has at most ``max_qubit`` qubits.
   When the open block admits no ready item, it is closed and a new one opened.
5. Each block is then split into its connected pieces (items joined by a direct dependency
   inside the block).  Pieces are found in the order given by the first remaining element of
   a Python set of the block's items, elements leaving the set one at a time.
6. A second pass rebuilds the blocks: this time the open block admits exactly the items of
   the next piece.  The second pass's blocks become the sub-circuits, and the parameter order
   records where each item's parameters move.

The result is identical to the reference's on the same circuit; the fixture
tests/golden/partition_kahn.json, produced by running the reference's own modules, checks it.

The optimal strategies ("ilp", "ilp-fusion", "ilp-fusion-ca") are in partitioning_ilp.py and
solve their models with SciPy's HiGHS in place of the reference's PuLP with CBC or Gurobi.  The
"qiskit*" / "bqskit*" strategies need those frameworks, which this package does not include,
so PartitionCircuit raises NotImplementedError for them.

A partitioned circuit (a Circuit of sub-circuits) hands its block boundaries to the engine:
the state-vector plan then starts fused passes only at partition boundaries, merging
consecutive partitions while they fit one shared-memory chunk (Circuit.native).
"""
import heapq

import numpy as np

from .circuit import Circuit


def get_qubits(gate):
    """Set of qubit indices a gate (or sub-circuit) acts on."""
    return set(gate.get_Involved_Qbits())


class _Dag:
    """Dependency graph of a circuit's top-level items."""

    def __init__(self, circuit):
        self.items = list(circuit.get_Gates())
        count = len(self.items)
        self.qubits = [frozenset(item.get_Involved_Qbits()) for item in self.items]
        self.heap_key = [(tuple(sorted(q)), i) for i, q in enumerate(self.qubits)]
        self.succ = [set() for _ in range(count)]
        self.pred = [set() for _ in range(count)]
        for i, item in enumerate(self.items):
            for j in circuit.get_Children(item):
                self.succ[i].add(j)
                self.pred[j].add(i)

    def sources(self):
        """Indices without predecessors, as a set filled in index order (rule 3)."""
        found = set()
        for i, p in enumerate(self.pred):
            if not p:
                found.add(i)
        return found


class _ReadyHeap:
    """The ready items of rule 2: a heapq array scanned front to back."""

    def __init__(self, dag):
        self._key = dag.heap_key
        self._arr = [self._key[i] for i in dag.sources()]
        heapq.heapify(self._arr)

    def __len__(self):
        return len(self._arr)

    def take_first(self, admits):
        for pos in range(len(self._arr)):
            item = self._arr[pos][1]
            if admits(item):
                self._arr.pop(pos)
                return item
        return None

    def push(self, item):
        heapq.heappush(self._arr, self._key[item])


def _greedy_blocks(dag, admits):
    """Rules 2-4 (and 6 with a membership test): the blocks of item indices, in placement
    order.  admits(block_number, block_qubits, item) says whether the open block takes item."""
    ready = _ReadyHeap(dag)
    waiting = [len(p) for p in dag.pred]
    blocks = [[]]
    block_qubits = set()
    while len(ready):
        item = ready.take_first(lambda i: admits(len(blocks) - 1, block_qubits, i))
        if item is None:
            blocks.append([])
            block_qubits = set()
            item = ready.take_first(lambda i: admits(len(blocks) - 1, block_qubits, i))
            if item is None:
                raise ValueError("a gate acts on more than max_partition_size qubits")
        blocks[-1].append(item)
        block_qubits |= dag.qubits[item]
        for child in set(dag.succ[item]):
            waiting[child] -= 1
            if waiting[child] == 0:
                ready.push(child)
    if sum(len(b) for b in blocks) != len(dag.items):
        raise RuntimeError("partitioning lost gates")
    return blocks


def _pieces(dag, blocks):
    """Rule 5: every block split into its connected pieces, pieces in discovery order."""
    out = []
    for block in blocks:
        left = set(block)
        while left:
            first = next(iter(left))
            piece = {first}
            left.remove(first)
            frontier = [first]
            while frontier:
                node = frontier.pop()
                for other in list(dag.pred[node]) + list(dag.succ[node]):
                    if other in left:
                        left.remove(other)
                        piece.add(other)
                        frontier.append(other)
            out.append(piece)
    return out


def _assemble(circuit, dag, blocks):
    """Sub-circuit per block and the parameter moves [(source start, destination start, count)]."""
    n = circuit.get_Qbit_Num()
    top = Circuit(n)
    moves = []
    dest = 0
    for block in blocks:
        sub = Circuit(n)
        for item in block:
            gate = dag.items[item]
            sub.add_Gate(gate)
            count = gate.get_Parameter_Num()
            moves.append((gate.get_Parameter_Start_Index(), dest, count))
            dest += count
        top.add_Circuit(sub)
    return top, moves


def kahn_partition_preparts(c, max_qubit, preparts):
    """Partitioned circuit of c whose blocks follow the given partitions (each split into its
    connected pieces first).  Returns (partitioned circuit, parameter moves, blocks)."""
    dag = _Dag(c)
    pieces = _pieces(dag, preparts)
    blocks = _greedy_blocks(dag, lambda k, _q, item: item in pieces[k])
    top, moves = _assemble(c, dag, blocks)
    return top, moves, blocks


def kahn_partition(c, max_qubit, preparts=None):
    """Greedy partitioning of circuit c into blocks of at most max_qubit qubits.  Returns
    (partitioned circuit, parameter moves [(source start, destination start, count)], blocks
    [[item index]])."""
    if preparts is None:
        dag = _Dag(c)
        preparts = _greedy_blocks(dag, lambda _k, q, item: len(q | dag.qubits[item]) <= max_qubit)
    return kahn_partition_preparts(c, max_qubit, preparts)


def translate_param_order(params, param_order):
    """Parameters of the original circuit rearranged for the partitioned circuit."""
    src = np.asarray(params)
    out = np.empty_like(src)
    for start, dest, count in param_order:
        out[dest:dest + count] = src[start:start + count]
    return out


def get_float_ops(num_qubit, gate_qubits, control_qubits, is_pure=False, io_penalty=48):
    """FLOP model of one gate application to a num_qubit register.  The gate acts as a dense
    2^(gate_qubits - control_qubits) square block: each output amplitude is a row of that
    block times the input, 6 flops per complex product and 2 per complex addition, plus
    io_penalty for moving the amplitude.  A pure controlled gate touches only the
    2^(num_qubit - control_qubits) amplitudes with its controls set; any other gate all
    2^num_qubit."""
    row = 1 << (gate_qubits - control_qubits)
    per_amplitude = 8 * row - 2 + io_penalty
    touched = 1 << (num_qubit - control_qubits) if is_pure else 1 << num_qubit
    return touched * per_amplitude


def parts_to_float_ops(num_qubit, gate_to_qubit, gate_to_tqubit, allparts):
    """FLOP model of each block applied as one fused gate on num_qubit qubits.  With
    gate_to_tqubit (item -> target qubit) the qubits that are no item's target count as
    controls, and a block whose items all carry the same set of non-target qubits is a pure
    controlled gate; without it every block is an uncontrolled dense gate."""
    out = []
    for part in allparts:
        used = set()
        for item in part:
            used |= gate_to_qubit[item]
        if gate_to_tqubit is None:
            out.append(get_float_ops(num_qubit, len(used), 0, False))
            continue
        targets = {gate_to_tqubit[item] for item in part}
        others = {frozenset(gate_to_qubit[item] - {gate_to_tqubit[item]}) for item in part}
        out.append(get_float_ops(num_qubit, len(used), len(used) - len(targets), len(others) == 1))
    return out


def total_float_ops(num_qubit, max_qubits_per_partition, gate_to_qubit, gate_to_tqubit, allparts):
    """FLOP model of the whole partitioned circuit on num_qubit qubits: the blocks' figures on a
    max_qubits_per_partition register, repeated for each of the 2^(num_qubit -
    max_qubits_per_partition) sub-registers (a fraction when the register is smaller than a
    block)."""
    per_block = parts_to_float_ops(max_qubits_per_partition, gate_to_qubit, gate_to_tqubit, allparts)
    spare = num_qubit - max_qubits_per_partition
    return (1 << spare if spare >= 0 else 0.5 ** -spare) * sum(per_block)


_OPTIMAL = {"ilp": (False, False), "ilp-fusion": (True, False), "ilp-fusion-ca": (True, True)}

_UNAVAILABLE = {
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
    if strategy in _OPTIMAL:
        from .partitioning_ilp import max_partitions

        fusion_cost, control_aware = _OPTIMAL[strategy]
        partitioned, param_order, parts = max_partitions(circ, max_partition_size, fusion_cost, control_aware)
    else:
        partitioned, param_order, parts = kahn_partition(circ, max_partition_size)
    return partitioned, translate_param_order(parameters, param_order), parts
