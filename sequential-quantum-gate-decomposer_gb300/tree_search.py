"""Structure search over CNOT placements: the drop-in for SQUANDER's
``N_Qubit_Decomposition_Tree_Search`` (src-cpp/decomposition/N_Qubit_Decomposition_Tree_Search.cpp).

The reference walks levels of increasing CNOT count; a level enumerates every sequence of
`level` CNOTs over the allowed qubit pairs (its N-ary Gray code), drops duplicates
(is_unique_structure: no CNOT repeated more than three times in a row, and only the
canonical order among sequences that differ by commuting CNOTs on disjoint qubits, :96-165),
builds for each sequence the structure [U3(t), U3(c), CNOT(t, c)] per CNOT plus a final U3
layer (:1518-1619) and decomposes it with N_Qubit_Decomposition_custom (:1453-1511, BFGS with 4
outer iterations up to five qubits), stopping at the first level that reaches the tolerance
(:622-776 with use_osr = use_graph_search = 0, tree_search_over_gate_structures :1269-1451).

Here every candidate structure of a level is decomposed on the GPU in one launch
(sqg_decompose_structures: one CTA per structure, each with its own gate list), in chunks;
consecutive small levels (together at most one wave of resident CTAs) run at the same time on
separate streams, and the lowest level that reaches the tolerance still decides.
Among the structures that reach the tolerance the one with the lowest cost is kept.  The
reference's threads instead stop at whichever solution they find first, so ties may resolve
differently.  The reference's default operator-Schmidt-rank bounds and best-first graph search
(use_osr, use_graph_search) are not restated: Start_Decomposition always runs this exhaustive
level search, which is the reference's use_osr = 0, use_graph_search = 0 mode.
"""
import math

import numpy as np

from . import _device as dev
from . import _native
from .batched import adam_decompose_graph
from .circuit import CNOT, U3, Circuit
from .decomposition import N_Qubit_Decomposition_custom


def normalize_topology(topology, qbit_num):
    """Qubit pairs (a < b) the CNOTs may use; all pairs when topology is empty (constructor of
    N_Qubit_Decomposition_Tree_Search, :397-470)."""
    if not topology:
        return [(a, b) for a in range(qbit_num) for b in range(a + 1, qbit_num)]
    out = []
    for e in topology:
        e = tuple(int(v) for v in e)
        if len(e) != 2:
            raise ValueError("invalid topology: each element should be a pair of integers")
        if not (0 <= e[0] < qbit_num and 0 <= e[1] < qbit_num):
            raise ValueError("invalid topology: qubit indices should be between 0 and qbit_num-1")
        if e[0] == e[1]:
            raise ValueError("invalid topology: target and control qubits should be different")
        out.append((min(e), max(e)))
    return out


def canonical_prefix_ok(code, topology):
    """-1 if the CNOT sequence is the canonical (Kahn, smallest pair first, then position)
    order of its commutation class, else the first position where it deviates (:96-155)."""
    import heapq

    m = len(code)
    if m <= 1:
        return -1
    succ = [[] for _ in range(m)]
    indeg = [0] * m
    last_on = {}
    for k in range(m):
        a, b = topology[code[k]]
        for q in (a, b):
            if q in last_on:
                succ[last_on[q]].append(k)
                indeg[k] += 1
            last_on[q] = k
    pq = [(topology[code[k]], k) for k in range(m) if indeg[k] == 0]
    heapq.heapify(pq)
    for pos in range(m):
        if not pq:
            return pos
        _, idx = heapq.heappop(pq)
        if idx != pos:
            return pos
        for v in succ[idx]:
            indeg[v] -= 1
            if indeg[v] == 0:
                heapq.heappush(pq, (topology[code[v]], v))
    return -1


def is_unique_structure(code, topology):
    """is_unique_structure (:157-165): at most three identical consecutive CNOTs, canonical order."""
    for i in range(len(code) - 3):
        if code[i] == code[i + 1] == code[i + 2] == code[i + 3]:
            return False
    return canonical_prefix_ok(code, topology) < 0


def _chain_topology(topology):
    """True when every two allowed pairs share a qubit: no two CNOTs commute, every sequence
    is canonical."""
    return all(set(p) & set(q) for p in topology for q in topology)


def level_codes(level, topology):
    """The unique CNOT sequences of one level (int array, level columns), in lexicographic
    order of the pair indices."""
    T = len(topology)
    if level == 0:
        return np.zeros((1, 0), dtype=np.int64)
    if _chain_topology(topology):
        codes = np.indices((T,) * level).reshape(level, -1).T
        if level >= 4:
            rep = np.zeros(codes.shape[0], dtype=bool)
            for i in range(level - 3):
                rep |= (codes[:, i] == codes[:, i + 1]) & (codes[:, i] == codes[:, i + 2]) & (codes[:, i] == codes[:, i + 3])
            codes = codes[~rep]
        return codes.astype(np.int64)
    out = []

    def grow(prefix):  # both filters are prefix-closed: prune early
        if len(prefix) == level:
            out.append(list(prefix))
            return
        for p in range(T):
            cand = prefix + [p]
            if is_unique_structure(cand, topology):
                grow(cand)

    grow([])
    return np.asarray(out, dtype=np.int64).reshape(-1, level)


def structure_records(codes, topology, qbit_num):
    """Gate records (type, target, control, param_start) of the structures of CNOT sequences
    (B x level array) as a B x L x 4 int32 array: per CNOT U3(target), U3(control),
    CNOT(target, control) (add_two_qubit_block, the pair's lower qubit as target), then U3 on
    every qubit (add_finalyzing_layer); the same records as structure_circuit(...).gate_records()."""
    codes = np.asarray(codes, dtype=np.int64).reshape(len(codes), -1)
    B, level = codes.shape
    topo = np.asarray(topology, dtype=np.int32).reshape(-1, 2)
    rec = np.zeros((B, 3 * level + qbit_num, 4), dtype=np.int32)
    for j in range(level):
        t, c = topo[codes[:, j], 0], topo[codes[:, j], 1]
        rec[:, 3 * j] = np.stack([np.full(B, U3), t, np.full(B, -1), np.full(B, 6 * j)], axis=1)
        rec[:, 3 * j + 1] = np.stack([np.full(B, U3), c, np.full(B, -1), np.full(B, 6 * j + 3)], axis=1)
        rec[:, 3 * j + 2] = np.stack([np.full(B, CNOT), t, c, np.full(B, 6 * j + 6)], axis=1)
    for q in range(qbit_num):
        rec[:, 3 * level + q] = (U3, q, -1, 6 * level + 3 * q)
    return rec


def structure_circuit(code, topology, qbit_num):
    """The structure of a CNOT sequence as a Circuit of blocks (one per CNOT, one final layer)."""
    top = Circuit(qbit_num)
    for d in code:
        t, c = topology[int(d)]
        blk = Circuit(qbit_num)
        blk.add_U3(t)
        blk.add_U3(c)
        blk.add_CNOT(t, c)
        top.add_Circuit(blk)
    fin = Circuit(qbit_num)
    for q in range(qbit_num):
        fin.add_U3(q)
    top.add_Circuit(fin)
    return top


class N_Qubit_Decomposition_Tree_Search(N_Qubit_Decomposition_custom):
    """Drop-in for squander.N_Qubit_Decomposition_Tree_Search(Umtx, qbit_num=-1, topology=None,
    config=None, accelerator_num=0) (qgd_N_Qubit_Decompositions_Wrapper.cpp:396-447)."""

    #: structures decomposed per launch (each holds its BFGS matrix, P^2 doubles, in HBM)
    chunk = 32768

    def __init__(self, Umtx, qbit_num=-1, topology=None, config=None, accelerator_num=0):
        super().__init__(Umtx, qbit_num, None, config, accelerator_num)
        self.topology = normalize_topology(topology, self.qbit_num)
        self.level_limit = min(max(int(self.config.get("tree_level_max", 14)), 0), 14)
        self.levels_done = 0

    def _launch_structures(self, codes, tol, max_inner, max_outer, loops, target, stream=None):
        """One launch of BFGS decompositions of the structures of `codes` (one level, at most
        `chunk` of them) on `stream`.  Returns the device results (x, cost, calls) and the
        buffers that must outlive the launch."""
        n, topo = self.qbit_num, self.topology
        circ = structure_circuit(codes[0], topo, n)
        nc = circ.native()
        P, B = nc.param_num, codes.shape[0]
        lib = _native.lib()
        recs = np.ascontiguousarray(structure_records(codes, topo, n))
        x = dev.to_device_real(self.rng.uniform(0.0, 2 * math.pi, (B, P)))
        cost = dev.torch.empty(B, dtype=dev.torch.float64, device="cuda")
        calls = dev.torch.empty(B, dtype=dev.torch.int32, device="cuda")
        w = dev.Workspace().get(lib.sqg_decompose_structures_workspace_bytes(nc.handle, B, target.shape[1]))
        dev.after_current(stream)  # the start points and the target were copied on the current stream
        _native.check(lib.sqg_decompose_structures(
            nc.handle, recs.ctypes.data, dev.ptr(target), 0, target.shape[1], B, self.trace_offset,
            self.cost_variant, dev.ptr(x), dev.ptr(cost), dev.ptr(calls), None, tol, max_inner, max_outer, loops, 0,
            int(self.rng.integers(1 << 62)), dev.ptr(w), w.numel(), dev.stream_ptr(stream)),
            "sqg_decompose_structures")
        return (x, cost, calls), (circ, w)

    @staticmethod
    def _collect(results, offset=0):
        """(best cost, its index + offset, best point, evaluations) of one launch's results."""
        x, cost, calls = results
        c = cost.cpu().numpy()
        k = int(np.argmin(c))
        return float(c[k]), offset + k, x[k].cpu().numpy(), int(calls.sum().item())

    def _decompose_level_small(self, codes, tol, max_inner, max_outer, loops, target):
        """BFGS decompositions of every structure of `codes` in chunks of one launch each
        (qbit_num <= 5).  Returns (best cost, its code index, best point, evaluations)."""
        best = (math.inf, -1, None)
        evals = 0
        for s in range(0, codes.shape[0], self.chunk):
            res, _keep = self._launch_structures(codes[s:s + self.chunk], tol, max_inner, max_outer, loops, target)
            f, k, x, ev = self._collect(res, s)
            evals += ev
            if f < best[0]:
                best = (f, k, x)
            if best[0] < tol:
                break
        return best[0], best[1], best[2], evals

    def _decompose_levels_concurrently(self, level_list, tol, max_inner, max_outer, loops, target):
        """Small levels (together at most one wave of resident CTAs) launched at once, one stream
        per level: a level's launch lasts as long as its slowest decomposition, so running
        them side by side costs no more than the slowest one.  Returns the per-level
        (best cost, index, best point, evaluations) in level order."""
        streams = [dev.torch.cuda.Stream() for _ in level_list]
        launched = []
        for (lv, codes), st in zip(level_list, streams):
            launched.append(self._launch_structures(codes, tol, max_inner, max_outer, loops, target, stream=st))
        for st in streams:
            st.synchronize()
        return [self._collect(res) for res, _keep in launched]

    # structures per level from which six-qubit ADAM decompositions run one CTA each in a single
    # launch (sqg_decompose_structures_adam) instead of one whole-GPU graph launch per structure
    batch_adam_min = 4

    @staticmethod
    def _adam_budget(P):
        """ADAM evaluations per candidate above five qubits (max_inner_iterations P / 852 * 1e7,
        N_Qubit_Decomposition_Tree_Search.cpp:1487-1495)."""
        return max(1, int(P / 852 * 10000000.0))

    def _launch_structures_adam(self, codes, tol, iters, target):
        """One launch of ADAM decompositions of the structures of `codes` (six qubits at most),
        one CTA each.  Returns (x, cost, evals) on the device and the buffers that must outlive
        the launch."""
        n, topo = self.qbit_num, self.topology
        nc = structure_circuit(codes[0], topo, n).native()
        P, B = nc.param_num, codes.shape[0]
        lib = _native.lib()
        recs = np.ascontiguousarray(structure_records(codes, topo, n))
        x = dev.to_device_real(self.rng.uniform(0.0, 2 * math.pi, (B, P)))
        cost = dev.torch.empty(B, dtype=dev.torch.float64, device="cuda")
        evals = dev.torch.empty(B, dtype=dev.torch.int32, device="cuda")
        w = dev.Workspace().get(lib.sqg_decompose_structures_adam_workspace_bytes(nc.handle, B))
        _native.check(lib.sqg_decompose_structures_adam(
            nc.handle, recs.ctypes.data, dev.ptr(target), 0, target.shape[1], B, self.trace_offset,
            self.cost_variant, dev.ptr(x), dev.ptr(cost), dev.ptr(evals), None, tol, iters, 1e-3, 1, 5, 2500000, 1,
            int(self.rng.integers(1 << 62)), dev.ptr(w), w.numel(), dev.stream_ptr()),
            "sqg_decompose_structures_adam")
        return (x, cost, evals), (nc, w)

    def _decompose_level_large(self, codes, tol, target):
        """ADAM decompositions (the reference's choice above five qubits: max_inner_iterations
        P / 852 * 1e7, random_shift_count_max 5, :1487-1495).  At six qubits a level of at least
        batch_adam_min structures runs in launches of `chunk` structures, one CTA each, stopping
        after the first launch that reaches the tolerance (as the BFGS levels below six qubits);
        otherwise one graph launch per structure, stopping at the first that reaches it."""
        n, topo = self.qbit_num, self.topology
        best = (math.inf, -1, None)
        evals = 0
        if n <= 6 and codes.shape[0] >= self.batch_adam_min:
            iters = self._adam_budget(structure_circuit(codes[0], topo, n).get_Parameter_Num())
            for s in range(0, codes.shape[0], self.chunk):
                res, _keep = self._launch_structures_adam(codes[s:s + self.chunk], tol, iters, target)
                f, k, x, ev = self._collect(res, s)
                evals += ev
                if f < best[0]:
                    best = (f, k, x)
                if best[0] < tol:
                    break
            return best[0], best[1], best[2], evals
        for i, code in enumerate(codes):
            circ = structure_circuit(code, topo, n)
            P = circ.get_Parameter_Num()
            iters = self._adam_budget(P)
            x, cost, ev, _ = adam_decompose_graph(circ, target, self.rng.uniform(0.0, 2 * math.pi, P), tol, iters,
                                                  random_shift_count_max=5, seed=int(self.rng.integers(1 << 62)),
                                                  trace_offset=self.trace_offset, cost_variant=self.cost_variant)
            f = float(cost.item())
            evals += int(ev.item())
            if f < best[0]:
                best = (f, i, x.cpu().numpy())
            if best[0] < tol:
                break
        return best[0], best[1], best[2], evals

    def Start_Decomposition(self):
        """determine_gate_structure (:622-776) with the level search: levels 0..tree_level_max,
        stop at the first level whose best structure reaches the tolerance."""
        tol = float(self.config.get("optimization_tolerance", self.optimization_tolerance))
        target = self.evaluator().target
        max_inner = int(self.config.get("max_inner_iterations_bfgs", self.config.get("max_inner_iterations", 10000)))
        max_outer = int(self.config.get("max_outer_iterations", 4 if self.qbit_num <= 5 else 1))
        loops = int(self.config.get("max_iteration_loops", 3 if self.qbit_num == 2 else 1))
        best_f, best_code, best_x = math.inf, None, None
        props = dev.torch.cuda.get_device_properties(dev.torch.cuda.current_device())
        wave = 8 * props.multi_processor_count  # resident decomposition CTAs (8 per SM)
        level = 0
        while level <= self.level_limit:
            codes = level_codes(level, self.topology)
            if codes.shape[0] == 0:  # e.g. one qubit pair: four equal CNOTs in a row are excluded
                level += 1
                continue
            group = [(level, codes)]
            total = codes.shape[0]
            while self.qbit_num <= 5 and group[-1][0] < self.level_limit:
                nxt = level_codes(group[-1][0] + 1, self.topology)
                if nxt.shape[0] == 0 or total + nxt.shape[0] > wave:
                    break
                group.append((group[-1][0] + 1, nxt))
                total += nxt.shape[0]
            if len(group) > 1:
                results = self._decompose_levels_concurrently(group, tol, max_inner, max_outer, loops, target)
            elif self.qbit_num <= 5:
                results = [self._decompose_level_small(codes, tol, max_inner, max_outer, loops, target)]
            else:
                results = [self._decompose_level_large(codes, tol, target)]
            for (lv, lcodes), (f, k, x, ev) in zip(group, results):
                # levels above the solving one ran ahead on idle SMs: not counted as the search's work
                self.num_iters += ev
                self.levels_done = lv + 1
                if f < best_f:
                    best_f, best_code, best_x = f, lcodes[k], x
                if best_f < tol:
                    break
            if best_f < tol:
                break
            level = group[-1][0] + 1
        self.circuit = structure_circuit(best_code, self.topology, self.qbit_num)
        self._evaluator = None
        self.optimized_parameters = best_x
        self.decomposition_error = self.Optimization_Problem(best_x)
        self.best_cnot_sequence = [self.topology[int(d)] for d in best_code]
        return 0


def insert_into_best_solution(best_solutions, code, minimum):
    """Keeps (code, minimum) pairs sorted by minimum, at most 40
    (N_Qubit_Decomposition_Tabu_Search::insert_into_best_solution): the pair goes before the
    first entry with a larger minimum (into an empty list at the front; after the last entry
    it is not added)."""
    if not best_solutions:
        best_solutions.insert(0, (tuple(code), minimum))
    for i, (_, m) in enumerate(best_solutions):
        if m > minimum:
            best_solutions.insert(i, (tuple(code), minimum))
            break
    if len(best_solutions) > 40:
        best_solutions.pop()


def determine_mutated_structures(code, n_pairs, level_limit, tested):
    """Untested neighbours of a CNOT sequence: every single-position change, every single
    removal and, below the level limit, every one-CNOT extension at the end
    (determine_mutated_structures)."""
    code = tuple(int(v) for v in code)
    out = []
    for i in range(len(code)):
        for e in range(n_pairs):
            m = code[:i] + (e,) + code[i + 1:]
            if m not in tested:
                out.append(m)
    for i in range(len(code)):
        m = code[:i] + code[i + 1:]
        if m not in tested:
            out.append(m)
    if len(code) == level_limit:
        return out
    for e in range(n_pairs):
        m = code + (e,)
        if m not in tested:
            out.append(m)
    return out


def draw_gate_structure_from_list(codes, rng):
    """Removes and returns one sequence, drawn with weight 4 * (len(codes[0]) - len(code))
    (draw_gate_structure_from_list): a uniform integer r in [0, sum of weights] picks the first
    entry whose running weight sum exceeds r, else the first entry (also when the weights sum
    to a negative number, where the reference's unsigned draw exceeds every partial sum)."""
    if not codes:
        raise ValueError("the list of gate structures is empty")
    levels = len(codes[0])
    weights = [4 * levels - 4 * len(c) for c in codes]
    total = sum(weights)
    chosen = 0
    if total >= 0:
        r = int(rng.integers(0, total + 1))
        part = 0
        for i, w in enumerate(weights):
            part += w
            if r < part:
                chosen = i
                break
    return codes.pop(chosen)


class N_Qubit_Decomposition_Tabu_Search(N_Qubit_Decomposition_Tree_Search):
    """Drop-in for squander.N_Qubit_Decomposition_Tabu_Search(Umtx, qbit_num=-1, topology=None,
    config=None, accelerator_num=0): the tabu walk over CNOT structures of
    N_Qubit_Decomposition_Tabu_Search::tabu_search_over_gate_structures
    (src-cpp/decomposition/N_Qubit_Decomposition_Tabu_Search.cpp:160-400, use_osr = 0).  Each step
    decomposes one structure on the device (one k_decompose launch: BFGS up to five qubits,
    the graph-driven ADAM loop above), accepts it when its minimum is lower, or else with
    probability exp(-(f - f_current)), keeps the 40 best structures, and draws the next
    structure among the untested neighbours of the current one.  Random draws come from the
    decomposer's seeded generator instead of the reference's default_random_engine and
    random_device."""

    def Start_Decomposition(self):
        tol = float(self.config.get("optimization_tolerance", self.optimization_tolerance))
        target = self.evaluator().target
        max_inner = int(self.config.get("max_inner_iterations_bfgs", self.config.get("max_inner_iterations", 10000)))
        max_outer = int(self.config.get("max_outer_iterations", 4 if self.qbit_num <= 5 else 1))
        loops = int(self.config.get("max_iteration_loops", 3 if self.qbit_num == 2 else 1))
        T = len(self.topology)
        code = ()
        best_code, best_x = (), None
        current = math.inf
        possible, tested, best_solutions = [], set(), []
        accepted = {}  # parameters of every accepted structure
        self.structures_tested = 0
        while True:
            codes = np.asarray([code], dtype=np.int64).reshape(1, len(code))
            if self.qbit_num <= 5:
                f, _, x, ev = self._decompose_level_small(codes, tol, max_inner, max_outer, loops, target)
            else:
                f, _, x, ev = self._decompose_level_large(codes, tol, target)
            self.num_iters += ev
            self.structures_tested += 1
            tested.add(code)
            if f < current or self.rng.uniform() < math.exp(-1.0 * (f - current)):
                current, best_code, best_x = f, code, x
                accepted[code] = x
                possible = []
                insert_into_best_solution(best_solutions, code, f)
            if current < tol:
                break
            if not possible:
                possible = determine_mutated_structures(best_code, T, self.level_limit, tested)
            if not possible:
                while best_solutions:
                    best_code, current = best_solutions.pop(0)
                    possible = determine_mutated_structures(best_code, T, self.level_limit, tested)
                    if possible or not best_solutions:
                        break
            if not possible:
                break
            code = draw_gate_structure_from_list(possible, self.rng)
        best_x = accepted[best_code]  # the structure may come back from the list of best ones
        self.circuit = structure_circuit(best_code, self.topology, self.qbit_num)
        self._evaluator = None
        self.optimized_parameters = best_x
        self.decomposition_error = self.Optimization_Problem(best_x)
        self.best_cnot_sequence = [self.topology[int(d)] for d in best_code]
        return 0
