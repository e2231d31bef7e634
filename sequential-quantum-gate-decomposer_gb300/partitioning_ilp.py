"""Optimal partitioning: the strategies "ilp", "ilp-fusion" and "ilp-fusion-ca" of
PartitionCircuit (squander/partitioning/partition.py:32-44, squander/partitioning/ilp.py:
max_partitions 935-971).  Solved with SciPy's HiGHS MILP solver.

What is optimised, stated as the rules this module implements:

1. Single-qubit chains.  A chain is a maximal run of consecutive single-qubit items on one
   qubit.  Chains are taken out of the dependency graph; the multi-qubit items keep an edge
   u -> w when w follows u on some qubit, directly or through a chain
   (ilp.py:contract_single_qubit_chains 267-306).
2. Candidates.  Every set X of multi-qubit items that is convex (every dependency path between
   two members stays in X), weakly connected through edges inside X, and acts on at most
   max_qubit qubits (ilp.py:get_all_partitions 859-933 enumerates exactly this family).
3. Selection.  Binary x_i per candidate; every multi-qubit item is covered exactly once; the
   chosen parts' dependency graph must be acyclic, enforced by cutting every strongly
   connected group of chosen parts (sum of its x <= size - 1) and solving again
   (ilp.py:ilp_global_optimal 600-857).  Objectives:
     "ilp"          sum x_i                                   (fewest parts)
     "ilp-fusion"   sum (F_i N + 1) x_i, F_i the FLOP model of part i as a dense gate on a
                    max_qubit register, N the number of candidates (least work, then fewest)
     "ilp-fusion-ca"  N * (control-aware FLOP cost) + sum x_i, with chain placement variables;
                    the cost model is rule 5.
4. Chains go back (ilp.py:recombine_single_qubit_chains 309-348): with no placement decided
   ("ilp", "ilp-fusion") a chain joins its predecessor's part, else its successor's, else it
   is a part of its own; with "ilp-fusion-ca" it joins the part the solution placed it in (a
   chain between two items of one part always joins that part).
5. Control-aware cost of a chosen part P (unit(g) = 8 g - 2 flops per amplitude of a dense
   g x g gate, R = 2^max_qubit): the part's full set F adds the chains enclosed between two of
   its items; Q, T are F's qubits and target qubits, C = Q - T its control-only qubits; F is
   "pure" when all its items carry the same set of non-target qubits.  A chain adjacent to P on
   a qubit of C that is placed into P turns that qubit into a target (j such qubits);
   cost = R unit(2^(|Q| - |C| + j)), divided by 2^|C| when F is pure, j = 0 and no adjacent
   chain on a target qubit is placed into P.  For an impure P an adjacent chain on a target
   qubit must be placed into P; a chain after P may instead go to its successor's part, and
   so may a chain before P that is a single gate (the reference's model offers that choice to
   a chain before P only when its last gate is also its first, ilp.py:786-790, and this model
   is the same).  A chain with a predecessor only
   (successor only) costs R unit(2) unless placed into it; a chain between two parts costs
   R unit(2) when placed in neither, and is placed at most once.

Optimal solutions need not be unique: the parts chosen can differ from the reference's run on
the same circuit while the optimum value is the same.  The final order of the parts is a
topological order (ties by the sorted qubits of a part, then its first item); the partitioned
circuit is then assembled by kahn_partition_preparts, as the reference does.
"""
import heapq

import numpy as np

_CHAIN_UNIT = 8 * 2 - 2  # a single-qubit gate: unit(2)


class _Items:
    """The circuit's top-level items with their qubits, target qubits and dependencies."""

    def __init__(self, circuit):
        self.items = list(circuit.get_Gates())
        count = len(self.items)
        self.qubits = [frozenset(it.get_Involved_Qbits()) for it in self.items]
        # a sub-circuit item has no target qubit of its own
        self.target = [it.get_Target_Qbit() if hasattr(it, "get_Target_Qbit") else -1 for it in self.items]
        self.succ = [set() for _ in range(count)]
        self.pred = [set() for _ in range(count)]
        for i, it in enumerate(self.items):
            for j in circuit.get_Children(it):
                self.succ[i].add(j)
                self.pred[j].add(i)
        self.single = [len(q) == 1 for q in self.qubits]

    def only(self, s):
        """The single element of a (one-element or empty) neighbour set, or None."""
        return next(iter(s)) if s else None


class _Contracted:
    """Rule 1: the multi-qubit items, their contracted edges and the chains."""

    def __init__(self, it):
        self.it = it
        self.nodes = [i for i in range(len(it.items)) if not it.single[i]]
        self.local = {v: k for k, v in enumerate(self.nodes)}
        self.chains = []
        self.chain_of = {}
        for i in range(len(it.items)):
            if it.single[i] and not (it.pred[i] and it.single[it.only(it.pred[i])]):
                chain = [i]
                while it.succ[chain[-1]] and it.single[it.only(it.succ[chain[-1]])]:
                    chain.append(it.only(it.succ[chain[-1]]))
                chain = tuple(chain)
                self.chains.append(chain)
                for g in chain:
                    self.chain_of[g] = chain
        m = len(self.nodes)
        self.succ = [set() for _ in range(m)]
        for a, u in enumerate(self.nodes):
            for s in it.succ[u]:
                while s is not None and it.single[s]:
                    s = it.only(it.succ[s])
                if s is not None:
                    self.succ[a].add(self.local[s])
        self.pred = [set() for _ in range(m)]
        for a in range(m):
            for b in self.succ[a]:
                self.pred[b].add(a)
        self.order = self._topological()
        self.desc = [0] * m
        self.anc = [0] * m
        for a in reversed(self.order):
            for b in self.succ[a]:
                self.desc[a] |= self.desc[b] | (1 << b)
        for a in self.order:
            for b in self.pred[a]:
                self.anc[a] |= self.anc[b] | (1 << b)
        self.adj = [0] * m
        for a in range(m):
            for b in self.succ[a] | self.pred[a]:
                self.adj[a] |= 1 << b
        self.qmask = [sum(1 << q for q in it.qubits[u]) for u in self.nodes]

    def _topological(self):
        waiting = [len(p) for p in self.pred]
        ready = [a for a in range(len(waiting)) if waiting[a] == 0]
        heapq.heapify(ready)
        out = []
        while ready:
            a = heapq.heappop(ready)
            out.append(a)
            for b in self.succ[a]:
                waiting[b] -= 1
                if waiting[b] == 0:
                    heapq.heappush(ready, b)
        return out


def _bits(mask):
    while mask:
        low = mask & -mask
        yield low.bit_length() - 1
        mask ^= low


def candidate_parts(cg, max_qubit):
    """Rule 2: the candidate family as bitmasks over the contracted nodes.  Grown from each
    node t over the nodes after t in topological order: a set is extended by one neighbour
    and closed under convexity (the nodes that are both descendants and ancestors of
    members), so every member of the family is reached and each is kept once."""
    pos = {a: k for k, a in enumerate(cg.order)}
    family = []
    for t in cg.order:
        after = 0
        for a in cg.order[pos[t] + 1:]:
            after |= 1 << a
        start = 1 << t
        seen = {start}
        stack = [(start, cg.desc[t], cg.anc[t], cg.adj[t], cg.qmask[t])]
        while stack:
            members, desc, anc, adj, qm = stack.pop()
            family.append(members)
            for v in _bits(adj & after & ~members):
                grown = members | (1 << v)
                d, a = desc | cg.desc[v], anc | cg.anc[v]
                closed = grown | (d & a)
                if closed in seen:
                    continue
                q, nb = qm, adj
                for w in _bits(closed & ~members):
                    q |= cg.qmask[w]
                    nb |= cg.adj[w]
                if bin(q).count("1") > max_qubit:
                    continue
                seen.add(closed)
                stack.append((closed, d, a, nb, q))
    return family


class _Model:
    """A mixed-integer linear model in the form scipy.optimize.milp takes."""

    def __init__(self):
        self.lo, self.hi, self.integer, self.cost = [], [], [], []
        self.rows, self.cols, self.vals, self.rlo, self.rhi = [], [], [], [], []
        self.constant = 0.0

    def var(self, lo=0.0, hi=1.0, integer=True):
        self.lo.append(lo)
        self.hi.append(hi)
        self.integer.append(1 if integer else 0)
        self.cost.append(0.0)
        return len(self.lo) - 1

    def row(self, coefs, lo, hi):
        r = len(self.rlo)
        for j, c in coefs:
            self.rows.append(r)
            self.cols.append(j)
            self.vals.append(float(c))
        self.rlo.append(lo)
        self.rhi.append(hi)

    def both(self, a, b):
        """A binary equal to the product of binaries a and b (b given as (j, negated))."""
        z = self.var()
        j, neg = b
        self.row([(z, 1), (a, -1)], -np.inf, 0)
        if neg:  # b = 1 - y_j
            self.row([(z, 1), (j, 1)], -np.inf, 1)
            self.row([(a, 1), (j, -1), (z, -1)], -np.inf, 0)
        else:
            self.row([(z, 1), (j, -1)], -np.inf, 0)
            self.row([(a, 1), (j, 1), (z, -1)], -np.inf, 1)
        return z

    def solve(self):
        from scipy.optimize import Bounds, LinearConstraint, milp
        from scipy.sparse import coo_matrix

        n = len(self.lo)
        if n == 0:
            return np.zeros(0), self.constant
        cons = []
        if self.rlo:
            A = coo_matrix((self.vals, (self.rows, self.cols)), shape=(len(self.rlo), n)).tocsr()
            cons = [LinearConstraint(A, np.array(self.rlo, dtype=float), np.array(self.rhi, dtype=float))]
        res = milp(np.array(self.cost), integrality=np.array(self.integer), bounds=Bounds(self.lo, self.hi),
                   constraints=cons, options={"mip_rel_gap": 0.0})
        if res.x is None:
            raise ValueError("no partitioning satisfies the qubit limit (%s)" % res.message)
        x = np.where(np.array(self.integer) == 1, np.round(res.x), res.x)
        return x, float(np.dot(self.cost, x)) + self.constant


def _cyclic_groups(cg, parts, chosen):
    """Strongly connected groups (more than one part) of the chosen parts' dependencies."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    owner = {}
    for k, i in enumerate(chosen):
        for a in _bits(parts[i]):
            owner[a] = k
    src, dst = [], []
    for a, k in owner.items():
        for b in cg.succ[a]:
            if owner.get(b, k) != k:
                src.append(k)
                dst.append(owner[b])
    m = len(chosen)
    graph = coo_matrix((np.ones(len(src)), (src, dst)), shape=(m, m))
    count, label = connected_components(graph, directed=True, connection="strong")
    groups = {}
    for k in range(m):
        groups.setdefault(label[k], []).append(chosen[k])
    return [g for g in groups.values() if len(g) > 1]


def _control_aware_terms(model, cg, parts, x, max_qubit):
    """Rule 5 on the model: placement variables of the chains, the cost of every candidate.
    Returns (pre, post) variable maps keyed by chain."""
    it = cg.it
    R = 1 << max_qubit
    chain_cost = R * _CHAIN_UNIT
    has_pred = {ch: bool(it.pred[ch[0]]) for ch in cg.chains}
    has_succ = {ch: bool(it.succ[ch[-1]]) for ch in cg.chains}
    pre = {ch: model.var() for ch in cg.chains if has_pred[ch]}
    post = {ch: model.var() for ch in cg.chains if has_succ[ch]}
    neither = {ch: model.var() for ch in cg.chains if has_pred[ch] and has_succ[ch]}
    enclosing = {ch: [] for ch in neither}
    N = len(parts)
    for i, mask in enumerate(parts):
        part = [cg.nodes[a] for a in _bits(mask)]
        inside = set(part)
        enclosed = []
        for p in part:
            for s in it.succ[p]:
                ch = cg.chain_of.get(s)
                if ch is not None and ch in neither and it.only(it.succ[ch[-1]]) in inside:
                    enclosed.append(ch)
        full = set(inside)
        for ch in enclosed:
            enclosing[ch].append(i)
            full.update(ch)
        qubits = set().union(*(it.qubits[g] for g in full))
        control_only = qubits - {it.target[g] for g in full}
        pure = len({it.qubits[g] - {it.target[g]} for g in full}) == 1
        converts = {}
        impurities = []
        for p in part:
            for s in it.succ[p]:
                ch = cg.chain_of.get(s)
                if ch is None or s != ch[0]:
                    continue
                q = it.target[s]
                if q in control_only:
                    converts.setdefault(q, []).append(model.both(x[i], (pre[ch], False)))
                elif s not in full:
                    if pure:
                        impurities.append(pre[ch])
                    elif ch in post:
                        model.row([(pre[ch], 1), (post[ch], 1), (x[i], -1)], 0, np.inf)
                    else:
                        model.row([(pre[ch], 1), (x[i], -1)], 0, np.inf)
            for s in it.pred[p]:
                ch = cg.chain_of.get(s)
                if ch is None or s != ch[-1]:
                    continue
                q = it.target[s]
                if q in control_only:
                    converts.setdefault(q, []).append(model.both(x[i], (post[ch], False)))
                elif s not in full:
                    if pure:
                        impurities.append(post[ch])
                    elif ch in pre and len(ch) == 1:
                        model.row([(post[ch], 1), (pre[ch], 1), (x[i], -1)], 0, np.inf)
                    else:
                        model.row([(post[ch], 1), (x[i], -1)], 0, np.inf)
        # j = number of control-only qubits turned into targets, one-hot in t[0..len(converts)]
        t = [model.var() for _ in range(len(converts) + 1)]
        u = {}
        for q, placed in converts.items():
            u[q] = model.var()
            model.row([(u[q], 1), (x[i], -1)], -np.inf, 0)
            for a in placed:
                model.row([(u[q], 1), (a, -1)], 0, np.inf)
        model.row([(v, 1) for v in t] + [(x[i], -1)], 0, 0)
        model.row([(t[j], j) for j in range(len(t))] + [(u[q], -1) for q in u], 0, 0)
        impure = None
        if pure and impurities:
            impure = model.var()
            for z in impurities:
                model.row([(impure, 1), (z, -1)], 0, np.inf)
        for j in range(len(t)):
            controls = len(control_only) - j
            unit = 8 * (1 << (len(qubits) - controls)) - 2
            if pure and j == 0 and impure is not None:
                model.cost[model.both(t[0], (impure, False))] += N * R * unit
                model.cost[model.both(t[0], (impure, True))] += N * (R >> controls) * unit
            else:
                model.cost[t[j]] += N * (R >> (controls if pure and j == 0 else 0)) * unit
    for ch in cg.chains:
        if ch in neither:
            model.row([(pre[ch], 1), (post[ch], 1), (neither[ch], 1)] + [(x[i], 1) for i in enclosing[ch]], 1, 1)
            model.cost[neither[ch]] += N * chain_cost
        elif ch in pre:
            model.constant += N * chain_cost
            model.cost[pre[ch]] -= N * chain_cost
        elif ch in post:
            model.constant += N * chain_cost
            model.cost[post[ch]] -= N * chain_cost
    return pre, post


def select_parts(cg, parts, max_qubit, objective="ilp"):
    """Rule 3: the chosen candidates (indices into parts), the optimum, and for the
    control-aware objective the chains placed before / after (sets of chains)."""
    from .partitioning import parts_to_float_ops

    model = _Model()
    N = len(parts)
    x = [model.var() for _ in range(N)]
    covering = [[] for _ in cg.nodes]
    for i, mask in enumerate(parts):
        for a in _bits(mask):
            covering[a].append(i)
    for lst in covering:
        model.row([(i, 1) for i in lst], 1, 1)
    pre = post = None
    if objective == "ilp":
        for i in range(N):
            model.cost[x[i]] = 1.0
    elif objective == "ilp-fusion":
        qubits = {a: set(cg.it.qubits[cg.nodes[a]]) for a in range(len(cg.nodes))}
        flops = parts_to_float_ops(max_qubit, qubits, None, [list(_bits(m)) for m in parts])
        for i in range(N):
            model.cost[x[i]] = float(flops[i] * N + 1)
    else:
        pre, post = _control_aware_terms(model, cg, parts, x, max_qubit)
        for i in range(N):
            model.cost[x[i]] += 1.0
    while True:
        sol, best = model.solve()
        chosen = [i for i in range(N) if sol[x[i]] == 1]
        groups = _cyclic_groups(cg, parts, chosen)
        if not groups:
            break
        for g in groups:
            model.row([(i, 1) for i in g], -np.inf, len(g) - 1)
    placed = None
    if pre is not None:
        placed = ({ch for ch, v in pre.items() if sol[v] == 1}, {ch for ch, v in post.items() if sol[v] == 1})
    return chosen, best, placed


def _with_chains(cg, groups, placed):
    """Rule 4: the chosen parts (sets of item indices) with the chains put back."""
    it = cg.it
    owner = {}
    for k, grp in enumerate(groups):
        for g in grp:
            owner[g] = k
    out = [set(g) for g in groups]
    before, after = placed if placed is not None else (None, None)
    for ch in cg.chains:
        p = it.only(it.pred[ch[0]])
        s = it.only(it.succ[ch[-1]])
        home = None
        if p is not None and s is not None and owner[p] == owner[s]:
            home = owner[p]
        elif p is not None and (before is None or ch in before):
            home = owner[p]
        elif s is not None and (after is None or ch in after):
            home = owner[s]
        if home is None:
            out.append(set(ch))
        else:
            out[home].update(ch)
    return out


def _topological_parts(it, parts):
    """The parts in a topological order of their dependencies; ready parts leave by (sorted
    qubits of the part, first item)."""
    owner = {}
    for k, p in enumerate(parts):
        for g in p:
            owner[g] = k
    succ = [set() for _ in parts]
    waiting = [0] * len(parts)
    for g, k in owner.items():
        for h in it.succ[g]:
            if owner[h] != k and owner[h] not in succ[k]:
                succ[k].add(owner[h])
                waiting[owner[h]] += 1
    key = [(tuple(sorted(set().union(*(it.qubits[g] for g in p)))), min(p)) for p in parts]
    ready = [(key[k], k) for k in range(len(parts)) if waiting[k] == 0]
    heapq.heapify(ready)
    out = []
    while ready:
        k = heapq.heappop(ready)[1]
        out.append(k)
        for m in succ[k]:
            waiting[m] -= 1
            if waiting[m] == 0:
                heapq.heappush(ready, (key[m], m))
    if len(out) != len(parts):
        raise RuntimeError("the chosen parts depend on each other cyclically")
    return [sorted(parts[k]) for k in out]


def assemble(c, max_qubit, groups, placed=None):
    """Rules 4 and the final order: the partitioned circuit from chosen groups of multi-qubit
    item indices and, for the control-aware objective, the chain placement given as (first
    items of the chains placed before, last items of the chains placed after).  Returns what
    kahn_partition returns."""
    from .partitioning import kahn_partition_preparts

    it = _Items(c)
    cg = _Contracted(it)
    if placed is not None:
        before, after = placed
        placed = ({cg.chain_of[g] for g in before}, {cg.chain_of[g] for g in after})
    full = _with_chains(cg, [list(g) for g in groups], placed)
    return kahn_partition_preparts(c, max_qubit, _topological_parts(it, full))


def max_partitions(c, max_qubit, fusion_cost=False, control_aware=False):
    """Optimal partitioning of circuit c into parts of at most max_qubit qubits (rules 1-5).
    Returns (partitioned circuit, parameter moves [(source start, destination start, count)],
    parts [[item index]]), as kahn_partition does."""
    from .partitioning import kahn_partition_preparts

    it = _Items(c)
    if not it.items:
        return kahn_partition_preparts(c, max_qubit, [])
    cg = _Contracted(it)
    parts = candidate_parts(cg, max_qubit)
    objective = "ilp-fusion-ca" if fusion_cost and control_aware else "ilp-fusion" if fusion_cost else "ilp"
    if cg.nodes:
        chosen, _, placed = select_parts(cg, parts, max_qubit, objective)
    else:
        chosen, placed = [], (set(), set())
    groups = [[cg.nodes[a] for a in _bits(parts[i])] for i in chosen]
    full = _with_chains(cg, groups, placed)
    return kahn_partition_preparts(c, max_qubit, _topological_parts(it, full))
