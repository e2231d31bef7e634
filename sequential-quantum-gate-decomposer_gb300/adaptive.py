"""Adaptive decomposition: the drop-in for SQUANDER's ``N_Qubit_Decomposition_adaptive``
(src-cpp/decomposition/N_Qubit_Decomposition_adaptive.cpp, Python class in
qgd_N_Qubit_Decompositions_Wrapper.cpp:281-330).

The reference grows a circuit of "adaptive" layers until it decomposes the target, compresses it
by removing two-qubit blocks while the decomposition still converges, and finalises it by
replacing the adaptive controlled rotations with CNOT/CZ constructions:

  get_initial_circuit / determine_initial_gate_structure   :289-370, :787-1044
  compress_circuit / compress_gate_structure              :372-497, :1046-1335
  get_panelty, replace_trivial_CRY_gates                  :1337-1582
  remove_trivial_gates, create_reduced_parameters         :1584-1800
  construct_adaptive_gate_layers, add_finalyzing_layer    :1829-1977
  finalize_circuit                                         :499-685

Its Adaptive gate is a CRY whose angle passes through activation_function
(src-cpp/common/common.cpp:35-38), which returns the angle unchanged, so the layers here use the
engine's CRY.  Every inner decomposition is an N_Qubit_Decomposition_custom run on the device
(BFGS up to five qubits, ADAM above, with the reference's budgets).  The candidates of one
compression step (the circuit without one of its blocks, all with the same gate types) are
decomposed together in one launch, one CTA each: sqg_decompose_structures (BFGS) up to five
qubits, sqg_decompose_structures_adam at six qubits when there are at least batch_adam_min of
them; the reference runs them one after another.  Random choices (randomized layer order, the subset of blocks tried, ties of the
penalty) come from the decomposer's seeded generator instead of the reference's std::mt19937.
"""
import math

import numpy as np

from . import _device as dev
from . import _native
from .circuit import CNOT, CRY, CZ, PARAM_NUM, RX, RY, RZ, U3, Circuit
from .decomposition import N_Qubit_Decomposition_custom


def _u3(t2, p, l):
    """SQUANDER's U3 kernel from (theta/2, phi, lambda) (Gate::calc_one_qubit_u3)."""
    c, s = math.cos(t2), math.sin(t2)
    return np.array([[c, -np.exp(1j * l) * s], [np.exp(1j * p) * s, np.exp(1j * (p + l)) * c]])


class _Structure:
    """Top-level blocks of a circuit, each a list of (type, target, control) gates; the last
    block is the final U3 layer."""

    def __init__(self, n, blocks):
        self.n = n
        self.blocks = [list(b) for b in blocks]

    def copy(self):
        return _Structure(self.n, self.blocks)

    def param_num(self, b=None):
        blocks = self.blocks if b is None else [self.blocks[b]]
        return sum(PARAM_NUM[g[0]] for blk in blocks for g in blk)

    def block_start(self, b):
        return sum(PARAM_NUM[g[0]] for blk in self.blocks[:b] for g in blk)

    def types(self):
        return tuple(g[0] for blk in self.blocks for g in blk)

    def circuit(self):
        top = Circuit(self.n)
        for blk in self.blocks:
            sub = Circuit(self.n)
            for t, tg, c in blk:
                sub._add(t, tg, c)
            top.add_Circuit(sub)
        return top

    def records(self):
        recs, p = [], 0
        for blk in self.blocks:
            for t, tg, c in blk:
                recs.append((t, tg, c, p))
                p += PARAM_NUM[t]
        return np.asarray(recs, dtype=np.int32).reshape(-1, 4)

    def without(self, b):
        s = self.copy()
        del s.blocks[b]
        return s


class N_Qubit_Decomposition_adaptive(N_Qubit_Decomposition_custom):
    """Drop-in for squander.N_Qubit_Decomposition_adaptive(Umtx, qbit_num=-1, level_limit_max=8,
    level_limit_min=0, topology=None, config=None, accelerator_num=0)."""

    def __init__(self, Umtx, qbit_num=-1, level_limit_max=8, level_limit_min=0, topology=None, config=None,
                 accelerator_num=0):
        super().__init__(Umtx, qbit_num, None, config, accelerator_num)
        self.level_limit = int(level_limit_max)
        self.level_limit_min = int(level_limit_min)
        self.topology = [tuple(int(v) for v in e) for e in topology] if topology else None
        self.randomized_adaptive_layers = bool(self.config.get("randomized_adaptive_layers", False))
        self.structure = None

    # ---- circuit construction ------------------------------------------------------------
    def _adaptive_layer(self):
        """construct_adaptive_gate_layers: a block [U3(t), U3(c), CRY(t, c)] per qubit pair (the
        topology's (control, target) pairs, else every t < c), in order or shuffled."""
        n = self.qbit_num
        if self.topology:
            pairs = []
            for e in self.topology:
                if len(e) != 2:
                    raise ValueError("The connectivity data should contains two qubits.")
                c, t = e
                if c >= n or t >= n:
                    raise ValueError("Label of control/target qubit should be less than the number of qubits "
                                     "in the register.")
                pairs.append((t, c))
        else:
            pairs = [(t, c) for t in range(n) for c in range(t + 1, n)]
        layers = [[(U3, t, -1), (U3, c, -1), (CRY, t, c)] for t, c in pairs]
        out = []
        while layers:
            idx = int(self.rng.integers(0, 5001)) % len(layers) if self.randomized_adaptive_layers else 0
            out.append(layers.pop(idx))
        return out

    def _final_layer(self):
        return [(U3, q, -1) for q in range(self.qbit_num)]

    # ---- gate structure built by the caller (wrapper methods of the reference class) -----
    def _append_blocks(self, blocks):
        for blk in blocks:
            sub = Circuit(self.qbit_num)
            for t, tg, c in blk:
                sub._add(t, tg, c)
            self.circuit.add_Circuit(sub)
        self._evaluator = None

    def add_Adaptive_Layers(self):
        """add_adaptive_layers (N_Qubit_Decomposition_adaptive.cpp:1802-1820, wrapper
        qgd_N_Qubit_Decompositions_Wrapper.cpp:2174): appends one level of adaptive layers,
        a [U3(t), U3(c), CRY(t, c)] block per qubit pair, to the gate structure that the
        Optimization_Problem family evaluates."""
        self._append_blocks(self._adaptive_layer())
        return 0

    def add_Finalyzing_Layer_To_Gate_Structure(self):
        """add_finalyzing_layer (N_Qubit_Decomposition_adaptive.cpp:1938-1968, wrapper :874):
        appends a block of U3 gates on every qubit to the gate structure."""
        self._append_blocks([self._final_layer()])
        return 0

    # ---- inner decompositions (N_Qubit_Decomposition_custom runs) ---------------------------
    def _phase_target(self, factor):
        """apply_global_phase_factor on the decomposer's target."""
        self.Umtx = np.ascontiguousarray(self.Umtx * factor)
        self._evaluator = None

    # candidates of one step from which six-qubit ADAM decompositions run one CTA each in a
    # single launch (sqg_decompose_structures_adam) instead of one whole-GPU graph launch each
    batch_adam_min = 4

    def _stage_budget(self, stage, adam, P):
        """Evaluation budget of a stage's custom decompositions.  The reference copies
        max_inner_iterations_compression / _final into the stage's config as
        max_inner_iterations (N_Qubit_Decomposition_adaptive.cpp:574-579, 1269-1275); the
        engines read max_inner_iterations_bfgs / _adam, then max_inner_iterations
        (BFGS.cpp:91-97, ADAM.cpp:98-103), before the value the stage sets: BFGS 10000 (100
        for compression), ADAM P / 852 * 1e7 (100000 for compression), :600-616, :1303-1313."""
        cfg = self.config
        own = "max_inner_iterations_adam" if adam else "max_inner_iterations_bfgs"
        key = {"compression": "max_inner_iterations_compression", "final": "max_inner_iterations_final"}.get(stage)
        if own in cfg:
            return int(cfg[own])
        if key and key in cfg:
            return int(cfg[key])
        if "max_inner_iterations" in cfg:
            return int(cfg["max_inner_iterations"])
        if adam:
            return 100000 if stage == "compression" else int(P / 852 * 10000000.0)
        return 100 if stage == "compression" else 10000

    def _adam_settings(self, stage, tol):
        """ADAM engine settings of a stage: (tolerance, eta, adaptive eta, random shifts at most,
        randomization threshold), with the config keys ADAM.cpp:98-170 reads."""
        cfg = self.config
        tol_a = float(cfg.get("optimization_tolerance_adam", tol))
        eta = float(cfg["eta"]) if "eta" in cfg else 1e-3
        adaptive = bool(cfg["adaptive_eta"]) if "adaptive_eta" in cfg else True
        thr = int(cfg.get("randomization_threshold_adam", cfg.get("randomization_threshold", 2500000)))
        shifts = 1 if stage == "compression" else 10000
        return tol_a, eta, adaptive, shifts, thr

    def _groups(self, structs):
        groups = {}
        for i, s in enumerate(structs):
            groups.setdefault(s.types(), []).append(i)
        return groups

    def _start_points(self, structs, starts, idx, P):
        return np.stack([starts[i] if starts[i] is not None else self.rng.uniform(0, 2 * math.pi, P) for i in idx])

    def _inner_adam_batched(self, structs, starts, idx, stage, tol, max_outer, out):
        """The ADAM decompositions of structures idx (same gate types, six qubits) in one
        launch, one CTA each (sqg_decompose_structures_adam)."""
        nc = structs[idx[0]].circuit().native()
        P, B = nc.param_num, len(idx)
        target = self.evaluator().target
        tol_a, eta, adaptive, shifts, thr = self._adam_settings(stage, tol)
        recs = np.ascontiguousarray(np.stack([structs[i].records() for i in idx]))
        x = dev.to_device_real(self._start_points(structs, starts, idx, P))
        cost = dev.torch.empty(B, dtype=dev.torch.float64, device="cuda")
        evals = dev.torch.empty(B, dtype=dev.torch.int32, device="cuda")
        lib = _native.lib()
        w = dev.Workspace().get(lib.sqg_decompose_structures_adam_workspace_bytes(nc.handle, B))
        _native.check(lib.sqg_decompose_structures_adam(
            nc.handle, recs.ctypes.data, dev.ptr(target), 0, target.shape[1], B, self.trace_offset, self.cost_variant,
            dev.ptr(x), dev.ptr(cost), dev.ptr(evals), None, tol_a, self._stage_budget(stage, True, P), eta,
            1 if adaptive else 0, shifts, thr, max_outer, int(self.rng.integers(1 << 62)), dev.ptr(w), w.numel(),
            dev.stream_ptr()), "sqg_decompose_structures_adam")
        c, xs, ev = cost.cpu().numpy(), x.cpu().numpy(), evals.cpu().numpy()
        for j, i in enumerate(idx):
            out[i] = (float(c[j]), xs[j].copy(), int(ev[j]))

    def _inner(self, structs, starts, stage, tol):
        """One custom decomposition per (structure, start point or None for a random start).
        Returns [(minimum, best point, evaluations)]."""
        n = self.qbit_num
        max_outer = int(self.config.get("max_outer_iterations", self.max_outer_iterations))
        loops = int(self.config.get("max_iteration_loops", 3 if n == 2 else 1))
        out = [None] * len(structs)
        if n <= 5:
            groups = self._groups(structs)
            target = self.evaluator().target
            lib = _native.lib()
            for idx in groups.values():
                nc = structs[idx[0]].circuit().native()
                P, B = nc.param_num, len(idx)
                max_inner = self._stage_budget(stage, False, P)
                recs = np.ascontiguousarray(np.stack([structs[i].records() for i in idx]))
                x = dev.to_device_real(self._start_points(structs, starts, idx, P))
                cost = dev.torch.empty(B, dtype=dev.torch.float64, device="cuda")
                calls = dev.torch.empty(B, dtype=dev.torch.int32, device="cuda")
                w = dev.Workspace().get(lib.sqg_decompose_structures_workspace_bytes(nc.handle, B, target.shape[1]))
                _native.check(lib.sqg_decompose_structures(
                    nc.handle, recs.ctypes.data, dev.ptr(target), 0, target.shape[1], B, self.trace_offset,
                    self.cost_variant, dev.ptr(x), dev.ptr(cost), dev.ptr(calls), None, tol, max_inner, max_outer,
                    loops, 0, int(self.rng.integers(1 << 62)), dev.ptr(w), w.numel(), dev.stream_ptr()),
                    "sqg_decompose_structures")
                c, xs, ev = cost.cpu().numpy(), x.cpu().numpy(), calls.cpu().numpy()
                for j, i in enumerate(idx):
                    out[i] = (float(c[j]), xs[j].copy(), int(ev[j]))
            return out
        single = list(range(len(structs)))
        if n == 6:
            for idx in self._groups(structs).values():
                if len(idx) >= self.batch_adam_min:
                    self._inner_adam_batched(structs, starts, idx, stage, tol, max_outer, out)
            single = [i for i in single if out[i] is None]
        for i in single:  # ADAM above five qubits, one graph launch per run
            s = structs[i]
            P = s.param_num()
            cfg = dict(self.config)
            cfg.pop("max_inner_iterations_adam", None)
            cfg["max_inner_iterations"] = self._stage_budget(stage, True, P)
            cfg["random_shift_count_max"] = 1 if stage == "compression" else 10000
            cfg["optimization_tolerance"] = tol
            d = N_Qubit_Decomposition_custom(self.Umtx, self.qbit_num, None, cfg)
            d.rng = self.rng
            d.set_Gate_Structure(s.circuit())
            d.set_Optimizer("ADAM")
            d.max_outer_iterations = max_outer
            if starts[i] is not None:
                d.set_Optimized_Parameters(starts[i])
            d.trace_offset, d.cost_variant = self.trace_offset, self.cost_variant
            d.Start_Decomposition()
            out[i] = (d.get_Decomposition_Error(), d.get_Optimized_Parameters(), d.get_Num_of_Iters())
        return out

    # ---- the three stages ----------------------------------------------------------------
    def _initial(self, tol):
        """determine_initial_gate_structure: levels level_limit_min..level_limit of adaptive
        layers plus the final layer, each decomposed from a random start; the best one wins."""
        if self.level_limit_min > self.level_limit:
            raise ValueError("level_limit_min exceeds level_limit_max: no circuit to optimize")
        results = []
        level = self.level_limit_min
        while level <= self.level_limit:
            blocks = []
            for _ in range(level):
                blocks += self._adaptive_layer()
            s = _Structure(self.qbit_num, blocks + [self._final_layer()])
            f, x, ev = self._inner([s], [None], "initial", tol)[0]
            self.num_iters += ev
            results.append((f, s, x))
            if f < tol:
                break
            level += 1
        return min(results, key=lambda r: r[0])

    def _theta_of_layer(self, s, x, b):
        """extract_theta_from_layer: sin^2 of the block's controlled-rotation parameter."""
        p = s.block_start(b)
        for t, _, _ in s.blocks[b]:
            if t == CRY:
                return math.sin(x[p]) ** 2
            p += PARAM_NUM[t]
        return 0.0

    def _reduced(self, s, x, b):
        """create_reduced_parameters: x without block b's parameters."""
        p0, k = s.block_start(b), s.param_num(b)
        return np.concatenate([x[:p0], x[p0 + k:]])

    def _panelty(self, s, x):
        """get_panelty: 0 for a CRY at the identity, 1 for a CRY at a CNOT (as written in the
        reference, |sin| < 0.999 with |cos| < 1e-3 never holds), 2 otherwise."""
        pen, p = 0, 0
        for blk in s.blocks:
            for t, _, _ in blk:
                par = x[p] if p < len(x) else 0.0
                p += PARAM_NUM[t]
                if t != CRY:
                    continue
                if abs(math.sin(par)) < 0.999 and abs(math.cos(par)) < 1e-3:
                    pen += 1
                elif abs(math.sin(par)) < 1e-3 and abs(1 - math.cos(par)) < 1e-3:
                    pass
                else:
                    pen += 2
        return pen

    def _compress_one(self, s, b, x, tol):
        """compress_gate_structure(structure, layer, ...): decompose the circuit without block b
        from the reduced parameters (budget of the compression stage); kept when it converges."""
        red = s.without(b)
        f, xr, ev = self._inner([red], [self._reduced(s, x, b)], "compression", tol)[0]
        self.num_iters += ev
        if f < tol:
            return red, xr, f
        return s.copy(), x, math.inf

    def _fold_block(self, s, x, b):
        """The U3 gates of block b folded into the next U3 on the same qubit in a later block
        (the merge of remove_trivial_gates, :1600-1700): block b's U3 parameters become zero, the
        matching U3 takes the product's angles when they reproduce it, and the product's global
        phase is returned (the reference moves it onto the target).  Returns (x, phase)."""
        x = x.copy()
        phase = 1.0 + 0.0j
        blk = s.blocks[b]
        involved = sorted({q for _, t, c in blk for q in ((t, c) if c >= 0 else (t,))})
        pr = s.block_start(b)
        for rdx in range(len(involved)):
            g = blk[rdx]
            match = None
            for kb in range(b + 1, len(s.blocks)):
                pk = s.block_start(kb)
                for t, tg, _c in s.blocks[kb]:
                    if t == U3 and tg == g[1]:
                        match = pk
                        break
                    pk += PARAM_NUM[t]
                if match is not None:
                    break
            if match is None:
                raise RuntimeError("N_Qubit_Decomposition_adaptive::remove_trivial_gates: No matching U3 gate was "
                                   "found. Need to append a U3 gate to the end, but this functionality is not "
                                   "developed yet.")
            prod = _u3(*x[match:match + 3]) @ _u3(*x[pr:pr + 3])
            x[pr:pr + 3] = 0.0
            pr += PARAM_NUM[g[0]]
            c3, s3 = abs(prod[0, 0]), abs(prod[1, 0])
            t3 = math.atan2(s3, c3)
            alpha = math.atan2(prod[0, 0].imag, prod[0, 0].real)
            if abs(s3) < 4e-8:
                l3 = (math.atan2(prod[1, 1].imag, prod[1, 1].real) - alpha) / 2
                p3 = l3
            else:
                l3 = math.atan2(-prod[0, 1].imag, -prod[0, 1].real) - alpha
                p3 = math.atan2(prod[1, 0].imag, prod[1, 0].real) - alpha
            f = complex(math.cos(alpha), math.sin(alpha))
            new = _u3(t3, p3, l3) * f
            if (abs(new[1, 1].real - prod[1, 1].real) + abs(new[1, 1].imag - prod[1, 1].imag) < 1e-8
                    and s3 * s3 + c3 * c3 > 0.99):
                x[match:match + 3] = (t3, p3, l3)
                phase *= f
        return x, phase

    def _remove_trivial(self, s, x, fmin, tol):
        """remove_trivial_gates: the first block whose CRY is at the identity is folded away
        (_fold_block, its phase moved onto the target) and the circuit without it is decomposed
        again."""
        for b in range(len(s.blocks) - 1):
            blk = s.blocks[b]
            if len(blk) < 3 or blk[2][0] != CRY:
                continue
            par = x[s.block_start(b) + 6]
            if not (abs(math.sin(par)) < 1e-3 and abs(1 - math.cos(par)) < 1e-3):
                continue
            x2, phase = self._fold_block(s, x, b)
            if phase != 1.0:
                self._phase_target(phase)
            red, xr, f = self._compress_one(s, b, x2, tol)
            return red, xr, min(fmin, f)
        return s, x, fmin

    def _compress(self, s, x, fmin, uncompressed, tol):
        """compress_gate_structure(structure, uncompressed_iter_num): try to remove a few blocks
        (the five with the smallest CRY angle in the first round, a random subset later), keep the
        candidate of the lowest penalty."""
        L = len(s.blocks) - 1  # the final U3 layer is never removed
        lmax = L if L < 50 else (4 if L < 60 else 2)
        if uncompressed == 0:
            lmax = min(5, L)
            order = sorted(range(L), key=lambda b: self._theta_of_layer(s, x, b))
            trial = order[:lmax]
        else:
            trial = list(range(L))
            while len(trial) > lmax:
                trial.pop(int(self.rng.integers(0, 5001)) % len(trial))
        nt = min(lmax, L)
        if nt == 0:
            return s, x, fmin
        target_save = self.Umtx.copy()
        # the candidates' decompositions are independent: one launch for all of them
        reds = [s.without(b) for b in trial[:nt]]
        res = self._inner(reds, [self._reduced(s, x, b) for b in trial[:nt]], "compression", tol)
        cands = []
        for k, b in enumerate(trial[:nt]):
            self.Umtx = target_save.copy()
            self._evaluator = None
            f, xr, ev = res[k]
            self.num_iters += ev
            if f < tol:
                red, xk, fk = reds[k], xr, f
                tmp, xk, fk = self._remove_trivial(red, xk, fk, tol)
            else:
                tmp, xk, fk = s.copy(), x.copy(), math.inf
            cands.append((self._panelty(tmp, xk), tmp, xk, fk, self.Umtx.copy()))
        best = 0
        pmin = cands[0][0]
        for k in range(len(cands)):
            if pmin > cands[k][0]:
                pmin, best = cands[k][0], k
            elif pmin == cands[k][0] and int(self.rng.integers(0, 5001)) % 2 == 1:
                pmin, best = cands[k][0], k
        _, s2, x2, f2, target = cands[best]
        self.Umtx = target
        self._evaluator = None
        return s2, x2, (f2 if f2 < math.inf else fmin)

    def _replace_trivial_cry(self, s, x):
        """replace_trivial_CRY_gates: a CRY at the identity is dropped, a CRY at +-pi (a CNOT up to
        phases) becomes RX(-pi/4) CZ RX(pi/4) RZ(+-pi/4) with the phase e^{+-i pi/4} moved onto the
        target, any other CRY becomes RY(t/2) CNOT RY(-t/2) CNOT."""
        blocks, xs, p = [], [], 0
        for blk in s.blocks:
            nb = []
            for t, tg, c in blk:
                k = PARAM_NUM[t]
                par = x[p] if p < len(x) else 0.0
                if t == CRY and abs(math.sin(par)) > 0.999 and abs(math.cos(par)) < 1e-3:
                    nb += [(RX, tg, -1), (CZ, tg, c), (RX, tg, -1), (RZ, c, -1)]
                    sgn = -1.0 if math.sin(par) < 0 else 1.0
                    xs += [-math.pi / 4, math.pi / 4, sgn * math.pi / 4]
                    self._phase_target(complex(math.cos(sgn * math.pi / 4), math.sin(sgn * math.pi / 4)))
                elif t == CRY and abs(math.sin(par)) < 1e-3 and abs(1 - math.cos(par)) < 1e-3:
                    pass
                elif t == CRY:
                    nb += [(RY, tg, -1), (CNOT, tg, c), (RY, tg, -1), (CNOT, tg, c)]
                    xs += [par / 2, -par / 2]
                else:
                    nb.append((t, tg, c))
                    xs += list(x[p:p + k])
                p += k
            blocks.append(nb)
        return _Structure(self.qbit_num, blocks), np.asarray(xs, dtype=np.float64)

    # ---- the stages as the reference's wrapper exposes them --------------------------------
    def _held(self):
        """The gate structure the decomposer holds (built by add_Adaptive_Layers /
        add_Finalyzing_Layer_To_Gate_Structure, or left by an earlier stage), one block per
        top-level item, with its parameters (None when they do not fit it)."""
        c = self.circuit
        s = _Structure(self.qbit_num, [list(c._gates[a:b]) for a, b in c._item_ranges()])
        x = self.optimized_parameters
        return s, (x.copy() if x is not None and x.size == s.param_num() else None)

    def _hold(self, s, x):
        self.structure = s
        self.circuit = s.circuit()
        self._evaluator = None
        self.optimized_parameters = np.asarray(x, dtype=np.float64)
        self.decomposition_error = self.Optimization_Problem(self.optimized_parameters)

    def _final_tolerance(self):
        """finalize_circuit reads the config's optimization_tolerance into an integer
        (N_Qubit_Decomposition_adaptive.cpp:538-543; Config_Element keeps a float entry's integer
        field at 0), so a float entry makes the final tolerance 0 and the final optimisation runs
        its whole budget; an integer entry is used as it is; without one the tolerance is 1e-4."""
        v = self.config.get("optimization_tolerance")
        if v is None:
            return 1e-4
        if isinstance(v, (int, np.integer)) and not isinstance(v, bool):
            return float(v)
        return 0.0

    def get_Initial_Circuit(self):
        """get_initial_circuit (:289-370): nothing when level_limit is 0; with a gate structure
        already held, one decomposition of it from the held parameters
        (optimize_imported_gate_structure, :687-776); otherwise the level search of
        determine_initial_gate_structure.  The result is held for the next stage."""
        if self.level_limit == 0:
            return 0
        tol = float(self.config.get("optimization_tolerance", self.optimization_tolerance))
        if self.circuit.get_Gate_Num() > 0:
            s, x0 = self._held()
            f, x, ev = self._inner([s], [x0], "initial", tol)[0]
            self.num_iters += ev
        else:
            f, s, x = self._initial(tol)
        self._current_minimum = f
        self._hold(s, x)
        return 0

    def Compress_Circuit(self):
        """compress_circuit (:372-497): rounds of compress_gate_structure while fewer than 25
        rounds ran or at most five rounds in a row removed nothing, stopping after the second
        such round; nothing without a held gate structure."""
        if self.circuit.get_Gate_Num() == 0:
            return 0
        tol = float(self.config.get("optimization_tolerance", self.optimization_tolerance))
        s, x = self._held()
        if x is None:
            x = self.rng.uniform(0, 2 * math.pi, s.param_num())
        f = getattr(self, "_current_minimum", math.inf)
        it, unc = 0, 0
        while it < 25 or unc <= 5:
            s2, x2, f2 = self._compress(s, x, f, unc, tol)
            unc = 0 if len(s2.blocks) < len(s.blocks) else unc + 1
            s, x, f = s2, x2, f2
            it += 1
            if unc > 1:
                break
        self.compressed_structure = s
        self._current_minimum = f
        self._hold(s, x)
        return 0

    def Finalize_Circuit(self):
        """finalize_circuit (:499-685): the controlled rotations replaced by CNOT / CZ
        constructions (replace_trivial_CRY_gates) and one final decomposition from the held
        parameters; nothing without a held gate structure."""
        if self.circuit.get_Gate_Num() == 0:
            return 0
        s, x = self._held()
        if x is None:
            x = np.zeros(s.param_num())
        s, x = self._replace_trivial_cry(s, x)
        f, x, ev = self._inner([s], [x], "final", self._final_tolerance())[0]
        self.num_iters += ev
        self._current_minimum = f
        self._hold(s, x)
        return 0

    def Start_Decomposition(self):
        """start_decomposition (:245-260): get_Initial_Circuit, Compress_Circuit,
        Finalize_Circuit."""
        if self.level_limit == 0:
            print("please increase level limit")
            return 0
        self.get_Initial_Circuit()
        self.Compress_Circuit()
        self.Finalize_Circuit()
        return 0


class N_Qubit_State_Preparation_adaptive(N_Qubit_Decomposition_adaptive):
    """Drop-in for squander.N_Qubit_State_Preparation_adaptive(State, level_limit_max=8,
    level_limit_min=0, topology=None, config={})
    (squander/decomposition/qgd_N_Qubit_State_Preparation_adaptive.py): the adaptive decomposition
    of a state given as a complex128 column vector, so that the circuit maps it to |0...0>
    (the cost 1 - Re (C psi)_0 of a one-column target)."""

    def __init__(self, State, level_limit_max=8, level_limit_min=0, topology=None, config=None):
        if not isinstance(State, np.ndarray):
            raise Exception("Initial state should be a numpy array")
        if State.dtype != np.complex128:
            raise Exception("Initial state should be made of complex values")
        if not State.flags.c_contiguous:
            raise Exception("Initial state should be contiguous in memory")
        if State.ndim == 1:
            State = State.reshape((State.size, 1))
        if not (State.ndim == 2 and State.shape[1] == 1):
            raise Exception("Initial state not properly formatted. Input state must be a column vector")
        super().__init__(State, -1, level_limit_max, level_limit_min, topology=topology, config=config)

    def get_Qiskit_Circuit(self):
        raise NotImplementedError("Qiskit is not part of this engine")
