"""Drop-in ``N_Qubit_Decomposition_custom`` on the GB300 engine.

Mirrors squander.N_Qubit_Decomposition_custom
(squander/decomposition/qgd_N_Qubit_Decompositions_Wrapper.cpp:347-400 and the method
table at :3125-3250): the same constructor arguments, the same U^dagger target
convention, parameter layout, cost-function variants and return shapes.  The cost and
gradient run in the engine's CUDA kernels; the decomposition driver follows
N_Qubit_Decomposition_custom::start_decomposition (src-cpp/decomposition/
N_Qubit_Decomposition_custom.cpp:116-190) with BFGS for qbit_num <= 5 and ADAM above
(:59-76).
"""
import math

import numpy as np

from . import _device as dev
from . import _native
from . import sharding
from .circuit import Circuit, combined_unitary_device
from .evaluator import FROBENIUS_NORM, SUPPORTED_VARIANTS, CostEvaluator
from .batched import BatchedDecomposer, adam_decompose_graph, bfgs_decompose_graph
from .optim import adam_squander, bfgs_powell

_GUESS = {"zeros": "ZEROS", "random": "RANDOM", "close_to_zero": "CLOSE_TO_ZERO"}


class N_Qubit_Decomposition_custom:
    def __init__(self, Umtx, qbit_num=-1, initial_guess=None, config=None, accelerator_num=0):
        U = np.asarray(Umtx)
        if U.dtype == np.complex64:
            raise NotImplementedError("the GB300 engine computes in FP64; pass a complex128 target")
        if U.dtype != np.complex128 or U.ndim != 2:
            raise TypeError("Umtx must be a 2-D complex128 array")
        self.Umtx = np.ascontiguousarray(U)
        if qbit_num == -1:
            qbit_num = int(round(math.log2(self.Umtx.shape[0])))
        if self.Umtx.shape[0] != (1 << qbit_num):
            raise ValueError("the target must have 2**qbit_num rows")
        self.qbit_num = int(qbit_num)
        self.config = dict(config or {})
        g = "random" if initial_guess is None else str(initial_guess).lower()
        self.initial_guess = _GUESS.get(g, "RANDOM")
        self.accelerator_num = accelerator_num
        self.circuit = Circuit(self.qbit_num)
        self.cost_variant = FROBENIUS_NORM
        self.trace_offset = 0
        self.optimization_tolerance = float(self.config.get("optimization_tolerance", 1e-7))
        self.verbose = int(self.config.get("verbose", 0))
        seed = self.config.get("random_seed")
        self.rng = np.random.default_rng(None if seed is None else int(seed))
        if self.qbit_num <= 5:
            self.set_Optimizer("BFGS")
            self.max_outer_iterations = 4
        else:
            self.set_Optimizer("ADAM")
            self.max_outer_iterations = 1
        self.optimized_parameters = np.zeros(0)
        self.decomposition_error = None
        self.num_iters = 0
        self._evaluator = None
        self._loop_ws = dev.Workspace()
        # True: drive every evaluation from the host (optim.py), the form the device loops are
        # tested against
        self._host_loops = False

    # ---- configuration -----------------------------------------------------------------
    def set_Gate_Structure(self, gate_structure):
        if not isinstance(gate_structure, Circuit):
            raise TypeError("set_Gate_Structure expects a Circuit")
        if gate_structure.qbit_num != self.qbit_num:
            raise ValueError("the gate structure must span %d qubits" % self.qbit_num)
        self.circuit = gate_structure
        self._evaluator = None
        return 0

    def get_Circuit(self):
        return self.circuit

    def get_Parameter_Num(self):
        return self.circuit.get_Parameter_Num()

    def get_Qbit_Num(self):
        return self.qbit_num

    def set_Cost_Function_Variant(self, costfnc=0):
        if int(costfnc) not in SUPPORTED_VARIANTS:
            raise Exception("Optimization_Interface::optimization_problem: Cost function variant not implmented.")
        self.cost_variant = int(costfnc)
        self._evaluator = None

    def set_Trace_Offset(self, trace_offset=0):
        if trace_offset < 0 or trace_offset + self.Umtx.shape[1] > self.Umtx.shape[0]:
            raise ValueError("trace offset out of range")
        self.trace_offset = int(trace_offset)
        self._evaluator = None

    def get_Trace_Offset(self):
        return self.trace_offset

    def set_Optimizer(self, optimizer="BFGS"):
        name = str(optimizer).upper()
        if name not in ("BFGS", "ADAM"):
            print("Wrong optimizer: %s. Using default: BFGS" % optimizer)
            name = "BFGS"
        self.optimizer = name
        # Optimization_Interface::set_optimizer (Optimization_Interface.cpp:1619-1670): BFGS runs
        # 10000 evaluations per run and outer iterations until the tolerance; ADAM 100000
        # evaluations in one outer iteration with up to 100 randomisations.  The constructor
        # then sets 4 (BFGS) or 1 (ADAM) outer iterations, N_Qubit_Decomposition_custom.cpp:59-76.
        if name == "BFGS":
            self.max_inner_iterations, self.max_outer_iterations, self.random_shift_count_max = 10000, 100000000, 1
        else:
            self.max_inner_iterations, self.max_outer_iterations, self.random_shift_count_max = 100000, 1, 100
        return 0

    def set_Optimization_Tolerance(self, tolerance):
        self.optimization_tolerance = float(tolerance)

    def set_Max_Iterations(self, max_iterations):
        self.max_inner_iterations = int(max_iterations)

    def set_Verbose(self, verbose):
        self.verbose = int(verbose)

    def set_Optimized_Parameters(self, new_params):
        p = np.asarray(new_params, dtype=np.float64).reshape(-1)
        if p.size != self.get_Parameter_Num():
            raise ValueError("wrong number of parameters")
        self.optimized_parameters = p.copy()
        return 0

    def get_Optimized_Parameters(self):
        return self.optimized_parameters.copy()

    def get_Decomposition_Error(self):
        return self.decomposition_error

    def get_Num_of_Iters(self):
        return self.num_iters

    def get_Unitary(self):
        """The matrix being decomposed (the U^dagger handed to the constructor)."""
        return self.Umtx.copy()

    def set_Unitary(self, Umtx):
        U = np.asarray(Umtx)
        if U.dtype != np.complex128 or U.shape != self.Umtx.shape:
            raise ValueError("the new target must be complex128 with shape %s" % (self.Umtx.shape,))
        self.Umtx = np.ascontiguousarray(U)
        self._evaluator = None

    def get_Gate_Num(self):
        return self.circuit.get_Gate_Num()

    def set_Iteration_Loops(self, iteration_loops):
        """{qbit_num: loops} or an int: BFGS restarts per outer iteration (BFGS.cpp:67-99)."""
        if isinstance(iteration_loops, dict):
            loops = iteration_loops.get(self.qbit_num)
            if loops is not None:
                self.config["max_iteration_loops"] = int(loops)
        else:
            self.config["max_iteration_loops"] = int(iteration_loops)
        return 0

    def set_Convergence_Threshold(self, threshold):
        self.config["convergence_threshold"] = float(threshold)

    # ---- bookkeeping methods of the reference wrapper (DECOMPOSITION_WRAPPER_BASE_METHODS,
    # qgd_N_Qubit_Decompositions_Wrapper.cpp) ------------------------------------------------
    def get_Gates(self):
        """Gate dictionaries with the optimized parameters (Wrapper get_Gates: "type",
        "target_qbit", "control_qbit", U3 "Theta"/"Phi"/"Lambda", RX/RY/CRY "Theta", RZ "Phi")."""
        out = []
        params = self.optimized_parameters
        for d in self.circuit.get_Flat_Gates():
            g = {"type": d["type"], "target_qbit": d["target_qbit"]}
            if "control_qbit" in d:
                g["control_qbit"] = d["control_qbit"]
            ps = d["parameter_start_index"]
            if d["type"] == "U3" and params.size >= ps + 3:
                g["Theta"], g["Phi"], g["Lambda"] = float(params[ps]), float(params[ps + 1]), float(params[ps + 2])
            elif d["type"] in ("RX", "RY", "CRY") and params.size >= ps + 1:
                g["Theta"] = float(params[ps])
            elif d["type"] == "RZ" and params.size >= ps + 1:
                g["Phi"] = float(params[ps])
            out.append(g)
        return out

    def List_Gates(self):
        """Prints the gate structure with the optimized parameters."""
        for k, g in enumerate(self.get_Gates()):
            print("%d-th gate: %s" % (k, ", ".join("%s %s" % (key, val) for key, val in g.items())))

    def get_Project_Name(self):
        return getattr(self, "project_name", "")

    def set_Project_Name(self, name):
        self.project_name = str(name)

    def set_Debugfile(self, filename):
        self.debugfile = str(filename)

    def set_Max_Layer_Num(self, max_layer_num):
        """Stored for structure-building decompositions; a custom gate structure is used as given."""
        self.max_layer_num = max_layer_num

    def set_Optimization_Blocks(self, optimization_blocks):
        """Stored; the custom decomposition optimizes all gates of the structure at once."""
        self.optimization_blocks = int(optimization_blocks)

    def get_Global_Phase(self):
        gp = getattr(self, "global_phase_factor", 1.0 + 0.0j)
        return math.atan2(gp.imag, gp.real)

    def set_Global_Phase(self, phase):
        """Decomposition_Base::set_global_phase (Decomposition_Base.cpp:1098-1101), including
        its sqrt(2) magnitude."""
        self.global_phase_factor = complex(math.sqrt(2) * math.cos(phase), math.sqrt(2) * math.sin(phase))

    def apply_Global_Phase_Factor(self):
        """Multiplies the target by the global phase factor and resets the phase
        (Decomposition_Base.cpp:1117-1121)."""
        self.Umtx = np.ascontiguousarray(self.Umtx * getattr(self, "global_phase_factor", 1.0 + 0.0j))
        self.set_Global_Phase(0)
        self._evaluator = None

    def export_Unitary(self, filename):
        """Decomposition_Base::export_unitary (Decomposition_Base.cpp:1128-1143): int32 rows,
        int32 cols, then the complex128 entries row by row, the project name prefixed."""
        name = str(filename)
        if self.get_Project_Name():
            name = self.get_Project_Name() + "_" + name
        with open(name, "wb") as f:
            np.asarray([self.Umtx.shape[0], self.Umtx.shape[1]], dtype=np.int32).tofile(f)
            np.ascontiguousarray(self.Umtx, dtype=np.complex128).tofile(f)

    def Reorder_Qubits(self, qbit_list):
        """Decomposition_Base::reorder_qubits (Decomposition_Base.cpp:910-950) with
        Gate::reorder_qubits (Gate.cpp:1151-1195): qubit qbit_list[k] becomes qubit k, in the
        gate structure and in the rows and columns of the target."""
        ql = [int(q) for q in qbit_list]
        n = self.qbit_num
        if sorted(ql) != list(range(n)):
            raise ValueError("Gate::reorder_qubits: Wrong number of qubits.")
        new_of_old = [0] * n
        for k, q in enumerate(ql):
            new_of_old[q] = k
        self.circuit = self.circuit.Remap_Qbits({q: new_of_old[q] for q in range(n)})
        idx = np.arange(self.Umtx.shape[0])
        perm = np.zeros_like(idx)
        for k, q in enumerate(ql):
            perm |= ((idx >> q) & 1) << k
        U = np.empty_like(self.Umtx)
        U[np.ix_(perm, perm)] = self.Umtx
        self.Umtx = U
        self._evaluator = None

    # ---- cost / gradient -----------------------------------------------------------------
    def evaluator(self):
        if self._evaluator is None:
            self._evaluator = CostEvaluator(self.circuit, self.Umtx, self.trace_offset, self.cost_variant)
        return self._evaluator

    def _params(self, parameters):
        p = np.asarray(parameters)
        if p.dtype == np.float32:
            p = p.astype(np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1)
        if p.size != self.get_Parameter_Num():
            raise Exception("Optimization_Interface::optimization_problem: Wrong number of parameters.")
        return p

    def Optimization_Problem(self, parameters):
        p = self._params(parameters)
        cost, _ = self.evaluator().cost_grad(dev.to_device_real(p), with_grad=False)
        self.num_iters += 1
        return float(cost.item())

    def Optimization_Problem_Combined(self, parameters):
        p = self._params(parameters)
        cost, grad = self.evaluator().cost_grad(dev.to_device_real(p), with_grad=True)
        self.num_iters += p.size + 1
        return float(cost.item()), grad.reshape(-1, 1).cpu().numpy()

    def Optimization_Problem_Grad(self, parameters):
        return self.Optimization_Problem_Combined(parameters)[1]

    def Optimization_Problem_Batch(self, parameters):
        p = np.asarray(parameters)
        if p.dtype == np.float32:
            p = p.astype(np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        if p.ndim != 2 or p.shape[1] != self.get_Parameter_Num():
            raise Exception("Optimization_Interface::optimization_problem: Wrong number of parameters.")
        def evaluate(rows):
            if rows.shape[0] == 0:
                return np.zeros(0), None
            cost, _ = self.evaluator().cost_grad(dev.to_device_real(np.ascontiguousarray(rows)), with_grad=False)
            return cost.cpu().numpy(), None

        if sharding.distributed() is not None:
            # one process per GPU: each rank evaluates its share, then all ranks gather (the
            # reference's MPI path, Optimization_Interface.cpp:962-1006)
            costs, _ = sharding.sharded_batch(evaluate, p)
        else:
            costs, _ = evaluate(p)
        return np.asarray(costs).reshape(-1, 1)

    def Optimization_Problem_Combined_Unitary(self, parameters):
        p = self._params(parameters)
        out = combined_unitary_device(self.circuit.native(), dev.to_device_real(p), dev.to_device_complex(self.Umtx),
                                      self.circuit._ws)
        host = out.cpu().numpy()
        return host[0], [host[k] for k in range(1, host.shape[0])]

    def get_Matrix(self, parameters):
        return self.circuit.get_Matrix(self._params(parameters))

    # ---- decomposition driver --------------------------------------------------------------
    def _fg(self, x):
        cost, grad = self.evaluator().cost_grad(dev.to_device_real(x), with_grad=True)
        return float(cost.item()), grad.reshape(-1).cpu().numpy()

    def _initial(self, P):
        if self.optimized_parameters.size == P:
            return self.optimized_parameters.copy()
        if self.initial_guess == "ZEROS":
            return np.zeros(P)
        x = self.rng.uniform(0.0, 2 * math.pi, P)
        return x / 100 if self.initial_guess == "CLOSE_TO_ZERO" else x

    def _bfgs_on_device(self, target, guess, tol, max_inner, loops):
        """iteration_loops BFGS runs of one outer iteration in one k_decompose launch (batch 1).
        Returns (minimum, evaluations, best point), or None (and switches to host-driven BFGS)
        when the gate structure does not fit one CTA."""
        dec = BatchedDecomposer(self.circuit, tolerance=tol, max_calls=max_inner, max_outer=1,
                                iteration_loops=loops, stop_at_tolerance=False, trace_offset=self.trace_offset,
                                cost_variant=self.cost_variant)
        try:
            xd, cd, ed = dec.run(target.unsqueeze(0), guess.reshape(1, -1), seed=int(self.rng.integers(1 << 62)))
        except _native.SQGError as e:
            if "unsupported" not in str(e):
                raise
            self._host_loops = True
            return None
        return float(cd.item()), int(ed.item()), xd.reshape(-1).cpu().numpy()

    def Start_Decomposition(self):
        """Decomposition_Base::solve_optimization_problem for the custom structure
        (Decomposition_Base.cpp:375-700 with optimization_block = all gates) with the
        BFGS restarts of optimization_engines/BFGS.cpp:121-150 or the ADAM engine of
        optimization_engines/ADAM.cpp:44-330.

        Every outer iteration runs on the device without a host round trip per evaluation:
        ADAM as one CUDA graph launch (batched.adam_decompose_graph), BFGS up to five qubits
        as one k_decompose launch of iteration_loops runs and above five qubits as one CUDA
        graph launch of those runs (batched.bfgs_decompose_graph).  The outer loop and
        its tolerance test stay on the host, so each launch is bounded by one outer
        iteration's evaluation budget."""
        P = self.get_Parameter_Num()
        if P == 0:
            self.optimized_parameters = np.zeros(0)
            self.decomposition_error = self.Optimization_Problem(np.zeros(0))
            return 0
        tol = float(self.config.get("optimization_tolerance", self.optimization_tolerance))
        max_inner = int(self.config.get("max_inner_iterations_bfgs" if self.optimizer == "BFGS" else
                                        "max_inner_iterations_adam", self.config.get("max_inner_iterations",
                                                                                     self.max_inner_iterations)))
        max_outer = int(self.config.get("max_outer_iterations", self.max_outer_iterations))
        loops = int(self.config.get("max_iteration_loops", 3 if self.qbit_num == 2 else 1))
        guess = self._initial(P)
        best_x, best_f = guess.copy(), math.inf
        target = self.evaluator().target
        for _outer in range(max_outer):
            if self.optimizer == "ADAM":
                # solve_layer_optimization_problem_ADAM (optimization_engines/ADAM.cpp:44-330); the
                # config lookups keep the reference's precedence (an "eta" or "adaptive_eta" key
                # decides over its "_adam" variant, ADAM.cpp:150-185)
                cfg = self.config
                eta = float(cfg["eta"]) if "eta" in cfg else 1e-3
                adaptive = bool(cfg["adaptive_eta"]) if "adaptive_eta" in cfg else True
                thr = int(cfg.get("randomization_threshold_adam", cfg.get("randomization_threshold", 2500000)))
                tol_a = float(cfg.get("optimization_tolerance_adam", tol))
                shift_max = int(cfg.get("random_shift_count_max", self.random_shift_count_max))
                seed = int(self.rng.integers(1 << 62))
                if self._host_loops:
                    x = guess.copy()
                    f, calls = adam_squander(self._fg, x, max_inner, tol_a, eta, adaptive, shift_max, thr,
                                             seed=seed, current_minimum=best_f)
                else:
                    xd, cd, ed, _sd = adam_decompose_graph(
                        self.circuit, target, guess, tol_a, max_inner, eta, adaptive, shift_max, thr, max_outer=1,
                        current_minimum=best_f, seed=seed, trace_offset=self.trace_offset,
                        cost_variant=self.cost_variant, workspace=self._loop_ws)
                    f, calls, x = float(cd.item()), int(ed.item()), xd.cpu().numpy()
                self.num_iters += calls
                if f < best_f:
                    best_f, best_x = f, x.copy()
            else:
                if self.qbit_num <= 5 and not self._host_loops:
                    run = self._bfgs_on_device(target, guess, tol, max_inner, loops)
                    if run is not None:
                        f, calls, x = run
                        self.num_iters += calls
                        if f < best_f:
                            best_f, best_x = f, x
                if self.qbit_num > 5 and not self._host_loops:
                    # the BFGS runs of one outer iteration as one CUDA graph launch
                    xd, cd, ed, _it = bfgs_decompose_graph(
                        self.circuit, target, guess, tol, max_inner, max_outer=1, iteration_loops=loops,
                        stop_at_tolerance=False, seed=int(self.rng.integers(1 << 62)),
                        trace_offset=self.trace_offset, cost_variant=self.cost_variant, workspace=self._loop_ws)
                    f, calls = float(cd.item()), int(ed.item())
                    self.num_iters += calls
                    if f < best_f:
                        best_f, best_x = f, xd.cpu().numpy()
                elif self.qbit_num > 5 or self._host_loops:
                    for _loop in range(loops):
                        f, calls = bfgs_powell(self._fg, guess, max_inner)
                        self.num_iters += calls
                        if f < best_f:
                            best_f, best_x = f, guess.copy()
                            guess += self.rng.uniform(0.0, 2 * math.pi, P) / 100
            guess = best_x.copy()
            if abs(best_f) < tol:
                break
        self.optimized_parameters = best_x
        self.decomposition_error = self.Optimization_Problem(best_x)
        return 0
