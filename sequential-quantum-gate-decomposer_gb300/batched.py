"""Batched decompositions on the device (one BFGS decomposition per CTA, one launch).

This is the throughput form of SQUANDER's ``N_Qubit_Decomposition_custom`` with the
BFGS optimizer (src-cpp/decomposition/N_Qubit_Decomposition_custom.cpp:116-190) or its
ADAM engine (src-cpp/optimization_engines/ADAM.cpp:44-330): every target of the batch is
decomposed with the same gate structure, each from its own start point, without a host
round trip per iteration.
"""
import numpy as np

from . import _device as dev
from . import _native
from .circuit import Circuit


class BatchedDecomposer:
    """Decomposes batches of targets (each given as U^dagger) with one gate structure."""

    def __init__(self, circuit, tolerance=1e-8, max_calls=10000, max_outer=4, iteration_loops=1,
                 stop_at_tolerance=True, trace_offset=0, cost_variant=0, optimizer="BFGS", eta=1e-3,
                 adaptive_eta=True, random_shift_count_max=100, randomization_threshold=2500000):
        """optimizer "BFGS": BFGS_Powell runs of at most max_calls evaluations each, restarted
        iteration_loops times per outer iteration.  optimizer "ADAM": one ADAM engine call of at
        most max_calls evaluations per outer iteration (SQUANDER sets max_outer_iterations 1,
        max_inner_iterations 100000 and random_shift_count_max 100 for ADAM)."""
        dev.require_cuda()
        self.optimizer = str(optimizer).upper()
        if self.optimizer not in ("BFGS", "ADAM"):
            raise ValueError("optimizer must be BFGS or ADAM")
        self.eta = float(eta)
        self.adaptive_eta = bool(adaptive_eta)
        self.random_shift_count_max = int(random_shift_count_max)
        self.randomization_threshold = int(randomization_threshold)
        if not isinstance(circuit, Circuit):
            raise TypeError("circuit must be a Circuit")
        self.circuit = circuit
        self.native = circuit.native()
        self.tolerance = float(tolerance)
        self.max_calls = int(max_calls)
        self.max_outer = int(max_outer)
        self.iteration_loops = int(iteration_loops)
        self.stop_at_tolerance = bool(stop_at_tolerance)
        self.trace_offset = int(trace_offset)
        self.cost_variant = int(cost_variant)
        self._ws = dev.Workspace()

    def run(self, targets_udag, x0, seed=0, stream=None):
        """targets_udag: (B, rows, cols) complex128; x0: (B, P) float64 (host or device).
        Returns CUDA tensors (x (B, P), cost (B,), calls (B,) int32); asynchronous.  The BFGS
        iteration counts (ADAM: randomisation counts) of the call are left in self.iters."""
        t = dev.to_device_complex(targets_udag)
        if t.dim() != 3 or t.shape[1] != (1 << self.native.qbit_num):
            raise ValueError("targets must be (B, 2**qbit_num, cols)")
        B, _, cols = t.shape
        x = dev.to_device_real(x0).clone()
        if x.shape != (B, self.native.param_num):
            raise ValueError("x0 must be (B, %d)" % self.native.param_num)
        cost = dev.torch.empty(B, dtype=dev.torch.float64, device="cuda")
        calls = dev.torch.empty(B, dtype=dev.torch.int32, device="cuda")
        self.iters = dev.torch.empty(B, dtype=dev.torch.int32, device="cuda")
        lib = _native.lib()
        dev.after_current(stream)
        if self.optimizer == "ADAM":
            _native.check(lib.sqg_decompose_batched_adam(
                self.native.handle, dev.ptr(t), cols, B, self.trace_offset, self.cost_variant, dev.ptr(x),
                dev.ptr(cost), dev.ptr(calls), dev.ptr(self.iters), self.tolerance, self.max_calls, self.eta,
                1 if self.adaptive_eta else 0, self.random_shift_count_max, self.randomization_threshold,
                self.max_outer, int(seed) & 0xFFFFFFFFFFFFFFFF, dev.stream_ptr(stream)), "sqg_decompose_batched_adam")
            self._keep = t
            return x, cost, calls
        ws = self._ws.get(lib.sqg_decompose_workspace_bytes(self.native.handle, B, cols))
        _native.check(lib.sqg_decompose_batched(
            self.native.handle, dev.ptr(t), cols, B, self.trace_offset, self.cost_variant, dev.ptr(x), dev.ptr(cost),
            dev.ptr(calls), dev.ptr(self.iters), self.tolerance, self.max_calls, self.max_outer, self.iteration_loops,
            1 if self.stop_at_tolerance else 0, int(seed) & 0xFFFFFFFFFFFFFFFF, dev.ptr(ws), ws.numel(),
            dev.stream_ptr(stream)), "sqg_decompose_batched")
        self._keep = t  # keep the target buffer alive until the caller synchronises
        return x, cost, calls


    def run_sharded(self, targets_udag, x0, seed=0, group=None):
        """run() across the ranks of a torch.distributed group (one process per GPU): each rank
        decomposes its contiguous share of the batch, with the restart draws every instance
        gets in the unsharded batch, and every rank receives the full results as host arrays
        (x (B, P), cost (B,), calls (B,)).  The only exchange is the final gather, as in the
        MPI_Allgather of optimization_problem_batched (Optimization_Interface.cpp:962-1006)."""
        from . import sharding

        T = np.asarray(targets_udag.cpu() if hasattr(targets_udag, "cpu") else targets_udag)
        X = np.asarray(x0.cpu() if hasattr(x0, "cpu") else x0, dtype=np.float64)

        def local(t, x, s):
            if t.shape[0] == 0:
                return np.zeros((0, X.shape[1])), np.zeros(0), np.zeros(0, dtype=np.int64)
            xr, cr, nr = self.run(np.ascontiguousarray(t), np.ascontiguousarray(x), seed=s)
            return xr.cpu().numpy(), cr.cpu().numpy(), nr.cpu().numpy().astype(np.int64)

        return sharding.sharded_decompose(local, T, X, seed=seed, group=group)


def adam_decompose_graph(circuit, target_udag, x0, tolerance=1e-8, max_iters=100000, eta=1e-3, adaptive_eta=True,
                         random_shift_count_max=100, randomization_threshold=2500000, max_outer=1,
                         current_minimum=None, seed=0, trace_offset=0, cost_variant=0, workspace=None, stream=None):
    """One decomposition of target_udag ((2**n, cols) complex128, U^dagger) with SQUANDER's ADAM
    engine for any register the gradient supports, run on the device as a single CUDA graph
    launch (sqg_decompose_adam_loop: a conditional while-node over [cost + gradient kernels,
    one engine pass]), with no host round trip between evaluations.  Starts at x0 (P,) with
    the running minimum current_minimum (None: a fresh decomposition).  Returns CUDA tensors
    (x (P,) best point, cost (1,), evals (1,) int32, shifts (1,) int32); asynchronous on stream."""
    dev.require_cuda()
    native = circuit.native() if isinstance(circuit, Circuit) else circuit
    t = dev.to_device_complex(target_udag)
    if t.dim() != 2 or t.shape[0] != (1 << native.qbit_num):
        raise ValueError("target must be (2**qbit_num, cols)")
    x = dev.to_device_real(x0).reshape(-1).clone()
    if x.numel() != native.param_num:
        raise ValueError("x0 must hold %d parameters" % native.param_num)
    cost = dev.torch.empty(1, dtype=dev.torch.float64, device="cuda")
    evals = dev.torch.empty(1, dtype=dev.torch.int32, device="cuda")
    shifts = dev.torch.empty(1, dtype=dev.torch.int32, device="cuda")
    lib = _native.lib()
    cols = int(t.shape[1])
    ws = (workspace or dev.Workspace()).get(lib.sqg_adam_loop_workspace_bytes(native.handle, cols))
    dev.after_current(stream)
    cur = np.finfo(np.float64).max if current_minimum is None or not np.isfinite(current_minimum) else current_minimum
    _native.check(lib.sqg_decompose_adam_loop(
        native.handle, dev.ptr(t), cols, int(trace_offset), int(cost_variant), dev.ptr(x), dev.ptr(cost),
        dev.ptr(evals), dev.ptr(shifts), float(tolerance), int(max_iters), float(eta), 1 if adaptive_eta else 0,
        int(random_shift_count_max), int(randomization_threshold), int(max_outer), float(cur),
        int(seed) & 0xFFFFFFFFFFFFFFFF, dev.ptr(ws), ws.numel(), dev.stream_ptr(stream)), "sqg_decompose_adam_loop")
    if stream is not None:  # the scratch and the target stay allocated until that stream is past the graph
        ws.record_stream(stream)
        t.record_stream(stream)
    return x, cost, evals, shifts


def bfgs_decompose_graph(circuit, target_udag, x0, tolerance=1e-8, max_calls=10000, max_outer=4, iteration_loops=1,
                         stop_at_tolerance=True, seed=0, trace_offset=0, cost_variant=0, workspace=None, stream=None):
    """One BFGS decomposition (the driver of BatchedDecomposer for a single target) for any
    register the gradient supports, run on the device as a single CUDA graph launch
    (sqg_decompose_bfgs_loop: a conditional while-node over [cost + gradient kernels, BFGS
    step]).  Returns CUDA tensors (x (P,) best point, cost (1,), calls (1,) int32, BFGS
    iterations (1,) int32); asynchronous on stream."""
    dev.require_cuda()
    native = circuit.native() if isinstance(circuit, Circuit) else circuit
    t = dev.to_device_complex(target_udag)
    if t.dim() != 2 or t.shape[0] != (1 << native.qbit_num):
        raise ValueError("target must be (2**qbit_num, cols)")
    x = dev.to_device_real(x0).reshape(-1).clone()
    if x.numel() != native.param_num:
        raise ValueError("x0 must hold %d parameters" % native.param_num)
    cost = dev.torch.empty(1, dtype=dev.torch.float64, device="cuda")
    calls = dev.torch.empty(1, dtype=dev.torch.int32, device="cuda")
    iters = dev.torch.empty(1, dtype=dev.torch.int32, device="cuda")
    lib = _native.lib()
    cols = int(t.shape[1])
    ws = (workspace or dev.Workspace()).get(lib.sqg_bfgs_loop_workspace_bytes(native.handle, cols))
    dev.after_current(stream)
    _native.check(lib.sqg_decompose_bfgs_loop(
        native.handle, dev.ptr(t), cols, int(trace_offset), int(cost_variant), dev.ptr(x), dev.ptr(cost),
        dev.ptr(calls), dev.ptr(iters), float(tolerance), int(max_calls), int(max_outer), int(iteration_loops),
        1 if stop_at_tolerance else 0, int(seed) & 0xFFFFFFFFFFFFFFFF, dev.ptr(ws), ws.numel(),
        dev.stream_ptr(stream)), "sqg_decompose_bfgs_loop")
    if stream is not None:
        ws.record_stream(stream)
        t.record_stream(stream)
    return x, cost, calls, iters


def random_start(B, P, rng):
    """RANDOM initial guess of Decomposition_Base (U[0, 2 pi), Decomposition_Base.cpp:415-436)."""
    return rng.uniform(0.0, 2 * np.pi, (B, P))
