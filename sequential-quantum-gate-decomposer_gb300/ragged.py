"""Ragged batches: instances with different circuits and qubit counts evaluated in one
persistent launch (sqg_ragged_cost_grad), optionally replayed from a captured CUDA graph,
with a small autotuner choosing the column-tile width per qubit count.

SQUANDER's batched cost (Optimization_Interface::optimization_problem_batched,
src-cpp/decomposition/Optimization_Interface.cpp:940-1033) evaluates many parameter
vectors of one circuit; this is the device form for many circuits at once.
"""
import ctypes

import numpy as np

from . import _device as dev
from . import _native
from .circuit import Circuit


class RaggedBatch:
    """circuits: list of Circuit; targets: list of (2^n_i, cols_i) complex128 arrays
    (U^dagger of each instance)."""

    def __init__(self, circuits, targets, with_grad=True, tile_cols=None):
        dev.require_cuda()
        torch = dev.torch
        if len(circuits) != len(targets) or not circuits:
            raise ValueError("need one target per circuit")
        self.circuits = [c if isinstance(c, Circuit) else None for c in circuits]
        if any(c is None for c in self.circuits):
            raise TypeError("circuits must be Circuit objects")
        self.natives = [c.native() for c in self.circuits]
        self.count = len(circuits)
        self.with_grad = bool(with_grad)
        cols = np.array([int(np.asarray(t).shape[-1]) for t in targets], dtype=np.int32)
        handles = (ctypes.c_void_p * self.count)(*[n.handle for n in self.natives])
        tc = None
        if tile_cols is not None:
            tc = np.ascontiguousarray(np.asarray(tile_cols, dtype=np.int32))
        lib = _native.lib()
        h = ctypes.c_void_p()
        _native.check(lib.sqg_ragged_create(ctypes.cast(handles, ctypes.c_void_p), cols.ctypes.data, self.count,
                                            int(self.with_grad), tc.ctypes.data if tc is not None else None,
                                            ctypes.byref(h)), "sqg_ragged_create")
        self.handle = h.value
        self.theta_off = np.zeros(self.count + 1, dtype=np.int64)
        self.target_off = np.zeros(self.count + 1, dtype=np.int64)
        _native.check(lib.sqg_ragged_layout(self.handle, self.theta_off.ctypes.data, self.target_off.ctypes.data),
                      "sqg_ragged_layout")
        flat = torch.empty(int(self.target_off[-1]), dtype=torch.complex128, device="cuda")
        for i, t in enumerate(targets):
            flat[self.target_off[i]:self.target_off[i + 1]] = dev.to_device_complex(np.ascontiguousarray(t)).reshape(-1)
        self.targets = flat
        self.ws = torch.empty(max(lib.sqg_ragged_workspace_bytes(self.handle), 256), dtype=torch.uint8, device="cuda")
        self.param_total = int(self.theta_off[-1])
        self.cost = torch.empty(self.count, dtype=torch.float64, device="cuda")
        self.grad = torch.empty(max(self.param_total, 1), dtype=torch.float64, device="cuda")
        self._graph = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                _native.lib().sqg_ragged_destroy(h)
            except Exception:
                pass

    def pack(self, thetas):
        """List of per-instance parameter arrays -> flat CUDA tensor."""
        return dev.to_device_real(np.concatenate([np.asarray(t, dtype=np.float64).reshape(-1) for t in thetas]))

    def split(self, flat):
        return [flat[self.theta_off[i]:self.theta_off[i + 1]] for i in range(self.count)]

    def _launch(self, theta_flat, variant, with_grad, stream=None):
        dev.after_current(stream)
        _native.check(_native.lib().sqg_ragged_cost_grad(
            self.handle, dev.ptr(theta_flat) if self.param_total else None, dev.ptr(self.targets), int(variant),
            dev.ptr(self.cost), dev.ptr(self.grad) if with_grad else None, dev.ptr(self.ws), self.ws.numel(),
            dev.stream_ptr(stream)), "sqg_ragged_cost_grad")

    def cost_grad(self, theta_flat, variant=0, with_grad=None):
        """theta_flat: packed parameters (CUDA float64).  Returns (cost (count,), packed
        gradient or None); the result tensors are reused by the next call."""
        g = self.with_grad if with_grad is None else bool(with_grad)
        th = dev.to_device_real(theta_flat).reshape(-1)
        if th.numel() != self.param_total:
            raise ValueError("expected %d packed parameters, got %d" % (self.param_total, th.numel()))
        self._launch(th, variant, g)
        return self.cost, (self.grad[:self.param_total] if g else None)

    def capture(self, variant=0, with_grad=None):
        """Captures one evaluation into a CUDA graph; replay() re-runs it on the contents
        of self.theta_static (copy new parameters into it first)."""
        torch = dev.torch
        g = self.with_grad if with_grad is None else bool(with_grad)
        self.theta_static = torch.zeros(max(self.param_total, 1), dtype=torch.float64, device="cuda")
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._launch(self.theta_static, variant, g, stream=s)  # warm-up outside the graph
        torch.cuda.current_stream().wait_stream(s)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self._launch(self.theta_static, variant, g)
        self._graph = graph
        self._graph_grad = g
        return graph

    def replay(self):
        self._graph.replay()
        return self.cost, (self.grad[:self.param_total] if self._graph_grad else None)


def autotune_tile_cols(circuits, targets, with_grad=True, candidates=(1, 2, 4, 8, 16, 32, 64), reps=2, rng=None):
    """Per qubit count, times the ragged launch of that group's instances for every
    candidate tile width that fits and returns the per-instance choice."""
    torch = dev.torch
    rng = rng or np.random.default_rng(0)
    nq = np.array([c.qbit_num for c in circuits])
    cols = np.array([np.asarray(t).shape[-1] for t in targets])
    choice = np.zeros(len(circuits), dtype=np.int32)
    report = {}
    for n in sorted(set(nq.tolist())):
        idx = np.nonzero(nq == n)[0]
        sub_c = [circuits[i] for i in idx]
        sub_t = [targets[i] for i in idx]
        best = None
        for tc in candidates:
            if tc > cols[idx].max():
                break
            try:
                rb = RaggedBatch(sub_c, sub_t, with_grad=with_grad, tile_cols=[tc] * len(idx))
            except _native.SQGError:
                continue
            th = rb.pack([rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()) for c in sub_c])
            rb.cost_grad(th)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                rb.cost_grad(th)
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1) / reps
            report.setdefault(int(n), {})[int(tc)] = t
            if best is None or t < best[1]:
                best = (tc, t)
        choice[idx] = best[0] if best else 0
    return choice, report
