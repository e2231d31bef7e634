"""Batched cost / adjoint-gradient evaluation on CUDA tensors, and its autograd face.

``CostEvaluator`` is the device-level form of SQUANDER's
``Optimization_Interface::optimization_problem{,_batched,_combined}``
(src-cpp/decomposition/Optimization_Interface.cpp:634-668, 940-1033, 1145-1485):
B parameter vectors are evaluated against one shared target U^dagger or one target per
instance in a single launch of the column-tile kernels (sqg_cost_grad).
"""
from . import _device as dev
from . import _native
from .circuit import Circuit, NativeCircuit

FROBENIUS_NORM, HILBERT_SCHMIDT_TEST, INFIDELITY = 0, 3, 9
SUPPORTED_VARIANTS = (FROBENIUS_NORM, HILBERT_SCHMIDT_TEST, INFIDELITY)


class CostEvaluator:
    """Cost and gradient of a circuit against a target held on the GPU.

    target: (rows, cols) shared by every instance, or (B, rows, cols) one per instance.
    """

    def __init__(self, circuit, target, trace_offset=0, cost_variant=FROBENIUS_NORM):
        dev.require_cuda()
        self.native = circuit.native() if isinstance(circuit, Circuit) else circuit
        if not isinstance(self.native, NativeCircuit):
            raise TypeError("circuit must be a Circuit or NativeCircuit")
        if cost_variant not in SUPPORTED_VARIANTS:
            raise ValueError("cost function variant %r is not implemented by the GB300 engine "
                             "(supported: FROBENIUS_NORM=0, HILBERT_SCHMIDT_TEST=3, INFIDELITY=9)" % (cost_variant,))
        self.variant = int(cost_variant)
        self.trace_offset = int(trace_offset)
        self.set_target(target)
        self._ws = dev.Workspace()

    def set_target(self, target):
        t = dev.to_device_complex(target)
        if t.dim() not in (2, 3):
            raise ValueError("target must be (rows, cols) or (B, rows, cols)")
        if t.shape[-2] != (1 << self.native.qbit_num):
            raise ValueError("target rows must equal 2**qbit_num")
        self.target = t
        self.cols = int(t.shape[-1])
        self.per_instance = t.dim() == 3

    @property
    def param_num(self):
        return self.native.param_num

    def workspace_bytes(self, batch, with_grad, checkpoint_interval=0):
        lib = _native.lib()
        if with_grad and checkpoint_interval > 0:
            return lib.sqg_cost_grad_checkpoint_workspace_bytes(self.native.handle, batch, self.cols,
                                                                checkpoint_interval)
        return lib.sqg_cost_grad_workspace_bytes(self.native.handle, batch, self.cols, 1 if with_grad else 0)

    def cost_grad(self, theta, with_grad=True, checkpoint_interval=0, stream=None, out=None):
        """theta: (B, P) or (P,) float64 CUDA tensor.  Returns (cost (B,), grad (B, P) or None)."""
        th = theta if theta.dim() == 2 else theta.reshape(1, -1)
        if th.dtype != dev.torch.float64 or not th.is_cuda:
            th = th.to(device="cuda", dtype=dev.torch.float64)
        th = th.contiguous()
        B, P = th.shape
        if P != self.param_num:
            raise ValueError("Optimization_Interface::optimization_problem: Wrong number of parameters. "
                             "Expected %d, got %d" % (self.param_num, P))
        if self.per_instance and self.target.shape[0] != B:
            raise ValueError("per-instance targets (%d) do not match the batch (%d)" % (self.target.shape[0], B))
        if out is None:
            cost = dev.torch.empty(B, dtype=dev.torch.float64, device="cuda")
            grad = dev.torch.empty((B, P), dtype=dev.torch.float64, device="cuda") if with_grad else None
        else:
            cost, grad = out
        ws_bytes = self.workspace_bytes(B, with_grad and P > 0, checkpoint_interval)
        ws = self._ws.get(ws_bytes)
        tstride = self.target.shape[-2] * self.target.shape[-1] if self.per_instance else 0
        dev.after_current(stream)
        _native.check(_native.lib().sqg_cost_grad(
            self.native.handle, dev.ptr(th) if P else None, B, dev.ptr(self.target), self.cols, tstride,
            self.trace_offset, self.variant, dev.ptr(cost), dev.ptr(grad) if (with_grad and P) else None,
            int(checkpoint_interval) if with_grad else 0, dev.ptr(ws), ws.numel(), dev.stream_ptr(stream)),
            "sqg_cost_grad")
        if with_grad and P == 0:
            grad = dev.torch.zeros((B, 0), dtype=dev.torch.float64, device="cuda")
        return cost, grad


def _make_autograd():
    torch = dev.torch

    class CircuitCost(torch.autograd.Function):
        """Differentiable cost C(theta) -> f(theta) backed by the adjoint kernel.

        forward returns the (B,) costs; backward scales the adjoint gradient computed in
        the same launch by the incoming gradient.
        """

        @staticmethod
        def forward(ctx, theta, evaluator, checkpoint_interval=0):
            need = theta.requires_grad
            cost, grad = evaluator.cost_grad(theta.detach(), with_grad=need, checkpoint_interval=checkpoint_interval)
            if need:
                ctx.save_for_backward(grad)
            ctx.squeeze = theta.dim() == 1
            return cost[0] if ctx.squeeze else cost

        @staticmethod
        def backward(ctx, gcost):
            (grad,) = ctx.saved_tensors
            if ctx.squeeze:
                return gcost * grad[0], None, None
            return gcost.reshape(-1, 1) * grad, None, None

    return CircuitCost


CircuitCost = _make_autograd() if dev.torch is not None else None


def circuit_cost(theta, evaluator, checkpoint_interval=0):
    """Differentiable cost of ``theta`` ((P,) or (B, P) CUDA float64 tensor)."""
    return CircuitCost.apply(theta, evaluator, checkpoint_interval)
