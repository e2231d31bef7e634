"""Learned initialiser: an MLP mapping a small target U^dagger to starting angles of a
fixed ansatz, trained on the GPU with the engine's own BF16/FP32-accumulate kernels
(csrc/mlp.cu) on decompositions produced by the batched decomposition kernel.

The network only proposes start points.  Every result still comes from the FP64
decomposition kernels and counts only if its FP64 cost drops below the tolerance; the
plain random start of SQUANDER (U[0, 2 pi), Decomposition_Base.cpp:415-436) remains the
fallback.  No counterpart exists in the reference.

Architecture: 2*rows*cols real inputs (Re/Im of U^dagger) -> 4 hidden layers of 1024
(ReLU) -> 2*P outputs read as (cos, sin) pairs, theta_k = atan2(s_k, c_k).
Training: supervised on solutions reached from one fixed start point (a consistent
branch of the many-valued map U -> theta), then optionally fine-tuned on the FP64
decomposition cost itself (the adjoint gradient chained through atan2 and the MLP).
"""
import math

import numpy as np

from . import _device as dev
from . import _native


def _lib():
    return _native.lib()


def _declare():
    import ctypes

    lib = _lib()
    if getattr(lib, "_mlp_declared", False):
        return lib
    vp, ci, cll, cf = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
    lib.sqg_mlp_gemm_bf16.argtypes = [ci, ci, ci, vp, ci, ci, vp, ci, ci, vp, ci, vp, ci, vp, ci, vp]
    lib.sqg_mlp_to_bf16.argtypes = [vp, vp, cll, vp]
    lib.sqg_mlp_relu_backward.argtypes = [vp, vp, vp, cll, vp]
    lib.sqg_mlp_col_sum.argtypes = [vp, ci, ci, vp, vp]
    lib.sqg_mlp_adam.argtypes = [vp, vp, vp, vp, vp, cll, cf, cf, cf, cf, ci, cf, vp]
    lib.sqg_mlp_angle_head.argtypes = [vp, ci, ci, vp, vp, ci, cf, vp, vp, vp]
    lib.sqg_mlp_features.argtypes = [vp, cll, vp, vp]
    lib.sqg_mlp_gemm_tc.argtypes = [ci, ci, ci, vp, ci, vp, ci, vp, ci, vp, ci, vp, vp, vp]
    lib.sqg_mlp_transpose_bf16.argtypes = [vp, ci, ci, ci, vp, ci, vp]
    lib._mlp_declared = True
    return lib


def _p(t):
    return None if t is None else int(t.data_ptr())


def _pad64(v):
    return (int(v) + 63) // 64 * 64


class MLP:
    """Fully connected ReLU network with fp32 master weights and bf16 working copies.

    use_tc selects the layer GEMMs: True = tcgen05 tensor cores fed by TMA
    (csrc/gemm_tc.cu, both operands K-major, so the backward pass works on transposed
    copies), False = the mma.sync kernel (csrc/mlp.cu).  The output width is padded to a
    multiple of 64 with zero rows (their gradients are zero, so they stay zero)."""

    def __init__(self, sizes, seed=0, use_tc=False):
        dev.require_cuda()
        torch = dev.torch
        self.out_dim = int(sizes[-1])
        sizes = list(sizes[:-1]) + [_pad64(sizes[-1])]
        self.sizes = list(sizes)
        self.use_tc = bool(use_tc)
        self.err = torch.zeros(1, dtype=torch.int32, device="cuda")
        g = torch.Generator(device="cpu").manual_seed(int(seed))
        self.W, self.b, self.Wb = [], [], []
        for i in range(len(sizes) - 1):
            fan_in, fan_out = sizes[i], sizes[i + 1]
            std = math.sqrt(2.0 / fan_in) if i < len(sizes) - 2 else math.sqrt(1.0 / fan_in)
            w = torch.randn((fan_out, fan_in), generator=g, dtype=torch.float32) * std
            if i == len(sizes) - 2:
                w[self.out_dim:] = 0.0
            w = w.cuda()
            self.W.append(w)
            self.b.append(torch.zeros(fan_out, dtype=torch.float32, device="cuda"))
            self.Wb.append(w.to(torch.bfloat16))
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step = 0

    def state_dict(self):
        return {"sizes": self.sizes, "W": [w.cpu() for w in self.W], "b": [b.cpu() for b in self.b]}

    def load_state_dict(self, d):
        torch = dev.torch
        self.W = [w.cuda() for w in d["W"]]
        self.b = [b.cuda() for b in d["b"]]
        self.Wb = [w.to(torch.bfloat16) for w in self.W]

    def _tc(self, A, B, M, N, K, C=None, Cb=None, bias=None, relu=False):
        """C = A B^T on the tensor cores; A (M, K), B (N, K), both bf16 row-major."""
        lib = _declare()
        _native.check(lib.sqg_mlp_gemm_tc(M, N, K, _p(A), K, _p(B), K, _p(C), N, _p(bias), int(relu), _p(Cb),
                                          _p(self.err), dev.stream_ptr()), "sqg_mlp_gemm_tc")

    def _t(self, X):
        """bf16 transpose of a 2-D CUDA tensor."""
        lib = _declare()
        r, c = X.shape
        out = dev.torch.empty((c, r), dtype=dev.torch.bfloat16, device="cuda")
        _native.check(lib.sqg_mlp_transpose_bf16(_p(X), r, c, c, _p(out), r, dev.stream_ptr()), "sqg_mlp_transpose_bf16")
        return out

    def check_errors(self):
        """Raises if a tensor-core GEMM reported a timed-out wait."""
        if int(self.err.item()) != 0:
            raise _native.SQGError("tensor-core GEMM reported error code %d" % int(self.err.item()))

    def _gemm(self, A, transA, B, transB, M, N, K, C=None, Cb=None, bias=None, relu=False, accumulate=False,
              lda=None, ldb=None):
        lib = _declare()
        _native.check(lib.sqg_mlp_gemm_bf16(M, N, K, _p(A), lda, int(transA), _p(B), ldb, int(transB), _p(C), N,
                                            _p(bias), int(relu), _p(Cb), int(accumulate), dev.stream_ptr()),
                      "sqg_mlp_gemm_bf16")

    def forward(self, xb, keep=True):
        """xb: (M, in) bf16 CUDA tensor.  Returns (out fp32 (M, out), cache)."""
        torch = dev.torch
        M = xb.shape[0]
        acts, pre = [xb], []
        a = xb
        L = len(self.W)
        for i in range(L):
            fan_out, fan_in = self.W[i].shape
            last = i == L - 1
            # inference needs the fp32 pre-activations of the output layer only
            z = torch.empty((M, fan_out), dtype=torch.float32, device="cuda") if (keep or last) else None
            ab = None if last else torch.empty((M, fan_out), dtype=torch.bfloat16, device="cuda")
            # Z = A W^T + b; the next layer's input is ReLU(Z) in bf16
            if self.use_tc:
                if z is not None:
                    self._tc(a, self.Wb[i], M, fan_out, fan_in, C=z, bias=self.b[i])
                if not last:
                    self._tc(a, self.Wb[i], M, fan_out, fan_in, Cb=ab, bias=self.b[i], relu=True)
            else:
                if z is not None:
                    self._gemm(a, False, self.Wb[i], True, M, fan_out, fan_in, C=z, bias=self.b[i], lda=fan_in,
                               ldb=fan_in)
                if not last:
                    self._gemm(a, False, self.Wb[i], True, M, fan_out, fan_in, Cb=ab, bias=self.b[i], relu=True,
                               lda=fan_in, ldb=fan_in)
            if not last:
                acts.append(ab)
                a = ab
            pre.append(z)
        return pre[-1], (acts, pre) if keep else None

    def backward(self, dout, cache):
        """dout: (M, out) fp32 gradient of the loss w.r.t. the network output.
        Returns (dW list, db list)."""
        torch = dev.torch
        lib = _declare()
        acts, pre = cache
        M = dout.shape[0]
        L = len(self.W)
        dW = [None] * L
        db = [None] * L
        dz = dout.contiguous()
        dzb = torch.empty(dz.shape, dtype=torch.bfloat16, device="cuda")
        _native.check(lib.sqg_mlp_to_bf16(_p(dz), _p(dzb), dz.numel(), dev.stream_ptr()), "sqg_mlp_to_bf16")
        for i in range(L - 1, -1, -1):
            fan_out, fan_in = self.W[i].shape
            a_prev = acts[i]
            gw = torch.empty((fan_out, fan_in), dtype=torch.float32, device="cuda")
            # dW = dZ^T A_prev
            if self.use_tc:
                self._tc(self._t(dzb), self._t(a_prev), fan_out, fan_in, M, C=gw)
            else:
                self._gemm(dzb, True, a_prev, False, fan_out, fan_in, M, C=gw, lda=fan_out, ldb=fan_in)
            gb = torch.empty(fan_out, dtype=torch.float32, device="cuda")
            _native.check(lib.sqg_mlp_col_sum(_p(dz), M, fan_out, _p(gb), dev.stream_ptr()), "sqg_mlp_col_sum")
            dW[i], db[i] = gw, gb
            if i > 0:
                # dA_prev = dZ W, then through the ReLU of layer i-1
                da = torch.empty((M, fan_in), dtype=torch.float32, device="cuda")
                if self.use_tc:
                    self._tc(dzb, self._t(self.Wb[i]), M, fan_in, fan_out, C=da)
                else:
                    self._gemm(dzb, False, self.Wb[i], False, M, fan_in, fan_out, C=da, lda=fan_out, ldb=fan_in)
                dzb = torch.empty((M, fan_in), dtype=torch.bfloat16, device="cuda")
                _native.check(lib.sqg_mlp_relu_backward(_p(da), _p(pre[i - 1]), _p(dzb), da.numel(),
                                                        dev.stream_ptr()), "sqg_mlp_relu_backward")
                dz = da
        return dW, db

    def adam(self, dW, db, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        lib = _declare()
        self.step += 1
        for i in range(len(self.W)):
            _native.check(lib.sqg_mlp_adam(_p(self.W[i]), _p(dW[i]), _p(self.mW[i]), _p(self.vW[i]), _p(self.Wb[i]),
                                           self.W[i].numel(), lr, beta1, beta2, eps, self.step, weight_decay,
                                           dev.stream_ptr()), "sqg_mlp_adam")
            _native.check(lib.sqg_mlp_adam(_p(self.b[i]), _p(db[i]), _p(self.mb[i]), _p(self.vb[i]), None,
                                           self.b[i].numel(), lr, beta1, beta2, eps, self.step, 0.0,
                                           dev.stream_ptr()), "sqg_mlp_adam")


def features(targets_dev):
    """(B, rows, cols) complex128 CUDA tensor -> (B, 2*rows*cols) bf16 network input."""
    torch = dev.torch
    lib = _declare()
    B = targets_dev.shape[0]
    n = targets_dev[0].numel()
    x = torch.empty((B, 2 * n), dtype=torch.bfloat16, device="cuda")
    _native.check(lib.sqg_mlp_features(_p(targets_dev), B * n, _p(x), dev.stream_ptr()), "sqg_mlp_features")
    return x


def angle_head(out, P, mode=0, target=None, dtheta=None, scale=1.0):
    """out: (M, W >= 2P) network output (padding columns ignored).  Returns
    (theta (M, P) float64, out_grad (M, W) with zero padding, or None, loss_rows or None)."""
    torch = dev.torch
    lib = _declare()
    M = out.shape[0]
    if out.shape[1] != 2 * P:
        res = angle_head(out[:, :2 * P].contiguous(), P, mode, target, dtheta, scale)
        if res[1] is None:
            return res
        og = torch.zeros_like(out)
        og[:, :2 * P] = res[1]
        return res[0], og, res[2]
    theta = torch.empty((M, P), dtype=torch.float64, device="cuda")
    og = torch.empty_like(out) if mode else None
    lr = torch.empty(M, dtype=torch.float32, device="cuda") if mode == 1 else None
    aux = target if mode == 1 else dtheta
    _native.check(lib.sqg_mlp_angle_head(_p(out), M, P, _p(theta), _p(aux), mode, scale, _p(og), _p(lr),
                                         dev.stream_ptr()), "sqg_mlp_angle_head")
    return theta, og, lr


class LearnedInitializer:
    """MLP initialiser for one ansatz (a Circuit with P parameters) on rows x cols targets."""

    def __init__(self, circuit, rows, cols, hidden=(1024, 1024, 1024, 1024), seed=0, use_tc=True):
        self.circuit = circuit
        self.P = circuit.get_Parameter_Num()
        self.in_dim = 2 * rows * cols
        self.mlp = MLP([self.in_dim] + list(hidden) + [2 * self.P], seed=seed, use_tc=use_tc)
        self.history = []

    def predict(self, targets_dev):
        out, _ = self.mlp.forward(features(targets_dev), keep=False)
        theta, _, _ = angle_head(out, self.P)
        return theta

    def train_supervised(self, targets_dev, theta_star, epochs=10, batch=512, lr=1e-3, seed=0, log=None):
        """Regress (cos, sin) of theta_star (S, P) from the targets (S, rows, cols)."""
        torch = dev.torch
        S = targets_dev.shape[0]
        x_all = features(targets_dev)
        th = dev.to_device_real(theta_star)
        gen = torch.Generator(device="cpu").manual_seed(int(seed))
        for ep in range(epochs):
            perm = torch.randperm(S, generator=gen).cuda()
            tot, nb = 0.0, 0
            for s0 in range(0, S - batch + 1, batch):
                idx = perm[s0:s0 + batch]
                xb = x_all.index_select(0, idx)
                tb = th.index_select(0, idx).contiguous()
                out, cache = self.mlp.forward(xb)
                _, og, loss_rows = angle_head(out, self.P, mode=1, target=tb, scale=1.0 / (batch * self.P))
                dW, db = self.mlp.backward(og, cache)
                self.mlp.adam(dW, db, lr * (0.5 * (1 + math.cos(math.pi * ep / max(1, epochs)))))
                tot += float(loss_rows.mean())
                nb += 1
            self.history.append(("supervised", ep, tot / max(nb, 1)))
            if log:
                log("epoch %d supervised loss %.5f" % (ep, tot / max(nb, 1)))

    def train_cost(self, evaluator_factory, targets_dev, steps=200, batch=512, lr=2e-4, seed=0, log=None):
        """Fine-tune on the FP64 decomposition cost: dL/dtheta from the adjoint kernel is
        chained through the angle head and the MLP.  evaluator_factory(targets) returns a
        CostEvaluator with one target per instance."""
        torch = dev.torch
        S = targets_dev.shape[0]
        x_all = features(targets_dev)
        gen = torch.Generator(device="cpu").manual_seed(int(seed))
        for st in range(steps):
            idx = torch.randint(0, S, (batch,), generator=gen).cuda()
            xb = x_all.index_select(0, idx)
            tb = targets_dev.index_select(0, idx).contiguous()
            out, cache = self.mlp.forward(xb)
            theta, _, _ = angle_head(out, self.P)
            ev = evaluator_factory(tb)
            cost, grad = ev.cost_grad(theta)
            _, og, _ = angle_head(out, self.P, mode=2, dtheta=grad.contiguous(), scale=1.0 / batch)
            dW, db = self.mlp.backward(og, cache)
            self.mlp.adam(dW, db, lr)
            if log and st % 20 == 0:
                log("step %d mean cost %.4f" % (st, float(cost.mean())))
            self.history.append(("cost", st, float(cost.mean())))


def generate_solutions(decomposer, targets_dev, start, seed=0):
    """Decompose every target from the same start point `start` (P,); returns
    (solved mask (S,), theta (S, P)) as CUDA tensors."""
    torch = dev.torch
    S = targets_dev.shape[0]
    x0 = dev.to_device_real(np.asarray(start, dtype=np.float64)).reshape(1, -1).expand(S, -1).contiguous()
    x, cost, calls = decomposer.run(targets_dev, x0, seed=seed)
    return cost < decomposer.tolerance, x


def train_initializer(circuit, n_samples=131072, epochs=8, cost_steps=0, batch=512, seed=0, start=0.3,
                      max_calls=1000, use_tc=True, log=None):
    """End-to-end training of a LearnedInitializer for 3-qubit targets on the GPU.

    1. synthetic targets (half Haar-random, half random CNOT+U3 circuits with 1..14 blocks);
    2. the batched decomposition kernel solves them from one fixed start point, which picks
       a consistent branch of the many-valued map target -> angles;
    3. supervised regression of the (cos, sin) of the solved angles;
    4. fine-tuning on the FP64 decomposition cost itself (adjoint gradient through atan2).
    Returns (initializer, stats)."""
    import time

    from .batched import BatchedDecomposer
    from .evaluator import CostEvaluator
    from .workloads import haar_unitaries, random_circuit_targets

    torch = dev.torch
    rng = np.random.default_rng(seed)
    n = circuit.qbit_num
    N = 1 << n
    t0 = time.perf_counter()
    U = np.concatenate([haar_unitaries(n_samples // 2, N, rng), random_circuit_targets(n_samples - n_samples // 2, n, rng)])
    T = torch.from_numpy(np.ascontiguousarray(np.conj(np.transpose(U, (0, 2, 1))))).cuda()
    dec = BatchedDecomposer(circuit, tolerance=1e-8, max_calls=max_calls, max_outer=1)
    P = circuit.get_Parameter_Num()
    solved, X = generate_solutions(dec, T, np.full(P, float(start)), seed=seed)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    init = LearnedInitializer(circuit, N, N, seed=seed, use_tc=use_tc)
    t1 = time.perf_counter()
    init.train_supervised(T[solved], X[solved], epochs=epochs, batch=batch, lr=1e-3, seed=seed, log=log)
    if cost_steps:
        init.train_cost(lambda tb: CostEvaluator(circuit, tb), T, steps=cost_steps, batch=batch, lr=2e-4, seed=seed,
                        log=log)
    torch.cuda.synchronize()
    init.mlp.check_errors()
    stats = {"samples": int(n_samples), "solved_for_training": int(solved.sum()), "generation_s": t_gen,
             "training_s": time.perf_counter() - t1, "epochs": epochs, "cost_steps": cost_steps}
    return init, stats
