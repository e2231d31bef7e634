"""ORACLE — test infrastructure only (CPU checker, never part of the engine).

NumPy restatement of the learned initialiser's network arithmetic: BF16 operands
(round-to-nearest-even from FP32), accumulation in FP64 here (FP32 on the GPU), ReLU
hidden layers, the (cos, sin) angle head with its supervised loss and the chain rule of an
external dL/dtheta through atan2, and the backward pass.  Used by tests to check the GPU
forward/backward kernels.  The initialiser has no counterpart in the reference, so this
oracle is pinned by its own definition and by finite differences (tests/test_mlp_gpu.py).
"""
import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    bias = ((u >> 16) & 1) + 0x7FFF
    r = ((u + bias) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(a.shape)


def forward(x, W, b):
    """x (M, in) float32; W list of (out, in); b list of (out,).  Returns (out, cache)."""
    a = bf16(x)
    acts, pre = [a], []
    for i, (w, bb) in enumerate(zip(W, b)):
        z = (a.astype(np.float64) @ bf16(w).astype(np.float64).T + bb).astype(np.float32)
        pre.append(z)
        if i < len(W) - 1:
            a = bf16(np.maximum(z, 0.0))
            acts.append(a)
    return pre[-1], (acts, pre)


def backward(dout, W, cache):
    """dout (M, out) float32 -> (dW list, db list) with bf16 operands as on the GPU."""
    acts, pre = cache
    L = len(W)
    dW, db = [None] * L, [None] * L
    dz = dout.astype(np.float32)
    for i in range(L - 1, -1, -1):
        dzb = bf16(dz).astype(np.float64)
        dW[i] = (dzb.T @ acts[i].astype(np.float64)).astype(np.float32)
        db[i] = dz.astype(np.float64).sum(axis=0).astype(np.float32)
        if i > 0:
            da = (dzb @ bf16(W[i]).astype(np.float64)).astype(np.float32)
            dz = np.where(pre[i - 1] > 0, da, 0.0).astype(np.float32)
    return dW, db


def angle_head(out, P):
    c = out[:, 0::2].astype(np.float64)
    s = out[:, 1::2].astype(np.float64)
    return np.arctan2(s, c)


def supervised_loss_grad(out, theta_star, scale):
    c = out[:, 0::2].astype(np.float64)
    s = out[:, 1::2].astype(np.float64)
    dc = c - np.cos(theta_star)
    ds = s - np.sin(theta_star)
    g = np.empty_like(out, dtype=np.float64)
    g[:, 0::2] = 2 * dc * scale
    g[:, 1::2] = 2 * ds * scale
    return (dc * dc + ds * ds).mean(axis=1), g.astype(np.float32)


def chain_dtheta(out, dtheta, scale):
    c = out[:, 0::2].astype(np.float64)
    s = out[:, 1::2].astype(np.float64)
    r2 = c * c + s * s + 1e-12
    g = np.empty_like(out, dtype=np.float64)
    g[:, 0::2] = -s / r2 * dtheta * scale
    g[:, 1::2] = c / r2 * dtheta * scale
    return g.astype(np.float32)
