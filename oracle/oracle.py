"""ORACLE — test infrastructure only (CPU checker, never part of the engine).

ctypes front end of ``sqg_oracle.c``, the plain-C restatement of SQUANDER's
decomposition hot path (gate application, cost, gradient, batched cost and the
BFGS decomposition driver).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import this module.

Gate records are ``(type, target, control, param_start)`` with SQUANDER's gate-type
ids (src-cpp/gates/include/Gate.h:37-50).  Matrices are complex128, C-contiguous,
``rows = 2**qbit_num``; the decomposer is handed U^dagger as in SQUANDER.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libsqg_oracle.so")
SRC = os.path.join(HERE, "sqg_oracle.c")

CZ, CNOT, U3, RY, RX, RZ, CRY = 4, 5, 7, 8, 9, 10, 14
PARAM_NUM = {CZ: 0, CNOT: 0, U3: 3, RY: 1, RX: 1, RZ: 1, CRY: 1}

FROBENIUS_NORM, HILBERT_SCHMIDT_TEST, INFIDELITY = 0, 3, 9


def build(force=False):
    """Compile the oracle with gcc into oracle/_build (portable C, no -march flags)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-Wall", "-o", tmp, SRC, "-lm", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_long)
        i = ctypes.c_int
        _lib.sqgo_apply_to.argtypes = [i, ip, i, dp, i, dp, i, i, i]
        _lib.sqgo_apply_from_right.argtypes = [i, ip, i, dp, i, dp, i, i, i]
        _lib.sqgo_apply_derivate_to.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp]
        _lib.sqgo_cost_of_matrix.argtypes = [dp, i, i, i, i]
        _lib.sqgo_cost_of_matrix.restype = ctypes.c_double
        _lib.sqgo_cost.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp]
        _lib.sqgo_cost_grad.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp, dp]
        _lib.sqgo_batch.argtypes = [i, ip, i, dp, i, i, dp, i, i, i, i, dp, dp, i]
        _lib.sqgo_batch2.argtypes = [i, ip, i, dp, i, i, dp, i, i, i, i, dp, dp, i, i]
        _lib.sqgo_cost_grad_sweep.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp, dp]
        _lib.sqgo_decompose.argtypes = [i, ip, i, i, dp, i, i, i, dp, ctypes.c_double, ctypes.c_long, i, i,
                                        ctypes.c_uint64, dp, lp]
        _lib.sqgo_decompose_batch.argtypes = [i, ip, i, i, i, dp, i, i, i, dp, ctypes.c_double, ctypes.c_long, i,
                                              i, ctypes.c_uint64, dp, lp, i]
        _lib.sqgo_adam_batch.argtypes = [i, ip, i, i, i, dp, i, i, i, dp, ctypes.c_double, ctypes.c_long,
                                         ctypes.c_double, i, i, ctypes.c_long, ctypes.c_uint64, dp, lp, lp, i]
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _gates(gates):
    g = np.ascontiguousarray(np.asarray(gates, dtype=np.int32).reshape(-1, 4))
    return g, g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), g.shape[0]


def param_count(gates):
    return int(sum(PARAM_NUM[int(t)] for t, _, _, _ in np.asarray(gates).reshape(-1, 4)))


def _check(rc, what):
    if rc != 0:
        raise ValueError("oracle %s failed with status %d" % (what, rc))


def apply_to(qbit_num, gates, params, mtx):
    """In-place left application C(params) @ mtx (Gates_block::apply_to)."""
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    assert mtx.dtype == np.complex128 and mtx.flags.c_contiguous
    rows, cols = mtx.shape
    _check(lib().sqgo_apply_to(qbit_num, gp, L, _dp(p), p.size, _dp(mtx.view(np.float64)), rows, cols, cols), "apply_to")
    return mtx


def apply_from_right(qbit_num, gates, params, mtx):
    """In-place right application mtx @ C(params) (Gates_block::apply_from_right)."""
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    rows, cols = mtx.shape
    _check(lib().sqgo_apply_from_right(qbit_num, gp, L, _dp(p), p.size, _dp(mtx.view(np.float64)), rows, cols, cols),
           "apply_from_right")
    return mtx


def get_matrix(qbit_num, gates, params):
    m = np.eye(1 << qbit_num, dtype=np.complex128)
    return apply_to(qbit_num, gates, params, m)


def apply_derivate_to(qbit_num, gates, params, mtx):
    """List of P matrices d(C mtx)/d params[k] (Gates_block::apply_derivate_to)."""
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    m = np.ascontiguousarray(mtx, dtype=np.complex128)
    rows, cols = m.shape
    out = np.zeros((max(p.size, 1), rows, cols), dtype=np.complex128)
    _check(lib().sqgo_apply_derivate_to(qbit_num, gp, L, _dp(p), p.size, _dp(m.view(np.float64)), rows, cols, cols,
                                        _dp(out.view(np.float64))), "apply_derivate_to")
    return [out[k] for k in range(p.size)]


def cost_of_matrix(mtx, trace_offset=0, variant=FROBENIUS_NORM):
    m = np.ascontiguousarray(mtx, dtype=np.complex128)
    return lib().sqgo_cost_of_matrix(_dp(m.view(np.float64)), m.shape[1], m.shape[1], trace_offset, variant)


def cost(qbit_num, gates, params, target, trace_offset=0, variant=FROBENIUS_NORM):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    t = np.ascontiguousarray(target, dtype=np.complex128)
    out = np.zeros(1)
    _check(lib().sqgo_cost(qbit_num, gp, L, _dp(p), p.size, _dp(t.view(np.float64)), t.shape[1], trace_offset, variant,
                           _dp(out)), "cost")
    return float(out[0])


def cost_grad(qbit_num, gates, params, target, trace_offset=0, variant=FROBENIUS_NORM):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    t = np.ascontiguousarray(target, dtype=np.complex128)
    out = np.zeros(1)
    grad = np.zeros(max(p.size, 1))
    _check(lib().sqgo_cost_grad(qbit_num, gp, L, _dp(p), p.size, _dp(t.view(np.float64)), t.shape[1], trace_offset,
                                variant, _dp(out), _dp(grad)), "cost_grad")
    return float(out[0]), grad[:p.size].copy()


def cost_grad_sweep(qbit_num, gates, params, target, trace_offset=0, variant=FROBENIUS_NORM):
    """cost_grad by the reverse sweep (three matrices instead of P derivative matrices)."""
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    t = np.ascontiguousarray(target, dtype=np.complex128)
    out = np.zeros(1)
    grad = np.zeros(max(p.size, 1))
    _check(lib().sqgo_cost_grad_sweep(qbit_num, gp, L, _dp(p), p.size, _dp(t.view(np.float64)), t.shape[1],
                                      trace_offset, variant, _dp(out), _dp(grad)), "cost_grad_sweep")
    return float(out[0]), grad[:p.size].copy()


def batch(qbit_num, gates, params, target, trace_offset=0, variant=FROBENIUS_NORM, with_grad=False, nthreads=None,
          sweep=False):
    """Costs (and gradients) of B parameter rows; target is (rows, cols) shared or
    (B, rows, cols) per instance.  sweep=True computes the gradients by the reverse sweep
    (sqgo_cost_grad_sweep), for sizes whose P derivative matrices do not fit in memory."""
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    B, P = p.shape
    t = np.ascontiguousarray(target, dtype=np.complex128)
    per = 1 if t.ndim == 3 else 0
    cols = t.shape[-1]
    costs = np.zeros(B)
    grads = np.zeros((B, max(P, 1))) if with_grad else None
    nthreads = nthreads or os.cpu_count() or 1
    _check(lib().sqgo_batch2(qbit_num, gp, L, _dp(p), P, B, _dp(t.view(np.float64)), cols, per, trace_offset,
                             variant, _dp(costs), _dp(grads) if with_grad else None, nthreads, 1 if sweep else 0),
           "batch")
    return (costs, grads[:, :P]) if with_grad else costs


def decompose(qbit_num, gates, targets, x0, tolerance=1e-8, max_inner=10000, max_outer=4, iteration_loops=1,
              seed=0, nthreads=None, trace_offset=0, variant=FROBENIUS_NORM):
    """SQUANDER's custom-structure BFGS decomposition of each target (B, rows, cols)
    from the start points x0 (B, P).  Returns (x, final_cost, calls)."""
    g, gp, L = _gates(gates)
    t = np.ascontiguousarray(targets, dtype=np.complex128)
    x = np.array(x0, dtype=np.float64, order="C", copy=True)
    B, P = x.shape
    costs = np.zeros(B)
    calls = np.zeros(B, dtype=np.int64)
    nthreads = nthreads or os.cpu_count() or 1
    _check(lib().sqgo_decompose_batch(qbit_num, gp, L, P, B, _dp(t.view(np.float64)), t.shape[-1], trace_offset,
                                      variant, _dp(x), tolerance, max_inner, max_outer, iteration_loops, seed,
                                      _dp(costs), calls.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), nthreads),
           "decompose")
    return x, costs, calls


def adam_decompose(qbit_num, gates, targets, x0, tolerance=1e-8, max_iters=100000, eta=1e-3, adaptive_eta=True,
                   random_shift_count_max=100, randomization_threshold=2500000, seed=0, nthreads=None,
                   trace_offset=0, variant=FROBENIUS_NORM):
    """SQUANDER's ADAM decomposition engine (optimization_engines/ADAM.cpp) of each target
    (B, rows, cols) from the start points x0 (B, P).  Returns (x, minimum cost, evaluations,
    randomisations)."""
    g, gp, L = _gates(gates)
    t = np.ascontiguousarray(targets, dtype=np.complex128)
    x = np.array(x0, dtype=np.float64, order="C", copy=True)
    B, P = x.shape
    costs = np.zeros(B)
    evals = np.zeros(B, dtype=np.int64)
    shifts = np.zeros(B, dtype=np.int64)
    nthreads = nthreads or os.cpu_count() or 1
    _check(lib().sqgo_adam_batch(qbit_num, gp, L, P, B, _dp(t.view(np.float64)), t.shape[-1], trace_offset, variant,
                                 _dp(x), tolerance, max_iters, eta, 1 if adaptive_eta else 0, random_shift_count_max,
                                 randomization_threshold, seed, _dp(costs),
                                 evals.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                 shifts.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), nthreads), "adam_decompose")
    return x, costs, evals, shifts
