"""ORACLE — test infrastructure only (never part of the engine).

ctypes front end of ``oracle/_ref/libsqg_ref.so``: SQUANDER's own C++ decomposition path,
compiled from the reference's sources by ``oracle/build_ref.py``.  The tests use it to pin
the C restatement (``oracle.py``) to the reference itself and to generate golden fixtures
for the GPU tests.  It exists only where the reference tree exists; ``available()`` says
whether it could be built.

The call signatures follow ``oracle.py`` (gate records ``(type, target, control,
param_start)``, complex128 matrices, U^dagger as the target).  With ``SQG_REF_AVX=1`` it loads
the reference's AVX build instead (x86-64 only; for timing comparisons).
"""
import ctypes
import os

import numpy as np

from . import build_ref

_lib = None
_tried = False


def available():
    return lib() is not None


def lib():
    global _lib, _tried
    if _lib is None and not _tried:
        _tried = True
        path = build_ref.build(avx=os.environ.get("SQG_REF_AVX") == "1")
        if path is None:
            return None
        _lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_long)
        i = ctypes.c_int
        _lib.sqgr_cost.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp]
        _lib.sqgr_cost_grad.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp, dp]
        _lib.sqgr_batch.argtypes = [i, ip, i, dp, i, i, dp, i, i, i, dp]
        _lib.sqgr_apply_to.argtypes = [i, ip, i, dp, i, dp, i, i, i]
        _lib.sqgr_apply_from_right.argtypes = [i, ip, i, dp, i, dp, i, i]
        _lib.sqgr_apply_derivate_to.argtypes = [i, ip, i, dp, i, dp, i, i, i, dp]
        _lib.sqgr_combined_unitary.argtypes = [i, ip, i, dp, i, dp, i, dp, dp]
        _lib.sqgr_bfgs_run.argtypes = [i, ip, i, i, dp, i, i, i, dp, ctypes.c_long, dp, lp]
        _lib.sqgr_tree_search.argtypes = [i, dp, i, i, i, ctypes.c_double, ctypes.c_longlong, ip, dp]
        _lib.sqgr_init()
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _gates(gates):
    g = np.ascontiguousarray(np.asarray(gates, dtype=np.int32).reshape(-1, 4))
    return g, g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), g.shape[0]


def _check(rc, what):
    if rc == 1:
        raise ValueError("reference %s: gate list not in the reference's parameter layout" % what)
    if rc != 0:
        raise RuntimeError("reference %s threw (status %d)" % (what, rc))


def _target(target):
    return np.array(target, dtype=np.complex128, order="C", copy=True)


def cost(qbit_num, gates, params, target, trace_offset=0, variant=0):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    t = _target(target)
    out = np.zeros(1)
    _check(lib().sqgr_cost(qbit_num, gp, L, _dp(p), p.size, _dp(t.view(np.float64)), t.shape[1], trace_offset,
                           variant, _dp(out)), "cost")
    return float(out[0])


def cost_grad(qbit_num, gates, params, target, trace_offset=0, variant=0):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    t = _target(target)
    out = np.zeros(1)
    grad = np.zeros(max(p.size, 1))
    _check(lib().sqgr_cost_grad(qbit_num, gp, L, _dp(p), p.size, _dp(t.view(np.float64)), t.shape[1], trace_offset,
                                variant, _dp(out), _dp(grad)), "cost_grad")
    return float(out[0]), grad[:p.size].copy()


def batch(qbit_num, gates, params, target, trace_offset=0, variant=0):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    B, P = p.shape
    t = _target(target)
    costs = np.zeros(B)
    _check(lib().sqgr_batch(qbit_num, gp, L, _dp(p), P, B, _dp(t.view(np.float64)), t.shape[1], trace_offset,
                            variant, _dp(costs)), "batch")
    return costs


def apply_to(qbit_num, gates, params, mtx, parallel=0):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    assert mtx.dtype == np.complex128 and mtx.flags.c_contiguous
    rows, cols = mtx.shape
    _check(lib().sqgr_apply_to(qbit_num, gp, L, _dp(p), p.size, _dp(mtx.view(np.float64)), rows, cols, parallel),
           "apply_to")
    return mtx


def apply_from_right(qbit_num, gates, params, mtx):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    rows, cols = mtx.shape
    _check(lib().sqgr_apply_from_right(qbit_num, gp, L, _dp(p), p.size, _dp(mtx.view(np.float64)), rows, cols),
           "apply_from_right")
    return mtx


def get_matrix(qbit_num, gates, params):
    return apply_to(qbit_num, gates, params, np.eye(1 << qbit_num, dtype=np.complex128))


def apply_derivate_to(qbit_num, gates, params, mtx, parallel=0):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    m = np.ascontiguousarray(mtx, dtype=np.complex128)
    rows, cols = m.shape
    out = np.zeros((max(p.size, 1), rows, cols), dtype=np.complex128)
    _check(lib().sqgr_apply_derivate_to(qbit_num, gp, L, _dp(p), p.size, _dp(m.view(np.float64)), rows, cols,
                                        parallel, _dp(out.view(np.float64))), "apply_derivate_to")
    return [out[k] for k in range(p.size)]


def combined_unitary(qbit_num, gates, params, target):
    g, gp, L = _gates(gates)
    p = np.ascontiguousarray(params, dtype=np.float64)
    t = _target(target)
    rows, cols = t.shape
    U = np.zeros((rows, cols), dtype=np.complex128)
    dU = np.zeros((max(p.size, 1), rows, cols), dtype=np.complex128)
    _check(lib().sqgr_combined_unitary(qbit_num, gp, L, _dp(p), p.size, _dp(t.view(np.float64)), cols,
                                       _dp(U.view(np.float64)), _dp(dU.view(np.float64))), "combined_unitary")
    return U, [dU[k] for k in range(p.size)]


def bfgs_run(qbit_num, gates, target, x0, max_iters, trace_offset=0, variant=0):
    """One BFGS_Powell run from x0: returns (x, final cost, evaluations)."""
    g, gp, L = _gates(gates)
    t = _target(target)
    x = np.array(x0, dtype=np.float64, order="C", copy=True)
    out = np.zeros(1)
    calls = ctypes.c_long(0)
    _check(lib().sqgr_bfgs_run(qbit_num, gp, L, x.size, _dp(t.view(np.float64)), t.shape[1], trace_offset, variant,
                               _dp(x), max_iters, _dp(out), ctypes.byref(calls)), "bfgs_run")
    return x, float(out[0]), int(calls.value)


def tree_search(qbit_num, target, use_osr=0, use_graph_search=0, level_max=14, tolerance=1e-8, seed=1):
    """N_Qubit_Decomposition_Tree_Search on U^dagger: (CNOT count found, decomposition error)."""
    t = _target(target)
    cn = ctypes.c_int(0)
    err = np.zeros(1)
    _check(lib().sqgr_tree_search(qbit_num, _dp(t.view(np.float64)), use_osr, use_graph_search, level_max, tolerance,
                                  seed, ctypes.byref(cn), _dp(err)), "tree_search")
    return int(cn.value), float(err[0])
