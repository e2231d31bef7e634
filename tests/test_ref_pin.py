"""The oracle pinned to SQUANDER itself (CPU).

Two kinds of checks:
* against the reference's own C++ path, compiled from its sources by oracle/build_ref.py
  (run where the reference tree exists; skipped elsewhere): gate application from the left
  and right, the derivative matrices, the combined unitary, cost and gradient for the three
  cost variants with rectangular targets and trace offsets, the batched cost, and BFGS_Powell
  trajectories;
* against the golden fixtures that tests/golden/make_golden.py made from the reference (run
  everywhere): the oracle must reproduce them.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as R

    if not R.available():
        pytest.skip("the reference tree is not present here")
    return R


@pytest.fixture(scope="module")
def wl(sqg):
    import importlib

    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")


def _close(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    err = np.max(np.abs(a - b)) if a.size else 0.0
    assert err <= tol, err


@pytest.mark.parametrize("n", [1, 2, 3, 4, 6])
def test_gate_application_and_derivatives_equal_the_reference(ref, wl, n):
    rng = np.random.default_rng(100 + n)
    c = wl.all_gates_circuit(n, 40, rng)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    th = rng.uniform(0, 2 * np.pi, P)
    N = 1 << n
    M = np.ascontiguousarray(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N)))
    _close(O.apply_to(n, recs, th, M.copy()), ref.apply_to(n, recs, th, M.copy()), 1e-15)
    _close(O.apply_from_right(n, recs, th, M.copy()), ref.apply_from_right(n, recs, th, M.copy()), 1e-15)
    _close(np.stack(O.apply_derivate_to(n, recs, th, M)), np.stack(ref.apply_derivate_to(n, recs, th, M)), 1e-15)
    T = np.ascontiguousarray(wl.haar_unitary(N, rng).conj().T)
    U, dU = ref.combined_unitary(n, recs, th, T)
    _close(O.apply_to(n, recs, th, T.copy()), U, 1e-15)
    _close(np.stack(O.apply_derivate_to(n, recs, th, T)), np.stack(dU), 1e-15)


@pytest.mark.parametrize("n,blocks", [(2, 6), (3, 14), (4, 40), (5, 12), (7, 6), (8, 4)])
@pytest.mark.parametrize("variant", [0, 3, 9])
def test_cost_and_gradient_equal_the_reference(ref, wl, n, blocks, variant):
    rng = np.random.default_rng(10 * n + variant)
    c = wl.cnot_u3_ansatz(n, blocks)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    N = 1 << n
    T = np.ascontiguousarray(wl.haar_unitary(N, rng).conj().T)
    th = rng.uniform(0, 2 * np.pi, (2, P))
    for cols, off in ((N, 0), (N // 2, N // 4), (1, N - 1)):
        Tt = np.ascontiguousarray(T[:, :cols])
        for x in th:
            c_ref, g_ref = ref.cost_grad(n, recs, x, Tt, trace_offset=off, variant=variant)
            c_o, g_o = O.cost_grad(n, recs, x, Tt, trace_offset=off, variant=variant)
            _close(c_o, c_ref, 1e-15)
            _close(g_o, g_ref, 1e-15)
            c_s, g_s = O.cost_grad_sweep(n, recs, x, Tt, trace_offset=off, variant=variant)
            _close(c_s, c_ref, 1e-15)
            _close(g_s, g_ref, 1e-14)
        _close(O.batch(n, recs, th, Tt, trace_offset=off, variant=variant),
               ref.batch(n, recs, th, Tt, trace_offset=off, variant=variant), 1e-15)
        assert ref.cost(n, recs, th[0], Tt, trace_offset=off, variant=variant) == pytest.approx(
            O.cost(n, recs, th[0], Tt, trace_offset=off, variant=variant), abs=1e-15)


def test_all_gate_kinds_cost_and_gradient_equal_the_reference(ref, wl):
    rng = np.random.default_rng(77)
    for n in (2, 3, 5):
        c = wl.all_gates_circuit(n, 60, rng)
        recs, P = c.gate_records(), c.get_Parameter_Num()
        N = 1 << n
        T = np.ascontiguousarray(wl.haar_unitary(N, rng).conj().T)
        x = rng.uniform(0, 2 * np.pi, P)
        for variant in (0, 3, 9):
            c_ref, g_ref = ref.cost_grad(n, recs, x, T, variant=variant)
            c_o, g_o = O.cost_grad(n, recs, x, T, variant=variant)
            _close(c_o, c_ref, 1e-15)
            _close(g_o, g_ref, 1e-15)


def test_bfgs_runs_follow_the_reference(ref, wl):
    """One BFGS_Powell run (BFGS.cpp:121-125): same evaluation count, same point, same cost."""
    c = wl.cnot_u3_ansatz(3, 14)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    rng = np.random.default_rng(31)
    for k in range(6):
        T = np.ascontiguousarray(wl.haar_unitary(8, rng).conj().T) if k % 2 == 0 else np.ascontiguousarray(
            wl.circuit_matrix(c, rng.uniform(0, 2 * np.pi, P)).conj().T)
        x0 = rng.uniform(0, 2 * np.pi, P)
        xr, fr, nr = ref.bfgs_run(3, recs, T, x0, 400)
        xo, fo, no = O.decompose(3, recs, T[None], x0[None], max_inner=400, max_outer=1, iteration_loops=1, nthreads=1)
        assert no[0] == nr
        _close(xo[0], xr, 1e-12)
        assert fo[0] == pytest.approx(fr, abs=1e-14)


def test_bfgs_with_trace_offset_and_variants_follows_the_reference(ref, wl):
    c = wl.cnot_u3_ansatz(3, 6)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    rng = np.random.default_rng(32)
    U = wl.haar_unitary(8, rng)
    T = np.ascontiguousarray(U[2:6, :].conj().T)
    for variant in (0, 3, 9):
        x0 = rng.uniform(0, 2 * np.pi, P)
        off = 2 if variant == 0 else 0
        xr, fr, nr = ref.bfgs_run(3, recs, T, x0, 150, trace_offset=off, variant=variant)
        xo, fo, no = O.decompose(3, recs, T[None], x0[None], max_inner=150, max_outer=1, iteration_loops=1,
                                 nthreads=1, trace_offset=off, variant=variant)
        assert no[0] == nr
        _close(xo[0], xr, 1e-12)


# ---------------------------------------------------------------- golden fixtures


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_oracle_reproduces_the_reference_fixture_umtx4():
    d = _load("umtx4_golden.npz")
    g, th = d["gates"], d["theta"]
    for name, v in (("frob", 0), ("hs", 3), ("infid", 9)):
        c, gr = O.batch(4, g, th, d["target"], variant=v, with_grad=True, nthreads=1)
        _close(c, d["cost_" + name], 1e-15)
        _close(gr, d["grad_" + name], 1e-15)
    c, gr = O.batch(4, g, th, d["target_offset4"], trace_offset=4, with_grad=True, nthreads=1)
    _close(c, d["cost_offset4"], 1e-15)
    _close(gr, d["grad_offset4"], 1e-15)
    x, f, calls = O.decompose(4, g, d["target"][None], d["bfgs_x0"][None], max_inner=int(d["bfgs_max_iters"]),
                              max_outer=1, iteration_loops=1, nthreads=1)
    assert calls[0] == int(d["bfgs_calls"])
    _close(x[0], d["bfgs_x"], 1e-10)


def test_oracle_reproduces_the_reference_fixture_config1():
    d = _load("config1_n4.npz")
    g, th = d["gates"], d["theta"]
    for name, v in (("frob", 0), ("hs", 3), ("infid", 9)):
        c, gr = O.batch(4, g, th, d["target"], variant=v, with_grad=True)
        _close(c, d["cost_" + name], 1e-15)
        _close(gr, d["grad_" + name], 1e-15)


def test_oracle_reproduces_the_reference_fixture_config2():
    d = _load("config2_n8.npz")
    for blocks in (120, 360):
        k = "b%d_" % blocks
        c, gr = O.batch(8, d[k + "gates"], d[k + "theta"][:2], d[k + "target"], with_grad=True, sweep=True)
        _close(c, d[k + "cost"][:2], 1e-14)
        _close(gr, d[k + "grad"][:2], 1e-13)


def test_oracle_reproduces_the_reference_fixture_config4():
    d = _load("config4_3q.npz")
    sel = np.arange(0, 64, 8)
    x, f, calls = O.decompose(3, d["gates"], d["targets"][sel], d["x0"][sel], max_inner=int(d["max_iters"]),
                              max_outer=1, iteration_loops=1)
    assert np.array_equal(calls, d["calls"][sel])
    _close(x, d["x"][sel], 1e-10)


def test_oracle_reproduces_the_reference_fixture_config5():
    from golden.inputs import config5_inputs

    d = _load("config5_n12.npz")
    c, theta, X, S, T = config5_inputs()
    assert np.array_equal(c.gate_records(), d["gates"])
    Y = O.apply_to(12, d["gates"], theta[0], X.copy())
    _close(S @ Y, d["sketch"][0], 1e-11)
    cst = O.cost(12, d["gates"], theta[1], T, trace_offset=1000)
    assert cst == pytest.approx(d["cost"][1], abs=1e-14)


def test_oracle_reproduces_the_reference_fixture_config3():
    """10 qubits: the reference's costs (two of the 64 vectors) and the checksum of the target."""
    from golden.inputs import config3_inputs

    d = _load("config3_n10.npz")
    c, angles, theta, pick = config3_inputs()
    U = O.get_matrix(10, d["gates"], angles)
    target = np.ascontiguousarray(U.conj().T)
    assert np.max(np.abs(np.array([target.sum(), (target * target).sum()]) - d["target_checksum"])) < 1e-9
    costs = O.batch(10, d["gates"], theta[:2], target)
    _close(costs, d["cost"][:2], 1e-13)


def test_oracle_reproduces_the_reference_fixture_adaptive8():
    d = _load("adaptive_n8.npz")
    U = O.get_matrix(8, d["gates"], d["exact"])
    target = np.ascontiguousarray(U[80:240, :].conj().T)
    c, g = O.cost_grad(8, d["gates"], d["theta"][0], target, trace_offset=80)
    assert c == pytest.approx(float(d["cost"][0]), abs=1e-14)
    _close(g, d["grad"][0], 1e-14)
