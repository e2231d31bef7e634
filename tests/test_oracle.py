"""CPU tests that pin the oracle (oracle/sqg_oracle.c) to the reference's own
known-answer tests, so it can serve as the parity checker of the CUDA engine.

Pins, each following a test of the SQUANDER tree:
  * gate matrices equal the published U/RX/RY/RZ/CRY/CX/CZ definitions with the first
    parameter doubled, up to a global phase (tests/gates/test_gates.py:157-206, 758-769);
  * apply_to on the identity equals get_Matrix; the derivative matrices match central
    finite differences with eps=1e-5 to 1e-5 (tests/gates/test_circuit.py:120-133, 987-1008);
  * cost < 1e-8 at exactly representable parameters, also with a trace offset
    (tests/decomposition/test_optmization_problem_combined.py:123-184);
  * batch == repeated single cost, Grad == gradient of Combined, Combined_Unitary[0] ==
    get_Matrix (same file :189-219);
  * an independent dense (Kronecker) restatement agrees with the row-pair kernels.
"""
import numpy as np
import pytest

from oracle import oracle as O

CZ, CNOT, U3, RY, RX, RZ, CRY = O.CZ, O.CNOT, O.U3, O.RY, O.RX, O.RZ, O.CRY


# ---- published gate definitions (not derived from the oracle) --------------------------
def published_u(theta, phi, lam):
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return np.array([[c, -np.exp(1j * lam) * s], [np.exp(1j * phi) * s, np.exp(1j * (phi + lam)) * c]])


def published_rx(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[c, -1j * s], [-1j * s, c]])


def published_ry(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=complex)


def published_rz(t):
    return np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])


X = np.array([[0, 1], [1, 0]], dtype=complex)
Z = np.diag([1.0 + 0j, -1.0])


def embed(n, gate2, target, control=-1):
    """Dense 2^n matrix of a (controlled) one-qubit gate, qubit q = bit q of the index."""
    N = 1 << n
    M = np.zeros((N, N), dtype=complex)
    for col in range(N):
        if control >= 0 and not (col >> control) & 1:
            M[col, col] = 1
            continue
        b = (col >> target) & 1
        for a in range(2):
            row = (col & ~(1 << target)) | (a << target)
            M[row, col] += gate2[a, b]
    return M


def dense_circuit(n, gates, params):
    M = np.eye(1 << n, dtype=complex)
    for t, tg, c, ps in gates:
        if t == U3:
            G = embed(n, published_u(2 * params[ps], params[ps + 1], params[ps + 2]), tg)
        elif t == RX:
            G = embed(n, published_rx(2 * params[ps]), tg)
        elif t == RY:
            G = embed(n, published_ry(2 * params[ps]), tg)
        elif t == RZ:
            G = embed(n, published_rz(2 * params[ps]), tg)
        elif t == CRY:
            G = embed(n, published_ry(2 * params[ps]), tg, c)
        elif t == CNOT:
            G = embed(n, X, tg, c)
        else:
            G = embed(n, Z, tg, c)
        M = G @ M
    return M


def close_up_to_phase(a, b, tol):
    overlap = np.vdot(a.reshape(-1), b.reshape(-1))
    if abs(overlap) > 0:
        b = b * np.exp(-1j * np.angle(overlap))
    return np.linalg.norm(a - b) < tol


def records(spec):
    """[(type, target, control)] -> (L, 4) records with contiguous param_start."""
    out, p = [], 0
    for t, tg, c in spec:
        out.append((t, tg, c, p))
        p += O.PARAM_NUM[t]
    return np.asarray(out, dtype=np.int32), p


def random_spec(n, L, rng, types=(U3, RX, RY, RZ, CNOT, CZ, CRY)):
    spec = []
    for _ in range(L):
        t = types[rng.integers(len(types))]
        tg = int(rng.integers(n))
        c = -1
        if t in (CNOT, CZ, CRY):
            if n < 2:
                t, c = U3, -1
            else:
                c = int(rng.integers(n - 1))
                c = c + 1 if c >= tg else c
        spec.append((t, tg, c))
    return spec


@pytest.mark.parametrize("gtype", [U3, RX, RY, RZ, CRY, CNOT, CZ])
def test_gate_matches_published_definition(gtype):
    n, target, control = 4, 0, 3
    ctl = control if gtype in (CRY, CNOT, CZ) else -1
    g, P = records([(gtype, target, ctl)])
    params = np.linspace(0.1, 0.1 * P, P) if P else np.zeros(0)
    M = O.get_matrix(n, g, params)
    if gtype == U3:
        ref = embed(n, published_u(2 * params[0], params[1], params[2]), target)
    elif gtype == RX:
        ref = embed(n, published_rx(2 * params[0]), target)
    elif gtype == RY:
        ref = embed(n, published_ry(2 * params[0]), target)
    elif gtype == RZ:
        ref = embed(n, published_rz(2 * params[0]), target)
    elif gtype == CRY:
        ref = embed(n, published_ry(2 * params[0]), target, control)
    elif gtype == CNOT:
        ref = embed(n, X, target, control)
    else:
        ref = embed(n, Z, target, control)
    assert close_up_to_phase(M, ref, 1e-7)
    # the oracle's gates carry no stray global phase either
    assert np.allclose(M, ref, atol=1e-14)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_apply_matches_dense_restatement(n):
    rng = np.random.default_rng(100 + n)
    g, P = records(random_spec(n, 25, rng))
    params = rng.uniform(0, 2 * np.pi, P)
    M = O.get_matrix(n, g, params)
    assert np.allclose(M, dense_circuit(n, g, params), atol=1e-12)
    # rectangular input and right application
    A = rng.standard_normal((1 << n, 3)) + 1j * rng.standard_normal((1 << n, 3))
    B = O.apply_to(n, g, params, A.copy())
    assert np.allclose(B, M @ A, atol=1e-12)
    R = rng.standard_normal((5, 1 << n)) + 1j * rng.standard_normal((5, 1 << n))
    assert np.allclose(O.apply_from_right(n, g, params, R.copy()), R @ M, atol=1e-12)


@pytest.mark.parametrize("n", [2, 3])
def test_derivative_finite_difference(n):
    # test_circuit.py:_build_rx_rz_cnot_circuit + :987-1008
    spec = [(RX, 0, -1), (RZ, 0, -1)] + ([(CNOT, 0, 1), (RY, 1, -1)] if n >= 2 else [])
    spec += [(U3, n - 1, -1), (CRY, 0, n - 1)]
    g, P = records(spec)
    params = np.linspace(0.1, 0.1 * P, P)
    derivs = O.apply_derivate_to(n, g, params, np.eye(1 << n, dtype=complex))
    eps = 1e-5
    for k in range(P):
        pp, pm = params.copy(), params.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (O.get_matrix(n, g, pp) - O.get_matrix(n, g, pm)) / (2 * eps)
        assert np.linalg.norm(derivs[k] - fd) < 1e-5


def test_cost_zero_at_exact_parameters_and_trace_offset():
    n = 5
    rng = np.random.default_rng(42)
    g, P = records(random_spec(n, 40, rng))
    params = rng.uniform(0, 2 * np.pi, P)
    U = O.get_matrix(n, g, params)
    assert abs(O.cost(n, g, params, U.conj().T)) < 1e-8
    off = 8
    sub = U[off:off + 20, :]
    assert abs(O.cost(n, g, params, np.ascontiguousarray(sub.conj().T), trace_offset=off)) < 1e-8
    f, grad = O.cost_grad(n, g, params, np.ascontiguousarray(sub.conj().T), trace_offset=off)
    assert abs(f) < 1e-8 and np.max(np.abs(grad)) < 1e-7


@pytest.mark.parametrize("variant", [O.FROBENIUS_NORM, O.HILBERT_SCHMIDT_TEST, O.INFIDELITY])
def test_batch_grad_and_combined_consistency(variant):
    n = 3
    rng = np.random.default_rng(7)
    g, P = records(random_spec(n, 20, rng))
    target = np.ascontiguousarray(dense_circuit(n, g, rng.uniform(0, 2 * np.pi, P)).conj().T)
    x = rng.uniform(0, 2 * np.pi, (3, P))
    costs, grads = O.batch(n, g, x, target, variant=variant, with_grad=True)
    for b in range(3):
        f, gr = O.cost_grad(n, g, x[b], target, variant=variant)
        assert f == pytest.approx(costs[b], abs=1e-15)
        assert np.allclose(gr, grads[b], atol=1e-15)
        assert O.cost(n, g, x[b], target, variant=variant) == pytest.approx(f, abs=1e-14)
        # gradient matches central differences of the cost
        eps = 1e-6
        for k in range(0, P, 3):
            xp, xm = x[b].copy(), x[b].copy()
            xp[k] += eps
            xm[k] -= eps
            fd = (O.cost(n, g, xp, target, variant=variant) - O.cost(n, g, xm, target, variant=variant)) / (2 * eps)
            assert abs(fd - gr[k]) < 1e-7


def test_bfgs_decomposition_reaches_tolerance():
    n = 2
    rng = np.random.default_rng(3)
    spec = [(U3, 0, -1), (U3, 1, -1)]
    for _ in range(3):
        spec += [(CNOT, 1, 0), (U3, 0, -1), (U3, 1, -1)]
    g, P = records(spec)
    U = O.get_matrix(n, g, rng.uniform(0, 2 * np.pi, P))
    x0 = rng.uniform(0, 2 * np.pi, (2, P))
    x, costs, calls = O.decompose(n, g, np.stack([U.conj().T] * 2), x0, tolerance=1e-8, iteration_loops=3)
    assert np.all(costs < 1e-8)
    for b in range(2):
        assert O.cost(n, g, x[b], U.conj().T) < 1e-8


def test_oracle_reproduces_golden_fixture_of_the_reference_target():
    """tests/golden/umtx4_golden.npz holds the reference's own 4-qubit test target
    (data/Umtx.mat) with costs and gradients; the oracle must keep reproducing them."""
    import os

    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "umtx4_golden.npz"))
    g, th = d["gates"], d["theta"]
    for name, v in (("frob", O.FROBENIUS_NORM), ("hs", O.HILBERT_SCHMIDT_TEST), ("infid", O.INFIDELITY)):
        c, gr = O.batch(4, g, th, d["target"], variant=v, with_grad=True, nthreads=1)
        assert np.array_equal(c, d["cost_" + name]) and np.array_equal(gr, d["grad_" + name])
    c, gr = O.batch(4, g, th, d["target_offset4"], trace_offset=4, with_grad=True, nthreads=1)
    assert np.array_equal(c, d["cost_offset4"]) and np.array_equal(gr, d["grad_offset4"])
    # the stored target is unitary to the precision it was saved with (about 1e-8)
    T = d["target"]
    assert np.allclose(T @ T.conj().T, np.eye(16), atol=1e-7)
