"""Parity of the CUDA engine (libsqg.so) with the oracle, through the C ABI.

Tolerance: the cost and every gradient component must agree with the oracle within
1e-12 relative to max(1, |reference|) (costs and gradients are O(1) or smaller);
matrices within 1e-12 absolute entry-wise.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

RTOL = 1e-12


def assert_close(a, b, rtol=RTOL):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    err = float(np.max(np.abs(a - b))) if b.size else 0.0
    assert err <= rtol * scale, "max abs error %.3e exceeds %.1e * %.3g" % (err, rtol, scale)


def spec_circuit(sqg, n, L, rng, types=("U3", "RX", "RY", "RZ", "CNOT", "CZ", "CRY")):
    c = sqg.Circuit(n)
    for _ in range(L):
        t = types[rng.integers(len(types))]
        tg = int(rng.integers(n))
        if t in ("CNOT", "CZ", "CRY") and n >= 2:
            ctl = int(rng.integers(n - 1))
            ctl = ctl + 1 if ctl >= tg else ctl
            getattr(c, "add_" + t)(tg, ctl)
        elif t in ("CNOT", "CZ", "CRY"):
            c.add_U3(tg)
        else:
            getattr(c, "add_" + t)(tg)
    return c


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8])
def test_get_matrix_and_apply(sqg, n):
    rng = np.random.default_rng(10 + n)
    c = spec_circuit(sqg, n, 30, rng)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    ref = O.get_matrix(n, c.gate_records(), p)
    assert_close(c.get_Matrix(p), ref)
    # unfused (one HBM pass per gate), rectangular input
    A = rng.standard_normal((1 << n, 5)) + 1j * rng.standard_normal((1 << n, 5))
    dA = torch.from_numpy(A.copy()).cuda()
    c.apply_to_device(torch.from_numpy(p).cuda(), dA, fused=False)
    assert_close(dA.cpu().numpy(), ref @ A)
    B = A.copy()
    c.apply_to(p, B)
    assert_close(B, ref @ A)
    R = rng.standard_normal((3, 1 << n)) + 1j * rng.standard_normal((3, 1 << n))
    R2 = R.copy()
    c.apply_from_right(p, R2)
    assert_close(R2, R @ ref)


@pytest.mark.parametrize("n", [2, 3, 5])
def test_combined_unitary_matches_reference_derivatives(sqg, n):
    rng = np.random.default_rng(20 + n)
    c = spec_circuit(sqg, n, 12, rng)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    T = np.ascontiguousarray(O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, p.size)).conj().T)
    got = c.apply_to_combined(p, T.copy())
    fwd = O.apply_to(n, c.gate_records(), p, T.copy())
    ders = O.apply_derivate_to(n, c.gate_records(), p, T)
    assert len(got) == p.size + 1
    assert_close(got[0], fwd)
    for k in range(p.size):
        assert_close(got[k + 1], ders[k])


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 8])
@pytest.mark.parametrize("variant", [0, 3, 9])
def test_cost_and_adjoint_gradient_match_oracle(sqg, n, variant):
    rng = np.random.default_rng(30 + n + variant)
    c = spec_circuit(sqg, n, 40 if n < 8 else 60, rng)
    P = c.get_Parameter_Num()
    recs = c.gate_records()
    target = np.ascontiguousarray(O.get_matrix(n, recs, rng.uniform(0, 2 * np.pi, P)).conj().T)
    theta = rng.uniform(0, 2 * np.pi, (3, P))
    ev = sqg.CostEvaluator(c, target, cost_variant=variant)
    cost, grad = ev.cost_grad(torch.from_numpy(theta).cuda())
    rc, rg = O.batch(n, recs, theta, target, variant=variant, with_grad=True)
    assert_close(cost.cpu().numpy(), rc)
    assert_close(grad.cpu().numpy(), rg)
    cost_only, none = ev.cost_grad(torch.from_numpy(theta).cuda(), with_grad=False)
    assert none is None
    assert_close(cost_only.cpu().numpy(), rc)


def test_rectangular_target_with_trace_offset(sqg):
    n, off, cols = 6, 8, 40
    rng = np.random.default_rng(5)
    c = spec_circuit(sqg, n, 50, rng)
    P = c.get_Parameter_Num()
    recs = c.gate_records()
    U = O.get_matrix(n, recs, rng.uniform(0, 2 * np.pi, P))
    target = np.ascontiguousarray(U[off:off + cols, :].conj().T)
    theta = rng.uniform(0, 2 * np.pi, (2, P))
    ev = sqg.CostEvaluator(c, target, trace_offset=off)
    cost, grad = ev.cost_grad(torch.from_numpy(theta).cuda())
    rc, rg = O.batch(n, recs, theta, target, trace_offset=off, with_grad=True)
    assert_close(cost.cpu().numpy(), rc)
    assert_close(grad.cpu().numpy(), rg)


def test_per_instance_targets(sqg):
    n = 4
    rng = np.random.default_rng(6)
    c = spec_circuit(sqg, n, 30, rng)
    P = c.get_Parameter_Num()
    recs = c.gate_records()
    targets = np.stack([np.ascontiguousarray(O.get_matrix(n, recs, rng.uniform(0, 2 * np.pi, P)).conj().T)
                        for _ in range(5)])
    theta = rng.uniform(0, 2 * np.pi, (5, P))
    ev = sqg.CostEvaluator(c, targets)
    cost, grad = ev.cost_grad(torch.from_numpy(theta).cuda())
    rc, rg = O.batch(n, recs, theta, targets, with_grad=True)
    assert_close(cost.cpu().numpy(), rc)
    assert_close(grad.cpu().numpy(), rg)


def test_checkpointed_gradient_equals_uncomputed(sqg):
    n = 7
    rng = np.random.default_rng(8)
    wl = __import__("importlib").import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    c = wl.cnot_u3_ansatz(n, 60, pairs="random", rng=rng)
    P = c.get_Parameter_Num()
    target = np.ascontiguousarray(O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, P)).conj().T)
    theta = torch.from_numpy(rng.uniform(0, 2 * np.pi, (2, P))).cuda()
    ev = sqg.CostEvaluator(c, target)
    c0, g0 = ev.cost_grad(theta)
    c1, g1 = ev.cost_grad(theta, checkpoint_interval=17)
    assert_close(c1.cpu().numpy(), c0.cpu().numpy())
    assert_close(g1.cpu().numpy(), g0.cpu().numpy())
    rc, rg = O.batch(n, c.gate_records(), theta.cpu().numpy(), target, with_grad=True)
    assert_close(c1.cpu().numpy(), rc)
    assert_close(g1.cpu().numpy(), rg)


def test_exact_parameters_give_zero_cost_and_gradient(sqg):
    n = 8
    rng = np.random.default_rng(9)
    wl = __import__("importlib").import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    c = wl.cnot_u3_ansatz(n, 40)
    P = c.get_Parameter_Num()
    p = rng.uniform(0, 2 * np.pi, P)
    U = c.get_Matrix(p)
    ev = sqg.CostEvaluator(c, np.ascontiguousarray(U.conj().T))
    cost, grad = ev.cost_grad(torch.from_numpy(p).cuda())
    assert abs(cost.item()) < 1e-8
    assert float(grad.abs().max()) < 1e-8


def test_autograd_function(sqg):
    n = 3
    rng = np.random.default_rng(11)
    c = spec_circuit(sqg, n, 20, rng)
    P = c.get_Parameter_Num()
    recs = c.gate_records()
    target = np.ascontiguousarray(O.get_matrix(n, recs, rng.uniform(0, 2 * np.pi, P)).conj().T)
    ev = sqg.CostEvaluator(c, target)
    theta = torch.tensor(rng.uniform(0, 2 * np.pi, (4, P)), device="cuda", requires_grad=True)
    f = sqg.circuit_cost(theta, ev)
    (2.0 * f.sum()).backward()
    rc, rg = O.batch(n, recs, theta.detach().cpu().numpy(), target, with_grad=True)
    assert_close(f.detach().cpu().numpy(), rc)
    assert_close(theta.grad.cpu().numpy(), 2.0 * rg)
    # central finite differences of the cost (h = 1e-6) along every coordinate
    x = theta.detach()[0].clone()
    h = 1e-6
    g = torch.zeros(P, dtype=torch.float64)
    for k in range(P):
        xp, xm = x.clone(), x.clone()
        xp[k] += h
        xm[k] -= h
        g[k] = (ev.cost_grad(xp, with_grad=False)[0] - ev.cost_grad(xm, with_grad=False)[0]).item() / (2 * h)
    assert float((g - theta.grad[0].cpu() / 2.0).abs().max()) < 1e-8


def test_decomposition_api_shapes_and_errors(sqg):
    n = 3
    rng = np.random.default_rng(12)
    wl = __import__("importlib").import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    c = wl.cnot_u3_ansatz(n, 4)
    P = c.get_Parameter_Num()
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, P))
    d = sqg.N_Qubit_Decomposition_custom(U.conj().T, config={"random_seed": 1})
    d.set_Gate_Structure(c)
    assert d.get_Parameter_Num() == P
    x = rng.uniform(0, 2 * np.pi, P)
    f = d.Optimization_Problem(x)
    f2, g = d.Optimization_Problem_Combined(x)
    assert g.shape == (P, 1)
    assert f == pytest.approx(f2, abs=1e-14)
    assert np.allclose(d.Optimization_Problem_Grad(x), g, atol=1e-14)
    batch = d.Optimization_Problem_Batch(np.vstack([x, x, x]))
    assert batch.shape == (3, 1) and np.allclose(batch[:, 0], f, atol=1e-14)
    M, dM = d.Optimization_Problem_Combined_Unitary(x)
    assert len(dM) == P
    assert_close(M, O.apply_to(n, c.gate_records(), x, np.ascontiguousarray(U.conj().T)))
    rc, rg = O.cost_grad(n, c.gate_records(), x, np.ascontiguousarray(U.conj().T))
    assert_close(f, rc)
    assert_close(g[:, 0], rg)
    with pytest.raises(Exception):
        d.Optimization_Problem(np.zeros(P + 1))
    with pytest.raises(Exception):
        d.set_Cost_Function_Variant(1)


def test_start_decomposition_reaches_tolerance(sqg):
    n = 2
    rng = np.random.default_rng(13)
    wl = __import__("importlib").import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    c = wl.cnot_u3_ansatz(n, 3)
    U = c.get_Matrix(rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    d = sqg.N_Qubit_Decomposition_custom(U.conj().T, config={"random_seed": 3, "optimization_tolerance": 1e-8})
    d.set_Gate_Structure(c)
    d.Start_Decomposition()
    assert d.get_Decomposition_Error() < 1e-8
    x = d.get_Optimized_Parameters()
    assert O.cost(n, c.gate_records(), x, np.ascontiguousarray(U.conj().T)) < 1e-8


def test_errors_do_not_fall_back(sqg):
    with pytest.raises(Exception):
        sqg.Circuit(14).get_Matrix(np.zeros(0))
    c = sqg.Circuit(2)
    c.add_U3(0)
    with pytest.raises(ValueError):
        c.get_Matrix(np.zeros(4))


def test_engine_matches_golden_fixture_of_the_reference_target(sqg):
    """Cost and adjoint gradient on the reference's own 4-qubit test target (golden fixture
    from the oracle, tests/golden/make_golden.py), all three cost variants and a trace offset."""
    import os

    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "umtx4_golden.npz"))
    c = sqg.Circuit(4)
    for t, tg, ctl, ps in d["gates"]:
        if t == 7:
            c.add_U3(int(tg))
        else:
            c.add_CNOT(int(tg), int(ctl))
    assert np.array_equal(c.gate_records(), d["gates"])
    theta = torch.from_numpy(d["theta"]).cuda()
    for name, v in (("frob", 0), ("hs", 3), ("infid", 9)):
        cost, grad = sqg.CostEvaluator(c, d["target"], cost_variant=v).cost_grad(theta)
        assert_close(cost.cpu().numpy(), d["cost_" + name])
        assert_close(grad.cpu().numpy(), d["grad_" + name])
    cost, grad = sqg.CostEvaluator(c, d["target_offset4"], trace_offset=4).cost_grad(theta)
    assert_close(cost.cpu().numpy(), d["cost_offset4"])
    assert_close(grad.cpu().numpy(), d["grad_offset4"])


def test_apply_to_list_and_unitary_accessors(sqg):
    n = 3
    rng = np.random.default_rng(31)
    c = spec_circuit(sqg, n, 15, rng)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    ref = O.get_matrix(n, c.gate_records(), p)
    mats = [rng.standard_normal((8, k)) + 1j * rng.standard_normal((8, k)) for k in (8, 3, 8, 1)]
    orig = [m.copy() for m in mats]
    c.apply_to_list(mats, p)
    for m, o in zip(mats, orig):
        assert_close(m, ref @ o)
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, p.size))
    d = sqg.N_Qubit_Decomposition_custom(U.conj().T)
    assert np.array_equal(d.get_Unitary(), U.conj().T)
    d.set_Unitary(np.eye(8, dtype=np.complex128))
    d.set_Gate_Structure(c)
    assert_close(d.Optimization_Problem(p), 1.0 - np.trace(ref).real / 8)
    d.set_Iteration_Loops({3: 2})
    assert d.config["max_iteration_loops"] == 2


@pytest.mark.parametrize("kind", ["empty", "no_params"])
def test_circuits_without_gates_or_parameters(sqg, kind):
    """Edge cases of the reference's tests (test_circuit.py:1022-1041): an empty gate list and
    a circuit of constant gates only."""
    n = 3
    c = sqg.Circuit(n)
    if kind == "no_params":
        c.add_CNOT(1, 0)
        c.add_CZ(2, 1)
    rng = np.random.default_rng(40)


    target = np.ascontiguousarray((rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))))
    ev = sqg.CostEvaluator(c, target)
    cost, grad = ev.cost_grad(torch.zeros((2, 0), dtype=torch.float64, device="cuda"))
    rc = O.cost(n, c.gate_records(), np.zeros(0), target)
    assert np.allclose(cost.cpu().numpy(), rc, atol=1e-14)
    assert grad.shape == (2, 0)
    assert np.allclose(c.get_Matrix(np.zeros(0)), O.get_matrix(n, c.gate_records(), np.zeros(0)), atol=1e-14)
    assert c.apply_derivate_to(np.zeros(0), np.eye(8, dtype=np.complex128)) == []


def test_dropin_adam_above_five_qubits_follows_the_oracle(sqg):
    """N_Qubit_Decomposition_custom picks ADAM for qbit_num > 5 (N_Qubit_Decomposition_custom.cpp:
    59-76); its engine driven by the GPU cost and gradient follows the same engine driven by
    the oracle."""
    import importlib

    optim = importlib.import_module("sequential-quantum-gate-decomposer_gb300.optim")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    n = 6
    rng = np.random.default_rng(66)
    c = wl.cnot_u3_ansatz(n, 6)
    P = c.get_Parameter_Num()
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, P))
    T = np.ascontiguousarray(U.conj().T)
    dec = sqg.N_Qubit_Decomposition_custom(T, config={"max_inner_iterations": 200, "random_seed": 5})
    dec.set_Gate_Structure(c)
    assert dec.optimizer == "ADAM"
    x0 = rng.uniform(0, 2 * np.pi, P)
    xg, xo = x0.copy(), x0.copy()
    fg_gpu, ng = optim.adam_squander(dec._fg, xg, max_iters=200, seed=8)
    fg_orc, no = optim.adam_squander(lambda th: O.cost_grad(n, c.gate_records(), th, T), xo, max_iters=200, seed=8)
    assert ng == no == 200
    assert abs(fg_gpu - fg_orc) <= 1e-10 * max(1.0, abs(fg_orc))
    assert np.allclose(xg, xo, atol=1e-9)
    dec.set_Optimized_Parameters(x0)
    dec.Start_Decomposition()
    assert dec.get_Decomposition_Error() <= fg_orc + 1e-9


@pytest.mark.parametrize("n,cols,offset,variant", [(2, 4, 0, 0), (3, 8, 0, 0), (3, 6, 2, 0), (4, 16, 0, 3),
                                                   (4, 12, 4, 0), (4, 16, 0, 9)])
def test_small_register_cost_grad_forms_agree(sqg, monkeypatch, n, cols, offset, variant):
    """Up to five qubits sqg_cost_grad evaluates gradients with the environment-matrix kernel;
    it matches the oracle and the tile kernels (SQG_COSTGRAD_FORM=tile)."""
    import importlib

    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    rng = np.random.default_rng(300 + n + cols)
    c = wl.all_gates_circuit(n, 30, rng)
    P = c.get_Parameter_Num()
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, P))
    T = np.ascontiguousarray(U.conj().T[:, offset:offset + cols])
    th = rng.uniform(0, 2 * np.pi, (5, P))
    off = offset if variant == 0 else 0
    ev = sqg.CostEvaluator(c, T, trace_offset=off, cost_variant=variant)
    ce, ge = ev.cost_grad(torch.from_numpy(th).cuda())
    monkeypatch.setenv("SQG_COSTGRAD_FORM", "tile")
    ct, gt = ev.cost_grad(torch.from_numpy(th).cuda())
    torch.cuda.synchronize()
    cr, gr = O.batch(n, c.gate_records(), th, T, trace_offset=off, variant=variant, with_grad=True)
    scale = max(1.0, float(np.abs(gr).max()))
    for cost, grad in ((ce, ge), (ct, gt)):
        assert np.allclose(cost.cpu().numpy(), cr, rtol=0, atol=1e-12)
        assert float(np.abs(grad.cpu().numpy() - gr).max()) <= 1e-12 * scale


@pytest.mark.parametrize("n,cols", [(2, 4), (3, 5), (6, 12), (9, 64)])
def test_unfused_cnot_cz_passes_match_oracle(sqg, n, cols):
    """The HBM pass kernel of CNOT (row exchange) and CZ (sign flips of the target = 1 rows)
    used by unfused application to matrices, power-of-two widths and others."""
    rng = np.random.default_rng(400 + n)
    c = sqg.Circuit(n)
    for _ in range(12):
        t = int(rng.integers(n))
        ctl = int(rng.integers(n - 1))
        ctl = ctl + 1 if ctl >= t else ctl
        (c.add_CNOT if rng.integers(2) == 0 else c.add_CZ)(t, ctl)
    c.add_U3(0)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    A = rng.standard_normal((1 << n, cols)) + 1j * rng.standard_normal((1 << n, cols))
    dA = torch.from_numpy(np.stack([A, 2 * A])).cuda()
    c.apply_to_device(torch.from_numpy(np.stack([p, p])).cuda(), dA, fused=False)
    ref = O.get_matrix(n, c.gate_records(), p)
    got = dA.cpu().numpy()
    assert_close(got[0], ref @ A)
    assert_close(got[1], ref @ (2 * A))


@pytest.mark.parametrize("n", [1, 3, 7, 12])
def test_merged_single_qubit_runs_match_oracle(sqg, n):
    """Runs of single-qubit gates (U3, RX, RY, RZ) with no two-qubit gate on their qubit between
    them are applied as one general 2x2 gate by the fused forward paths (application and
    cost-only evaluation); their results equal the oracle's gate-by-gate ones."""
    rng = np.random.default_rng(500 + n)
    c = sqg.Circuit(n)
    for _ in range(40):
        t = int(rng.integers(n))
        for _ in range(int(rng.integers(1, 5))):
            getattr(c, "add_" + ("U3", "RX", "RY", "RZ")[int(rng.integers(4))])(t)
        if n > 1 and rng.integers(2):
            ctl = int(rng.integers(n - 1))
            ctl = ctl + 1 if ctl >= t else ctl
            getattr(c, "add_" + ("CNOT", "CZ", "CRY")[int(rng.integers(3))])(t, ctl)
    P = c.get_Parameter_Num()
    recs = c.gate_records()
    p = rng.uniform(0, 2 * np.pi, (2, P))
    N = 1 << n
    cols = min(N, 16)
    A = rng.standard_normal((N, cols)) + 1j * rng.standard_normal((N, cols))
    dA = torch.from_numpy(np.stack([A, A])).cuda()
    c.apply_to_device(torch.from_numpy(p).cuda(), dA, fused=True)
    got = dA.cpu().numpy()
    for b in range(2):
        assert_close(got[b], O.apply_to(n, recs, p[b], A.copy()))
    T = np.ascontiguousarray(A)
    ev = sqg.CostEvaluator(c, T, trace_offset=N - cols)
    cost, _ = ev.cost_grad(torch.from_numpy(p).cuda(), with_grad=False)
    ref = [O.cost(n, recs, p[b], T, trace_offset=N - cols) for b in range(2)]
    assert_close(cost.cpu().numpy(), np.array(ref))
