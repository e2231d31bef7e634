"""Full-size checks through size-independent properties (the oracle cannot evaluate these
sizes in seconds): n = 10 with 300 random-pair CNOT blocks (P = 1830) and n = 12 fused vs
unfused application."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def wl():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")


def test_n10_adjoint_gradient_finite_differences_and_checkpoints(sqg, wl):
    rng = np.random.default_rng(21)
    c = wl.cnot_u3_ansatz(10, 300, pairs="random", rng=rng)
    P = c.get_Parameter_Num()
    assert P == 1830
    U = c.get_Matrix(rng.uniform(0, 2 * np.pi, P))
    ev = sqg.CostEvaluator(c, np.ascontiguousarray(U.conj().T))
    theta = torch.tensor(rng.uniform(0, 2 * np.pi, (4, P)), device="cuda", requires_grad=True)
    f = sqg.circuit_cost(theta, ev)
    f.sum().backward()
    g = theta.grad.detach()
    # batch entries equal single evaluations
    c1, g1 = ev.cost_grad(theta.detach()[2])
    assert abs(c1.item() - f[2].item()) < 1e-13
    assert float((g1[0] - g[2]).abs().max()) < 1e-13
    # central differences with h = 1e-6 on coordinates and along a random direction
    h = 1e-6
    x = theta.detach()[0].clone()
    for k in rng.choice(P, 6, replace=False):
        xp, xm = x.clone(), x.clone()
        xp[k] += h
        xm[k] -= h
        fd = (ev.cost_grad(xp, with_grad=False)[0] - ev.cost_grad(xm, with_grad=False)[0]).item() / (2 * h)
        assert abs(fd - g[0, k].item()) < 1e-7
    v = torch.from_numpy(rng.standard_normal(P)).cuda()
    v /= v.norm()
    fd = (ev.cost_grad(x + h * v, with_grad=False)[0] - ev.cost_grad(x - h * v, with_grad=False)[0]).item() / (2 * h)
    assert abs(fd - float(g[0] @ v)) < 1e-7
    # checkpointed partial products give the same gradient
    c2, g2 = ev.cost_grad(theta.detach()[:2], checkpoint_interval=30)
    assert float((g2 - g[:2]).abs().max()) <= 1e-12 * max(1.0, float(g[:2].abs().max()))
    # away from the solution the cost does not vanish
    c0, _ = ev.cost_grad(torch.from_numpy(np.asarray(rng.uniform(0, 1, P))).cuda())
    assert c0.item() > 1e-3


def test_n10_adam_then_bfgs_with_and_without_checkpoints(sqg, wl):
    """n = 10 decomposition in two phases: torch.optim.Adam through the differentiable cost
    (the adjoint kernel behind torch.autograd.Function), once with the plain adjoint gradient
    and once with checkpointed partial products every 8 gates, then the device BFGS loop to
    cost < 1e-8.  The two Adam trajectories agree to rounding; the final cost is certified by a
    fresh evaluation."""
    batched = importlib.import_module("sequential-quantum-gate-decomposer_gb300.batched")
    rng = np.random.default_rng(23)
    c = wl.cnot_u3_ansatz(10, 12, pairs="random", rng=rng)
    P = c.get_Parameter_Num()
    p = rng.uniform(0, 2 * np.pi, P)
    T = np.ascontiguousarray(c.get_Matrix(p).conj().T)
    ev = sqg.CostEvaluator(c, T)
    start = p + rng.normal(0.0, 0.05, P)
    ends = []
    for interval in (0, 8):
        theta = torch.tensor(start, device="cuda", requires_grad=True)
        opt = torch.optim.Adam([theta], lr=2e-3)
        f0 = None
        for _ in range(100):
            opt.zero_grad()
            f = sqg.circuit_cost(theta, ev, checkpoint_interval=interval)
            f0 = f.item() if f0 is None else f0
            f.sum().backward()
            opt.step()
        ends.append((theta.detach().clone(), f.item(), f0))
    (xa, fa, f0a), (xb, fb, f0b) = ends
    assert f0a == pytest.approx(f0b, rel=1e-12)
    # Adam divides by the running gradient magnitude, so gradients that differ at rounding level
    # (checkpointed against plain uncomputation) part the trajectories slowly: 7e-7 relative on
    # the cost after 100 steps on GB300
    assert fa < 0.5 * f0a and fb == pytest.approx(fa, rel=1e-5)
    assert float((xa - xb).abs().max()) < 1e-9
    x, cost, calls, _ = batched.bfgs_decompose_graph(c, T, xa, tolerance=1e-8, max_calls=3000, max_outer=1)
    torch.cuda.synchronize()
    assert cost.item() < 1e-8
    check, _ = ev.cost_grad(x.reshape(1, -1), with_grad=False)
    assert check.item() < 1e-8
    assert 0 < int(calls.item()) <= 3000


def test_n10_exact_solution(sqg, wl):
    rng = np.random.default_rng(22)
    c = wl.cnot_u3_ansatz(10, 60, pairs="random", rng=rng)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    U = c.get_Matrix(p)
    ev = sqg.CostEvaluator(c, np.ascontiguousarray(U.conj().T))
    cost, grad = ev.cost_grad(torch.from_numpy(p).cuda())
    assert abs(cost.item()) < 1e-10
    assert float(grad.abs().max()) < 1e-10


def test_n12_fused_equals_unfused_and_stays_unitary(sqg, wl):
    rng = np.random.default_rng(23)
    c = wl.random_gate_circuit(12, 150, rng)
    th = torch.from_numpy(rng.uniform(0, 2 * np.pi, (1, c.get_Parameter_Num()))).cuda()
    N = 1 << 12
    a = torch.eye(N, dtype=torch.complex128, device="cuda").reshape(1, N, N).contiguous()
    b = a.clone()
    c.apply_to_device(th, a, fused=True)
    c.apply_to_device(th, b, fused=False)
    torch.cuda.synchronize()
    assert float((a - b).abs().max()) < 1e-12
    # unitarity of the applied circuit: columns stay orthonormal
    cols = a[0][:, :64]
    gram = cols.conj().T @ cols
    assert float((gram - torch.eye(64, dtype=torch.complex128, device="cuda")).abs().max()) < 1e-12
    # cost at n = 12 against a target built from the same circuit is zero
    U = a[0].clone()
    ev = sqg.CostEvaluator(c, U.conj().T.contiguous())
    cost, _ = ev.cost_grad(th[0], with_grad=False)
    assert abs(cost.item()) < 1e-10


def test_n13_maximum_size_cost_and_application(sqg, wl):
    """The largest supported register: n = 13 (8192 x 8192 complex128, 1 GiB), cost only."""
    rng = np.random.default_rng(24)
    c = wl.random_gate_circuit(13, 40, rng)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    N = 1 << 13
    a = torch.eye(N, dtype=torch.complex128, device="cuda").reshape(1, N, N).contiguous()
    th = torch.from_numpy(p).cuda().reshape(1, -1)
    c.apply_to_device(th, a, fused=True)
    b = torch.eye(N, dtype=torch.complex128, device="cuda").reshape(1, N, N).contiguous()
    c.apply_to_device(th, b, fused=False)
    torch.cuda.synchronize()
    assert float((a - b).abs().max()) < 1e-12
    del b
    ev = sqg.CostEvaluator(c, a[0].conj().T.contiguous())
    cost, _ = ev.cost_grad(th[0], with_grad=False)
    assert abs(cost.item()) < 1e-10
    with pytest.raises(Exception):
        ev.cost_grad(th[0], with_grad=True)  # gradients are limited to 12 qubits
