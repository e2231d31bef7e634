"""Parity of the CUDA engine at the sizes of the five benchmark workloads, against values
the reference itself produced (tests/golden/*.npz, made by tests/golden/make_golden.py from
SQUANDER's C++ path compiled by oracle/build_ref.py) and against the oracle run here.

Tolerances: costs and gradient components within 1e-12 relative to max(1, |reference|);
matrix products within 1e-12 relative to the largest entry (checked through a +-1 sketch,
so the bound is scaled by the sketch's row length); BFGS trajectories by their evaluation
counts and end points.
"""
import importlib
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL = 1e-12


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def assert_close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    err = float(np.max(np.abs(a - b))) if b.size else 0.0
    assert err <= rtol * scale, "max abs error %.3e exceeds %.1e * %.3g" % (err, rtol, scale)


@pytest.fixture(scope="module")
def wl():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")


def circuit_from_records(sqg, n, recs):
    c = sqg.Circuit(n)
    for t, tg, ctl, _ in recs:
        t, tg, ctl = int(t), int(tg), int(ctl)
        name = {7: "U3", 8: "RY", 9: "RX", 10: "RZ", 5: "CNOT", 4: "CZ", 14: "CRY"}[t]
        if t in (4, 5, 14):
            getattr(c, "add_" + name)(tg, ctl)
        else:
            getattr(c, "add_" + name)(tg)
    assert np.array_equal(c.gate_records(), recs)
    return c


def test_config1_cost_gradient_and_bfgs_run_against_the_reference(sqg):
    """4 qubits, 40 nearest-neighbour blocks (P = 252), Haar target: cost and gradient for three
    variants, and one BFGS run with a 2000-evaluation budget from the reference's start point."""
    d = _load("config1_n4.npz")
    c = circuit_from_records(sqg, 4, d["gates"])
    theta = torch.from_numpy(d["theta"]).cuda()
    for name, v in (("frob", 0), ("hs", 3), ("infid", 9)):
        cost, grad = sqg.CostEvaluator(c, d["target"], cost_variant=v).cost_grad(theta)
        assert_close(cost.cpu().numpy(), d["cost_" + name])
        assert_close(grad.cpu().numpy(), d["grad_" + name])
    # the device BFGS (one run, the drop-in's budget) and the reference's run
    dec = sqg.BatchedDecomposer(c, tolerance=1e-8, max_calls=int(d["bfgs_max_iters"]), max_outer=1,
                                stop_at_tolerance=False)
    x, cost, calls = dec.run(d["target"][None], d["bfgs_x0"][None])
    torch.cuda.synchronize()
    ref_calls, ref_cost = int(d["bfgs_calls"]), float(d["bfgs_cost"])
    got_calls, got_cost = int(calls.item()), float(cost.item())
    # the two runs take the same steps until rounding differences change a line search;
    # they end in the same minimum
    assert abs(got_cost - ref_cost) <= 1e-9, (got_cost, ref_cost)
    assert abs(got_calls - ref_calls) <= 0.1 * ref_calls, (got_calls, ref_calls)
    oc = O.cost(4, d["gates"], x.cpu().numpy()[0], d["target"])
    assert abs(oc - got_cost) <= 1e-12


@pytest.mark.parametrize("blocks", [120, 360])
def test_config2_batch_of_1024_against_the_reference(sqg, blocks):
    """8 qubits, ansatz target with an exact solution, B = 1024 parameter vectors in one launch
    (P = 744 or 2184): the four reference rows to 1e-12; every other row equal to its own
    single evaluation; cost-only equal to the cost of the cost+gradient call."""
    d = _load("config2_n8.npz")
    k = "b%d_" % blocks
    c = circuit_from_records(sqg, 8, d[k + "gates"])
    P = c.get_Parameter_Num()
    rng = np.random.default_rng(blocks)
    theta = rng.uniform(0, 2 * np.pi, (1024, P))
    theta[:4] = d[k + "theta"]
    ev = sqg.CostEvaluator(c, d[k + "target"])
    th = torch.from_numpy(theta).cuda()
    cost, grad = ev.cost_grad(th)
    cost_only, _ = ev.cost_grad(th, with_grad=False)
    torch.cuda.synchronize()
    cost, grad = cost.cpu().numpy(), grad.cpu().numpy()
    assert_close(cost[:4], d[k + "cost"])
    assert_close(grad[:4], d[k + "grad"])
    # cost-only runs the forward tile kernel, cost+gradient the adjoint one: same value to rounding
    assert_close(cost_only.cpu().numpy(), cost)
    for b in rng.choice(np.arange(4, 1024), 4, replace=False):
        c1, g1 = ev.cost_grad(th[b])
        assert_close(c1.cpu().numpy(), cost[b:b + 1])
        assert_close(g1.cpu().numpy(), grad[b:b + 1])
    assert np.all(np.isfinite(grad)) and np.all(cost > -1e-12) and np.all(cost <= 2.0)


@pytest.mark.parametrize("checkpoint", [0, 30])
def test_config3_n10_gradient_on_64_vectors(sqg, checkpoint):
    """10 qubits, 300 blocks over random pairs (P = 1830), 64 parameter vectors: costs against
    the reference, 32 gradient components per vector against the oracle's gradient (the
    reference's prefix form would need 30 GB), with and without checkpointed partial products."""
    from golden.inputs import config3_inputs

    d = _load("config3_n10.npz")
    c, angles, theta, pick = config3_inputs()
    assert np.array_equal(c.gate_records(), d["gates"]) and np.array_equal(pick, d["pick"])
    U = O.get_matrix(10, d["gates"], angles)
    target = np.ascontiguousarray(U.conj().T)
    chk = np.array([target.sum(), (target * target).sum()])
    assert np.max(np.abs(chk - d["target_checksum"])) < 1e-9
    ev = sqg.CostEvaluator(c, target)
    cost, grad = ev.cost_grad(torch.from_numpy(theta).cuda(), checkpoint_interval=checkpoint)
    torch.cuda.synchronize()
    assert_close(cost.cpu().numpy(), d["cost"])
    assert_close(np.take_along_axis(grad.cpu().numpy(), pick, axis=1), d["grad"])


def test_config4_first_bfgs_steps_equal_the_reference(sqg):
    """64 of the 3-qubit benchmark targets, 14-block ansatz (P = 93): a BFGS run of 20
    evaluations from the reference's start points lands where the reference's own run lands
    (same evaluation count, same point to 1e-8, same cost to 1e-9 relative)."""
    d = _load("config4_3q.npz")
    c = circuit_from_records(sqg, 3, d["gates"])
    dec = sqg.BatchedDecomposer(c, tolerance=0.0, max_calls=int(d["short_max_iters"]), max_outer=1,
                                stop_at_tolerance=False)
    x, cost, calls = dec.run(d["targets"], d["x0"])
    torch.cuda.synchronize()
    assert np.array_equal(calls.cpu().numpy(), d["short_calls"])
    assert np.max(np.abs(x.cpu().numpy() - d["short_x"])) < 1e-8
    # points equal to 1e-8 give costs equal to about 1e-9 relative
    assert np.allclose(cost.cpu().numpy(), d["short_cost"], rtol=1e-9, atol=1e-12)


def test_config4_full_bfgs_runs_reach_the_reference_outcomes(sqg):
    """The same targets and starts, one BFGS run of at most 1000 evaluations each, run to its own
    convergence.  Over hundreds of evaluations the device's and the reference's trajectories
    part at rounding level (their gradients agree to 1e-12, their summation orders differ, and a
    line search near convergence compares costs that differ by a few ulps), so the run lengths
    differ by a few per cent; the outcomes agree, and every device result is certified by the
    oracle's cost of its returned point."""
    d = _load("config4_3q.npz")
    c = circuit_from_records(sqg, 3, d["gates"])
    dec = sqg.BatchedDecomposer(c, tolerance=1e-8, max_calls=int(d["max_iters"]), max_outer=1, stop_at_tolerance=False)
    x, cost, calls = dec.run(d["targets"], d["x0"])
    torch.cuda.synchronize()
    calls, cost, xh = calls.cpu().numpy(), cost.cpu().numpy(), x.cpu().numpy()
    solved_ref, solved = d["cost"] < 1e-8, cost < 1e-8
    assert np.sum(solved != solved_ref) <= 4, (cost, d["cost"])
    assert abs(int(solved.sum()) - int(solved_ref.sum())) <= 3
    assert abs(float(calls.mean()) - float(d["calls"].mean())) <= 0.1 * float(d["calls"].mean())
    oc = np.array([O.cost(3, d["gates"], xh[b], d["targets"][b]) for b in range(64)])
    assert np.max(np.abs(oc - cost)) <= 1e-12


def test_config4_full_budget_decompositions_against_the_oracle(sqg):
    """The benchmark's budgets (1000 evaluations per run, 4 outer iterations, each restarting
    from the best point) on the same 64 targets against the oracle's restatement: the same
    outcomes per target up to the rounding-level parting of long trajectories, the same solved
    count within 3, and certified costs."""
    from golden.inputs import config4_inputs

    ansatz, targets, x0 = config4_inputs()
    recs = ansatz.gate_records()
    c = circuit_from_records(sqg, 3, recs)
    dec = sqg.BatchedDecomposer(c, tolerance=1e-8, max_calls=1000, max_outer=4, stop_at_tolerance=False)
    x, cost, calls = dec.run(targets, x0, seed=17)
    torch.cuda.synchronize()
    xo, co, callo = O.decompose(3, recs, targets, x0, tolerance=1e-8, max_inner=1000, max_outer=4, seed=17)
    calls, cost, xh = calls.cpu().numpy(), cost.cpu().numpy(), x.cpu().numpy()
    assert np.sum((cost < 1e-8) != (co < 1e-8)) <= 4
    assert abs(int((cost < 1e-8).sum()) - int((co < 1e-8).sum())) <= 3
    assert np.mean(cost < 1e-8) >= 0.85
    oc = np.array([O.cost(3, recs, xh[b], targets[b]) for b in range(64)])
    assert np.max(np.abs(oc - cost)) <= 1e-12


@pytest.mark.parametrize("fused", [True, False])
def test_config5_n12_application_against_the_reference(sqg, fused):
    """12 qubits, the benchmark's 2000-gate random circuit, 4 parameter vectors, applied to a
    4096 x 16 block (fused and one pass per gate); the reference's products are stored as a
    +-1 sketch S Y (8 x 16)."""
    from golden.inputs import config5_inputs

    d = _load("config5_n12.npz")
    c, theta, X, S, T = config5_inputs()
    assert np.array_equal(c.gate_records(), d["gates"])
    th = torch.from_numpy(theta).cuda()
    m = torch.from_numpy(np.broadcast_to(X, (4,) + X.shape).copy()).cuda()
    c.apply_to_device(th, m, fused=fused)
    torch.cuda.synchronize()
    Y = m.cpu().numpy()
    for b in range(4):
        got = S @ Y[b]
        scale = float(np.max(np.abs(Y[b])))
        err = float(np.max(np.abs(got - d["sketch"][b])))
        assert err <= RTOL * 4096 * scale, err


def test_config5_n12_cost_and_gradient_against_the_reference(sqg):
    """Cost (reference) and adjoint gradient (oracle sweep) of the same circuit on a 4096 x 16
    target with trace offset 1000, 4 parameter vectors."""
    from golden.inputs import config5_inputs

    d = _load("config5_n12.npz")
    c, theta, X, S, T = config5_inputs()
    ev = sqg.CostEvaluator(c, T, trace_offset=1000)
    cost, grad = ev.cost_grad(torch.from_numpy(theta).cuda())
    torch.cuda.synchronize()
    assert_close(cost.cpu().numpy(), d["cost"])
    assert_close(grad.cpu().numpy(), d["grad"])
