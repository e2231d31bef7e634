"""Graph-driven single-target decompositions (one CUDA graph launch per decomposition): the ADAM
engine (sqg_decompose_adam_loop) against the oracle's restatement of it, BFGS
(sqg_decompose_bfgs_loop) against k_decompose and the host-driven BFGS, and the drop-in
Start_Decomposition on its device loops against its host-driven loops."""
import importlib

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def wl():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")


@pytest.fixture(scope="module")
def batched():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.batched")


def _one_cnot_circuit(sqg):
    c = sqg.Circuit(2)
    for q in (0, 1):
        c.add_U3(q)
    c.add_CNOT(1, 0)
    for q in (0, 1):
        c.add_U3(q)
    return c


@pytest.mark.parametrize("case", ["n6_exact", "n7_rect_offset", "n3_env", "n2_randomised"])
def test_graph_adam_follows_the_oracle(sqg, wl, batched, case):
    """Tile-kernel evaluation (n = 6, 7) and environment-matrix evaluation (n <= 5) inside the
    graph body; the same evaluation and randomisation counts as the oracle's engine and the
    same trajectory to rounding (to the same minimum where a randomisation fires)."""
    rng = np.random.default_rng({"n6_exact": 61, "n7_rect_offset": 71, "n3_env": 31, "n2_randomised": 21}[case])
    offset, variant, adaptive, iters = 0, O.FROBENIUS_NORM, True, 300
    if case == "n2_randomised":
        n, c, adaptive, iters = 2, _one_cnot_circuit(sqg), False, 3000
        T = np.ascontiguousarray(wl.haar_unitary(4, rng).conj().T)
    else:
        n = {"n6_exact": 6, "n7_rect_offset": 7, "n3_env": 3}[case]
        c = wl.cnot_u3_ansatz(n, 3 if n > 5 else 4)
        P = c.get_Parameter_Num()
        T = np.ascontiguousarray(O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, P)).conj().T)
        if case == "n7_rect_offset":
            offset = 32
            T = np.ascontiguousarray(T[:, offset:offset + 64])
        if case == "n3_env":
            variant = O.HILBERT_SCHMIDT_TEST
    P = c.get_Parameter_Num()
    x0 = rng.uniform(0, 2 * np.pi, P)
    x, cost, evals, shifts = batched.adam_decompose_graph(c, T, x0, tolerance=1e-8, max_iters=iters, eta=1e-3,
                                                          adaptive_eta=adaptive, seed=9, trace_offset=offset,
                                                          cost_variant=variant)
    torch.cuda.synchronize()
    xr, cr, er, sr = O.adam_decompose(n, c.gate_records(), T[None], x0[None], tolerance=1e-8, max_iters=iters,
                                      eta=1e-3, adaptive_eta=adaptive, seed=9, trace_offset=offset, variant=variant)
    assert int(shifts.item()) == sr[0]
    assert int(evals.item()) == er[0]
    if case == "n2_randomised":
        assert sr[0] >= 1  # the randomisation branch ran
        assert np.isclose(cost.item(), cr[0], rtol=1e-4)
    else:
        assert np.isclose(cost.item(), cr[0], rtol=1e-9, atol=1e-12)
        assert np.allclose(x.cpu().numpy(), xr[0], atol=1e-8)


def test_graph_adam_outer_iterations_chain_engine_calls(sqg, wl, batched):
    """max_outer engine calls inside one graph launch equal successive single calls, each
    restarted at the best point with the running minimum; also on a side stream."""
    rng = np.random.default_rng(5)
    c = _one_cnot_circuit(sqg)
    T = np.ascontiguousarray(wl.haar_unitary(4, rng).conj().T)  # not reachable with one CNOT
    x0 = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        x3, c3, e3, s3 = batched.adam_decompose_graph(c, T, x0, max_iters=40, max_outer=3, adaptive_eta=False,
                                                      seed=3, stream=s)
    s.synchronize()
    assert int(e3.item()) == 120 and int(s3.item()) == 0
    x, cur = x0, None
    for _ in range(3):
        xd, cd, ed, _sd = batched.adam_decompose_graph(c, T, x, max_iters=40, adaptive_eta=False, seed=3,
                                                       current_minimum=cur)
        x, cur = xd.cpu().numpy(), float(cd.item())
        assert int(ed.item()) == 40
    assert cur == float(c3.item())
    assert np.array_equal(x, x3.cpu().numpy())


def test_graph_adam_rejects_bad_requests(sqg, wl, batched):
    lib = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    c = wl.cnot_u3_ansatz(3, 2)
    T = np.eye(8, dtype=np.complex128)
    x0 = np.zeros(c.get_Parameter_Num())
    with pytest.raises(lib.SQGError, match="iteration limits"):
        batched.adam_decompose_graph(c, T, x0, max_iters=0)
    with pytest.raises(lib.SQGError, match="trace offset"):
        batched.adam_decompose_graph(c, T[:, :4], x0, trace_offset=6)
    with pytest.raises(ValueError):
        batched.adam_decompose_graph(c, T, np.zeros(3))
    h = c.native().handle
    need = lib.lib().sqg_adam_loop_workspace_bytes(h, 8)
    ws = torch.empty(need // 2, dtype=torch.uint8, device="cuda")
    t = torch.from_numpy(T).cuda()
    x = torch.zeros(c.get_Parameter_Num(), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
    st = lib.lib().sqg_decompose_adam_loop(h, t.data_ptr(), 8, 0, 0, x.data_ptr(), out.data_ptr(), cnt.data_ptr(),
                                           None, 1e-8, 10, 1e-3, 1, 100, 2500000, 1, 1e300, 0, ws.data_ptr(),
                                           ws.numel(), torch.cuda.current_stream().cuda_stream)
    assert st == lib.SQG_ERR_WORKSPACE


@pytest.mark.parametrize("n,optimizer", [(3, "BFGS"), (2, "BFGS"), (6, "ADAM"), (4, "ADAM")])
def test_dropin_device_loops_match_host_loops(sqg, wl, n, optimizer):
    """Start_Decomposition on the device loops (ADAM: one graph launch per outer iteration;
    BFGS up to five qubits: one k_decompose launch) and on the host-driven loops from the
    same start and seeds: ADAM follows the same trajectory; BFGS reaches the tolerance."""
    rng = np.random.default_rng(100 + n)
    c = wl.cnot_u3_ansatz(n, 3 if n > 2 else 2)
    P = c.get_Parameter_Num()
    xt = rng.uniform(0, 2 * np.pi, P)
    T = np.ascontiguousarray(O.get_matrix(n, c.gate_records(), xt).conj().T)
    start = xt + 0.05 * rng.standard_normal(P)
    runs = []
    for host in (False, True):
        cfg = {"random_seed": 11, "optimization_tolerance": 1e-8}
        if optimizer == "ADAM":
            cfg["max_inner_iterations"] = 400
        dec = sqg.N_Qubit_Decomposition_custom(T, config=cfg)
        dec.set_Gate_Structure(c)
        dec.set_Optimizer(optimizer)
        dec.max_outer_iterations = 2
        dec._host_loops = host
        dec.set_Optimized_Parameters(start)
        dec.Start_Decomposition()
        runs.append((dec.get_Decomposition_Error(), dec.get_Num_of_Iters(), dec.get_Optimized_Parameters()))
    (fd, nd, xd), (fh, nh, xh) = runs
    if optimizer == "ADAM":
        assert nd == nh
        assert np.isclose(fd, fh, rtol=1e-7, atol=1e-13)
        assert np.allclose(xd, xh, atol=1e-7)
    else:
        assert fd < 1e-8 and fh < 1e-8


@pytest.mark.parametrize("n,blocks,max_outer,loops,early", [(3, 4, 4, 1, True), (3, 6, 2, 3, False), (4, 3, 2, 2, True)])
def test_graph_bfgs_equals_k_decompose(sqg, wl, batched, n, blocks, max_outer, loops, early):
    """Up to five qubits the graph loop evaluates with the same kernel and reduction order as
    k_decompose: every run, restart and perturbation gives the same bits."""
    rng = np.random.default_rng(300 + 10 * n + blocks)
    c = wl.cnot_u3_ansatz(n, blocks)
    P = c.get_Parameter_Num()
    T = np.ascontiguousarray(wl.haar_unitary(1 << n, rng).conj().T)  # not reachable: all runs happen
    x0 = rng.uniform(0, 2 * np.pi, P)
    dec = sqg.BatchedDecomposer(c, tolerance=1e-8, max_calls=200, max_outer=max_outer, iteration_loops=loops,
                                stop_at_tolerance=early)
    xk, ck, nk = dec.run(T[None], x0[None], seed=21)
    xg, cg, ng, ig = batched.bfgs_decompose_graph(c, T, x0, tolerance=1e-8, max_calls=200, max_outer=max_outer,
                                                  iteration_loops=loops, stop_at_tolerance=early, seed=21)
    torch.cuda.synchronize()
    assert int(ng.item()) == int(nk[0].item()) and int(ig.item()) == int(dec.iters[0].item())
    assert float(cg.item()) == float(ck[0].item())
    assert torch.equal(xg, xk[0])
    assert int(ng.item()) >= max_outer * loops


@pytest.mark.parametrize("n,blocks,cols,offset", [(6, 4, 64, 0), (6, 25, 64, 0), (7, 6, 48, 64)])
def test_graph_bfgs_above_five_qubits_follows_host_bfgs(sqg, wl, batched, n, blocks, cols, offset):
    """Tile-kernel evaluation in the graph body (P = 42 on 64 threads, P = 168 on 256, and a
    rectangular target with a trace offset): one BFGS run follows the host-driven BFGS_Powell
    restatement over the same cost and gradient."""
    optim = importlib.import_module("sequential-quantum-gate-decomposer_gb300.optim")
    rng = np.random.default_rng(600 + blocks)
    c = wl.cnot_u3_ansatz(n, blocks)
    P = c.get_Parameter_Num()
    T = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, P)).conj().T
    T = np.ascontiguousarray(T[:, offset:offset + cols])
    x0 = rng.uniform(0, 2 * np.pi, P)
    ev = sqg.CostEvaluator(c, T, trace_offset=offset)

    def fg(x):
        cost, grad = ev.cost_grad(torch.from_numpy(x).cuda())
        return float(cost.item()), grad.reshape(-1).cpu().numpy()

    xh = x0.copy()
    fh, nh = optim.bfgs_powell(fg, xh, 40)
    xg, cg, ng, _ = batched.bfgs_decompose_graph(c, T, x0, max_calls=40, max_outer=1, iteration_loops=1,
                                                 stop_at_tolerance=False, seed=1, trace_offset=offset)
    torch.cuda.synchronize()
    assert int(ng.item()) == nh
    assert np.isclose(float(cg.item()), fh, rtol=1e-7, atol=1e-12)
    assert np.allclose(xg.cpu().numpy(), xh, atol=1e-6)


def test_dropin_bfgs_above_five_qubits_on_the_device(sqg, wl):
    rng = np.random.default_rng(66)
    n, c = 6, wl.cnot_u3_ansatz(6, 3)
    P = c.get_Parameter_Num()
    xt = rng.uniform(0, 2 * np.pi, P)
    T = np.ascontiguousarray(O.get_matrix(n, c.gate_records(), xt).conj().T)
    dec = sqg.N_Qubit_Decomposition_custom(T, config={"optimization_tolerance": 1e-8, "random_seed": 3})
    dec.set_Gate_Structure(c)
    dec.set_Optimizer("BFGS")
    dec.max_outer_iterations = 4
    dec.set_Optimized_Parameters(xt + 0.05 * rng.standard_normal(P))
    dec.Start_Decomposition()
    assert dec.get_Decomposition_Error() < 1e-8
    assert abs(O.cost(n, c.gate_records(), dec.get_Optimized_Parameters(), T)) < 1e-8
