"""Adaptive decomposition (adaptive.py): the circuit transformations of
N_Qubit_Decomposition_adaptive checked on the CPU through the oracle's circuit matrix (the fold
of a trivial block and the replacement of controlled rotations keep the operator, up to the
global phase the reference moves onto the target), the penalty and parameter bookkeeping, and
on the GPU whole decompositions."""
import importlib

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def ad():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.adaptive")


def _three_qubit(ad, sqg):
    U3, CRY = sqg.U3, sqg.CRY
    blocks = [[(U3, 0, -1), (U3, 1, -1), (CRY, 0, 1)], [(U3, 1, -1), (U3, 2, -1), (CRY, 1, 2)],
              [(U3, 0, -1), (U3, 2, -1), (CRY, 0, 2)], [(U3, 0, -1), (U3, 1, -1), (U3, 2, -1)]]
    return ad._Structure(3, blocks)


def _dec(ad, n=3):
    U = np.eye(1 << n, dtype=np.complex128)
    return ad.N_Qubit_Decomposition_adaptive(U, level_limit_max=2, config={"random_seed": 1})


def test_fold_of_a_trivial_block_keeps_the_operator(sqg, ad):
    s = _three_qubit(ad, sqg)
    rng = np.random.default_rng(3)
    x = rng.uniform(-3, 3, s.param_num())
    x[6] = 0.0  # block 0's CRY at the identity
    d = _dec(ad)
    x2, phase = d._fold_block(s, x, 0)
    assert np.all(x2[:6] == 0.0) and abs(abs(phase) - 1) < 1e-14
    before = O.get_matrix(3, s.records(), x)
    after = O.get_matrix(3, s.records(), x2)
    assert np.allclose(after * phase, before, atol=1e-12)
    # the circuit without the folded block computes the same operator
    red = s.without(0)
    assert np.allclose(O.get_matrix(3, red.records(), d._reduced(s, x2, 0)) * phase, before, atol=1e-12)


@pytest.mark.parametrize("angle", [0.0, np.pi / 2, -np.pi / 2, 0.7])
def test_replacement_of_controlled_rotations_keeps_the_operator(sqg, ad, angle):
    s = _three_qubit(ad, sqg)
    rng = np.random.default_rng(4)
    x = rng.uniform(-3, 3, s.param_num())
    x[6] = angle
    d = _dec(ad)
    t0 = d.Umtx.copy()
    s2, x2 = d._replace_trivial_cry(s, x)
    phase = d.Umtx[0, 0] / t0[0, 0]  # the factor moved onto the target (U^dagger)
    assert sqg.CRY not in [g[0] for g in s2.blocks[0]]
    assert x2.size == s2.param_num()
    # cost invariance: C_new (phase U^dagger) = C_old U^dagger
    assert np.allclose(O.get_matrix(3, s2.records(), x2) * phase, O.get_matrix(3, s.records(), x), atol=1e-12)


def test_penalty_and_parameter_bookkeeping(sqg, ad):
    s = _three_qubit(ad, sqg)
    x = np.zeros(s.param_num())
    d = _dec(ad)
    x[6], x[13], x[20] = 0.0, np.pi / 2, 0.7
    # identity CRY 0; the reference's CNOT test (|sin| < 0.999 with |cos| < 1e-3) never holds, so 2 each
    assert d._panelty(s, x) == 4
    assert d._theta_of_layer(s, x, 1) == pytest.approx(1.0) and d._theta_of_layer(s, x, 0) == 0.0
    r = d._reduced(s, np.arange(s.param_num(), dtype=float), 1)
    assert r.size == s.param_num() - 7 and r[6] == 6 and r[7] == 14
    layer = d._adaptive_layer()
    assert [(b[0][1], b[1][1]) for b in layer] == [(0, 1), (0, 2), (1, 2)]
    bad = ad.N_Qubit_Decomposition_adaptive(np.eye(8, dtype=np.complex128), level_limit_max=1, level_limit_min=2)
    with pytest.raises(ValueError, match="level_limit_min"):
        bad._initial(1e-8)


@pytest.mark.gpu
@pytest.mark.parametrize("n,blocks", [(3, 2), (2, 1)])
def test_adaptive_decomposition_reaches_tolerance(sqg, ad, n, blocks):
    torch = pytest.importorskip("torch")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    rng = np.random.default_rng(20 + n)
    c = wl.cnot_u3_ansatz(n, blocks)
    U = O.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    T = np.ascontiguousarray(U.conj().T)
    dec = sqg.N_Qubit_Decomposition_adaptive(T, level_limit_max=3, level_limit_min=1,
                                             config={"optimization_tolerance": 1e-8, "random_seed": 7})
    dec.Start_Decomposition()
    torch.cuda.synchronize()
    assert dec.get_Decomposition_Error() < 1e-8
    C = O.get_matrix(n, dec.get_Circuit().gate_records(), dec.get_Optimized_Parameters())
    assert abs(abs(np.trace(C @ T)) / (1 << n) - 1.0) < 1e-8  # up to the global phase moved onto the target
    gates = dec.get_Circuit().get_Gate_Nums()
    assert gates.get("CRY", 0) == 0  # finalised into CNOT / CZ constructions


def test_state_preparation_input_checks(sqg):
    with pytest.raises(Exception, match="numpy array"):
        sqg.N_Qubit_State_Preparation_adaptive([1, 0])
    with pytest.raises(Exception, match="complex"):
        sqg.N_Qubit_State_Preparation_adaptive(np.zeros(4))
    with pytest.raises(Exception, match="column vector"):
        sqg.N_Qubit_State_Preparation_adaptive(np.zeros((4, 2), dtype=np.complex128))
    sp = sqg.N_Qubit_State_Preparation_adaptive(np.ones(8, dtype=np.complex128) / np.sqrt(8), 3)
    assert sp.qbit_num == 3 and sp.level_limit == 3 and sp.get_Unitary().shape == (8, 1)


@pytest.mark.gpu
def test_state_preparation_maps_the_state_to_zero(sqg):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    psi = rng.standard_normal(8) + 1j * rng.standard_normal(8)
    psi = np.ascontiguousarray(psi / np.linalg.norm(psi))
    sp = sqg.N_Qubit_State_Preparation_adaptive(psi, level_limit_max=4, level_limit_min=1,
                                                config={"optimization_tolerance": 1e-8, "random_seed": 2})
    sp.Start_Decomposition()
    torch.cuda.synchronize()
    assert sp.get_Decomposition_Error() < 1e-8
    C = O.get_matrix(3, sp.get_Circuit().gate_records(), sp.get_Optimized_Parameters())
    assert abs(abs((C @ psi)[0]) - 1.0) < 1e-8


def test_stage_budgets_follow_the_reference_precedence(ad):
    """max_inner_iterations_bfgs / _adam, then the stage's own key, then max_inner_iterations,
    then the stage's value (N_Qubit_Decomposition_adaptive.cpp:574-616, 1269-1313)."""
    d = _dec(ad)
    assert [d._stage_budget(s, False, 93) for s in ("initial", "compression", "final")] == [10000, 100, 10000]
    assert [d._stage_budget(s, True, 852) for s in ("initial", "compression", "final")] == [10000000, 100000,
                                                                                              10000000]
    d.config = {"max_inner_iterations": 7, "max_inner_iterations_compression": 5}
    assert [d._stage_budget(s, False, 93) for s in ("initial", "compression", "final")] == [7, 5, 7]
    d.config["max_inner_iterations_adam"] = 3
    assert [d._stage_budget(s, True, 93) for s in ("initial", "compression", "final")] == [3, 3, 3]
    assert [d._stage_budget(s, False, 93) for s in ("initial", "compression", "final")] == [7, 5, 7]


@pytest.mark.gpu
def test_six_qubit_compression_candidates_run_in_one_adam_launch(sqg, ad):
    """At six qubits the candidates of a compression step (the circuit without one of its
    blocks) run as one sqg_decompose_structures_adam launch: each candidate's result equals, bit
    for bit, a batched ADAM run of its own structure from the same start with the same seed (the
    stage's settings: the compression budget from the config, one random shift), and the
    evaluations stop at that budget."""
    torch = pytest.importorskip("torch")
    import copy

    n, budget = 6, 60
    builder = ad.N_Qubit_Decomposition_adaptive(np.eye(64, dtype=np.complex128), config={"random_seed": 2})
    s = ad._Structure(n, builder._adaptive_layer()[:6] + [builder._final_layer()])
    rng = np.random.default_rng(61)
    theta = rng.uniform(0, 2 * np.pi, s.param_num())
    T = np.ascontiguousarray(O.get_matrix(n, s.records(), theta).conj().T)
    dec = ad.N_Qubit_Decomposition_adaptive(T, config={"optimization_tolerance": 1e-8, "random_seed": 9,
                                                       "max_inner_iterations_compression": budget})
    cands = [s.without(b) for b in range(5)]
    starts = [dec._reduced(s, theta, b) for b in range(5)]
    state = copy.deepcopy(dec.rng.bit_generator.state)
    out = dec._inner(cands, starts, "compression", 1e-8)
    replay = np.random.default_rng()
    replay.bit_generator.state = state
    seed = int(replay.integers(1 << 62))
    targets = torch.from_numpy(np.stack([T] * len(cands))).cuda()
    for k, cand in enumerate(cands):
        bd = sqg.BatchedDecomposer(cand.circuit(), tolerance=1e-8, max_calls=budget, max_outer=1, optimizer="ADAM",
                                   eta=1e-3, random_shift_count_max=1)
        xk, ck, ek = bd.run(targets, np.stack(starts), seed=seed)
        torch.cuda.synchronize()
        f, x, ev = out[k]
        assert float(ck[k]) == f and np.array_equal(xk[k].cpu().numpy(), x) and int(ek[k]) == ev
        assert ev <= budget
