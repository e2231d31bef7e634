"""The reference's decomposition-level tests on its own 4-qubit target data/Umtx.mat (the IBM
challenge unitary, kept in tests/golden/umtx4_golden.npz as U^dagger), restated.  The reference
files rebuild the found circuit's matrix through Qiskit (get_Qiskit_Circuit,
utils.get_unitary_from_qiskit_circuit), which is not in this image; the oracle's circuit matrix
takes that role.  Every check keeps the reference's error measure and bound:
Re tr(2 I - P - P^dagger) / 2 < 1e-3 with P = U D^dagger, its global phase taken off by P[0, 0].

  tests/decomposition/test_IBM.py          adaptive (square and 14-row input), tree search,
                                           tabu search
  tests/decomposition/test_Compression.py  the stepwise adaptive calls with the file's config
                                           (full: initial, compression, final; no compression)
  tests/decomposition/test_Unitary.py,     get/set of the target and of the global phase
  test_Global_Phase.py
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
COMPRESSION_CONFIG = {"max_outer_iterations": 10, "max_inner_iterations": 300000,
                      "max_inner_iterations_compression": 10000, "max_inner_iterations_final": 1000,
                      "randomized_adaptive_layers": 1, "export_circuit_2_binary": 1,
                      "optimization_tolerance": 1e-8}


@pytest.fixture(scope="module")
def umtx():
    d = np.load(os.path.join(HERE, "golden", "umtx4_golden.npz"))
    return np.ascontiguousarray(d["target"].conj().T)  # data/Umtx.mat


def _error(U, D):
    P = U @ D.conj().T
    P = P * np.exp(-1j * np.angle(P[0, 0]))
    M = np.eye(P.shape[0]) * 2 - P - P.conj().T
    return float(np.real(np.trace(M)) / 2)


def _found(dec):
    return O.get_matrix(4, dec.get_Circuit().gate_records(), dec.get_Optimized_Parameters())


def _random_parameters(dec):
    rng = np.random.default_rng(42)
    dec.set_Optimized_Parameters(rng.random(dec.get_Parameter_Num()) * 2 * np.pi)


@pytest.mark.gpu
def test_ibm_challenge_adaptive(sqg, umtx):
    dec = sqg.N_Qubit_Decomposition_adaptive(umtx.conj().T, level_limit_max=5, level_limit_min=0,
                                             config={"random_seed": 42})
    _random_parameters(dec)
    dec.Start_Decomposition()
    assert _error(umtx, _found(dec)) < 1e-3


@pytest.mark.gpu
def test_ibm_challenge_adaptive_rectangular_input(sqg, umtx):
    U = np.ascontiguousarray(umtx[0:14, :])
    dec = sqg.N_Qubit_Decomposition_adaptive(np.ascontiguousarray(U.conj().T), level_limit_max=5,
                                             level_limit_min=0, config={"random_seed": 42})
    _random_parameters(dec)
    dec.Start_Decomposition()
    assert _error(U, _found(dec)[0:14, :]) < 1e-3


@pytest.mark.gpu
def test_ibm_challenge_tree_search(sqg, umtx):
    """Also the CNOT count: the reference's own search (both modes, run on this target for
    tests/golden/tree_search_ref.npz) needs 4 CNOTs."""
    d = np.load(os.path.join(HERE, "golden", "tree_search_ref.npz"))
    k = int(np.flatnonzero(d["generating_cnots"] < 0)[0])
    dec = sqg.N_Qubit_Decomposition_Tree_Search(umtx.conj().T, config={"random_seed": 42})
    dec.Start_Decomposition()
    assert _error(umtx, _found(dec)) < 1e-3
    assert len(dec.best_cnot_sequence) == int(d["default_cnots"][k]) == int(d["level_cnots"][k])


@pytest.mark.gpu
def test_ibm_challenge_tabu_search(sqg, umtx):
    dec = sqg.N_Qubit_Decomposition_Tabu_Search(umtx.conj().T, config={"random_seed": 42})
    dec.Start_Decomposition()
    assert _error(umtx, _found(dec)) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("levels,compress", [(2, True), (3, False)])
def test_ibm_challenge_stepwise_adaptive(sqg, umtx, levels, compress):
    """test_IBM_Chellenge_full (two levels: initial circuit, compression, finalisation) and
    test_IBM_Chellenge_no_compression (three levels: initial circuit, finalisation), with the
    file's config."""
    dec = sqg.N_Qubit_Decomposition_adaptive(umtx.conj().T, config=dict(COMPRESSION_CONFIG, random_seed=42))
    for _ in range(levels):
        dec.add_Adaptive_Layers()
    dec.add_Finalyzing_Layer_To_Gate_Structure()
    _random_parameters(dec)
    dec.get_Initial_Circuit()
    if compress:
        dec.Compress_Circuit()
    dec.Finalize_Circuit()
    assert _error(umtx, _found(dec)) < 1e-3
    assert dec.get_Circuit().get_Gate_Nums().get("CRY", 0) == 0


def test_target_and_global_phase_accessors(sqg, umtx):
    """test_Unitary.py and test_Global_Phase.py."""
    dec = sqg.N_Qubit_Decomposition_adaptive(umtx.conj().T, level_limit_max=5, level_limit_min=0)
    U = dec.get_Unitary()
    assert np.sum(np.abs(U - umtx.conj().T)) < 1e-5
    U[0, 0] = 1
    dec.set_Unitary(U)
    assert dec.get_Unitary()[0, 0] == 1
    dec = sqg.N_Qubit_Decomposition_adaptive(umtx.conj().T, level_limit_max=5, level_limit_min=0)
    assert abs(dec.get_Global_Phase()) < 2 * np.pi
    before = dec.get_Unitary()
    angle = np.pi / 3
    dec.set_Global_Phase(angle)
    factor = np.sqrt(2) * np.cos(angle) + 1j * np.sqrt(2) * np.sin(angle)
    dec.apply_Global_Phase_Factor()
    assert abs(dec.get_Global_Phase()) < 1e-8
    assert np.sum(np.abs(before * factor - dec.get_Unitary())) < 1e-5
