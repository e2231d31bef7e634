"""Inputs of the golden fixtures, rebuilt from their seeds by tests/golden/make_golden.py and by
the tests that compare against the fixtures (numpy's Generator streams are the same on every
platform, so only the stored outputs need to travel)."""
import importlib

import numpy as np

wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")


def config3_inputs():
    """10 qubits: 300 CNOT+U3 blocks over uniformly drawn ordered pairs (P = 1830), the
    angles of the target circuit, 64 parameter vectors and 32 gradient components per vector."""
    rng = np.random.default_rng(12)
    c = wl.cnot_u3_ansatz(10, 300, pairs="random", rng=rng)
    P = c.get_Parameter_Num()
    angles = rng.uniform(0, 2 * np.pi, P)
    theta = rng.uniform(0, 2 * np.pi, (64, P))
    pick = np.stack([np.sort(rng.choice(P, 32, replace=False)) for _ in range(64)])
    return c, angles, theta, pick


def config4_inputs():
    """64 of the 3-qubit benchmark targets (the first 32 Haar and the first 32 random-circuit
    ones of the 4096 the benchmark draws with seed 1234), as U^dagger, the 14-block ansatz and
    seeded start points."""
    rng = np.random.default_rng(1234)
    ansatz = wl.cnot_u3_ansatz(3, 14)
    U = wl.three_qubit_targets(4096, rng, wl.circuit_matrix)
    pick = np.r_[0:32, 2048:2080]
    targets = np.ascontiguousarray(np.conj(np.transpose(U[pick], (0, 2, 1))))
    x0 = np.random.default_rng(4321).uniform(0, 2 * np.pi, (64, ansatz.get_Parameter_Num()))
    return ansatz, targets, x0


def config5_inputs():
    """12 qubits: the benchmark's 2000-gate random circuit (seed 5), 4 parameter vectors, a
    4096 x 16 input block X, an 8 x 4096 +-1 sketch matrix S and a 4096 x 16 target T."""
    rng = np.random.default_rng(5)
    c = wl.random_gate_circuit(12, 2000, rng)
    P = c.get_Parameter_Num()
    theta = rng.uniform(0, 2 * np.pi, (4, P))
    r2 = np.random.default_rng(55)
    X = (r2.random((4096, 16)) - 0.5) + 1j * (r2.random((4096, 16)) - 0.5)
    sketch = 2.0 * r2.integers(0, 2, (8, 4096)) - 1.0
    T = (r2.random((4096, 16)) - 0.5) + 1j * (r2.random((4096, 16)) - 0.5)
    return c, theta, np.ascontiguousarray(X), sketch, np.ascontiguousarray(T)
