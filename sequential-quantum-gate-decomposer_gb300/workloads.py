"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: targets are Haar-random unitaries (QR of a seeded complex
Gaussian with the phase of diag(R) removed, as squander's tests/gates/test_circuit.py:86-95
builds them) or products of seeded random circuits, so that an exact solution exists.
"""
import numpy as np

from .circuit import Circuit


def haar_unitary(dim, rng):
    a = rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))
    q, r = np.linalg.qr(a)
    d = np.diag(r)
    phase = np.where(np.abs(d) > 0, d / np.abs(d), 1.0)
    return np.ascontiguousarray(q * phase, dtype=np.complex128)


def nearest_neighbour_pairs(n):
    """Ordered nearest-neighbour (control, target) pairs: (0,1), (1,0), (1,2), (2,1), ..."""
    out = []
    for q in range(n - 1):
        out += [(q, q + 1), (q + 1, q)]
    return out


def cnot_u3_ansatz(n, blocks, pairs=None, rng=None):
    """U3 on every qubit, then `blocks` x [CNOT(c, t), U3(c), U3(t)].

    pairs=None cycles through the ordered nearest-neighbour pairs; pairs="random" draws
    each (c, t) uniformly from all ordered pairs with `rng`."""
    c = Circuit(n)
    for q in range(n):
        c.add_U3(q)
    cyc = nearest_neighbour_pairs(n)
    allpairs = [(a, b) for a in range(n) for b in range(n) if a != b]
    for k in range(blocks):
        if pairs == "random":
            ctl, tgt = allpairs[rng.integers(len(allpairs))]
        elif pairs is None:
            ctl, tgt = cyc[k % len(cyc)]
        else:
            ctl, tgt = pairs[k % len(pairs)]
        c.add_CNOT(tgt, ctl)
        c.add_U3(ctl)
        c.add_U3(tgt)
    return c


def random_gate_circuit(n, gates, rng):
    """`gates` gates drawn uniformly from {U3, RY, CNOT, CZ, CRY} on uniform qubits."""
    c = Circuit(n)
    for _ in range(gates):
        kind = rng.integers(5)
        t = int(rng.integers(n))
        if kind == 0:
            c.add_U3(t)
        elif kind == 1:
            c.add_RY(t)
        else:
            ctl = int(rng.integers(n - 1))
            ctl = ctl + 1 if ctl >= t else ctl
            if kind == 2:
                c.add_CNOT(t, ctl)
            elif kind == 3:
                c.add_CZ(t, ctl)
            else:
                c.add_CRY(t, ctl)
    return c


def random_angles(P, rng, size=None):
    shape = (P,) if size is None else (size, P)
    return rng.uniform(0.0, 2 * np.pi, shape)


def three_qubit_targets(count, rng, matrix_fn):
    """Held-out 3-qubit targets U (not yet daggered): half Haar-random, half products of
    random circuits with a CNOT count uniform in 1..14 and U3 angles U[0, 2 pi).
    matrix_fn(circuit, theta) returns the circuit's 8x8 matrix."""
    out = np.empty((count, 8, 8), dtype=np.complex128)
    half = count // 2
    for i in range(half):
        out[i] = haar_unitary(8, rng)
    for i in range(half, count):
        k = int(rng.integers(1, 15))
        c = cnot_u3_ansatz(3, k, pairs="random", rng=rng)
        out[i] = matrix_fn(c, random_angles(c.get_Parameter_Num(), rng))
    return out
