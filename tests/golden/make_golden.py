"""Generates tests/golden/umtx4_golden.npz from the reference's own 4-qubit test target
(data/Umtx.mat of the SQUANDER tree, loaded by its tests/decomposition/test_Unitary.py) with
the oracle: the decomposer's target U^dagger, the 40-block nearest-neighbour CNOT+U3 ansatz of
the 4-qubit benchmark configuration, seeded parameters, and the oracle's cost and gradient for
the FROBENIUS_NORM, HILBERT_SCHMIDT_TEST and INFIDELITY variants (plus a trace-offset case).

Run once in a checkout that has the reference tree next to it:
    python tests/golden/make_golden.py /path/to/sequential-quantum-gate-decomposer/data/Umtx.mat
"""
import os
import sys

import numpy as np
import scipy.io

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def ansatz_records(n, blocks):
    recs, p = [], 0
    for q in range(n):
        recs.append((O.U3, q, -1, p))
        p += 3
    pairs = []
    for q in range(n - 1):
        pairs += [(q, q + 1), (q + 1, q)]
    for k in range(blocks):
        c, t = pairs[k % len(pairs)]
        recs.append((O.CNOT, t, c, p))
        recs.append((O.U3, c, -1, p))
        p += 3
        recs.append((O.U3, t, -1, p))
        p += 3
    return np.asarray(recs, dtype=np.int32), p


def main(path):
    U = scipy.io.loadmat(path)["Umtx"].astype(np.complex128)
    target = np.ascontiguousarray(U.conj().T)
    recs, P = ansatz_records(4, 40)
    rng = np.random.default_rng(20241203)
    theta = rng.uniform(0, 2 * np.pi, (3, P))
    out = {"target": target, "gates": recs, "theta": theta}
    for name, v in (("frob", O.FROBENIUS_NORM), ("hs", O.HILBERT_SCHMIDT_TEST), ("infid", O.INFIDELITY)):
        c, g = O.batch(4, recs, theta, target, variant=v, with_grad=True, nthreads=1)
        out["cost_" + name] = c
        out["grad_" + name] = g
    sub = np.ascontiguousarray(U[4:12, :].conj().T)
    c, g = O.batch(4, recs, theta, sub, trace_offset=4, with_grad=True, nthreads=1)
    out["target_offset4"] = sub
    out["cost_offset4"] = c
    out["grad_offset4"] = g
    np.savez_compressed(os.path.join(HERE, "umtx4_golden.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1])
