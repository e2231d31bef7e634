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


def all_gates_circuit(n, gates, rng):
    """`gates` gates drawn uniformly from all seven supported kinds on uniform qubits."""
    c = Circuit(n)
    for _ in range(gates):
        kind = int(rng.integers(7))
        t = int(rng.integers(n))
        ctl = int(rng.integers(n - 1)) if n > 1 else 0
        ctl = ctl + 1 if ctl >= t else ctl
        if kind == 0 or n == 1:
            c.add_U3(t)
        elif kind == 1:
            c.add_RX(t)
        elif kind == 2:
            c.add_RY(t)
        elif kind == 3:
            c.add_RZ(t)
        elif kind == 4:
            c.add_CNOT(t, ctl)
        elif kind == 5:
            c.add_CZ(t, ctl)
        else:
            c.add_CRY(t, ctl)
    return c


def qc_sim_circuit(n, levels=4):
    """The circuit of SQUANDER's state-vector simulation benchmark
    (examples/simulation/QC_sim_benchmark.py): `levels` sweeps over all qubit pairs
    c < t of [U3(t), U3(c), CRY(target t, control c)], then a U3 on qubit 0."""
    c = Circuit(n)
    for _ in range(levels):
        for ctl in range(n - 1):
            for t in range(ctl + 1, n):
                c.add_U3(t)
                c.add_U3(ctl)
                c.add_CRY(t, ctl)
    c.add_U3(0)
    return c


def _one_qubit(t, p, ps):
    if t == 7:  # U3 (theta/2, phi, lambda)
        c, s = np.cos(p[ps]), np.sin(p[ps])
        ep, el = np.exp(1j * p[ps + 1]), np.exp(1j * p[ps + 2])
        return np.array([[c, -el * s], [ep * s, ep * el * c]])
    c, s = np.cos(p[ps]), np.sin(p[ps])
    if t == 9:  # RX
        return np.array([[c, -1j * s], [-1j * s, c]])
    if t == 10:  # RZ
        return np.diag([c - 1j * s, c + 1j * s])
    return np.array([[c, -s], [s, c]], dtype=complex)  # RY, CRY


def circuit_matrix(circuit, theta):
    """Dense matrix of a small circuit (n <= 8) on the host, for building synthetic targets
    without a device round trip per target."""
    n = circuit.qbit_num
    N = 1 << n
    p = np.asarray(theta, dtype=np.float64)
    M = np.eye(N, dtype=complex)
    idx = np.arange(N)
    for t, tg, ctl, ps in circuit.gate_records():
        t, tg, ctl, ps = int(t), int(tg), int(ctl), int(ps)
        lo = idx[((idx >> tg) & 1) == 0]
        if ctl >= 0:
            lo = lo[((lo >> ctl) & 1) == 1]
        hi = lo | (1 << tg)
        if t == 5:  # CNOT
            M[[lo, hi]] = M[[hi, lo]]
            continue
        if t == 4:  # CZ
            M[hi] = -M[hi]
            continue
        g = _one_qubit(t, p, ps)
        x, y = M[lo].copy(), M[hi].copy()
        M[lo] = g[0, 0] * x + g[0, 1] * y
        M[hi] = g[1, 0] * x + g[1, 1] * y
    return M


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


def _u3_batch(p):
    """(S, 3) stored U3 parameters -> (S, 2, 2) matrices."""
    c, s = np.cos(p[:, 0]), np.sin(p[:, 0])
    ep, el = np.exp(1j * p[:, 1]), np.exp(1j * p[:, 2])
    g = np.empty((p.shape[0], 2, 2), dtype=complex)
    g[:, 0, 0], g[:, 0, 1], g[:, 1, 0], g[:, 1, 1] = c, -el * s, ep * s, ep * el * c
    return g


def _embed_batch(g, q, n):
    """Per-instance one-qubit gates g (S, 2, 2) on qubits q (S,) -> (S, 2^n, 2^n)."""
    S, N = g.shape[0], 1 << n
    idx = np.arange(N)
    bit = (idx[None, :] >> q[:, None]) & 1                      # (S, N)
    partner = idx[None, :] ^ (1 << q[:, None])                  # (S, N)
    M = np.zeros((S, N, N), dtype=complex)
    rows = np.arange(S)[:, None]
    M[rows, idx[None, :], idx[None, :]] = g[rows, bit, bit]
    M[rows, idx[None, :], partner] = g[rows, bit, 1 - bit]
    return M


def random_circuit_targets(count, n, rng, max_blocks=14):
    """Vectorised generator of products of random CNOT+U3 circuits: U3 on every qubit, then
    k ~ U{1..max_blocks} blocks of [CNOT(c, t), U3(c), U3(t)] with (c, t) uniform over
    ordered pairs and U3 angles U[0, 2 pi).  Returns (count, 2^n, 2^n) matrices U."""
    N = 1 << n
    U = np.broadcast_to(np.eye(N, dtype=complex), (count, N, N)).copy()
    for q in range(n):
        g = _u3_batch(rng.uniform(0, 2 * np.pi, (count, 3)))
        U = _embed_batch(g, np.full(count, q), n) @ U
    k = rng.integers(1, max_blocks + 1, count)
    pairs = np.array([(a, b) for a in range(n) for b in range(n) if a != b])
    idx = np.arange(N)
    for blk in range(max_blocks):
        act = k > blk
        if not act.any():
            break
        sel = pairs[rng.integers(len(pairs), size=count)]
        ctl, tgt = sel[:, 0], sel[:, 1]
        # CNOT as a row permutation: rows with the control bit set swap across the target bit
        src = np.where(((idx[None, :] >> ctl[:, None]) & 1) == 1, idx[None, :] ^ (1 << tgt[:, None]), idx[None, :])
        Up = np.take_along_axis(U, src[:, :, None], axis=1)
        g1 = _embed_batch(_u3_batch(rng.uniform(0, 2 * np.pi, (count, 3))), ctl, n)
        g2 = _embed_batch(_u3_batch(rng.uniform(0, 2 * np.pi, (count, 3))), tgt, n)
        Up = g2 @ (g1 @ Up)
        U = np.where(act[:, None, None], Up, U)
    return U


def haar_unitaries(count, dim, rng):
    a = rng.standard_normal((count, dim, dim)) + 1j * rng.standard_normal((count, dim, dim))
    q, r = np.linalg.qr(a)
    d = np.diagonal(r, axis1=1, axis2=2)
    phase = np.where(np.abs(d) > 0, d / np.abs(d), 1.0)
    return np.ascontiguousarray(q * phase[:, None, :], dtype=np.complex128)
