"""OpenQASM 2.0 input (qasm.py) against an independent dense restatement of the qelib1 / Qiskit
gate definitions, on the CPU through the oracle's circuit matrix; and the partitioning of a
QASM program (the reference's test_CorrectnessOfPartitionedCircuit with a program given as
text)."""
import cmath
import importlib
import math

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def qasm():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.qasm")


def _u3(t, p, l):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -cmath.exp(1j * l) * s], [cmath.exp(1j * p) * s, cmath.exp(1j * (p + l)) * c]])


ONE = {
    "h": lambda: np.array([[1, 1], [1, -1]]) / math.sqrt(2), "x": lambda: np.array([[0, 1], [1, 0]]),
    "y": lambda: np.array([[0, -1j], [1j, 0]]), "z": lambda: np.diag([1, -1]), "s": lambda: np.diag([1, 1j]),
    "sdg": lambda: np.diag([1, -1j]), "t": lambda: np.diag([1, cmath.exp(1j * math.pi / 4)]),
    "tdg": lambda: np.diag([1, cmath.exp(-1j * math.pi / 4)]),
    "sx": lambda: 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]),
    "sxdg": lambda: 0.5 * np.array([[1 - 1j, 1 + 1j], [1 + 1j, 1 - 1j]]),
}
PAR1 = {
    "rx": lambda a: np.array([[math.cos(a / 2), -1j * math.sin(a / 2)], [-1j * math.sin(a / 2), math.cos(a / 2)]]),
    "ry": lambda a: np.array([[math.cos(a / 2), -math.sin(a / 2)], [math.sin(a / 2), math.cos(a / 2)]]),
    "rz": lambda a: np.diag([cmath.exp(-0.5j * a), cmath.exp(0.5j * a)]),
    "u1": lambda a: np.diag([1, cmath.exp(1j * a)]), "p": lambda a: np.diag([1, cmath.exp(1j * a)]),
}


def _full(n, ops):
    """Dense operator of [(2x2 or controlled 2x2 matrix, target, controls)] (qubit q = bit q)."""
    N = 1 << n
    U = np.eye(N, dtype=complex)
    for m, t, ctrls in ops:
        G = np.eye(N, dtype=complex)
        for i in range(N):
            if any(not (i >> c) & 1 for c in ctrls):
                continue
            if (i >> t) & 1:
                continue
            j = i | (1 << t)
            G[i, i], G[i, j], G[j, i], G[j, j] = m[0, 0], m[0, 1], m[1, 0], m[1, 1]
        U = G @ U
    return U


def test_qasm_matches_dense_gate_definitions(sqg, qasm):
    rng = np.random.default_rng(5)
    n = 4
    lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', "qreg a[2];", "qreg b[2];", "creg c[4];",
             "gate mix(t) p, q { ry(t) p; cx p, q; rz(t/2) q; }"]
    ops = []
    names = [("a", 0), ("a", 1), ("b", 0), ("b", 1)]
    for _ in range(60):
        k = rng.integers(6)
        q0, q1, q2 = rng.permutation(n)[:3]
        r = lambda q: "%s[%d]" % names[q]
        if k == 0:
            g = list(ONE)[rng.integers(len(ONE))]
            lines.append("%s %s;" % (g, r(q0)))
            ops.append((ONE[g](), q0, []))
        elif k == 1:
            g = list(PAR1)[rng.integers(len(PAR1))]
            a = float(rng.uniform(-4, 4))
            lines.append("%s(%r) %s;" % (g, a, r(q0)))
            ops.append((PAR1[g](a), q0, []))
        elif k == 2:
            t, p, l = map(float, rng.uniform(-4, 4, 3))
            lines.append("u3(%r, %r, %r) %s;" % (t, p, l, r(q0)))
            ops.append((_u3(t, p, l), q0, []))
        elif k == 3:
            g = ["cx", "cz", "cy", "ch"][rng.integers(4)]
            m = {"cx": ONE["x"](), "cz": ONE["z"](), "cy": ONE["y"](), "ch": ONE["h"]()}[g]
            lines.append("%s %s, %s;" % (g, r(q0), r(q1)))
            ops.append((m, q1, [q0]))
        elif k == 4:
            g = ["cry", "crz", "crx", "cu1", "cp"][rng.integers(5)]
            a = float(rng.uniform(-4, 4))
            m = {"cry": PAR1["ry"], "crz": PAR1["rz"], "crx": PAR1["rx"], "cu1": PAR1["u1"], "cp": PAR1["p"]}[g](a)
            lines.append("%s(%r) %s, %s;" % (g, a, r(q0), r(q1)))
            ops.append((m, q1, [q0]))
        else:
            g = ["ccx", "swap", "cswap", "cu3", "mix", "u2"][rng.integers(6)]
            if g == "ccx":
                lines.append("ccx %s, %s, %s;" % (r(q0), r(q1), r(q2)))
                ops.append((ONE["x"](), q2, [q0, q1]))
            elif g == "swap":
                lines.append("swap %s, %s;" % (r(q0), r(q1)))
                ops += [(ONE["x"](), q1, [q0]), (ONE["x"](), q0, [q1]), (ONE["x"](), q1, [q0])]
            elif g == "cswap":
                lines.append("cswap %s, %s, %s;" % (r(q0), r(q1), r(q2)))
                ops += [(ONE["x"](), q1, [q2]), (ONE["x"](), q2, [q0, q1]), (ONE["x"](), q1, [q2])]
            elif g == "cu3":
                t, p, l = map(float, rng.uniform(-4, 4, 3))
                lines.append("cu3(%r, %r, %r) %s, %s;" % (t, p, l, r(q0), r(q1)))
                ops.append((_u3(t, p, l), q1, [q0]))
            elif g == "mix":
                a = float(rng.uniform(-4, 4))
                lines.append("mix(%r) %s, %s;" % (a, r(q0), r(q1)))
                ops += [(PAR1["ry"](a), q0, []), (ONE["x"](), q1, [q0]), (PAR1["rz"](a / 2), q1, [])]
            else:
                p, l = map(float, rng.uniform(-4, 4, 2))
                lines.append("u2(%r, %r) %s;  // comment" % (p, l, r(q0)))
                ops.append((_u3(math.pi / 2, p, l), q0, []))
    lines += ["barrier a;", "measure a[0] -> c[0];", "x b;"]  # register broadcast
    ops += [(ONE["x"](), 2, []), (ONE["x"](), 3, [])]
    circ, params, phase = qasm.qasm_to_circuit("\n".join(lines))
    assert circ.get_Qbit_Num() == n and params.size == circ.get_Parameter_Num()
    got = np.exp(1j * phase) * O.get_matrix(n, circ.gate_records(), params)
    assert np.allclose(got, _full(n, ops), atol=1e-12)


def test_qasm_expressions_and_errors(sqg, qasm):
    c, p, ph = qasm.qasm_to_circuit("OPENQASM 2.0;\nqreg q[1];\nrz(-pi/4 + 2*sin(pi/6)^2) q[0];\n")
    assert np.isclose(p[0], (-math.pi / 4 + 0.5) / 2) and ph == 0.0
    for bad in ("OPENQASM 2.0;\nqreg q[1];\nfoo q[0];\n", "OPENQASM 2.0;\nqreg q[1];\nrx(__import__) q[0];\n",
                "OPENQASM 2.0;\nqreg q[1];\nx q[3];\n"):
        with pytest.raises(ValueError):
            qasm.qasm_to_circuit(bad)


def test_partition_qasm_program_keeps_the_operator(sqg, qasm, tmp_path):
    rng = np.random.default_rng(9)
    n = 6
    lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', "qreg q[%d];" % n]
    for _ in range(80):
        a, b = rng.permutation(n)[:2]
        lines.append(["h q[%d];" % a, "cx q[%d],q[%d];" % (a, b), "rz(%r) q[%d];" % (float(rng.uniform(-3, 3)), a),
                      "cz q[%d],q[%d];" % (a, b)][rng.integers(4)])
    f = tmp_path / "prog.qasm"
    f.write_text("\n".join(lines))
    circ, params, _ = qasm.qasm_to_squander_circuit(str(f))
    pc, pparams, parts = qasm.PartitionCircuitQasm(str(f), 4)
    assert pc.get_Parameter_Num() == params.size
    assert np.allclose(O.get_matrix(n, circ.gate_records(), params), O.get_matrix(n, pc.gate_records(), pparams),
                       atol=1e-12)
