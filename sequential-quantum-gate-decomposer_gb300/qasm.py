"""OpenQASM 2.0 input: the drop-in for squander.utils.qasm_to_squander_circuit
(squander/utils.py:122-160) and squander.partitioning.partition.PartitionCircuitQasm
(squander/partitioning/partition.py:94-117).

The reference parses the file with Qiskit, transpiles gates outside SQUANDER's gate set and
converts the result (squander/IO_interfaces/Qiskit_IO.py).  Qiskit is not part of this engine;
this module reads OpenQASM 2.0 itself (qreg declarations, qelib1 gates, user `gate`
definitions, parameter expressions with pi and the usual functions; barrier, measure, reset
and creg are ignored) and maps every gate onto the engine's gate set U3 / RX / RY / RZ / CNOT /
CZ / CRY.  Gates of fixed angles become U3 or RZ gates whose angles go into the returned
parameter vector, in SQUANDER's storage convention (theta/2 for U3's theta and for RX / RY /
RZ / CRY).  Controlled and compound gates are expanded into exact CNOT sequences (the qelib1
definitions, e.g. Nielsen & Chuang section 4.3).  rz is Qiskit's diag(e^{-i t/2}, e^{i t/2})
(the gate the reference's Qiskit parser produces), u1 / p is diag(1, e^{i t}).  sx and sxdg map
to RX(+-pi/2) up to the global phase e^{+-i pi/4}; that phase is accumulated and returned, so
that exp(i * phase) * C(params) is the operator of the file.
"""
import ast
import math
import operator
import re

import numpy as np

from .circuit import Circuit

_PI = math.pi
_FUNCS = {"sin": math.sin, "cos": math.cos, "tan": math.tan, "exp": math.exp, "ln": math.log, "sqrt": math.sqrt,
          "asin": math.asin, "acos": math.acos, "atan": math.atan}
_BINOPS = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
           ast.Pow: operator.pow}


def _eval_expr(text, env):
    """Value of an OpenQASM parameter expression (numbers, pi, parameters in env, + - * / ^,
    unary minus, sin cos tan exp ln sqrt)."""
    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return float(node.value)
        if isinstance(node, ast.Name):
            if node.id == "pi":
                return _PI
            if node.id in env:
                return env[node.id]
            raise ValueError("unknown name %r in a parameter expression" % node.id)
        if isinstance(node, ast.BinOp) and type(node.op) in _BINOPS:
            return _BINOPS[type(node.op)](ev(node.left), ev(node.right))
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id in _FUNCS:
            return _FUNCS[node.func.id](*[ev(a) for a in node.args])
        raise ValueError("unsupported parameter expression %r" % text)
    return ev(ast.parse(text.replace("^", "**"), mode="eval"))


def _split_args(s):
    """Top-level comma split (parentheses may nest)."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


class _Builder:
    """Emits engine gates with their parameters (SQUANDER storage) and the global phase."""

    def __init__(self, n):
        self.circuit = Circuit(n)
        self.params = []
        self.phase = 0.0

    def u3(self, q, theta, phi, lam):
        self.circuit.add_U3(q)
        self.params += [theta / 2, phi, lam]

    def rx(self, q, theta):
        self.circuit.add_RX(q)
        self.params.append(theta / 2)

    def ry(self, q, theta):
        self.circuit.add_RY(q)
        self.params.append(theta / 2)

    def rz(self, q, theta):
        self.circuit.add_RZ(q)
        self.params.append(theta / 2)

    def p(self, q, lam):  # diag(1, e^{i lam}) = U3(0, 0, lam)
        self.u3(q, 0.0, 0.0, lam)

    def cx(self, c, t):
        self.circuit.add_CNOT(t, c)

    def cz(self, c, t):
        self.circuit.add_CZ(t, c)

    def cry(self, c, t, theta):
        self.circuit.add_CRY(t, c)
        self.params.append(theta / 2)

    # ---- compound gates, exact (phases tracked) -------------------------------------------
    def h(self, q):
        self.u3(q, _PI / 2, 0.0, _PI)

    def cp(self, c, t, lam):  # diag(1, 1, 1, e^{i lam})
        self.p(c, lam / 2)
        self.cx(c, t)
        self.p(t, -lam / 2)
        self.cx(c, t)
        self.p(t, lam / 2)

    def crz(self, c, t, lam):  # diag(1, 1, e^{-i lam/2}, e^{i lam/2})
        self.rz(t, lam / 2)
        self.cx(c, t)
        self.rz(t, -lam / 2)
        self.cx(c, t)

    def crx(self, c, t, theta):  # H-conjugated CRZ on the target
        self.h(t)
        self.crz(c, t, theta)
        self.h(t)

    def cu3(self, c, t, theta, phi, lam):  # controlled U3 (Nielsen & Chuang figure 4.6)
        self.p(c, (lam + phi) / 2)
        self.p(t, (lam - phi) / 2)
        self.cx(c, t)
        self.u3(t, -theta / 2, 0.0, -(phi + lam) / 2)
        self.cx(c, t)
        self.u3(t, theta / 2, phi, 0.0)

    def cy(self, c, t):  # S^dagger . X . S on the target
        self.p(t, -_PI / 2)
        self.cx(c, t)
        self.p(t, _PI / 2)

    def ch(self, c, t):  # H = RY(pi/4) Z RY(-pi/4), so CH = RY(pi/4)_t CZ RY(-pi/4)_t
        self.ry(t, -_PI / 4)
        self.cz(c, t)
        self.ry(t, _PI / 4)

    def swap(self, a, b):
        self.cx(a, b)
        self.cx(b, a)
        self.cx(a, b)

    def ccx(self, a, b, t):  # Toffoli with six CNOTs (Nielsen & Chuang figure 4.9)
        self.h(t)
        self.cx(b, t)
        self.p(t, -_PI / 4)
        self.cx(a, t)
        self.p(t, _PI / 4)
        self.cx(b, t)
        self.p(t, -_PI / 4)
        self.cx(a, t)
        self.p(b, _PI / 4)
        self.p(t, _PI / 4)
        self.h(t)
        self.cx(a, b)
        self.p(a, _PI / 4)
        self.p(b, -_PI / 4)
        self.cx(a, b)

    def cswap(self, c, a, b):
        self.cx(b, a)
        self.ccx(c, a, b)
        self.cx(b, a)

    def emit(self, name, args, qs):
        """One qelib1 gate; False if the name is not a qelib1 gate."""
        g = name.lower()
        one = {
            "u3": lambda: self.u3(qs[0], *args), "u": lambda: self.u3(qs[0], *args),
            "u2": lambda: self.u3(qs[0], _PI / 2, args[0], args[1]),
            "u1": lambda: self.p(qs[0], args[0]), "p": lambda: self.p(qs[0], args[0]),
            "rx": lambda: self.rx(qs[0], args[0]), "ry": lambda: self.ry(qs[0], args[0]),
            "rz": lambda: self.rz(qs[0], args[0]),
            "h": lambda: self.h(qs[0]), "x": lambda: self.u3(qs[0], _PI, 0.0, _PI),
            "y": lambda: self.u3(qs[0], _PI, _PI / 2, _PI / 2), "z": lambda: self.p(qs[0], _PI),
            "s": lambda: self.p(qs[0], _PI / 2), "sdg": lambda: self.p(qs[0], -_PI / 2),
            "t": lambda: self.p(qs[0], _PI / 4), "tdg": lambda: self.p(qs[0], -_PI / 4),
            "id": lambda: None,
        }
        if g in one:
            one[g]()
            return True
        if g in ("sx", "sxdg"):  # sx = e^{i pi/4} RX(pi/2)
            sgn = 1.0 if g == "sx" else -1.0
            self.rx(qs[0], sgn * _PI / 2)
            self.phase += sgn * _PI / 4
            return True
        two = {
            "cx": lambda: self.cx(qs[0], qs[1]), "cnot": lambda: self.cx(qs[0], qs[1]),
            "cz": lambda: self.cz(qs[0], qs[1]), "cy": lambda: self.cy(qs[0], qs[1]),
            "ch": lambda: self.ch(qs[0], qs[1]), "swap": lambda: self.swap(qs[0], qs[1]),
            "cry": lambda: self.cry(qs[0], qs[1], args[0]), "crz": lambda: self.crz(qs[0], qs[1], args[0]),
            "crx": lambda: self.crx(qs[0], qs[1], args[0]),
            "cu1": lambda: self.cp(qs[0], qs[1], args[0]), "cp": lambda: self.cp(qs[0], qs[1], args[0]),
            "cu3": lambda: self.cu3(qs[0], qs[1], *args),
            "ccx": lambda: self.ccx(qs[0], qs[1], qs[2]), "cswap": lambda: self.cswap(qs[0], qs[1], qs[2]),
        }
        if g in two:
            two[g]()
            return True
        return False


_STMT = re.compile(r"^([A-Za-z_][\w]*)\s*(?:\((.*)\))?\s*(.*)$", re.S)


def qasm_to_circuit(source):
    """Reads OpenQASM 2.0 (a file name or the program text).  Returns (Circuit, parameters
    (float64, SQUANDER storage), global_phase): exp(1j * global_phase) * C(parameters) is the
    program's operator."""
    text = source
    if "\n" not in source and not source.lstrip().upper().startswith("OPENQASM"):
        with open(source) as f:
            text = f.read()
    text = re.sub(r"//[^\n]*", "", text)
    # user gate definitions: gate name(params) qargs { body }
    defs = {}

    def take_def(m):
        defs[m.group(1)] = ([a.strip() for a in (m.group(2) or "").split(",") if a.strip()],
                            [a.strip() for a in m.group(3).split(",") if a.strip()], m.group(4))
        return ""
    text = re.sub(r"gate\s+([A-Za-z_]\w*)\s*(?:\(([^)]*)\))?\s*([^{]*)\{([^}]*)\}", take_def, text)
    regs, n = {}, 0
    stmts = [s.strip() for s in text.split(";") if s.strip()]
    for s in stmts:
        m = re.match(r"qreg\s+([A-Za-z_]\w*)\s*\[\s*(\d+)\s*\]", s)
        if m:
            regs[m.group(1)] = (n, int(m.group(2)))
            n += int(m.group(2))
    if n == 0:
        raise ValueError("no qreg declared")
    b = _Builder(n)

    def qubits(arg):
        arg = arg.strip()
        m = re.match(r"([A-Za-z_]\w*)\s*\[\s*(\d+)\s*\]$", arg)
        if m:
            off, size = regs[m.group(1)]
            if int(m.group(2)) >= size:
                raise ValueError("qubit index out of range: %s" % arg)
            return [off + int(m.group(2))]
        off, size = regs[arg]  # a whole register: the gate is applied to every qubit
        return list(range(off, off + size))

    def apply(name, args, qargs_lists, depth=0):
        if depth > 64:
            raise ValueError("gate definitions nest too deeply")
        width = max(len(q) for q in qargs_lists) if qargs_lists else 1
        for k in range(width):  # register broadcast
            qs = [q[k] if len(q) > 1 else q[0] for q in qargs_lists]
            if name in defs:
                pnames, qnames, body = defs[name]
                env = dict(zip(pnames, args))
                qmap = dict(zip(qnames, qs))
                for st in [x.strip() for x in body.split(";") if x.strip()]:
                    m = _STMT.match(st)
                    sub_args = [_eval_expr(a, env) for a in _split_args(m.group(2))] if m.group(2) else []
                    sub_qs = [[qmap[a.strip()]] for a in m.group(3).split(",") if a.strip()]
                    apply(m.group(1), sub_args, sub_qs, depth + 1)
            elif not b.emit(name, args, qs):
                raise ValueError("gate %r is not supported" % name)

    for s in stmts:
        head = s.split()[0] if s.split() else ""
        if head in ("OPENQASM", "include", "qreg", "creg", "barrier", "measure", "reset", "opaque") or \
                s.startswith("if"):
            continue
        m = _STMT.match(s)
        if not m:
            raise ValueError("cannot parse %r" % s)
        args = [_eval_expr(a, {}) for a in _split_args(m.group(2))] if m.group(2) else []
        qargs = [qubits(a) for a in _split_args(m.group(3))]
        apply(m.group(1), args, qargs)
    return b.circuit, np.asarray(b.params, dtype=np.float64), b.phase


def qasm_to_squander_circuit(filename, return_transpiled=False):
    """squander.utils.qasm_to_squander_circuit: (circuit, parameters, None); the third item of
    the reference (a transpiled Qiskit circuit) does not exist here."""
    circ, params, _phase = qasm_to_circuit(filename)
    return circ, params, None


def PartitionCircuitQasm(filename, max_partition_size, strategy="kahn"):
    """squander.partitioning.partition.PartitionCircuitQasm."""
    from .partitioning import PartitionCircuit

    circ, params, _ = qasm_to_squander_circuit(filename)
    return PartitionCircuit(circ, params, max_partition_size, strategy, filename)


def CompareCircuits(circ1, parameters1, circ2, parameters2, parallel=1, tolerance=1e-10, initial_mapping=None,
                    final_mapping=None, is_f32=False):
    """squander.utils.CompareCircuits: the two circuits transform a random state alike (GPU
    state-vector application); returns True or raises AssertionError."""
    n = circ1.get_Qbit_Num()
    rng = np.random.default_rng()
    v = rng.uniform(-1, 1, 1 << n) + 1j * rng.uniform(-1, 1, 1 << n)
    v /= np.linalg.norm(v)
    a, b2 = v.copy(), v.copy()
    if initial_mapping is not None:
        raise NotImplementedError("qubit mappings are not supported")
    circ1.apply_to(np.asarray(parameters1, dtype=np.float64), a)
    circ2.apply_to(np.asarray(parameters2, dtype=np.float64), b2)
    diff = float(np.linalg.norm(a - b2))
    assert diff < tolerance, diff
    return True
