"""Generates tests/golden/partition_kahn.json: partitions, parameter orders and FLOP-model
figures computed by the reference's OWN partitioner (squander/partitioning/kahn.py and the
functions of squander/partitioning/tools.py, executed from the reference tree) on seeded random
circuits over the engine's gate set, to pin the restatement in partitioning.py.

The reference modules import SQUANDER's compiled circuit class and Qiskit at load time; neither
is needed by the functions used here, so the script loads them with this package's Circuit in
place of squander.Circuit (the partitioner only calls get_Gates, get_Children,
get_Involved_Qbits, get_Parameter_Start_Index / get_Parameter_Num, add_Gate and add_Circuit)
and with empty placeholder modules for the Qiskit imports.

Run once with the reference tree available:
    python tests/golden/make_partition_golden.py /path/to/sequential-quantum-gate-decomposer
"""
import importlib
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

CASES = [(3, 12, 1), (4, 20, 2), (5, 30, 3), (6, 40, 4), (7, 50, 5), (8, 60, 6), (6, 24, 7), (10, 80, 8)]
MAX_QUBITS = [2, 3, 4, 5]


def random_circuit(circuit_cls, n, count, seed):
    """Seeded random circuit over U3, RX, RY, RZ, CNOT, CZ, CRY; also returned as records."""
    rng = np.random.default_rng(seed)
    c = circuit_cls(n)
    recs = []
    for _ in range(count):
        kind = ["U3", "RX", "RY", "RZ", "CNOT", "CZ", "CRY"][rng.integers(7)]
        t = int(rng.integers(n))
        if kind in ("CNOT", "CZ", "CRY"):
            ctl = int(rng.integers(n - 1))
            ctl = ctl + 1 if ctl >= t else ctl
            getattr(c, "add_" + kind)(t, ctl)
            recs.append([kind, t, ctl])
        else:
            getattr(c, "add_" + kind)(t)
            recs.append([kind, t, -1])
    return c, recs


def load_reference(ref_root, circuit_cls, gate_cls):
    """The reference's tools and kahn modules, loaded from ref_root/squander/partitioning."""
    def module(name, attrs=None, package=False):
        m = types.ModuleType(name)
        if package:
            m.__path__ = []
        for k, v in (attrs or {}).items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    module("squander", {"Circuit": circuit_cls}, package=True)
    module("squander.utils")
    sys.modules["squander"].utils = sys.modules["squander.utils"]
    module("squander.gates", package=True)
    module("squander.gates.qgd_Circuit", {"qgd_Circuit": circuit_cls})
    module("squander.gates.gates_Wrapper", {"Gate": gate_cls})
    module("squander.partitioning", package=True)
    module("qiskit", package=True)
    module("qiskit.transpiler", {"PassManager": object}, package=True)
    module("qiskit.transpiler.passes", {"CollectMultiQBlocks": object})
    out = {}
    for name in ("tools", "kahn"):
        path = os.path.join(ref_root, "squander", "partitioning", name + ".py")
        m = module("squander.partitioning." + name)
        m.__file__ = path
        with open(path) as f:
            exec(compile(f.read(), path, "exec"), m.__dict__)
        out[name] = m
    return out["tools"], out["kahn"]


def main(ref_root):
    pkg = importlib.import_module("sequential-quantum-gate-decomposer_gb300")
    circuit_mod = importlib.import_module("sequential-quantum-gate-decomposer_gb300.circuit")
    tools, kahn = load_reference(ref_root, pkg.Circuit, circuit_mod.Gate)
    cases = []
    for n, count, seed in CASES:
        for mq in MAX_QUBITS:
            c, recs = random_circuit(pkg.Circuit, n, count, seed)
            top, param_order, parts = kahn.kahn_partition(c, mq)
            gates = c.get_Gates()
            g2q = {i: set(g.get_Involved_Qbits()) for i, g in enumerate(gates)}
            g2t = {i: g.get_Target_Qbit() for i, g in enumerate(gates)}
            cases.append({
                "qbit_num": n, "gates": recs, "max_qubit": mq,
                "parts": [list(map(int, p)) for p in parts],
                "param_order": [list(map(int, t)) for t in param_order],
                "block_sizes": [len(b._gates) for b in top.get_Gates()],
                "float_ops": int(tools.total_float_ops(n, mq, g2q, None, parts)),
                "float_ops_ctrl": int(tools.total_float_ops(n, mq, g2q, g2t, parts)),
            })
    with open(os.path.join(HERE, "partition_kahn.json"), "w") as f:
        json.dump({"generator": "squander/partitioning/kahn.py + tools.py of the reference tree", "cases": cases}, f)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main(sys.argv[1])
