"""A pytest plugin that makes `import squander` resolve to this package, so that test files of
SQUANDER's own suite can run unmodified against the drop-in.  Only the modules those tests
import are provided: squander (Circuit, the decomposition classes), squander.utils
(qasm_to_squander_circuit), squander.partitioning.{partition, kahn, tools}.  Loaded with
`-p reference_alias` by tests/test_reference_suite.py."""
import importlib
import os
import sys
import types

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

_PKG = "sequential-quantum-gate-decomposer_gb300"


def _module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


def _install():
    pkg = importlib.import_module(_PKG)
    part = importlib.import_module(_PKG + ".partitioning")
    qasm = importlib.import_module(_PKG + ".qasm")
    top = _module("squander", __path__=[], **{k: getattr(pkg, k) for k in pkg.__all__})
    top.gates = _module("squander.gates", __path__=[])
    top.gates.qgd_Circuit = _module("squander.gates.qgd_Circuit", qgd_Circuit=pkg.Circuit)
    top.utils = _module("squander.utils", qasm_to_squander_circuit=qasm.qasm_to_squander_circuit,
                        CompareCircuits=qasm.CompareCircuits)
    partitioning = _module("squander.partitioning", __path__=[])
    top.partitioning = partitioning
    partitioning.partition = _module("squander.partitioning.partition", PartitionCircuit=part.PartitionCircuit,
                                     PartitionCircuitQasm=qasm.PartitionCircuitQasm)
    partitioning.kahn = _module("squander.partitioning.kahn", kahn_partition=part.kahn_partition,
                                kahn_partition_preparts=part.kahn_partition_preparts)
    partitioning.tools = _module("squander.partitioning.tools", get_qubits=part.get_qubits,
                                 get_float_ops=part.get_float_ops, parts_to_float_ops=part.parts_to_float_ops,
                                 total_float_ops=part.total_float_ops,
                                 translate_param_order=part.translate_param_order)


_install()
