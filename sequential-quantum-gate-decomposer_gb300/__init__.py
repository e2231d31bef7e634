"""GB300-native engine for SQUANDER's decomposition hot path.

The cost ``1 - Re Tr(C(theta) U^dagger)/cols`` (and the HILBERT_SCHMIDT_TEST /
INFIDELITY variants) of a parametric U3/RX/RY/RZ/CNOT/CZ/CRY circuit and its adjoint
gradient run in hand-written sm_103a CUDA kernels (libsqg.so, C ABI in include/sqg.h).
This package mirrors the reference's Python surface for that path:
``Circuit`` (squander.Circuit), ``N_Qubit_Decomposition_custom``,
``N_Qubit_Decomposition_Tree_Search`` and ``PartitionCircuit`` (squander.partitioning).

The directory name contains hyphens, so import it with
``importlib.import_module("sequential-quantum-gate-decomposer_gb300")``; the package
also registers itself under the alias ``sqg_gb300``.
"""
import sys as _sys

from ._native import SQGError, build
from .batched import BatchedDecomposer
from .circuit import CNOT, CRY, CZ, RX, RY, RZ, U3, Circuit
from .decomposition import N_Qubit_Decomposition_custom
from .evaluator import (FROBENIUS_NORM, HILBERT_SCHMIDT_TEST, INFIDELITY, CircuitCost, CostEvaluator,
                        circuit_cost)
from .partitioning import PartitionCircuit
from .qasm import CompareCircuits, PartitionCircuitQasm, qasm_to_circuit, qasm_to_squander_circuit
from .adaptive import N_Qubit_Decomposition_adaptive, N_Qubit_State_Preparation_adaptive
from .tree_search import N_Qubit_Decomposition_Tabu_Search, N_Qubit_Decomposition_Tree_Search

_sys.modules.setdefault("sqg_gb300", _sys.modules[__name__])

__all__ = ["Circuit", "BatchedDecomposer", "N_Qubit_Decomposition_custom", "N_Qubit_Decomposition_Tree_Search",
           "N_Qubit_Decomposition_Tabu_Search", "N_Qubit_Decomposition_adaptive",
           "N_Qubit_State_Preparation_adaptive",
           "PartitionCircuit", "PartitionCircuitQasm", "qasm_to_circuit", "qasm_to_squander_circuit", "CompareCircuits", "CostEvaluator", "CircuitCost", "circuit_cost", "SQGError",
           "build", "FROBENIUS_NORM", "HILBERT_SCHMIDT_TEST", "INFIDELITY", "U3", "RX", "RY", "RZ", "CNOT", "CZ",
           "CRY"]
