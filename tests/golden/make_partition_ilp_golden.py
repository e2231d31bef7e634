"""Generates tests/golden/partition_ilp.json: what the reference's OWN optimal partitioner
(squander/partitioning/ilp.py, with tools.py and kahn.py, executed from the reference tree)
computes for seeded random circuits over the engine's gate set:

  family     every candidate part it enumerates (get_all_partitions: gate sets of the circuit
             with its single-qubit chains contracted), as sorted gate-index lists;
  chains     the contracted single-qubit chains;
  ilp        the optimum of strategy "ilp" (number of parts) and the final partitions;
  fusion     the optimum of strategy "ilp-fusion" (its objective sum of (flops * N + 1) over the
             chosen parts, N the number of candidates) and the chosen parts' FLOP total;
  fusion_ca  the optimum of strategy "ilp-fusion-ca" (control-aware objective) and its chain
             placement (first gates of the chains placed into their predecessor's part, last
             gates of those placed into their successor's part).
Each strategy also records the parts its solution chose and the final partitions.

The reference solves its models with PuLP and CBC (or Gurobi).  Neither is in this image, so
the script installs tests/golden/pulp_highs.py as `pulp`: the reference's own model is then
solved by SciPy's HiGHS with a zero gap.  Optimal partitions need not be unique, so the fixture
pins optimal objective values, the candidate family, and the final partitions that the
reference builds from its chosen parts; the tests compare objectives and families exactly,
rebuild the final partitions from the reference's choice, and check their own solutions'
validity.

Run once with the reference tree available:
    python tests/golden/make_partition_ilp_golden.py /path/to/sequential-quantum-gate-decomposer
"""
import importlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import make_partition_golden as base  # noqa: E402
import pulp_highs  # noqa: E402

CASES = [(3, 14, 11), (4, 20, 12), (5, 28, 13), (6, 36, 14), (5, 40, 15), (7, 44, 16), (8, 52, 17),
         (10, 120, 18), (6, 80, 19)]
MAX_QUBITS = [2, 3, 4, 5]


def load_ilp(ref_root):
    path = os.path.join(ref_root, "squander", "partitioning", "ilp.py")
    m = base.types.ModuleType("squander.partitioning.ilp")
    m.__file__ = path
    sys.modules[m.__name__] = m
    with open(path) as f:
        exec(compile(f.read(), path, "exec"), m.__dict__)
    return m


def main(ref_root):
    sys.modules["pulp"] = pulp_highs
    pkg = importlib.import_module("sequential-quantum-gate-decomposer_gb300")
    circuit_mod = importlib.import_module("sequential-quantum-gate-decomposer_gb300.circuit")
    tools, kahn = base.load_reference(ref_root, pkg.Circuit, circuit_mod.Gate)
    ilp = load_ilp(ref_root)

    record = {}
    original = ilp.ilp_global_optimal

    def recording(allparts, g, *args, **kwargs):
        L, info = original(allparts, g, *args, **kwargs)
        record["chosen"] = [sorted(allparts[i]) for i in L]
        record["objective"] = pulp_highs.LpProblem.last_objective
        record["placed"] = None if info is None else [sorted(map(int, info[0])), sorted(map(int, info[1]))]
        return L, info

    ilp.ilp_global_optimal = recording
    cases = []
    for n, count, seed in CASES:
        for mq in MAX_QUBITS if count >= 80 else MAX_QUBITS[:3]:
            c, recs = base.random_circuit(pkg.Circuit, n, count, seed)
            t0 = time.time()
            allparts, g, go, rgo, chains, g2q, g2t = ilp.get_all_partitions(c, mq)
            case = {"qbit_num": n, "gates": recs, "max_qubit": mq,
                    "family": sorted(sorted(map(int, p)) for p in allparts),
                    "chains": sorted(list(map(int, ch)) for ch in chains)}
            _, _, parts = ilp.max_partitions(c, mq)
            case["ilp"] = {"objective": record["objective"], "chosen": sorted(record["chosen"]),
                           "parts": [sorted(map(int, p)) for p in parts]}
            _, _, parts = ilp.max_partitions(c, mq, fusion_cost=True)
            chosen = record["chosen"]
            flops = tools.parts_to_float_ops(mq, g2q, None, [frozenset(p) for p in chosen])
            case["fusion"] = {"objective": record["objective"], "flops": int(sum(flops)),
                              "chosen": sorted(chosen), "parts": [sorted(map(int, p)) for p in parts]}
            _, _, parts = ilp.max_partitions(c, mq, fusion_cost=True, control_aware=True)
            case["fusion_ca"] = {"objective": record["objective"], "chosen": sorted(record["chosen"]),
                                 "placed": record["placed"], "parts": [sorted(map(int, p)) for p in parts]}
            cases.append(case)
            print("n=%d gates=%d k=%d family=%d ilp=%g fusion=%g ca=%g  %.1fs" % (
                n, count, mq, len(allparts), case["ilp"]["objective"], case["fusion"]["objective"],
                case["fusion_ca"]["objective"], time.time() - t0))
    with open(os.path.join(HERE, "partition_ilp.json"), "w") as f:
        json.dump({"generator": "squander/partitioning/ilp.py (+ tools.py, kahn.py) of the reference tree, "
                                "its models solved by HiGHS through tests/golden/pulp_highs.py",
                   "cases": cases}, f)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main(sys.argv[1])
