"""Generates the golden fixtures of tests/golden/ from SQUANDER itself.

The numbers come from the reference's own C++ decomposition path, compiled from its sources
by oracle/build_ref.py into oracle/_ref/libsqg_ref.so (driven through oracle/ref.py), so the
fixtures pin both the oracle and the CUDA engine to the reference.  Where the reference
cannot run at a workload's size (its gradient materialises one derivative matrix per
parameter: 30 GB at 10 qubits, 4096 matrices of 256 MB at 12 qubits) the gradient comes from
the oracle's reverse-sweep form (oracle/sqg_oracle.c:sqgo_cost_grad_sweep), which the CPU
tests check against the reference wherever both run; costs and matrix products still come
from the reference.  Each file records which source produced each array ("source_*").

Files (workloads as the benchmark configurations define them; seeds fixed below):
  umtx4_golden.npz  the reference's 4-qubit test target data/Umtx.mat, 40-block
                    nearest-neighbour CNOT+U3 ansatz (P = 252), costs and gradients for the
                    FROBENIUS_NORM / HILBERT_SCHMIDT_TEST / INFIDELITY variants and a trace
                    offset, and one BFGS_Powell run
  config1_n4.npz    4-qubit Haar target, the same ansatz, 4 parameter vectors x 3 variants,
                    and one BFGS run to the end of its 2000-iteration budget
  config2_n8.npz    8-qubit targets made by the ansatz with 120 blocks (P = 744) and 360
                    blocks (P = 2184) at seeded angles; costs and gradients of 4 vectors each
  config3_n10.npz   10-qubit, 300 blocks over random ordered pairs (P = 1830), 64 parameter
                    vectors: costs (reference) and 32 gradient components each (sweep)
  config4_3q.npz    64 of the 3-qubit benchmark targets (32 Haar, 32 random-circuit) with the
                    14-block ansatz (P = 93): one BFGS_Powell run of at most 1000 iterations
                    from seeded starts (evaluations, final cost, final point)
  config5_n12.npz   12 qubits, 2000 random U3/RY/CNOT/CZ/CRY gates, 4 parameter vectors: the
                    product with a 4096 x 16 column block, stored as an 8 x 16 sketch R Y with
                    a seeded +-1 matrix R; cost (reference) and gradient (sweep) on a 4096 x 16
                    target with trace offset 1000

Run in a checkout with the reference tree present:
    python tests/golden/make_golden.py [which ...]
"""
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402

sys.path.insert(0, HERE)
from inputs import config3_inputs, config4_inputs, config5_inputs  # noqa: E402

wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")

VARIANTS = (("frob", 0), ("hs", 3), ("infid", 9))


def _save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print("wrote", name, flush=True)


def umtx4():
    import scipy.io

    src = R.build_ref.reference_root()
    U = scipy.io.loadmat(os.path.join(src, "..", "..", "data", "Umtx.mat"))["Umtx"].astype(np.complex128)
    target = np.ascontiguousarray(U.conj().T)
    c = wl.cnot_u3_ansatz(4, 40)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    rng = np.random.default_rng(20241203)
    theta = rng.uniform(0, 2 * np.pi, (3, P))
    out = {"target": target, "gates": recs, "theta": theta, "source": "reference"}
    for name, v in VARIANTS:
        cg = [R.cost_grad(4, recs, th, target, variant=v) for th in theta]
        out["cost_" + name] = np.array([a for a, _ in cg])
        out["grad_" + name] = np.stack([b for _, b in cg])
    sub = np.ascontiguousarray(U[4:12, :].conj().T)
    cg = [R.cost_grad(4, recs, th, sub, trace_offset=4) for th in theta]
    out["target_offset4"] = sub
    out["cost_offset4"] = np.array([a for a, _ in cg])
    out["grad_offset4"] = np.stack([b for _, b in cg])
    x, f, calls = R.bfgs_run(4, recs, target, theta[0], 300)
    out.update(bfgs_x0=theta[0], bfgs_max_iters=300, bfgs_x=x, bfgs_cost=f, bfgs_calls=calls)
    _save("umtx4_golden.npz", **out)


def config1():
    rng = np.random.default_rng(11)
    target = np.ascontiguousarray(wl.haar_unitary(16, rng).conj().T)
    c = wl.cnot_u3_ansatz(4, 40)
    recs, P = c.gate_records(), c.get_Parameter_Num()
    theta = rng.uniform(0, 2 * np.pi, (4, P))
    out = {"target": target, "gates": recs, "theta": theta, "source": "reference"}
    for name, v in VARIANTS:
        cg = [R.cost_grad(4, recs, th, target, variant=v) for th in theta]
        out["cost_" + name] = np.array([a for a, _ in cg])
        out["grad_" + name] = np.stack([b for _, b in cg])
    t0 = time.time()
    x, f, calls = R.bfgs_run(4, recs, target, theta[0], 2000)
    print("config1 BFGS: %d evaluations, cost %.6g, %.0f s" % (calls, f, time.time() - t0), flush=True)
    out.update(bfgs_x0=theta[0], bfgs_max_iters=2000, bfgs_x=x, bfgs_cost=f, bfgs_calls=calls)
    _save("config1_n4.npz", **out)


def config2():
    out = {"source": "reference"}
    for blocks in (120, 360):
        rng = np.random.default_rng(6 + blocks)
        c = wl.cnot_u3_ansatz(8, blocks)
        recs, P = c.gate_records(), c.get_Parameter_Num()
        U = R.get_matrix(8, recs, rng.uniform(0, 2 * np.pi, P))
        target = np.ascontiguousarray(U.conj().T)
        theta = rng.uniform(0, 2 * np.pi, (4, P))
        t0 = time.time()
        cg = [R.cost_grad(8, recs, th, target) for th in theta]
        print("config2 P=%d: %.0f s" % (P, time.time() - t0), flush=True)
        k = "b%d_" % blocks
        out.update({k + "gates": recs, k + "target": target, k + "theta": theta,
                    k + "cost": np.array([a for a, _ in cg]), k + "grad": np.stack([b for _, b in cg])})
    _save("config2_n8.npz", **out)


def config3():
    c, angles, theta, pick = config3_inputs()
    recs = c.gate_records()
    t0 = time.time()
    U = R.get_matrix(10, recs, angles)
    target = np.ascontiguousarray(U.conj().T)
    costs = R.batch(10, recs, theta, target)
    print("config3 reference costs: %.0f s" % (time.time() - t0), flush=True)
    t0 = time.time()
    oc, og = O.batch(10, recs, theta, target, with_grad=True, sweep=True)
    print("config3 sweep gradients: %.0f s" % (time.time() - t0), flush=True)
    assert np.max(np.abs(oc - costs)) < 1e-12, np.max(np.abs(oc - costs))
    _save("config3_n10.npz", gates=recs, cost=costs, pick=pick, grad=np.take_along_axis(og, pick, axis=1),
          source_cost="reference", source_grad="oracle sweep",
          target_checksum=np.array([target.sum(), (target * target).sum()]))


def config4():
    ansatz, targets, x0 = config4_inputs()
    recs = ansatz.gate_records()
    xs, fs, calls = [], [], []
    t0 = time.time()
    for b in range(64):
        x, f, n = R.bfgs_run(3, recs, targets[b], x0[b], 1000)
        xs.append(x), fs.append(f), calls.append(n)
    print("config4: %.0f s, solved %d of 64 in one run" % (time.time() - t0, sum(f < 1e-8 for f in fs)), flush=True)
    short = [R.bfgs_run(3, recs, targets[b], x0[b], 20) for b in range(64)]
    _save("config4_3q.npz", gates=recs, targets=targets, x0=x0, max_iters=1000, x=np.stack(xs), cost=np.array(fs),
          calls=np.array(calls), short_max_iters=20, short_x=np.stack([s[0] for s in short]),
          short_cost=np.array([s[1] for s in short]), short_calls=np.array([s[2] for s in short]),
          source="reference")


def config5():
    c, theta, X, S, T = config5_inputs()
    recs = c.gate_records()
    t0 = time.time()
    sk = []
    for th in theta:
        Y = R.apply_to(12, recs, th, X.copy())
        sk.append(S @ Y)
    costs = np.array([R.cost(12, recs, th, T, trace_offset=1000) for th in theta])
    print("config5 reference: %.0f s" % (time.time() - t0), flush=True)
    oc, og = O.batch(12, recs, theta, T, trace_offset=1000, with_grad=True, sweep=True)
    assert np.max(np.abs(oc - costs)) < 1e-12
    _save("config5_n12.npz", gates=recs, sketch=np.stack(sk), cost=costs, grad=og, source_apply="reference",
          source_cost="reference", source_grad="oracle sweep")


def adaptive_n8_records(levels=2):
    """8 qubits, `levels` levels of adaptive layers ([U3(t), U3(c), CRY(t, c)] for every pair
    t < c) and the final U3 layer: the gate structure that add_Adaptive_Layers and
    add_Finalyzing_Layer_To_Gate_Structure build."""
    recs, p = [], 0
    for _ in range(levels):
        for t in range(8):
            for c in range(t + 1, 8):
                for g in ((7, t, -1), (7, c, -1), (14, t, c)):
                    recs.append(g + (p,))
                    p += 3 if g[0] == 7 else 1
    for q in range(8):
        recs.append((7, q, -1, p))
        p += 3
    return np.asarray(recs, dtype=np.int32), p


def adaptive8():
    """The reference's combined-optimisation check (tests/decomposition/
    test_optmization_problem_combined.py): 8 qubits, two levels of adaptive layers, the target
    cut to rows 80..239 with trace offset 80; cost and gradient at a second parameter set."""
    recs, P = adaptive_n8_records()
    rng = np.random.default_rng(880)
    exact = rng.uniform(0, 2 * np.pi, P)
    theta = rng.uniform(0, 2 * np.pi, (2, P))
    U = R.get_matrix(8, recs, exact)
    target = np.ascontiguousarray(U[80:240, :].conj().T)
    c0, _ = R.cost_grad(8, recs, exact, target, trace_offset=80)
    cg = [R.cost_grad(8, recs, th, target, trace_offset=80) for th in theta]
    _save("adaptive_n8.npz", gates=recs, exact=exact, theta=theta, cost_exact=c0,
          cost=np.array([a for a, _ in cg]), grad=np.stack([b for _, b in cg]), source="reference")


def tree_search():
    """The reference's structure search (N_Qubit_Decomposition_Tree_Search, all qubit pairs,
    tolerance 1e-8, levels up to 8) in its default mode (operator-Schmidt-rank bounds with the
    best-first graph search) and in its exhaustive level-search mode, on targets made from
    random CNOT+U3 structures with k CNOTs, and on the reference's own 4-qubit test target
    data/Umtx.mat (the last entry, k = -1).  Targets are stored as U^dagger padded to 16 x 16."""
    import scipy.io

    rng = np.random.default_rng(8)
    cases = [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 3), (3, 4), (4, 1), (4, 2), (4, -1)]
    T = np.zeros((len(cases), 16, 16), dtype=np.complex128)
    rows = []
    for idx, (n, k) in enumerate(cases):
        if k < 0:
            src = R.build_ref.reference_root()
            U = scipy.io.loadmat(os.path.join(src, "..", "..", "data", "Umtx.mat"))["Umtx"].astype(np.complex128)
        else:
            c = wl.cnot_u3_ansatz(n, k, pairs="random", rng=rng)
            U = R.get_matrix(n, c.gate_records(), rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
        N = 1 << n
        T[idx, :N, :N] = U.conj().T
        d_cn, d_err = R.tree_search(n, T[idx, :N, :N], 1, 1, 8, 1e-8, 1)
        e_cn, e_err = R.tree_search(n, T[idx, :N, :N], 0, 0, 8, 1e-8, 1)
        rows.append((n, k, d_cn, d_err, e_cn, e_err))
        print("tree search n=%d k=%d: default %d (%.1e), level search %d (%.1e)" % rows[-1], flush=True)
    r = np.array(rows)
    _save("tree_search_ref.npz", targets=T, qbit_num=r[:, 0].astype(int), generating_cnots=r[:, 1].astype(int),
          default_cnots=r[:, 2].astype(int), default_error=r[:, 3], level_cnots=r[:, 4].astype(int),
          level_error=r[:, 5], source="reference")


JOBS = {"umtx4": umtx4, "adaptive8": adaptive8, "tree_search": tree_search, "config1": config1, "config2": config2, "config3": config3, "config4": config4,
        "config5": config5}

if __name__ == "__main__":
    if not R.available():
        sys.exit("the reference tree is needed (oracle/build_ref.py)")
    O.build()
    for name in (sys.argv[1:] or JOBS):
        JOBS[name]()
