#!/usr/bin/env python3
"""Benchmark of the decomposition hot path on one GB300.

Headline metric: 3-qubit decompositions per second reaching FROBENIUS_NORM cost < 1e-8.
Workload: 4096 held-out 3-qubit targets (half Haar-random 8x8, half products of random
CNOT+U3 circuits with 1..14 CNOTs; seeded synthetic data), fixed 14-block
nearest-neighbour CNOT+U3 ansatz (93 parameters), batched 4096-wide on the device.  One
step = one batched decomposition pass over all 4096 targets from fresh random starts.
Secondary lines inside the same JSON object: gate application at n=12 (2000-gate random
circuit, batch of 4 parameter vectors, fused vs unfused, HBM GB/s) and the batched
cost+gradient evaluation at n=8 (B=1024, 360 blocks).

--impl reference times the reference algorithm on the host cores instead: the oracle's C
restatement of SQUANDER's BFGS decomposition, which equals the reference's own C++ path (built
from the reference's sources by oracle/build_ref.py where that tree exists) evaluation for
evaluation on the pinned cases; the reference's source tree is not present where the
benchmark runs, so its own build cannot be timed there.
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
PKG = "sequential-quantum-gate-decomposer_gb300"

METRIC = "3q decompositions/s to cost<1e-8"
UNIT = "decompositions/s"
N_TARGETS = 4096
ANSATZ_BLOCKS = 14
TOL = 1e-8
MAX_CALLS = 1000      # cost+gradient evaluations per BFGS run
MAX_OUTER = 4         # restarts (N_Qubit_Decomposition_custom uses 4 outer iterations)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# FP64 FMA pipe peak of the GB300 (TFLOP/s, an FMA counts 2 flops).  Measured live at the
# start of every run by the engine's probe kernel (sqg_probe_fp64_tflops); 1.20 is the
# value measured on the GB300s and is used only if the probe cannot run.
FP64_PEAK_TFLOPS = 1.20


class Clocks:
    """nvidia-smi sampler for the timed region."""

    def __init__(self):
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="sqg_bench_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        lines = open(self.path).read().splitlines()
        os.remove(self.path)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(sqg, wl, orc_matrix=None, seed=1234, rank=0, world=1):
    """The 3-qubit workload (as U^dagger).  With world > 1 ranks the global workload is
    world x 4096 targets and rank r decomposes its own shard (sharding.shard_range): one rank
    reproduces the single-GPU workload exactly, more ranks add distinct targets."""
    ansatz = wl.cnot_u3_ansatz(3, ANSATZ_BLOCKS)
    if orc_matrix is None:
        orc_matrix = wl.circuit_matrix
    if world == 1:
        U = wl.three_qubit_targets(N_TARGETS, np.random.default_rng(seed), orc_matrix)
    else:
        sharding = importlib.import_module(PKG + ".sharding")
        start, stop = sharding.shard_range(world * N_TARGETS, rank, world)
        # shard k of the global workload is drawn from its own seed, so a rank builds only its shard
        U = wl.three_qubit_targets(stop - start, np.random.default_rng(seed + 7919 * rank), orc_matrix)
    targets = np.ascontiguousarray(np.conj(np.transpose(U, (0, 2, 1))))
    return ansatz, targets


def flush_l2(buf):
    buf.add_(1)


def barrier():
    """Barrier across the ranks of a torchrun launch (no-op for a single process)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def fp64_ops_per_eval(circuit_records, N, cols):
    """FP64 instructions of one cost+gradient evaluation in the tile kernels (update
    rules of gates.cuh): forward per pair U3 14, RX/RY/RZ 8, CRY 8 on the controlled
    quarter of rows... reverse per pair: uncompute + R accumulation (16) + co-state."""
    ops = 0
    for t, tg, c, ps in circuit_records:
        pairs_all = (N // 2) * cols
        pairs_ctl = (N // 4) * cols
        if t == 7:
            fwd, pairs = 14, pairs_all
        elif t in (8, 9, 10):
            fwd, pairs = 8, pairs_all
        elif t == 14:
            fwd, pairs = 8, pairs_ctl
        else:
            continue
        ops += pairs * (fwd + fwd + 16 + fwd)
    return ops


def algorithmic_flops_per_eval(circuit_records, N, cols):
    """Algorithmic FP64 flops of one cost + adjoint-gradient evaluation: three passes
    (forward, left and right application) per parametric gate over the N x cols target,
    16 flops per touched complex element (two complex multiply-adds); CRY touches the
    control = 1 half; CNOT and CZ are exchanges and sign flips (no flops)."""
    flops = 0
    for t, tg, c, ps in circuit_records:
        if t in (7, 8, 9, 10):
            flops += 3 * 16 * N * cols
        elif t == 14:
            flops += 3 * 16 * N * cols // 2
    return flops


def bfgs_flops_per_iteration(P):
    """Flops of one BFGS_Powell iteration of the reference algorithm
    (BFGS_Powell.cpp:202-446): Z^T g 2P^2, Z (Z^T g) 2P^2, the Givens sweep 6P^2, Z^T gamma
    2P^2, rank-one update 2P^2, column norms 2P^2, column scaling P^2."""
    return 17 * P * P


# DRAM bytes of one k_decompose launch of the timed workload (4096 targets), measured once with
# ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum (one pass, --profile-case decompose_full)
K_DECOMPOSE_DRAM_BYTES = 25.60e9 + 45.09e9
K_DECOMPOSE_TRAFFIC_SOURCE = ("dram__bytes_read.sum + dram__bytes_write.sum of one k_decompose launch of this "
                              "workload (ncu): 25.60 GB read, 45.09 GB written; the BFGS matrices are kept in L2 "
                              "with the evict_last policy (78 GB written without it), and what reaches HBM is "
                              "mostly the out-of-line evaluation's register spills, whose local-memory window "
                              "(about 140 MB) does not fit in L2 beside them")


def decomposition_steps(torch, decs, streams, flush, tdev, start_fn, seeds):
    """Runs one batched decomposition step per seed, consecutive steps on alternating streams
    (each with its own decomposer and workspace), so that a step's end-of-batch tail overlaps
    the next step's start.  Each step writes the 256 MB flush buffer on its stream first (L2
    larger than the inputs).  Timed with CUDA events on the current stream, which waits for
    both streams; returns (seconds, [(x, cost, calls, iters) per step])."""
    main = torch.cuda.current_stream()
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(main)
    for s in streams:
        s.wait_event(e0)
    out = []
    for k, seed in enumerate(seeds):
        s, dec = streams[k % len(streams)], decs[k % len(decs)]
        with torch.cuda.stream(s):
            flush_l2(flush)
            x, cost, calls = dec.run(tdev, start_fn(k), seed=seed)
            out.append((x, cost, calls, dec.iters))
    for s in streams:
        main.wait_stream(s)
    e1.record(main)
    e1.synchronize()
    barrier()
    return e0.elapsed_time(e1) / 1e3, out


def decomposition_steps_e2e(torch, decs, streams, targets, start_fn, seeds):
    """The same steps through host buffers: each step copies the targets (and, when start_fn
    returns host start points, the starts) from pinned host memory to the device and reads the
    best parameters and costs back into pinned host memory, all inside the timed region (host
    clock around the whole run).  Returns (seconds, solved, h2d bytes per step, d2h bytes per step)."""
    tgt_pin = torch.from_numpy(targets).pin_memory()
    P = decs[0].native.param_num
    outs = [(torch.empty((N_TARGETS, P), dtype=torch.float64).pin_memory(),
             torch.empty(N_TARGETS, dtype=torch.float64).pin_memory()) for _ in seeds]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h2d = 0
    for k, seed in enumerate(seeds):
        s, dec = streams[k % len(streams)], decs[k % len(decs)]
        with torch.cuda.stream(s):
            tdev = tgt_pin.to("cuda", non_blocking=True)
            start = start_fn(k, tdev)
            if start.device.type == "cpu":
                h2d = tgt_pin.numel() * 16 + start.numel() * 8
                start = start.to("cuda", non_blocking=True)
            else:
                h2d = tgt_pin.numel() * 16
            x, cost, calls = dec.run(tdev, start, seed=seed)
            outs[k][0].copy_(x, non_blocking=True)
            outs[k][1].copy_(cost, non_blocking=True)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    solved = sum(int((c.numpy() < TOL).sum()) for _, c in outs)
    return dt, solved, h2d, N_TARGETS * P * 8 + N_TARGETS * 8


def breakdown(results, P):
    """Evaluation budget of the timed steps: where the evaluations went."""
    calls = np.concatenate([r[2].cpu().numpy().astype(np.int64) for r in results])
    cost = np.concatenate([r[1].cpu().numpy() for r in results])
    ok = cost < TOL
    return {"evaluations_per_target": float(calls.mean()),
            "evaluations_per_solved_target": float(calls[ok].mean()) if ok.any() else None,
            "evaluations_per_unsolved_target": float(calls[~ok].mean()) if (~ok).any() else None,
            "share_of_evaluations_in_unsolved": float(calls[~ok].sum() / max(1, calls.sum())),
            "solved_evaluations_quantiles_10_50_90": [float(q) for q in np.quantile(calls[ok], [0.1, 0.5, 0.9])]
            if ok.any() else None}


def path_stats(results, seconds, steps, P, flops_eval):
    solved = sum(int((r[1].cpu().numpy() < TOL).sum()) for r in results)
    calls = sum(int(r[2].cpu().numpy().astype(np.int64).sum()) for r in results)
    iters = sum(int(r[3].cpu().numpy().astype(np.int64).sum()) for r in results)
    tflops = (flops_eval * calls + bfgs_flops_per_iteration(P) * iters) / seconds / 1e12
    return {"value": solved / seconds, "ms_per_step": 1e3 * seconds / steps,
            "solved_fraction": solved / (N_TARGETS * steps), "evaluations_per_step": calls / steps,
            "bfgs_iterations_per_step": iters / steps, "achieved_tflops": tflops}


def bench_ours(args, rank=0, world=1):
    import torch

    global FP64_PEAK_TFLOPS
    sqg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    native = importlib.import_module(PKG + "._native")
    ini = importlib.import_module(PKG + ".initializer")
    if world == 1:
        torch.cuda.set_device(0)
    FP64_PEAK_TFLOPS = max(native.probe_fp64_tflops() for _ in range(3))
    ansatz, targets = make_workload(sqg, wl, rank=rank, world=world)
    P = ansatz.get_Parameter_Num()
    flops_eval = algorithmic_flops_per_eval(ansatz.gate_records(), 8, 8)
    tdev = torch.from_numpy(targets).cuda()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    decs = [sqg.BatchedDecomposer(ansatz, tolerance=TOL, max_calls=MAX_CALLS, max_outer=MAX_OUTER) for _ in streams]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    rng = np.random.default_rng(99 + 7919 * rank)
    seed0 = 1000 + 100000 * rank

    # learned initialiser: trained here, before any timed region, on decompositions the
    # batched kernel generates (204800 synthetic targets, tcgen05 GEMMs).  --skip-learned
    # (profiling runs only) reports the plain path alone.
    if args.skip_learned:
        init, train_stats = None, None
    else:
        init, train_stats = ini.train_initializer(ansatz, n_samples=204800, epochs=8, seed=4242)
    torch.cuda.synchronize()

    # plain path: random starts U[0, 2pi), generated on the host beforehand (part of the input)
    x0s = [torch.from_numpy(rng.uniform(0, 2 * np.pi, (N_TARGETS, P))).cuda() for _ in range(args.steps)]
    warm = [torch.from_numpy(rng.uniform(0, 2 * np.pi, (N_TARGETS, P))).cuda() for _ in range(args.warmup)]
    decomposition_steps(torch, decs, streams, flush, tdev, lambda k: warm[k], [seed0 + 50000 + k for k in range(args.warmup)])
    if init is not None:
        decomposition_steps(torch, decs, streams, flush, tdev, lambda k: init.predict(tdev),
                            [seed0 + 60000 + k for k in range(args.warmup)])
    clocks = Clocks()
    clocks.start()
    seeds = [seed0 + k for k in range(args.steps)]
    t_plain, res_plain = decomposition_steps(torch, decs, streams, flush, tdev, lambda k: x0s[k], seeds)
    if init is not None:
        t_learn, res_learn = decomposition_steps(torch, decs, streams, flush, tdev, lambda k: init.predict(tdev),
                                                 seeds)
    clk = clocks.stop()
    plain = path_stats(res_plain, t_plain, args.steps, P, flops_eval)
    plain["breakdown"] = breakdown(res_plain, P)
    if init is None:
        line = {"metric": METRIC, "value": plain["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": plain["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded Haar + random-circuit 3-qubit targets)",
                "config": {"workload": "4096 3-qubit targets, 14-block NN ansatz, plain random-start path only "
                                       "(profiling run)", "init": "random U[0,2pi)"},
                "plain": plain, "gpu_launches": args.steps}
        if clk:
            line["clocks"] = clk
        return line
    init.mlp.check_errors()
    learned = path_stats(res_learn, t_learn, args.steps, P, flops_eval)
    learned["breakdown"] = breakdown(res_learn, P)

    # end to end through host buffers (the same number of steps as the timed region)
    e2e_seeds = [seed0 + 20000 + k for k in range(args.steps)]
    x0h = [torch.from_numpy(rng.uniform(0, 2 * np.pi, (N_TARGETS, P))).pin_memory() for _ in range(args.steps)]
    t_pe, solved_pe, h2d_p, d2h_p = decomposition_steps_e2e(torch, decs, streams, targets, lambda k, t: x0h[k],
                                                           e2e_seeds)
    t_le, solved_le, h2d_l, d2h_l = decomposition_steps_e2e(torch, decs, streams, targets,
                                                           lambda k, t: init.predict(t), e2e_seeds)
    plain["e2e"] = {"value": solved_pe / t_pe, "unit": UNIT, "h2d_bytes_per_step": h2d_p, "d2h_bytes_per_step": d2h_p}
    learned_e2e = {"value": solved_le / t_le, "unit": UNIT, "h2d_bytes_per_step": h2d_l, "d2h_bytes_per_step": d2h_l}

    # kernels of ours per step: learned = features, 5 layer GEMMs (tcgen05), angle head, k_decompose
    launches_learned = 8 * args.steps
    line = {
        "metric": METRIC, "value": learned["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": learned["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Haar + random-circuit 3-qubit targets)",
        "config": {"workload": "4096 held-out 3-qubit targets (half Haar, half random CNOT+U3 circuits with 1..14 "
                               "CNOTs), 14-block NN CNOT+U3 ansatz (93 params), learned-initialiser path, BFGS "
                               "batched 4096-wide",
                   "targets": N_TARGETS, "params": P, "tolerance": TOL, "max_calls_per_bfgs": MAX_CALLS,
                   "restarts": MAX_OUTER, "init": "learned MLP initialiser (random-start plain path in 'plain')",
                   "steps_overlap": "consecutive steps on two streams",
                   "l2": "flushed before every step (256 MB write)"},
        "solved_fraction": learned["solved_fraction"],
        "evaluations_per_step": learned["evaluations_per_step"],
        "ratio_vs_plain": learned["value"] / plain["value"],
        "e2e": learned_e2e,
        "gpu_launches": launches_learned,
        "roofline": {"bound": "fp64", "achieved": learned["achieved_tflops"], "peak": FP64_PEAK_TFLOPS,
                     "unit": "TFLOP/s", "peak_source": "measured live by the FP64 probe kernel",
                     "frac": learned["achieved_tflops"] / FP64_PEAK_TFLOPS, "traffic": K_DECOMPOSE_DRAM_BYTES,
                     "traffic_source": K_DECOMPOSE_TRAFFIC_SOURCE,
                     "note": "k_decompose is FP64-issue bound; achieved = algorithmic flops of the evaluations "
                             "(3 passes x 16 flop per complex element per parametric gate) and BFGS iterations "
                             "(17 P^2) of the timed learned-path steps over their time",
                     "flops_per_eval": flops_eval, "flops_per_bfgs_iteration": bfgs_flops_per_iteration(P)},
        "learned": dict(learned, training=train_stats,
                        init="MLP 128 -> 4x1024 -> 186 (BF16, FP32 accumulate, tcgen05), trained on 204800 "
                             "decompositions"),
        "plain": plain,
    }
    if clk:
        line["clocks"] = clk
    if not args.skip_secondary:
        line["gate_apply_n12"] = bench_gate_apply(sqg, wl, torch)
        line["cost_grad_n8"] = bench_cost_grad(sqg, wl, torch)
        line["cost_grad_uneven"] = bench_ragged(sqg, wl, torch)
        line["cost_grad_n10"] = bench_cost_grad_n10(sqg, wl, torch)
        line["decompose_n4_single"] = bench_single_n4(sqg, wl, torch)
        line["dropin_loops"] = bench_dropin_loops(sqg, wl, torch)
        line["decompose_n6_batched"] = bench_decompose_n6(sqg, wl, torch)
        line["state_vector_n24"] = bench_state_vector(sqg, wl, torch)
        line["decompose_16384_one_launch"] = bench_large_batch(sqg, wl, torch, ansatz, targets)
    if not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(sqg, wl, ansatz, targets, P, budget_s=args.cpu_seconds)
    return line


def bench_large_batch(sqg, wl, torch, ansatz, targets):
    """The headline workload four times over in one launch (16384 targets: the 4096 of the
    headline with four independent random starts each): the end-of-batch tail of a single
    4096-target step is spread over four times the work."""
    P = ansatz.get_Parameter_Num()
    rng = np.random.default_rng(4242)
    T = torch.from_numpy(np.concatenate([targets] * 4)).cuda()
    dec = sqg.BatchedDecomposer(ansatz, tolerance=TOL, max_calls=MAX_CALLS, max_outer=MAX_OUTER)
    x0 = torch.from_numpy(rng.uniform(0, 2 * np.pi, (T.shape[0], P))).cuda()
    dec.run(T, x0, seed=1)
    torch.cuda.synchronize()
    x0 = torch.from_numpy(rng.uniform(0, 2 * np.pi, (T.shape[0], P))).cuda()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    x, cost, calls = dec.run(T, x0, seed=2)
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    solved = int((cost.cpu().numpy() < TOL).sum())
    return {"config": "16384 targets (the 4096 headline targets x 4 random starts) in one launch",
            "seconds": t, "decompositions_per_s": solved / t, "solved_fraction": solved / T.shape[0]}


def bench_gate_apply(sqg, wl, torch):
    """n=12, 2000 random gates of U3/RY/CNOT/CZ/CRY, batch of 4 parameter vectors."""
    hbm, src = peaks()
    n, L, B = 12, 2000, 4
    rng = np.random.default_rng(5)
    c = wl.random_gate_circuit(n, L, rng)
    P = c.get_Parameter_Num()
    N = 1 << n
    th = torch.from_numpy(rng.uniform(0, 2 * np.pi, (B, P))).cuda()
    m = torch.empty((B, N, N), dtype=torch.complex128, device="cuda")
    m.real.normal_()
    recs = c.gate_records()
    frac = {7: 1.0, 8: 1.0, 9: 1.0, 10: 1.0, 5: 0.5, 14: 0.5, 4: 0.25}
    alg_bytes = sum(32.0 * N * N * frac[int(t)] for t, _, _, _ in recs)  # per parameter vector
    res = {}
    for fused in (True, False):
        c.apply_to_device(th, m, fused=fused)  # warm-up
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        c.apply_to_device(th, m, fused=fused)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        key = "fused" if fused else "unfused"
        res[key] = {"seconds": t, "algorithmic_GBps": B * alg_bytes / t / 1e9}
        if fused:
            res[key]["hbm_pass_GBps"] = B * 32.0 * N * N / t / 1e9
    fwd_ops = 0
    for t_, tg, ctl, ps in recs:
        t_ = int(t_)
        if t_ == 7:
            fwd_ops += 14 * (N // 2) * N
        elif t_ in (8, 9, 10):
            fwd_ops += 8 * (N // 2) * N
        elif t_ == 14:
            fwd_ops += 8 * (N // 4) * N
    res["fused"]["fp64_tflops"] = 2.0 * B * fwd_ops / res["fused"]["seconds"] / 1e12
    res["fused"]["note"] = ("fp64_tflops counts every gate's own FP64 rule; the fused path applies runs of "
                            "single-qubit gates on one qubit as one general 2x2 gate, which executes fewer")
    res["fused"]["fp64_frac"] = res["fused"]["fp64_tflops"] / FP64_PEAK_TFLOPS
    res["unfused"]["hbm_frac"] = res["unfused"]["algorithmic_GBps"] / hbm
    res["unfused"]["fp64_tflops"] = 2.0 * B * fwd_ops / res["unfused"]["seconds"] / 1e12
    # permutation/sign passes alone (CNOT and CZ, no FP64 instruction): one HBM pass per gate
    crng = np.random.default_rng(55)
    cc = sqg.Circuit(n)
    for _ in range(200):
        t_ = int(crng.integers(n))
        ctl = int(crng.integers(n - 1))
        ctl = ctl + 1 if ctl >= t_ else ctl
        (cc.add_CNOT if crng.integers(2) == 0 else cc.add_CZ)(t_, ctl)
    cbytes = sum(32.0 * N * N * frac[int(t)] for t, _, _, _ in cc.gate_records())
    th0 = torch.zeros((B, 0), dtype=torch.float64, device="cuda")
    cc.apply_to_device(th0, m, fused=False)
    torch.cuda.synchronize()
    e0.record()
    cc.apply_to_device(th0, m, fused=False)
    e1.record()
    e1.synchronize()
    tc = e0.elapsed_time(e1) / 1e3
    res["unfused_cnot_cz_only"] = {"gates": 200, "seconds": tc, "algorithmic_GBps": B * cbytes / tc / 1e9,
                                   "hbm_frac": B * cbytes / tc / 1e9 / hbm,
                                   "note": "CNOT (exchange of the control=1 row pairs) and CZ (sign of a quarter "
                                           "of the rows) passes execute no FP64 instruction: this is the HBM "
                                           "bound of k_gate_hbm"}
    # one full cost + adjoint-gradient evaluation of the same circuit at n = 12
    ev = sqg.CostEvaluator(c, torch.eye(N, dtype=torch.complex128, device="cuda"))
    ev.cost_grad(th[:1])
    torch.cuda.synchronize()
    e0.record()
    ev.cost_grad(th[:1])
    e1.record()
    e1.synchronize()
    tg = e0.elapsed_time(e1) / 1e3
    gops = fp64_ops_per_eval(recs, N, N)
    res["cost_grad_eval"] = {"seconds": tg, "fp64_tflops": 2.0 * gops / tg / 1e12}
    del ev
    res["peak_hbm_GBps"] = hbm
    res["peak_source"] = src
    res["config"] = "n=12 (4096x4096 complex128), 2000 random gates U3/RY/CNOT/CZ/CRY, batch 4"
    del m
    return res


def bench_cost_grad(sqg, wl, torch):
    """n=8 target from a 360-block ansatz at seeded angles, B=1024 parameter vectors."""
    n, blocks, B = 8, 360, 1024
    rng = np.random.default_rng(6)
    c = wl.cnot_u3_ansatz(n, blocks)
    P = c.get_Parameter_Num()
    U = c.get_Matrix(rng.uniform(0, 2 * np.pi, P))
    ev = sqg.CostEvaluator(c, np.ascontiguousarray(U.conj().T))
    th = torch.from_numpy(rng.uniform(0, 2 * np.pi, (B, P))).cuda()
    ev.cost_grad(th[:8])
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    ev.cost_grad(th)
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    ops = fp64_ops_per_eval(c.gate_records(), 1 << n, 1 << n) + 0
    return {"config": "n=8, 360 blocks (P=2184), B=1024, cost+adjoint gradient", "seconds": t,
            "evals_per_s": B / t, "fp64_tflops": 2.0 * ops * B / t / 1e12,
            "fp64_frac": 2.0 * ops * B / t / 1e12 / FP64_PEAK_TFLOPS}


def bench_ragged(sqg, wl, torch):
    """Uneven batch: 512 instances with n ~ U{3..9}, 3n(n-1)/2 CNOT+U3 blocks each, target =
    the instance's own ansatz at seeded angles; one cost+gradient launch for all of them."""
    rg = importlib.import_module(PKG + ".ragged")
    rng = np.random.default_rng(8)
    circs, targets, thetas = [], [], []
    for _ in range(512):
        n = int(rng.integers(3, 10))
        c = wl.cnot_u3_ansatz(n, 3 * n * (n - 1) // 2)
        P = c.get_Parameter_Num()
        U = c.get_Matrix(rng.uniform(0, 2 * np.pi, P))
        circs.append(c)
        targets.append(np.ascontiguousarray(U.conj().T))
        thetas.append(rng.uniform(0, 2 * np.pi, P))
    choice, report = rg.autotune_tile_cols(circs, targets, candidates=(1, 2, 4, 8, 16), reps=1)
    rb = rg.RaggedBatch(circs, targets, tile_cols=choice)
    th = rb.pack(thetas)
    rb.capture()
    rb.theta_static.copy_(th)
    rb.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    rb.replay()
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    ops = sum(fp64_ops_per_eval(c.gate_records(), 1 << c.qbit_num, 1 << c.qbit_num) for c in circs)
    return {"config": "512 instances, n ~ U{3..9}, 3n(n-1)/2 blocks, one persistent CUDA-graph launch, "
                      "tile widths autotuned per n", "seconds": t, "evals_per_s": 512 / t,
            "fp64_tflops": 2.0 * ops / t / 1e12, "fp64_frac": 2.0 * ops / t / 1e12 / FP64_PEAK_TFLOPS,
            "tile_cols_by_n": {int(n): int(choice[[c.qbit_num for c in circs].index(n)]) for n in range(3, 10)
                               if n in [c.qbit_num for c in circs]}}


def bench_single_n4(sqg, wl, torch):
    """One 4-qubit Haar target, U3 layer + 40 nearest-neighbour CNOT blocks (P = 252), BFGS
    towards cost < 1e-8 through the drop-in class with its host-driven loop (one GPU
    cost+gradient call per evaluation) and through the device decomposer (B = 1)."""
    rng = np.random.default_rng(11)
    U = wl.haar_unitary(16, rng)
    c = wl.cnot_u3_ansatz(4, 40)
    P = c.get_Parameter_Num()
    x0 = rng.uniform(0, 2 * np.pi, P)
    d = sqg.N_Qubit_Decomposition_custom(U.conj().T, config={"optimization_tolerance": 1e-8, "max_outer_iterations": 1,
                                                             "max_inner_iterations": 2000})
    d.set_Gate_Structure(c)
    d._host_loops = True  # BFGS driven from the host, one GPU cost+gradient call per evaluation
    d.set_Optimized_Parameters(x0)
    t0 = time.perf_counter()
    d.Start_Decomposition()
    t_host = time.perf_counter() - t0
    host_calls = d.get_Num_of_Iters()
    bd = sqg.BatchedDecomposer(c, tolerance=1e-8, max_calls=2000, max_outer=1)
    tdev = torch.from_numpy(np.ascontiguousarray(U.conj().T)[None]).cuda()
    bd.run(tdev, x0[None])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, cost, calls = bd.run(tdev, x0[None])
    torch.cuda.synchronize()
    t_dev = time.perf_counter() - t0
    return {"config": "n=4 Haar target, 40 NN CNOT+U3 blocks (P=252), one BFGS run of at most 2000 evaluations",
            "host_bfgs": {"evals": host_calls, "seconds": t_host, "evals_per_s": host_calls / t_host,
                          "final_cost": d.get_Decomposition_Error()},
            "device_bfgs": {"evals": int(calls.item()), "seconds": t_dev, "evals_per_s": int(calls.item()) / t_dev,
                            "final_cost": float(cost.item())},
            "note": "40 CNOTs are below the 61-CNOT lower bound for generic 4-qubit unitaries, so the cost "
                    "cannot reach 1e-8 on a Haar target"}


def bench_dropin_loops(sqg, wl, torch):
    """Single decompositions through the drop-in class above five qubits: the device loops (one
    CUDA graph launch per outer iteration) against the host-driven loops over the same GPU
    cost and gradient, per evaluation; and the structure search of the tree-search class on a
    3-qubit target made from a 5-CNOT structure (all candidates of a level in one launch)."""
    out = {}
    for n, blocks, opt, iters in [(6, 20, "BFGS", 1000), (6, 20, "ADAM", 1000), (8, 120, "BFGS", 60)]:
        rng = np.random.default_rng(n + blocks)
        c = wl.cnot_u3_ansatz(n, blocks)
        P = c.get_Parameter_Num()
        T = np.ascontiguousarray(wl.haar_unitary(1 << n, rng).conj().T)
        start = rng.uniform(0, 2 * np.pi, P)
        row = {"qbit_num": n, "params": P}
        for host in (False, True):
            d = sqg.N_Qubit_Decomposition_custom(T, config={"random_seed": 1, "max_inner_iterations": iters})
            d.set_Gate_Structure(c)
            d.set_Optimizer(opt)
            d.max_outer_iterations = 1
            d._host_loops = host
            d.set_Optimized_Parameters(start)
            d.Start_Decomposition()  # warm-up: graph, kernels
            d.num_iters = 0
            d.set_Optimized_Parameters(start)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d.Start_Decomposition()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            ev = d.get_Num_of_Iters()
            row["host_loop" if host else "device_loop"] = {"evals": ev, "seconds": dt, "us_per_eval": 1e6 * dt / ev}
        row["speedup"] = row["host_loop"]["us_per_eval"] / row["device_loop"]["us_per_eval"]
        out["%s_n%d_P%d" % (opt.lower(), n, P)] = row
    ts = importlib.import_module(PKG + ".tree_search")
    topo = ts.normalize_topology(None, 3)
    rng = np.random.default_rng(5)
    code = [0, 2, 1, 0, 2]
    c = ts.structure_circuit(code, topo, 3)
    U = c.get_Matrix(rng.uniform(0, 2 * np.pi, c.get_Parameter_Num()))
    d = sqg.N_Qubit_Decomposition_Tree_Search(np.ascontiguousarray(U.conj().T),
                                              config={"optimization_tolerance": 1e-8, "random_seed": 2})
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d.Start_Decomposition()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    cand = sum(ts.level_codes(lv, topo).shape[0] for lv in range(d.levels_done))
    out["tree_search_3q"] = {"config": "3-qubit target from a 5-CNOT structure, level search over all pairs",
                             "seconds": dt, "levels": d.levels_done, "structures": cand,
                             "structures_per_s": cand / dt, "cnots_found": len(d.best_cnot_sequence),
                             "error": d.get_Decomposition_Error()}
    return out


def bench_decompose_n6(sqg, wl, torch):
    """Batched six-qubit decompositions, one CTA per target (target read from L2, four warps
    per CTA): 608 targets built by the ansatz from random parameters, BFGS with one run of at
    most 500 evaluations from random starts."""
    out = {}
    for blocks in (3, 8):
        rng = np.random.default_rng(5)
        c = wl.cnot_u3_ansatz(6, blocks)
        P = c.get_Parameter_Num()
        B = 608
        T = np.stack([np.ascontiguousarray(c.get_Matrix(rng.uniform(0, 2 * np.pi, P)).conj().T) for _ in range(B)])
        tdev = torch.as_tensor(T, device="cuda")
        x0 = torch.as_tensor(rng.uniform(0, 2 * np.pi, (B, P)), device="cuda")
        dec = sqg.BatchedDecomposer(c, tolerance=1e-8, max_calls=500, max_outer=1)
        dec.run(tdev, x0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, cost, calls = dec.run(tdev, x0)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        ev = int(calls.sum().item())
        out["P%d" % P] = {"targets": B, "seconds": dt, "decompositions_per_s": B / dt, "evaluations": ev,
                          "evaluations_per_s": ev / dt, "solved_fraction": float((cost < 1e-8).float().mean().item())}
    return out


def bench_cost_grad_n10(sqg, wl, torch):
    """The n = 10 workload: 300 CNOT blocks over uniformly drawn ordered pairs
    (P = 1830), cost + adjoint gradient of 64 parameter vectors, plain and checkpointed."""
    rng = np.random.default_rng(12)
    c = wl.cnot_u3_ansatz(10, 300, pairs="random", rng=rng)
    P = c.get_Parameter_Num()
    U = c.get_Matrix(rng.uniform(0, 2 * np.pi, P))
    ev = sqg.CostEvaluator(c, np.ascontiguousarray(U.conj().T))
    th = torch.from_numpy(rng.uniform(0, 2 * np.pi, (64, P))).cuda()
    out = {"config": "n=10, 300 random-pair blocks (P=1830), B=64, cost + adjoint gradient"}
    for ck in (0, 30):
        ev.cost_grad(th[:2], checkpoint_interval=ck)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ev.cost_grad(th, checkpoint_interval=ck)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        ops = fp64_ops_per_eval(c.gate_records(), 1024, 1024) * 64
        out["checkpoint_%d" % ck] = {"seconds": t, "evals_per_s": 64 / t, "fp64_tflops": 2.0 * ops / t / 1e12}
    return out


def state_flops(circuit_records, n):
    """Algorithmic flops of one application to a 2^n state vector: 16 flop per touched
    complex element (two complex multiply-adds), CRY on the control = 1 half; CNOT and CZ
    are exchanges and sign flips."""
    f = 0
    for t, tg, c, ps in circuit_records:
        if t in (7, 8, 9, 10):
            f += 16 * (1 << n)
        elif t == 14:
            f += 16 * (1 << (n - 1))
    return f


def bench_state_vector(sqg, wl, torch):
    """The state-vector simulation benchmark circuit of SQUANDER
    (examples/simulation/QC_sim_benchmark.py) at n = 24: 4 sweeps of [U3, U3, CRY] over all
    qubit pairs (3313 gates) applied to a random normalised state (256 MB), fused blocks vs one
    pass per gate."""
    hbm, src = peaks()
    n = 24
    rng = np.random.default_rng(24)
    c = wl.qc_sim_circuit(n, levels=4)
    th = torch.from_numpy(rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())).cuda()
    v = torch.randn(1 << n, dtype=torch.complex128, device="cuda")
    v /= torch.linalg.vector_norm(v)
    flops = state_flops(c.gate_records(), n)
    res = {"config": "n=24 state vector (256 MB), SQUANDER QC_sim_benchmark circuit, 4 levels, %d gates"
                     % c.get_Gate_Num(), "blocks": c.state_block_count()}
    for fused in (True, False):
        c.apply_state_device(th, v, fused=fused)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c.apply_state_device(th, v, fused=fused)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        passes = c.state_block_count() if fused else c.get_Gate_Num()
        hbm_gbs = passes * 2 * 16 * (1 << n) / t / 1e9
        res["fused" if fused else "unfused"] = {
            "seconds": t, "fp64_tflops": flops / t / 1e12, "fp64_frac": flops / t / 1e12 / FP64_PEAK_TFLOPS,
            "hbm_pass_GBps": hbm_gbs, "hbm_frac": hbm_gbs / hbm}
    res["norm_after"] = float(torch.linalg.vector_norm(v))
    res["peak_hbm_GBps"] = hbm
    res["peak_source"] = src
    return res


def cpu_baseline(sqg, wl, ansatz, targets, P, budget_s=20.0):
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    recs = ansatz.gate_records()
    rng = np.random.default_rng(77)
    # bounded sample: calls of 16 targets per host thread (the work queue balances the long
    # decompositions against the short ones) until about budget_s of CPU work
    n = 16 * threads
    t0 = time.perf_counter()
    solved, done = 0, 0
    while True:
        idx = np.arange(done, done + n) % N_TARGETS
        x0 = rng.uniform(0, 2 * np.pi, (n, P))
        _, cost, _ = orc.decompose(3, recs, targets[idx], x0, tolerance=TOL, max_inner=MAX_CALLS,
                                   max_outer=MAX_OUTER, nthreads=threads, seed=int(rng.integers(1 << 31)))
        solved += int((cost < TOL).sum())
        done += n
        if time.perf_counter() - t0 > budget_s or done >= N_TARGETS:
            break
    t = time.perf_counter() - t0
    return {"value": solved / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the 4096 targets, same ansatz, tolerance and BFGS budgets, oracle C restatement of "
                      "SQUANDER's BFGS decomposition with %d threads (%.1f s)" % (done, threads, t),
            "solved_fraction": solved / done}


def bench_reference(args):
    """Reference arm: the reference algorithm on the host cores (oracle C restatement)."""
    from oracle import oracle as orc

    sqg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")

    def mat(circ, theta):
        return orc.get_matrix(circ.qbit_num, circ.gate_records(), theta)

    ansatz, targets = make_workload(sqg, wl, orc_matrix=mat)
    P = ansatz.get_Parameter_Num()
    recs = ansatz.gate_records()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(77)
    # 16 targets per host thread and step: the work queue then balances the long-running
    # decompositions (up to 4000 evaluations) against the short ones, as the GPU's batch does
    per_step = int(args.ref_targets) if args.ref_targets > 0 else 16 * threads
    per_step = max(threads, per_step)

    def step(k, count=per_step):
        idx = (np.arange(count) + k * per_step) % N_TARGETS
        x0 = rng.uniform(0, 2 * np.pi, (count, P))
        t0 = time.perf_counter()
        _, cost, _ = orc.decompose(3, recs, targets[idx], x0, tolerance=TOL, max_inner=MAX_CALLS,
                                   max_outer=MAX_OUTER, nthreads=threads, seed=k)
        return time.perf_counter() - t0, int((cost < TOL).sum())

    for w in range(args.warmup):  # one target per thread: warms the library and the threads
        step(100 + w, count=threads)
    times, solved = [], 0
    for k in range(args.steps):
        t, s = step(k)
        times.append(t)
        solved += s
    value = solved / sum(times)
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "config 4 plain path, bounded sample of %d targets per step" % per_step,
                       "params": P, "tolerance": TOL},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d targets per step" % per_step},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def profile_case(case, profile_calls=60):
    """Small single-launch cases for ncu captures (one kernel of interest each)."""
    import torch

    sqg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    rng = np.random.default_rng(3)
    if case == "decompose":
        ansatz, targets = make_workload(sqg, wl)
        P = ansatz.get_Parameter_Num()
        B = 1216
        dec = sqg.BatchedDecomposer(ansatz, tolerance=TOL, max_calls=profile_calls, max_outer=1,
                                    stop_at_tolerance=profile_calls == 60)
        x, cost, calls = dec.run(torch.from_numpy(targets[:B]).cuda(), rng.uniform(0, 2 * np.pi, (B, P)))
    elif case == "decompose_full":
        # one launch of the timed step itself: all 4096 targets, the bench's budgets (for the
        # one-pass DRAM byte counters only)
        ansatz, targets = make_workload(sqg, wl)
        P = ansatz.get_Parameter_Num()
        dec = sqg.BatchedDecomposer(ansatz, tolerance=TOL, max_calls=MAX_CALLS, max_outer=MAX_OUTER)
        x, cost, calls = dec.run(torch.from_numpy(targets).cuda(), rng.uniform(0, 2 * np.pi, (N_TARGETS, P)), seed=1000)
        torch.cuda.synchronize()
        print(json.dumps({"evaluations": int(calls.sum().item()), "bfgs_iterations": int(dec.iters.sum().item())}))
    elif case == "decompose_n6":
        # six-qubit targets, one CTA each (608 targets, at most 60 evaluations, one run)
        c = wl.cnot_u3_ansatz(6, 3)
        P = c.get_Parameter_Num()
        T = np.stack([np.ascontiguousarray(c.get_Matrix(rng.uniform(0, 2 * np.pi, P)).conj().T) for _ in range(608)])
        dec = sqg.BatchedDecomposer(c, tolerance=TOL, max_calls=profile_calls, max_outer=1)
        x, cost, calls = dec.run(torch.from_numpy(T).cuda(), rng.uniform(0, 2 * np.pi, (608, P)))
        torch.cuda.synchronize()
    elif case == "gate_apply":
        c = wl.random_gate_circuit(12, 200, rng)
        th = torch.from_numpy(rng.uniform(0, 2 * np.pi, (1, c.get_Parameter_Num()))).cuda()
        m = torch.zeros((1, 4096, 4096), dtype=torch.complex128, device="cuda")
        c.apply_to_device(th, m, fused=True)
        c.apply_to_device(th, m, fused=False)
    elif case == "mlp_gemm":
        ini = importlib.import_module(PKG + ".initializer")
        net = ini.MLP([8, 8], use_tc=True)
        A = torch.randn((4096, 1024), device="cuda").to(torch.bfloat16)
        B = torch.randn((1024, 1024), device="cuda").to(torch.bfloat16)
        C = torch.empty((4096, 1024), dtype=torch.float32, device="cuda")
        for _ in range(3):
            net._tc(A, B, 4096, 1024, 1024, C=C)
        torch.cuda.synchronize()
        net.check_errors()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(20):
            net._tc(A, B, 4096, 1024, 1024, C=C)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 20 / 1e3
        print(json.dumps({"mlp_gemm_tc": {"M": 4096, "N": 1024, "K": 1024, "seconds": t,
                                          "tflops": 2.0 * 4096 * 1024 * 1024 / t / 1e12}}))
    elif case == "dropin_bfgs_n6":
        batched = importlib.import_module(PKG + ".batched")
        c = wl.cnot_u3_ansatz(6, 20)
        P = c.get_Parameter_Num()
        T = np.ascontiguousarray(wl.haar_unitary(64, rng).conj().T)
        batched.bfgs_decompose_graph(c, T, rng.uniform(0, 2 * np.pi, P), max_calls=profile_calls, max_outer=1,
                                     stop_at_tolerance=False)
    elif case == "state_vector":  # n = 24 simulation circuit, one level: fused blocks, then one pass per gate
        c = wl.qc_sim_circuit(24, levels=1)
        th = torch.from_numpy(rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())).cuda()
        v = torch.randn(1 << 24, dtype=torch.complex128, device="cuda")
        c.apply_state_device(th, v, fused=True)
        c.apply_state_device(th, v, fused=False)
    elif case == "env_costgrad":  # small-register cost + gradient, 4096 parameter vectors of the 3-qubit ansatz
        ansatz, targets = make_workload(sqg, wl)
        P = ansatz.get_Parameter_Num()
        ev = sqg.CostEvaluator(ansatz, torch.from_numpy(targets).cuda())
        ev.cost_grad(torch.from_numpy(rng.uniform(0, 2 * np.pi, (targets.shape[0], P))).cuda())
    elif case == "ragged":  # uneven batch: 128 instances, n ~ U{3..9}
        rg = importlib.import_module(PKG + ".ragged")
        circs, tg, ths = [], [], []
        for _ in range(128):
            n = int(rng.integers(3, 10))
            c = wl.cnot_u3_ansatz(n, 3 * n * (n - 1) // 2)
            P = c.get_Parameter_Num()
            circs.append(c)
            tg.append(np.ascontiguousarray(c.get_Matrix(rng.uniform(0, 2 * np.pi, P)).conj().T))
            ths.append(rng.uniform(0, 2 * np.pi, P))
        rb = rg.RaggedBatch(circs, tg)
        rb.cost_grad(rb.pack(ths))
    elif case == "cost_grad":
        c = wl.cnot_u3_ansatz(8, 60)
        P = c.get_Parameter_Num()
        U = c.get_Matrix(rng.uniform(0, 2 * np.pi, P))
        ev = sqg.CostEvaluator(c, np.ascontiguousarray(U.conj().T))
        ev.cost_grad(torch.from_numpy(rng.uniform(0, 2 * np.pi, (64, P))).cuda())
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": case, "ok": True}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--probe-fp64", action="store_true", help="print the live FP64 FMA peak by active lanes")
    ap.add_argument("--profile-case", choices=["decompose", "decompose_full", "decompose_n6", "gate_apply", "cost_grad", "mlp_gemm", "dropin_bfgs_n6",
                                                     "state_vector", "env_costgrad", "ragged"],
                    default=None)
    ap.add_argument("--profile-calls", type=int, default=60,
                    help="evaluations per BFGS run in the decompose profile case (below 60: no tolerance stop)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-secondary", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-learned", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--ref-targets", type=int, default=0, help="targets per reference step (0: 16 per host thread)")
    args = ap.parse_args()
    if args.probe_fp64:
        native = importlib.import_module(PKG + "._native")
        print(json.dumps({"fp64_fma_tflops_by_active_lanes": {k: native.probe_fp64_tflops(k) for k in (32, 16, 8, 1)}}))
        return
    if args.profile_case:
        profile_case(args.profile_case, args.profile_calls)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(bench_reference(args)))
        return
    if world > 1:
        # batch sharding: rank r decomposes its own shard of world x 4096 distinct targets with
        # its own seeds; no collective on the data path, only the final reduction of the counts
        import torch
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        args.skip_secondary = True
        args.skip_cpu = rank != 0
        line = bench_ours(args, rank=rank, world=world)
        t = torch.tensor([line["ms_per_step"]], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        solved = torch.tensor([line["solved_fraction"] * N_TARGETS * args.steps], device="cuda", dtype=torch.float64)
        dist.all_reduce(solved, op=dist.ReduceOp.SUM)
        if rank == 0:
            line["ms_per_step"] = float(t.item())
            line["value"] = float(solved.item()) / (args.steps * line["ms_per_step"] / 1e3)
            line["n_gpus"] = world
            print(json.dumps(line))
        dist.destroy_process_group()
        return
    print(json.dumps(bench_ours(args)))


if __name__ == "__main__":
    main()
