"""sqg_cost_grad_noalloc: the cost/gradient entry point for callers that cannot allocate
device memory (for instance a cost callback behind an optimizer interface that passes only
the parameters, the cost and the gradient).  It runs the same kernels as sqg_cost_grad on a
32 MiB scratch array built into the library.  This file is collected last so that a run
stopping at the first failure has run every other test first."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_noalloc_entry_point_matches_workspace_entry_point(sqg):
    native = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    lib = native.lib()
    rng = np.random.default_rng(77)
    n = 5
    circ = wl.cnot_u3_ansatz(n, 20)
    P = circ.get_Parameter_Num()
    U = circ.get_Matrix(rng.uniform(0, 2 * np.pi, P))
    target = torch.from_numpy(np.ascontiguousarray(U.conj().T)).cuda()
    ev = sqg.CostEvaluator(circ, target)
    handle = ev.native.handle
    stream = torch.cuda.current_stream().cuda_stream
    B = 4
    for call in range(2):  # two calls in a row share the scratch array
        theta = torch.from_numpy(rng.uniform(0, 2 * np.pi, (B, P))).cuda()
        ref_cost, ref_grad = ev.cost_grad(theta)
        cost = torch.full((B,), np.nan, dtype=torch.float64, device="cuda")
        grad = torch.full((B, P), np.nan, dtype=torch.float64, device="cuda")
        st = lib.sqg_cost_grad_noalloc(handle, theta.data_ptr(), B, target.data_ptr(), target.shape[1], 0, 0, 0,
                                       cost.data_ptr(), grad.data_ptr(), 0, stream)
        assert st == 0, lib.sqg_last_error()
        torch.cuda.synchronize()
        scale = max(1.0, float(ref_grad.abs().max()))
        assert float((cost - ref_cost).abs().max()) <= 1e-12
        assert float((grad - ref_grad).abs().max()) <= 1e-12 * scale
        cost_only = torch.full((B,), np.nan, dtype=torch.float64, device="cuda")
        st = lib.sqg_cost_grad_noalloc(handle, theta.data_ptr(), B, target.data_ptr(), target.shape[1], 0, 0, 0,
                                       cost_only.data_ptr(), None, 0, stream)
        assert st == 0, lib.sqg_last_error()
        torch.cuda.synchronize()
        assert float((cost_only - ref_cost).abs().max()) <= 1e-12


def test_noalloc_rejects_requests_beyond_its_scratch(sqg):
    native = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    lib = native.lib()
    circ = wl.cnot_u3_ansatz(8, 120)
    nc = circ.native()
    B = 1024
    need = lib.sqg_cost_grad_workspace_bytes(nc.handle, B, 256, 1)
    assert need > native.SQG_NOALLOC_SCRATCH_BYTES
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = lib.sqg_cost_grad_noalloc(nc.handle, dummy.data_ptr(), B, dummy.data_ptr(), 256, 0, 0, 0,
                                   dummy.data_ptr(), dummy.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    assert st == native.SQG_ERR_WORKSPACE
    assert b"built-in array" in lib.sqg_last_error()
