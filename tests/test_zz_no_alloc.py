"""sqg_cost_grad_noalloc: the cost/gradient entry point for callers that cannot allocate
device memory (for instance a cost callback behind an optimizer interface that passes only
the parameters, the cost and the gradient, so it has nowhere to keep a workspace).  It runs
the same kernels as sqg_cost_grad on a 32 MiB scratch array built into the library; the cases
below put both the forward and the adjoint tile kernels on that array.  This file is collected last so that a run
stopping at the first failure has run every other test first."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n,blocks,cols,offset,checkpoint", [
    (5, 20, 32, 0, 0),   # five qubits: the gradient takes the environment-matrix form (no scratch)
    (5, 20, 32, 0, 4),   # checkpointed partial products: tile kernels on the scratch array
    (7, 12, 128, 0, 0),  # seven qubits: forward and adjoint tile kernels on the scratch array
    (7, 12, 48, 40, 0),  # rectangular target with a trace offset
])
def test_noalloc_entry_point_matches_workspace_entry_point(sqg, n, blocks, cols, offset, checkpoint):
    native = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    lib = native.lib()
    rng = np.random.default_rng(77 + n + cols)
    circ = wl.cnot_u3_ansatz(n, blocks)
    P = circ.get_Parameter_Num()
    U = circ.get_Matrix(rng.uniform(0, 2 * np.pi, P))
    target = torch.from_numpy(np.ascontiguousarray(U.conj().T[:, :cols])).cuda()
    ev = sqg.CostEvaluator(circ, target, trace_offset=offset)
    handle = ev.native.handle
    stream = torch.cuda.current_stream().cuda_stream
    B = 4
    need = lib.sqg_cost_grad_workspace_bytes(handle, B, cols, checkpoint)
    assert 0 < need <= native.SQG_NOALLOC_SCRATCH_BYTES
    for call in range(2):  # two calls in a row share the scratch array
        theta = torch.from_numpy(rng.uniform(0, 2 * np.pi, (B, P))).cuda()
        ref_cost, ref_grad = ev.cost_grad(theta, checkpoint_interval=checkpoint)
        cost = torch.full((B,), np.nan, dtype=torch.float64, device="cuda")
        grad = torch.full((B, P), np.nan, dtype=torch.float64, device="cuda")
        st = lib.sqg_cost_grad_noalloc(handle, theta.data_ptr(), B, target.data_ptr(), cols, 0, offset, 0,
                                       cost.data_ptr(), grad.data_ptr(), checkpoint, stream)
        assert st == 0, lib.sqg_last_error()
        torch.cuda.synchronize()
        scale = max(1.0, float(ref_grad.abs().max()))
        assert float((cost - ref_cost).abs().max()) <= 1e-12
        assert float((grad - ref_grad).abs().max()) <= 1e-12 * scale
        cost_only = torch.full((B,), np.nan, dtype=torch.float64, device="cuda")
        st = lib.sqg_cost_grad_noalloc(handle, theta.data_ptr(), B, target.data_ptr(), cols, 0, offset, 0,
                                       cost_only.data_ptr(), None, 0, stream)
        assert st == 0, lib.sqg_last_error()
        torch.cuda.synchronize()
        assert float((cost_only - ref_cost).abs().max()) <= 1e-12


def test_noalloc_reports_argument_errors_before_the_scratch_limit(sqg):
    native = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    wl = importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")
    lib = native.lib()
    nc = wl.cnot_u3_ansatz(8, 120).native()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # batch above 65535: an argument error, not a scratch error
    st = lib.sqg_cost_grad_noalloc(nc.handle, dummy.data_ptr(), 70000, dummy.data_ptr(), 256, 0, 0, 0,
                                   dummy.data_ptr(), dummy.data_ptr(), 0, stream)
    assert st == native.SQG_ERR_INVALID_ARGUMENT
    # a cost variant the engine does not implement
    st = lib.sqg_cost_grad_noalloc(nc.handle, dummy.data_ptr(), 1024, dummy.data_ptr(), 256, 0, 0, 1,
                                   dummy.data_ptr(), dummy.data_ptr(), 0, stream)
    assert st == native.SQG_ERR_UNSUPPORTED


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
