"""The drop-in N_Qubit_Decomposition_adaptive with a caller-built gate structure
(add_Adaptive_Layers, add_Finalyzing_Layer_To_Gate_Structure) on the checks the reference's
own tests/decomposition/test_optmization_problem_combined.py makes: zero cost at the exact
parameters of a target cut by a trace offset, Combined_Unitary's matrix equal to get_Matrix,
the batch equal to single evaluations, Grad equal to the gradient of Combined; and the
reference's cost and gradient at other parameters (tests/golden/adaptive_n8.npz, made from the
reference by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LEVELS = 2


def _adaptive(sqg, Umtx, offset=0):
    d = sqg.N_Qubit_Decomposition_adaptive(Umtx, level_limit_max=5, level_limit_min=0, accelerator_num=0)
    if offset:
        d.set_Trace_Offset(offset)
    for _ in range(LEVELS):
        assert d.add_Adaptive_Layers() == 0
    assert d.add_Finalyzing_Layer_To_Gate_Structure() == 0
    return d


def test_adaptive_layers_trace_offset_and_combined_functions(sqg):
    f = np.load(os.path.join(GOLDEN, "adaptive_n8.npz"))
    builder = _adaptive(sqg, np.eye(256, dtype=np.complex128))
    assert builder.get_Parameter_Num() == f["exact"].size
    assert np.array_equal(builder.get_Circuit().gate_records(), f["gates"])
    # the matrix of the structure at the exact parameters, against the oracle
    U = builder.get_Matrix(f["exact"])
    Uo = O.get_matrix(8, f["gates"], f["exact"])
    assert np.max(np.abs(U - Uo)) < 1e-12
    # the decomposer of the cut target: zero cost at the exact parameters
    target = np.ascontiguousarray(Uo[80:240, :].conj().T)
    dec = _adaptive(sqg, target, offset=80)
    f0, g0 = dec.Optimization_Problem_Combined(f["exact"])
    assert abs(f0) < 1e-8 and abs(f0 - float(f["cost_exact"])) < 1e-12
    # the reference's cost and gradient elsewhere
    for k in range(f["theta"].shape[0]):
        c, g = dec.Optimization_Problem_Combined(f["theta"][k])
        assert abs(c - f["cost"][k]) <= 1e-12
        assert np.max(np.abs(g.reshape(-1) - f["grad"][k])) <= 1e-12 * max(1.0, np.max(np.abs(f["grad"][k])))
    # the consistency checks of the reference's test on the uncut identity target
    th = f["theta"][0]
    mat, mat_deriv = builder.Optimization_Problem_Combined_Unitary(th)
    assert np.allclose(builder.get_Matrix(th), mat, atol=1e-12) and len(mat_deriv) == th.size
    cost = builder.Optimization_Problem(th)
    batch = builder.Optimization_Problem_Batch(np.vstack([th, th, th]))
    assert np.allclose(batch.reshape(-1), cost, rtol=0, atol=1e-14)
    grad = builder.Optimization_Problem_Grad(th)
    fc, gc = builder.Optimization_Problem_Combined(th)
    assert np.allclose(grad, gc, rtol=0, atol=1e-14) and abs(fc - cost) < 1e-14
