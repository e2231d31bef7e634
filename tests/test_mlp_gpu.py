"""The learned initialiser's kernels (csrc/mlp.cu) against the NumPy oracle
(oracle/mlp_oracle.py): BF16 GEMM with FP32 accumulation in every transpose combination,
the forward pass, the backward pass (all weight and bias gradients) and the angle head.

Tolerances: GEMMs 1e-5 relative (exact bf16 products, FP32 vs FP64 accumulation order);
whole-network forward/backward 2e-2 in norm (a last-bit FP32 difference can move a bf16
rounding of an activation by one bf16 ulp, 2^-8, which then propagates)."""
import importlib

import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ini():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.initializer")


@pytest.mark.parametrize("ta,tb", [(False, True), (False, False), (True, False), (True, True)])
def test_gemm_bf16_all_layouts(ini, ta, tb):
    rng = np.random.default_rng(1)
    M, N, K = 70, 45, 100
    A = MO.bf16(rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32))
    B = MO.bf16(rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32))
    ref = (A.T if ta else A).astype(np.float64) @ (B.T if tb else B).astype(np.float64)
    Ad = torch.from_numpy(A).cuda().to(torch.bfloat16)
    Bd = torch.from_numpy(B).cuda().to(torch.bfloat16)
    C = torch.empty((M, N), dtype=torch.float32, device="cuda")
    mlp = ini.MLP([4, 4])
    mlp._gemm(Ad, ta, Bd, tb, M, N, K, C=C, lda=A.shape[1], ldb=B.shape[1])
    torch.cuda.synchronize()
    got = C.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref))


def test_forward_backward_match_oracle(ini):
    rng = np.random.default_rng(2)
    sizes = [128, 96, 96, 40]
    M = 48
    net = ini.MLP(sizes, seed=3)
    for i in range(len(net.b)):
        net.b[i].copy_(torch.randn(net.b[i].shape, dtype=torch.float32) * 0.1)
    net.b[-1][sizes[-1]:] = 0.0  # padding rows of the output layer stay zero
    x = rng.standard_normal((M, sizes[0])).astype(np.float32)
    xb = torch.from_numpy(x).cuda().to(torch.bfloat16)
    out, cache = net.forward(xb)
    W = [w.cpu().numpy() for w in net.W]
    b = [bb.cpu().numpy() for bb in net.b]
    ref_out, ref_cache = MO.forward(x, W, b)
    got = out.cpu().numpy()
    assert np.linalg.norm(got - ref_out) <= 2e-2 * np.linalg.norm(ref_out)
    P = sizes[-1] // 2
    assert got.shape[1] == 64 and np.all(got[:, 2 * P:] == 0)  # output padded to 64 with zero rows
    theta_star = rng.uniform(-np.pi, np.pi, (M, P))
    theta, og, loss_rows = ini.angle_head(out, P, mode=1, target=torch.from_numpy(theta_star).cuda(),
                                          scale=1.0 / (M * P))
    ref_loss, ref_og = MO.supervised_loss_grad(got[:, :2 * P], theta_star, 1.0 / (M * P))
    assert np.allclose(theta.cpu().numpy(), MO.angle_head(got[:, :2 * P], P), atol=1e-6)
    assert np.allclose(loss_rows.cpu().numpy(), ref_loss, rtol=1e-5, atol=1e-6)
    assert np.allclose(og.cpu().numpy()[:, :2 * P], ref_og, rtol=1e-5, atol=1e-9)
    assert np.all(og.cpu().numpy()[:, 2 * P:] == 0)
    dW, db = net.backward(og, cache)
    rdW, rdb = MO.backward(og.cpu().numpy(), W, ref_cache)
    for i in range(len(W)):
        g = dW[i].cpu().numpy()
        assert np.linalg.norm(g - rdW[i]) <= 2e-2 * np.linalg.norm(rdW[i]), i
        gb = db[i].cpu().numpy()
        assert np.linalg.norm(gb - rdb[i]) <= 2e-2 * np.linalg.norm(rdb[i]) + 1e-12, i
    # chain rule through atan2
    dth = rng.standard_normal((M, P))
    _, og2, _ = ini.angle_head(out, P, mode=2, dtheta=torch.from_numpy(dth).cuda(), scale=0.5)
    assert np.allclose(og2.cpu().numpy()[:, :2 * P], MO.chain_dtheta(got[:, :2 * P], dth, 0.5), rtol=1e-4, atol=1e-7)


def test_backward_matches_finite_differences_in_fp32(ini):
    """Directional derivative of the supervised loss along dW[0], by central differences of
    the oracle's loss (weights perturbed by a step far above the bf16 resolution)."""
    rng = np.random.default_rng(4)
    sizes = [16, 32, 8]
    M = 8
    net = ini.MLP(sizes, seed=5)
    x = rng.standard_normal((M, sizes[0])).astype(np.float32)
    theta_star = rng.uniform(-np.pi, np.pi, (M, sizes[-1] // 2))
    out, cache = net.forward(torch.from_numpy(x).cuda().to(torch.bfloat16))
    P = sizes[-1] // 2
    _, og, _ = ini.angle_head(out, P, mode=1, target=torch.from_numpy(theta_star).cuda(), scale=1.0 / (M * P))
    dW, db = net.backward(og, cache)
    W = [w.cpu().numpy() for w in net.W]
    b = [bb.cpu().numpy() for bb in net.b]

    def loss(Wl):
        o, _ = MO.forward(x, Wl, b)
        l, _ = MO.supervised_loss_grad(o[:, :2 * P], theta_star, 1.0)
        return l.mean()

    d = dW[0].cpu().numpy()
    h = 0.05 / np.linalg.norm(d)
    lp = loss([W[0] + h * d] + W[1:])
    lm = loss([W[0] - h * d] + W[1:])
    fd = (lp - lm) / (2 * h)
    an = float(np.sum(d * d))
    assert abs(fd - an) <= 0.1 * abs(an)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 130, 72), (512, 192, 1024), (1000, 1024, 128), (64, 8, 8)])
def test_tcgen05_gemm_matches_reference(ini, M, N, K):
    """C = A B^T on the tcgen05 tensor cores (TMA-staged, 128-byte swizzle) against an FP64
    product of the same bf16 operands."""
    rng = np.random.default_rng(M + N + K)
    A = MO.bf16(rng.standard_normal((M, K)).astype(np.float32))
    B = MO.bf16(rng.standard_normal((N, K)).astype(np.float32))
    bias = rng.standard_normal(N).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T + bias
    net = ini.MLP([8, 8], use_tc=True)
    Ad = torch.from_numpy(A).cuda().to(torch.bfloat16)
    Bd = torch.from_numpy(B).cuda().to(torch.bfloat16)
    C = torch.full((M, N), np.nan, dtype=torch.float32, device="cuda")
    Cb = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    net._tc(Ad, Bd, M, N, K, C=C, Cb=Cb, bias=torch.from_numpy(bias).cuda(), relu=False)
    torch.cuda.synchronize()
    net.check_errors()
    got = C.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref)) + 1e-5
    assert np.allclose(Cb.float().cpu().numpy(), got, rtol=1e-2, atol=1e-2)


def test_tcgen05_network_matches_mma_sync_network(ini):
    rng = np.random.default_rng(7)
    sizes = [128, 256, 256, 186]
    M = 256
    a = ini.MLP(sizes, seed=9, use_tc=False)
    b = ini.MLP(sizes, seed=9, use_tc=True)
    x = torch.from_numpy(rng.standard_normal((M, 128)).astype(np.float32)).cuda().to(torch.bfloat16)
    oa, ca = a.forward(x)
    ob, cb = b.forward(x)
    torch.cuda.synchronize()
    b.check_errors()
    assert float((oa - ob).abs().max()) <= 1e-4 * float(oa.abs().max())
    P = 93
    t = torch.from_numpy(rng.uniform(-np.pi, np.pi, (M, P))).cuda()
    _, ga, _ = ini.angle_head(oa, P, mode=1, target=t, scale=1.0 / (M * P))
    _, gb, _ = ini.angle_head(ob, P, mode=1, target=t, scale=1.0 / (M * P))
    dWa, dba = a.backward(ga, ca)
    dWb, dbb = b.backward(gb, cb)
    torch.cuda.synchronize()
    b.check_errors()
    for i in range(len(dWa)):
        assert float((dWa[i] - dWb[i]).norm()) <= 1e-3 * float(dWa[i].norm()) + 1e-12
        assert float((dba[i] - dbb[i]).norm()) <= 1e-3 * float(dba[i].norm()) + 1e-12
