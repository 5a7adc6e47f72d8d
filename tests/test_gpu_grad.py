"""Adjoints on the GPU (the differentiation form): max-min witnesses (saved and
recomputed), the max-min / ratio / B-spline MI backward kernels, and the whole
MCP3 edge-score loss, against the FP64 CPU oracle and finite differences.

The max-min adjoint is exact arithmetic (routing) and is compared to the
oracle run on the same float matrices; the MI adjoint runs in FP32 and is
compared to the FP64 oracle with a relative tolerance of 1e-3 (of the largest
gradient entry)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym01(rng, n):
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    return A


@pytest.mark.parametrize("rows,cols,k", [(1, 1, 1), (5, 3, 7), (129, 77, 200), (130, 130, 130)])
def test_witness_matches_oracle(gpu, port, rows, cols, k):
    rng = np.random.default_rng(rows + cols + k)
    A = rng.normal(size=(rows, k)).astype(np.float32)
    B = rng.normal(size=(cols, k)).astype(np.float32)
    C, K = gpu.maxmin_witness(A, B)
    assert np.array_equal(C, port.maxmin(A, B))
    Ko = port.maxmin_bwd(A, B, C, np.zeros_like(C), np.zeros_like(A), np.zeros_like(B))
    assert np.array_equal(K, Ko)


def test_witness_symmetric_and_ties(gpu, port):
    rng = np.random.default_rng(2)
    A = (rng.integers(0, 4, size=(150, 150)) * 0.25).astype(np.float32)  # many ties
    C, K = gpu.maxmin_witness(A)  # symmetric path
    Ko = port.maxmin_bwd(A, A, C, np.zeros_like(C), np.zeros_like(A), np.zeros_like(A))
    assert np.array_equal(C, port.maxmin(A)) and np.array_equal(K, Ko)


@pytest.mark.parametrize("saved", [True, False])
def test_maxmin_and_ratio_bwd_vs_oracle(gpu, port, saved):
    import torch
    rng = np.random.default_rng(7)
    n = 140
    A = _sym01(rng, n)
    S = rng.random((n, n)) < 0.05
    c = (rng.uniform(-1, 1, (n, n)) * S).astype(np.float32)
    M1 = port.maxmin(A)
    M2 = port.maxmin(A, M1)
    # oracle (float, sequential)
    dA_o, dM2_o, dM1_o = (np.zeros((n, n), np.float32) for _ in range(3))
    port.ratio_bwd(A, M2, c, dA_o, dM2_o)
    port.maxmin_bwd(A, M1, M2, dM2_o, dA_o, dM1_o)
    port.maxmin_bwd(A, A, M1, dM1_o, dA_o, dA_o)
    # GPU
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    Ad, M1d, M2d, cd = t(A), t(M1), t(M2), t(c)
    dA, dM2, dM1 = (torch.zeros((n, n), device="cuda") for _ in range(3))
    K1 = K2 = None
    if saved:
        K1 = torch.empty((n, n), dtype=torch.int32, device="cuda")
        K2 = torch.empty((n, n), dtype=torch.int32, device="cuda")
        tmp = torch.empty((n, n), device="cuda")
        gpu.maxmin_witness_dev(Ad, Ad, tmp, K1)
        gpu.maxmin_witness_dev(Ad, M1d, tmp, K2)
    gpu.ratio_bwd_dev(Ad, M2d, cd, dA, dM2)
    gpu.maxmin_bwd_dev(Ad, M1d, M2d, dM2, K2, dA, dM1)
    gpu.maxmin_bwd_dev(Ad, Ad, M1d, dM1, K1, dA, dA)
    gpu.synchronize()
    np.testing.assert_allclose(dM2.cpu().numpy(), dM2_o, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(dM1.cpu().numpy(), dM1_o, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(dA.cpu().numpy(), dA_o, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("n,m,bins,order", [(40, 96, 10, 3), (100, 300, 10, 3), (33, 80, 7, 2)])
def test_mi_bwd_vs_fp64(gpu, port, built_lib, n, m, bins, order):
    rng = np.random.default_rng(n + m)
    X = built_lib.synth_grn(n, m, seed=n * 7 + m)
    G = (rng.normal(size=(n, n)) * (rng.random((n, n)) < 0.2)).astype(np.float32)
    dX = gpu.bspline_mi_bwd(X, G, bins, order)
    ref = port.mi_bwd(X.astype(np.float64), G.astype(np.float64), bins, order)
    err = np.abs(dX - ref).max() / np.abs(ref).max()
    assert err < 1e-3, err


def test_mcp3_loss_grad_small_vs_oracle_and_fd(gpu, port, built_lib):
    """The whole differentiation form at 64 genes x 128 samples: GPU gradient vs
    (i) the oracle composed on the same float max-min values with the FP64 MI
    adjoint and (ii) central finite differences of the FP64 oracle forward."""
    import torch
    rng = np.random.default_rng(11)
    n, m = 64, 128
    X = built_lib.synth_grn(n, m, seed=4242)
    iu = np.array([(i, j) for i in range(n) for j in range(n) if i != j])
    pick = iu[rng.random(len(iu)) < 0.05]
    coef = rng.uniform(-1, 1, len(pick))
    Xd = torch.from_numpy(X).cuda()
    ri = torch.from_numpy(pick[:, 0]).cuda()
    ci = torch.from_numpy(pick[:, 1]).cuda()
    cf = torch.from_numpy(coef).cuda()
    L_s, dX_s = gpu.mcp3_loss_grad_dev(Xd, ri, ci, cf, witness="saved")
    L_r, dX_r = gpu.mcp3_loss_grad_dev(Xd, ri, ci, cf, witness="recompute")
    dX_s, dX_r = dX_s.cpu().numpy(), dX_r.cpu().numpy()
    assert L_s == L_r
    np.testing.assert_allclose(dX_s, dX_r, rtol=1e-5, atol=1e-6 * np.abs(dX_s).max())

    # (i) oracle on the GPU's float MI (identical max-min routing), FP64 MI adjoint
    A = gpu.bspline_mi(X, 10, 3, "fp32")
    np.fill_diagonal(A, 0)
    c = np.zeros((n, n), np.float32)
    np.add.at(c, (pick[:, 0], pick[:, 1]), coef.astype(np.float32))
    M1 = port.maxmin(A)
    M2 = port.maxmin(A, M1)
    dA, dM2, dM1 = (np.zeros((n, n), np.float32) for _ in range(3))
    port.ratio_bwd(A, M2, c, dA, dM2)
    port.maxmin_bwd(A, M1, M2, dM2, dA, dM1)
    port.maxmin_bwd(A, A, M1, dM1, dA, dA)
    np.fill_diagonal(dA, 0)
    ref = port.mi_bwd(X.astype(np.float64), dA.astype(np.float64))
    assert np.abs(dX_s - ref).max() / np.abs(ref).max() < 1e-3

    # (ii) central finite differences (step 1e-3) of the FP64 forward
    X64 = X.astype(np.float64)

    def loss(Xv):
        Av = port.bspline_mi(Xv)
        np.fill_diagonal(Av, 0)
        R = port.ratio(Av, port.maxmin(Av, port.maxmin(Av)))
        return float((coef * R[pick[:, 0], pick[:, 1]]).sum())

    agree = 0
    trials = 24
    for _ in range(trials):
        g, s = int(rng.integers(n)), int(rng.integers(m))
        Xp, Xm = X64.copy(), X64.copy()
        Xp[g, s] += 1e-3
        Xm[g, s] -= 1e-3
        fd = (loss(Xp) - loss(Xm)) / 2e-3
        agree += abs(fd - dX_s[g, s]) <= 0.05 * abs(fd) + 1e-3 * np.abs(dX_s).max()
    # a max-min witness can switch inside +-1e-3 (the loss is piecewise smooth)
    assert agree >= int(0.8 * trials), agree


def test_config4_scale_gradient_vs_fp64(gpu, port, built_lib):
    """Differentiation form at 4,096 genes x 1,024 samples with a seeded 5 % of
    gene pairs and U(-1, 1) weights: saved and recomputed witnesses agree, and
    the FP32 GPU gradient dL/dX matches the FP64 CPU adjoint given the same
    dL/dMI to 1e-4 of its largest entry."""
    import torch
    rng = np.random.default_rng(20260004)
    n, m = 4096, 1024
    X = built_lib.synth_grn(n, m, seed=20260001)
    iu = np.triu_indices(n, 1)
    sel = rng.random(len(iu[0])) < 0.05
    ri = torch.from_numpy(iu[0][sel].astype(np.int64)).cuda()
    ci = torch.from_numpy(iu[1][sel].astype(np.int64)).cuda()
    cf = torch.from_numpy(rng.uniform(-1, 1, int(sel.sum()))).cuda()
    Xd = torch.from_numpy(X).cuda()
    L1, dX1, dA = gpu.mcp3_loss_grad_dev(Xd, ri, ci, cf, witness="saved", return_dA=True)
    L2, dX2 = gpu.mcp3_loss_grad_dev(Xd, ri, ci, cf, witness="recompute")
    dX1, dX2 = dX1.cpu().numpy(), dX2.cpu().numpy()
    assert L1 == L2
    assert np.abs(dX1 - dX2).max() <= 1e-5 * np.abs(dX1).max()
    ref = port.mi_bwd(X.astype(np.float64), dA.cpu().numpy().astype(np.float64))
    assert np.abs(dX1 - ref).max() <= 1e-4 * np.abs(ref).max()
