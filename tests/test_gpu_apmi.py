"""Adaptive-partitioning MI on the GPU against the reference's own kernels
(golden fixtures) and the oracle.

Tolerance: given the same ranks every window decision (chi-square split,
counts) is exact and the sum has the reference's order; only log2 (CUDA's vs
the C library's, both within an ulp) can move the last bit of a term, so an
entry may differ from the reference by a few float ulps and most are equal:
|gpu - ref| <= 4 ulp(ref) + 1e-7, and at least 95% of entries bit-identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def assert_ap_close(got, want, exact_frac=0.95):
    got = np.asarray(got, np.float32)
    want = np.asarray(want, np.float32)
    tol = 4 * np.spacing(np.abs(want)) + 1e-7
    assert np.all(np.abs(got - want) <= tol), float(np.max(np.abs(got - want)))
    frac = float(np.mean(got.view(np.uint32) == want.view(np.uint32)))
    assert frac >= exact_frac, frac
    return frac


def test_ap_mi_golden(gpu, golden):
    g = golden("ap_mi")
    for name in g["names"]:
        mi = gpu.ap_mi_ranks(g[f"{name}_R"])
        assert_ap_close(mi, g[f"{name}_MI"])
        mi2 = gpu.ap_mi(g[f"{name}_X"])  # ranks on the GPU
        assert np.array_equal(mi2, mi), name


def test_ap_ranks_match_oracle(gpu, port):
    import torch
    rng = np.random.default_rng(3)
    for n, m in ((5, 1), (7, 33), (64, 1000), (3, 4097), (2, 16384)):
        X = rng.random((n, m)).astype(np.float32)
        if m > 10:
            X[:, ::7] = np.round(X[:, ::7] * 4) / 4  # ties
            X[0, 1] = -0.0
            X[0, 2] = 0.0
        R = torch.empty((n, m), dtype=torch.int32, device="cuda")
        gpu.ap_ranks_dev(torch.from_numpy(X).cuda(), R)
        assert np.array_equal(R.cpu().numpy(), port.ap_ranks(X)), (n, m)


@pytest.mark.parametrize("n,m", [(96, 2000), (40, 4096), (3, 16384), (130, 64)])
def test_ap_mi_vs_oracle(gpu, port, n, m):
    import mcpnet_gb300 as M
    X = M.synth_grn(n, m, seed=n + m)
    R = port.ap_ranks(X)
    assert_ap_close(gpu.ap_mi_ranks(R), port.ap_mi(R))


def test_ap_mi_noise_breaks_ties(gpu, port):
    import torch
    X = (np.round(np.random.default_rng(9).random((20, 500)) * 3) / 3).astype(np.float32)
    dX = torch.from_numpy(X).cuda()
    R = torch.empty((20, 500), dtype=torch.int32, device="cuda")
    gpu.ap_ranks_dev(dX, R, noise=1e-5, seed=7)
    Rh = R.cpu().numpy()
    # float32 holds only ~300 noisy values per level near 1/3 or 2/3, so some ties
    # survive (as in the reference's float mode); four levels become many ranks
    assert all(len(np.unique(r)) > 200 for r in Rh)
    assert np.all((Rh >= 0) & (Rh < 500))
    MI = torch.empty((20, 20), device="cuda")
    gpu.ap_mi_dev(dX, MI, noise=1e-5, seed=7)
    assert_ap_close(MI.cpu().numpy(), port.ap_mi(Rh))


def test_ap_mi_errors(gpu, built_lib):
    with pytest.raises(built_lib.MCPGError) as e:
        gpu.ap_mi(np.zeros((2, 16385), np.float32))
    assert e.value.status == built_lib.ERR_UNSUPPORTED
    with pytest.raises(built_lib.MCPGError):
        gpu.ap_mi_ranks(np.array([[0, 1, 5]], np.int32))  # rank outside [0, m)
    with pytest.raises(built_lib.MCPGError):
        gpu.ap_mi(np.array([[0.1, np.nan, 0.2]], np.float32))
    assert gpu.ap_mi(np.array([[0.3, 0.1]], np.float32)).shape == (1, 1)  # still usable


def test_ap_mi_4096_genes(gpu, port):
    """4096 genes x 1024 samples: symmetric, bounded by log2(m), and a
    48-gene subset equal to the oracle's."""
    import torch
    import mcpnet_gb300 as M
    n, m = 4096, 1024
    X = M.synth_grn(n, m, seed=20260001)
    dX = torch.from_numpy(X).cuda()
    MI = torch.empty((n, n), device="cuda")
    gpu.ap_mi_dev(dX, MI)
    A = MI.cpu().numpy()
    assert np.array_equal(A, A.T)
    assert np.all(np.isfinite(A)) and A.min() >= -1e-5 and A.max() <= np.log2(m) + 1e-4
    idx = np.random.default_rng(1).choice(n, 48, replace=False)
    R = port.ap_ranks(X[idx])
    assert_ap_close(A[np.ix_(idx, idx)], port.ap_mi(R))
