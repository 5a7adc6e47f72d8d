"""Stouffer / CLR transforms on the GPU.

The per-entry transforms are checked bit for bit against MCPNet's own
stouffer_vector_kernel / clr_vector_kernel (golden fixture, and the oracle's
restatement fed the GPU's statistics).  The row statistics (FP64 mean and
unbiased sd, rounded to float) stand in for the absent splash
GaussianParamsExclude1: they are checked against the oracle's FP64 two-pass
sums to one float ulp (the GPU sums in a different order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("mode", ["all", "exclude_diagonal"])
def test_transform_golden(gpu, port, golden, mode):
    import torch
    g = golden("stouffer")
    A = g["A"]
    dA = torch.from_numpy(A).cuda()
    n = A.shape[0]
    mean = torch.empty(n, device="cuda")
    sd = torch.empty(n, device="cuda")
    gpu.row_stats_dev(dA, mean, sd, stats=mode)
    m, s = mean.cpu().numpy(), sd.cpu().numpy()
    assert ulps(m, g[f"{mode}_mean"]).max() <= 1 and ulps(s, g[f"{mode}_sd"]).max() <= 1
    for kind in ("stouffer", "clr"):
        out = gpu.transform(A, kind, mode)
        want = port.transform_with_stats(A, m, s, clr=(kind == "clr"))  # the reference's kernels, the GPU's stats
        assert np.array_equal(out.view(np.uint32), want.view(np.uint32)), kind
        if np.array_equal(m, g[f"{mode}_mean"]) and np.array_equal(s, g[f"{mode}_sd"]):
            assert np.array_equal(out.view(np.uint32), g[f"{mode}_{kind}"].view(np.uint32))


@pytest.mark.parametrize("n", [1, 2, 3, 257, 1000])
def test_transform_vs_oracle(gpu, port, n):
    import torch
    rng = np.random.default_rng(n)
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    if n > 3:
        A[1, :] = 0.5  # sd 0
    dA = torch.from_numpy(A).cuda()
    mean = torch.empty(n, device="cuda")
    sd = torch.empty(n, device="cuda")
    gpu.row_stats_dev(dA, mean, sd)
    m, s = mean.cpu().numpy(), sd.cpu().numpy()
    om, osd = port.row_stats(A)
    assert ulps(m, om).max() <= 1 and ulps(s, osd).max() <= 1
    out = torch.empty_like(dA)
    for kind in ("stouffer", "clr"):
        gpu.transform_dev(dA, out, kind)
        want = port.transform_with_stats(A, m, s, clr=(kind == "clr"))
        assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32)), kind


def test_combo_stouffer_eval(gpu, port, golden):
    """The Stouffer half of the coefficient search equals its composition
    from the individual GPU calls, and the oracle's within 1e-9."""
    import torch
    g = golden("eval_truth")
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    A, M1, M2, M3, L, cs = d(g["A"]), d(g["M1"]), d(g["M2"]), d(g["M3"]), d(g["labels"]), g["coeffs"]
    pr, roc, best = gpu.combo_stouffer_eval_dev(A, M1, M2, M3, L, cs)
    n = A.shape[0]
    comb = torch.empty((n, n), device="cuda")
    tr = torch.empty((n, n), device="cuda")
    top, want_best = 0.0, 0
    for i, c in enumerate(cs):
        if c[0] == 1 and not c[1:].any():
            assert np.isnan(pr[i])
            continue
        gpu.combo_dev(A, M1, M2, M3, c, comb)
        gpu.transform_dev(comb, tr)
        a, b, _, _ = gpu.eval_truth_dev(tr, L)
        assert (pr[i], roc[i]) == (a, b)
        ca = port.combo(g["A"], g["M1"], g["M2"], g["M3"], c)
        oa, ob, _, _ = port.eval_truth(port.transform(ca), g["labels"])
        assert abs(oa - a) <= 1e-9 and abs(ob - b) <= 1e-9
        if a > top:
            top, want_best = a, i
    assert best == want_best
