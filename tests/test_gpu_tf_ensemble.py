"""The TF form of the ensemble on the GPU: compute_maxmins_tfs, the TF
Stouffer transform (compute_stouffer_tf) and the TF coefficient searches.

The max-min products are bit-exact against the reference's own masked kernel
(golden) and the oracle.  The TF Stouffer's statistics (FP64 population mean
and sd, standing in for the absent splash StandardScore) are checked to one
float ulp of the oracle's (the GPU sums in another order); the per-entry
transform, fed the GPU's statistics, is bit-exact against the oracle's
restatement of zscored_stouffer_kernel, itself pinned to the reference's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def test_maxmins_tf_golden(gpu, golden):
    g = golden("tf_ensemble")
    got = gpu.maxmins_tf(g["A"], g["tfs"])
    for name, m in zip(("T", "M1", "M2", "M3"), got):
        assert same_bits(m, g[name]), name


def test_maxmins_tf_dev_partial_outputs(gpu, golden):
    """Only M3 requested (M1 kept in scratch), on a padded leading dimension."""
    import torch
    g = golden("tf_ensemble")
    A = dev(g["A"])
    t, n = g["T"].shape
    M3 = torch.full((t, n + 5), -7.0, device="cuda")[:, :n]
    gpu.maxmins_tf_dev(A, g["tfs"], M3=M3)
    torch.cuda.synchronize()
    assert same_bits(M3.cpu().numpy(), g["M3"])


@pytest.mark.parametrize("n,frac", [(1, 1.0), (2, 0.5), (5, 0.0), (257, 0.1), (300, 1.0)])
def test_maxmins_tf_vs_oracle(gpu, port, n, frac):
    rng = np.random.default_rng(n)
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    tfs = np.where(rng.random(n) < frac, np.inf, -np.inf).astype(np.float32)
    if frac == 1.0:
        tfs[:] = np.inf
    got = gpu.maxmins_tf(A, tfs)
    want = port.maxmins_tf(A, tfs)
    for name, a, b in zip(("T", "M1", "M2", "M3"), got, want):
        assert a.shape == b.shape and same_bits(a, b), name


def test_stouffer_tf_golden(gpu, port, golden):
    import torch
    g = golden("tf_ensemble")
    S = g["st_in"]
    dS = dev(S)
    stats = [x.cpu().numpy() for x in gpu.stouffer_tf_stats_dev(dS)]
    for got, key in zip(stats, ("st_rmean", "st_rsd", "st_cmean", "st_csd")):
        assert ulps(got, g[key]).max() <= 1, key
    assert stats[1][3] == 0.0 and stats[3][7] == 0.0
    out = gpu.stouffer_tf(S)
    assert same_bits(out, port.stouffer_tf_with_stats(S, *stats))
    if all(np.array_equal(a, g[k]) for a, k in zip(stats, ("st_rmean", "st_rsd", "st_cmean", "st_csd"))):
        assert same_bits(out, g["st_out"])
    o2 = torch.empty_like(dS)
    gpu.stouffer_tf_dev(dS, o2)
    torch.cuda.synchronize()
    assert same_bits(o2.cpu().numpy(), out)
    assert same_bits(gpu.transform_tf(S, "stouffer"), out)
    clr = gpu.transform_tf(S, "clr")
    assert same_bits(clr, port.stouffer_tf_with_stats(S, *stats, clr=True))
    if all(np.array_equal(a, g[k]) for a, k in zip(stats, ("st_rmean", "st_rsd", "st_cmean", "st_csd"))):
        assert same_bits(clr, g["clr_out"])
    gpu.transform_tf_dev(dS, o2, "clr")
    torch.cuda.synchronize()
    assert same_bits(o2.cpu().numpy(), clr)


@pytest.mark.parametrize("rows,cols", [(1, 1), (1, 9), (9, 1), (33, 300), (300, 33), (64, 4100)])
def test_stouffer_tf_vs_oracle(gpu, port, rows, cols):
    rng = np.random.default_rng(rows * 1000 + cols)
    S = rng.random((rows, cols)).astype(np.float32)
    if rows > 2 and cols > 2:
        S[1, :] = 0.25
        S[:, 2] = 0.25
    S[0, 0] = np.float32(3.4028235e38)  # FLT_MAX, as compute_combo writes for a vanishing denominator
    dS = dev(S)
    stats = [x.cpu().numpy() for x in gpu.stouffer_tf_stats_dev(dS)]
    want = port.tf_stats(S)
    for a, b, k in zip(stats, want, ("rmean", "rsd", "cmean", "csd")):
        assert ulps(a, b).max() <= 1, k
    out = gpu.stouffer_tf(S)
    assert same_bits(out, port.stouffer_tf_with_stats(S, *stats))


def test_combo_stouffer_tf_eval(gpu, port, golden):
    """The TF Stouffer search equals its composition from the individual GPU
    calls, the oracle's within 1e-12, and its host form; the TF combo search
    over the same rows matches the reference's values."""
    import torch
    g = golden("tf_ensemble")
    T, M1, M2, M3 = (dev(g[k]) for k in ("T", "M1", "M2", "M3"))
    L, rg, ct, cs = dev(g["labels_tf"]), dev(g["row_gene"]), dev(g["col_tf"]), g["coeffs"]
    pr, roc, best = gpu.combo_stouffer_tf_eval_dev(T, M1, M2, M3, L, cs, "tf", rg, ct)
    want_pr, want_roc = g["st_aupr"], g["st_auroc"]
    assert np.array_equal(np.isnan(pr), np.isnan(want_pr))
    ok = ~np.isnan(want_pr)
    assert np.all(np.abs(pr[ok] - want_pr[ok]) <= TOL) and np.all(np.abs(roc[ok] - want_roc[ok]) <= TOL)
    t, n = g["T"].shape
    comb = torch.empty((t, n), device="cuda")
    st = torch.empty((t, n), device="cuda")
    top, want_best = 0.0, 0
    for i, c in enumerate(cs):
        if c[0] == 1 and not c[1:].any():
            continue
        gpu.combo_dev(T, M1, M2, M3, c, comb)
        gpu.stouffer_tf_dev(comb, st)
        a, b, _, _ = gpu.eval_truth_dev(st, L, "tf", rg, ct)
        assert (pr[i], roc[i]) == (a, b)
        if a > top:
            top, want_best = a, i
    assert best == want_best == int(g["st_best"])
    hp, hr, hb = gpu.combo_stouffer_tf_eval(g["T"], g["M1"], g["M2"], g["M3"], g["labels_tf"], cs, "tf",
                                            g["row_gene"], g["col_tf"])
    assert np.array_equal(hp, pr, equal_nan=True) and np.array_equal(hr, roc, equal_nan=True) and hb == best
    cp, cr, cb = gpu.combo_eval_dev(T, M1, M2, M3, L, cs, "tf", rg, ct)
    ok = ~np.isnan(g["combo_aupr"])
    assert np.all(np.abs(cp[ok] - g["combo_aupr"][ok]) <= TOL) and np.all(np.abs(cr[ok] - g["combo_auroc"][ok]) <= TOL)
    assert cb == int(g["combo_best"])


def test_combo_stouffer_tf_eval_errors(gpu):
    import mcpnet_gb300 as M
    with pytest.raises(M.MCPGError):
        gpu.combo_stouffer_tf_eval(np.zeros((2, 3), np.float32), None, None, None, np.zeros((2, 3), np.int8),
                                   [0.5, 0.5, 0, 0], "all")  # M1 null with a non-zero coefficient
