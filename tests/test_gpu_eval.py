"""Gold-standard evaluation on the GPU (AUPR / AUROC, truth selection, the
ensemble coefficient search) against the reference's kernels' golden values
and the oracle.

Tolerance: every curve term is rounded as the reference rounds it; only the
order of the double sum differs (a deterministic compensated reduction on the
GPU, a left-to-right loop in the reference), so the results agree to a few
ulps of the sum: |gpu - ref| <= 1e-12 here.  Selected score vectors, counts
and the chosen coefficient row are exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def close(a, b):
    return abs(a - b) <= TOL


def test_eval_cases_golden(gpu, golden):
    import torch
    g = golden("eval_cases")
    for k in range(int(g["ncases"])):
        pos, neg = g[f"pos_{k}"], g[f"neg_{k}"]
        ref = g[f"ref64_{k}"]
        a, b = gpu.aupr_auroc(pos, neg)
        assert close(a, ref[0]) and close(b, ref[1]), (k, a, b, ref)
        dp = torch.from_numpy(pos).cuda()
        dn = torch.from_numpy(neg).cuda()
        a2, b2 = gpu.aupr_auroc_dev(dp, dn)
        assert (a2, b2) == (a, b), k  # same device path, deterministic


def test_eval_edge_values(gpu):
    assert gpu.aupr_auroc([], []) == (0.0, 0.0)
    assert gpu.aupr_auroc([], [1.0]) == (0.0, 1.0)
    assert gpu.aupr_auroc([1.0], []) == (1.0, 0.0)
    assert gpu.aupr_auroc([2.0, 3.0], [0.0, 1.0, 1.5]) == (1.0, 1.0)
    a, b = gpu.aupr_auroc([0.0, 1.0], [2.0, 3.0, 4.0])  # reversed: AUROC 0
    assert abs(b) <= 1e-15


def test_eval_nan_rejected(gpu, built_lib):
    with pytest.raises(built_lib.MCPGError):
        gpu.aupr_auroc([0.5, np.nan], [0.1])
    with pytest.raises(built_lib.MCPGError):
        gpu.aupr_auroc([0.5, 0.7], [0.1, np.nan, 0.2])
    assert gpu.aupr_auroc([0.5], [0.1]) == (1.0, 1.0)  # handle still usable


@pytest.mark.parametrize("P,N,levels", [(200_000, 3_000_000, 0), (5_000, 2_000_000, 97), (300_000, 40_000, 0),
                                        (7_000, 6_000, 13), (1, 1_000_000, 0), (1_000_000, 1, 0)])
def test_eval_large_vs_oracle(gpu, port, P, N, levels):
    """Sizes past the shared-memory staging (splitter search, global histograms)."""
    rng = np.random.default_rng(P + N)
    pos = rng.normal(0.4, 1.0, P).astype(np.float32)
    neg = rng.normal(0.0, 1.0, N).astype(np.float32)
    if levels:
        pos = (np.round(pos * levels) / levels).astype(np.float32)
        neg = (np.round(neg * levels) / levels).astype(np.float32)
    want = port.aupr_auroc(pos, neg)
    got = gpu.aupr_auroc(pos, neg)
    assert abs(got[0] - want[0]) <= 1e-11 and abs(got[1] - want[1]) <= 1e-11, (got, want)
    assert gpu.aupr_auroc(pos, neg) == got  # reproducible


def test_eval_truth_golden(gpu, golden):
    import torch
    g = golden("eval_truth")
    A, L = g["A"], g["labels"]
    ti, ct = g["tf_idx"], g["col_tf"]
    for region, V, Lb, rg, c in (("lower", A, L, None, None), ("all", A, L, None, None),
                                  ("tf", A[ti], L[ti], ti, ct)):
        ref = g[f"{region}_ref"]
        a, b, npos, nneg = gpu.eval_truth(V, Lb, region, rg, c)
        assert (npos, nneg) == (g[f"{region}_pos"].size, g[f"{region}_neg"].size), region
        assert close(a, ref[0]) and close(b, ref[1]), (region, a, b, ref)
        dv = torch.from_numpy(np.ascontiguousarray(V)).cuda()
        dl = torch.from_numpy(np.ascontiguousarray(Lb)).cuda()
        drg = None if rg is None else torch.from_numpy(rg).cuda()
        dct = None if c is None else torch.from_numpy(c).cuda()
        assert gpu.eval_truth_dev(dv, dl, region, drg, dct) == (a, b, npos, nneg)
        pos, neg = gpu.select_truth_dev(dv, dl, region, drg, dct)
        assert np.array_equal(pos.cpu().numpy(), g[f"{region}_pos"]), region  # row-major order
        assert np.array_equal(neg.cpu().numpy(), g[f"{region}_neg"]), region


def test_combo_eval_golden(gpu, golden):
    import torch
    g = golden("eval_truth")
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    pr, roc, best = gpu.combo_eval_dev(d(g["A"]), d(g["M1"]), d(g["M2"]), d(g["M3"]), d(g["labels"]), g["coeffs"])
    want_pr, want_roc = g["combo_aupr"], g["combo_auroc"]
    assert np.array_equal(np.isnan(pr), np.isnan(want_pr))
    ok = ~np.isnan(want_pr)
    assert np.all(np.abs(pr[ok] - want_pr[ok]) <= TOL) and np.all(np.abs(roc[ok] - want_roc[ok]) <= TOL)
    assert best == int(g["combo_best"])


@pytest.mark.parametrize("n,region", [(1, "lower"), (2, "all"), (777, "lower"), (4100, "lower"), (4100, "all"),
                                      (1500, "tf")])
def test_eval_truth_vs_oracle(gpu, port, n, region):
    """Ragged row segments (4096-column chunks), sparse and dense labels."""
    import torch
    rng = np.random.default_rng(n)
    V = rng.random((n, n)).astype(np.float32)
    V = np.round(V * 512) / 512
    V = V.astype(np.float32)
    L = rng.choice(np.array([-1, 0, 1, 2], np.int8), size=(n, n), p=[0.3, 0.6, 0.05, 0.05])
    rg = ct = None
    if region == "tf":
        tf = rng.random(n) < 0.1
        rg = np.nonzero(tf)[0].astype(np.int32)
        ct = tf.astype(np.uint8)
        V, L = V[rg], L[rg]
    want = port.eval_truth(V, L, region, rg, ct)
    got = gpu.eval_truth(V, L, region, rg, ct)
    assert got[2:] == want[2:]
    assert abs(got[0] - want[0]) <= 1e-11 and abs(got[1] - want[1]) <= 1e-11, (got, want)
    dv, dl = torch.from_numpy(V).cuda(), torch.from_numpy(np.ascontiguousarray(L)).cuda()
    drg = None if rg is None else torch.from_numpy(rg).cuda()
    dct = None if ct is None else torch.from_numpy(ct).cuda()
    pos, neg = gpu.select_truth_dev(dv, dl, region, drg, dct)
    wp, wn = port.select_truth(V, L, region, rg, ct)
    assert np.array_equal(pos.cpu().numpy(), wp) and np.array_equal(neg.cpu().numpy(), wn)


def test_eval_truth_full_size_properties(gpu):
    """20000 x 20000 scores, every lower-triangle entry labelled (2e8 pairs):
    perfect separation gives AUPR = AUROC = 1, reversed scores AUROC = 0, and
    the fused evaluation equals the evaluation of the selected vectors."""
    import torch
    n = 20000
    g = torch.Generator(device="cuda").manual_seed(3)
    V = torch.rand((n, n), device="cuda", generator=g)
    L = (torch.rand((n, n), device="cuda", generator=g) < 0.01).to(torch.int8)  # 1 = positive, 0 = negative
    a, b, npos, nneg = gpu.eval_truth_dev(V, L)
    assert npos + nneg == n * (n - 1) // 2
    pos, neg = gpu.select_truth_dev(V, L)
    assert (pos.numel(), neg.numel()) == (npos, nneg)
    assert gpu.aupr_auroc_dev(pos, neg) == (a, b)
    assert abs(b - 0.5) < 1e-2  # uniform scores: chance level
    sep = torch.where(L == 1, V + 2.0, V)
    a1, b1, _, _ = gpu.eval_truth_dev(sep, L)
    assert abs(a1 - 1.0) <= 1e-12 and b1 == 1.0  # AUPR: a sum of (run / n_pos) terms
    a0, b0, _, _ = gpu.eval_truth_dev(-sep, L)
    assert abs(b0) <= 1e-12
