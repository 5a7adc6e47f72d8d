"""Pins the CPU oracle (the C restatement) against fixtures produced by
MCPNet's own kernels (tests/golden/make_golden.py), and -- where the reference
build exists in this checkout -- against the reference directly."""
import numpy as np
import pytest

MI_CASES = ["mi_37x211", "mi_64x500", "mi_3x7", "mi_1x5", "mi_20x64_b8k2"]


@pytest.mark.parametrize("name", MI_CASES)
def test_weights_bit_exact(port, golden, name):
    g = golden(name)
    W = port.bspline_weights(g["X"], int(g["bins"]), int(g["order"]))
    # the weight block is bit-exact; the trailing H_g slot follows the
    # reference's SIMD reduction order (entropy1d_2), so only ~1 ulp
    assert np.array_equal(W[:, :-1], g["W"][:, :-1])
    np.testing.assert_allclose(W[:, -1], g["W"][:, -1], rtol=0, atol=2e-6)


@pytest.mark.parametrize("name", MI_CASES)
def test_mi_matches_reference(port, golden, name):
    g = golden(name)
    bins, order = int(g["bins"]), int(g["order"])
    mi32 = port.bspline_mi(g["X"], bins, order)
    np.testing.assert_allclose(mi32, g["MI32"], rtol=0, atol=5e-6)  # bits
    mi64 = port.bspline_mi(g["X"].astype(np.float64), bins, order)
    np.testing.assert_allclose(mi64, g["MI64"], rtol=0, atol=1e-12)
    assert np.array_equal(mi32, mi32.T)


@pytest.mark.parametrize("name", ["mcp_70", "mcp_130"])
def test_mcp_bit_exact(port, golden, name):
    g = golden(name)
    A = g["A"]
    for pl in (2, 3, 4):
        M, R = port.mcp(A, pl)
        assert np.array_equal(M.view(np.uint32), g[f"M{pl}"].view(np.uint32)), pl
        assert np.array_equal(R.view(np.uint32), g[f"R{pl}"].view(np.uint32)), pl
    M, R = port.mcp(A, 3, symmetrize=True)
    assert np.array_equal(M, g["M3s"]) and np.array_equal(R, g["R3s"])


@pytest.mark.parametrize("name", ["mcp_70", "mcp_130"])
def test_dpi_bit_exact(port, golden, name):
    g = golden(name)
    out, mask, removed = port.dpi(g["A"], float(g["tol"]))
    assert np.array_equal(out.view(np.uint32), g["DPI_out"].view(np.uint32))
    assert np.array_equal(mask, g["DPI_mask"])
    assert removed == int(g["DPI_removed"])


def test_dpi_ties(port, golden):
    g = golden("dpi_ties")
    for tag in ("t0", "t1"):
        out, mask, removed = port.dpi(g["A"], float(g[f"tol_{tag}"]))
        assert np.array_equal(out, g[f"out_{tag}"])
        assert np.array_equal(mask, g[f"mask_{tag}"])
        assert removed == int(g[f"removed_{tag}"])


def test_maxmin_rect_negative(port, golden):
    g = golden("maxmin_rect")
    C = port.maxmin(g["A"], g["B"])
    assert np.array_equal(C.view(np.uint32), g["C"].view(np.uint32))


def test_maxmin_empty_k_is_minus_inf(port):
    A = np.zeros((3, 0), np.float32)
    C = port.maxmin(A)
    assert np.all(np.isneginf(C))


def test_ratio_edges(port):
    A = np.array([[0.0, 1e-8, 0.5, -0.25, 3.0]], np.float32)
    M = np.array([[0.0, 0.5, 0.0, 0.5, 7.0]], np.float32)
    R = port.ratio(A, M)
    assert R[0, 0] == 0 and R[0, 1] == 0
    assert R[0, 2] == np.finfo(np.float32).max
    assert R[0, 3] == np.float32(-0.5)
    assert R[0, 4] == np.float32(np.float64(np.float32(3.0)) / np.float64(np.float32(7.0)))


def test_closure_matches_spanning_tree_bottleneck(port):
    """The squaring closure equals the bottleneck (max-capacity) path value
    read off a maximum spanning tree, for every off-diagonal pair."""
    rng = np.random.default_rng(3)
    n = 40
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    B, it = port.closure(A)
    assert it > 0
    # Prim's maximum spanning tree, then widest path by DFS
    in_t = np.zeros(n, bool); in_t[0] = True
    best = A[0].astype(np.float64).copy(); par = np.zeros(n, int)
    adj = [[] for _ in range(n)]
    for _ in range(n - 1):
        c = np.where(~in_t, best, -np.inf).argmax()
        in_t[c] = True
        adj[c].append((par[c], A[c, par[c]])); adj[par[c]].append((c, A[c, par[c]]))
        upd = (~in_t) & (A[c] > best)
        best[upd] = A[c][upd]; par[upd] = c
    for s in range(n):
        cap = np.full(n, np.inf, np.float32); seen = np.zeros(n, bool); st = [s]; seen[s] = True
        while st:
            u = st.pop()
            for v, w in adj[u]:
                if not seen[v]:
                    seen[v] = True; cap[v] = min(cap[u], w); st.append(v)
        off = np.arange(n) != s
        assert np.array_equal(B[s, off], cap[off])


def test_port_against_reference_build(port):
    """Extra seeded shapes against MCPNet's own kernels (only where the
    reference sources were available to build them)."""
    from oracle import oracle as O
    R = O.ref()
    if R is None:
        pytest.skip("reference build not present in this checkout")
    rng = np.random.default_rng(7)
    for n, m in ((5, 33), (17, 129), (40, 64)):
        X = rng.random((n, m)).astype(np.float32)
        assert np.array_equal(port.bspline_weights(X)[:, :-1], R.bspline_weights(X)[:, :-1])
        np.testing.assert_allclose(port.bspline_mi(X), R.bspline_mi(X), rtol=0, atol=5e-6)
        A = port.bspline_mi(X); np.fill_diagonal(A, 0)
        for pl in (2, 3, 4):
            a, b = port.mcp(A, pl), R.mcp(A, pl)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        a, b = port.dpi(A, 0.1), R.dpi(A, 0.1)
        assert np.array_equal(a[0], b[0]) and a[2] == b[2]


def test_reference_fast_math_same_bytes(port):
    """The reference's Release flags include -ffast-math; on the max-min / ratio /
    DPI path that build gives the same bytes as the strict build."""
    from oracle import oracle as O
    R, RF = O.ref(), O.ref(fast_math=True)
    if R is None or RF is None:
        pytest.skip("reference build not present in this checkout")
    rng = np.random.default_rng(8)
    A = rng.random((60, 60)).astype(np.float32); A = np.maximum(A, A.T); np.fill_diagonal(A, 0)
    for pl in (2, 3, 4):
        a, b = R.mcp(A, pl), RF.mcp(A, pl)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(R.dpi(A, 0.1)[0], RF.dpi(A, 0.1)[0])


def test_tf_variants_bit_exact(port, golden):
    """compute_mcp{2,3,4}_tfs for every tf_gene_transition, dpi_tf_kernel and a
    general-valued mask, against the reference's own TF kernels."""
    g = golden("tf_90")
    A, tfs = g["A"], g["tfs"]
    for pl, ts in ((2, (0, 1)), (3, (0, 1, 2)), (4, (0, 1, 2, 3))):
        for t in ts:
            M, R = port.mcp_tf(A, tfs, pl, t)
            assert np.array_equal(M.view(np.uint32), g[f"M{pl}_t{t}"].view(np.uint32)), (pl, t)
            assert np.array_equal(R.view(np.uint32), g[f"R{pl}_t{t}"].view(np.uint32)), (pl, t)
    out, mask, removed = port.dpi_tf(A, tfs, float(g["tol"]))
    assert np.array_equal(out, g["DPI_out"]) and np.array_equal(mask, g["DPI_mask"])
    assert removed == int(g["DPI_removed"])
    assert np.array_equal(port.maxmin_masked(A, A, g["mask_general"]), g["MM_general"])


def test_eval_cases_bit_exact(port, golden):
    """The restated AUPR / AUROC equal MCPNet's aupr_kernel / auroc_kernel
    bit for bit (same sequential double sums), for float and double scores."""
    g = golden("eval_cases")
    for k in range(int(g["ncases"])):
        got = port.aupr_auroc(g[f"pos_{k}"], g[f"neg_{k}"])
        assert got == tuple(g[f"ref32_{k}"]) == tuple(g[f"ref64_{k}"]), k


def test_eval_truth_regions(port, golden):
    g = golden("eval_truth")
    A, L = g["A"], g["labels"]
    ti, ct = g["tf_idx"], g["col_tf"]
    for region, V, Lb, rg, c in (("lower", A, L, None, None), ("all", A, L, None, None),
                                  ("tf", A[ti], L[ti], ti, ct)):
        pos, neg = port.select_truth(V, Lb, region, rg, c)
        assert np.array_equal(pos, g[f"{region}_pos"]) and np.array_equal(neg, g[f"{region}_neg"]), region
        a, b, npos, nneg = port.eval_truth(V, Lb, region, rg, c)
        assert (a, b) == tuple(g[f"{region}_ref"]), region
        assert (npos, nneg) == (pos.size, neg.size)


def test_eval_truth_lower_matches_reference_loop(golden):
    """select_lower_triangle keeps (i, j) with j < i and label 0/1, row-major."""
    g = golden("eval_truth")
    A, L = g["A"], g["labels"]
    n = A.shape[0]
    pos = [A[i, j] for i in range(n) for j in range(i) if L[i, j] == 1]
    neg = [A[i, j] for i in range(n) for j in range(i) if L[i, j] == 0]
    assert np.array_equal(np.array(pos, np.float32), g["lower_pos"])
    assert np.array_equal(np.array(neg, np.float32), g["lower_neg"])


def test_combo_eval_oracle(port, golden):
    g = golden("eval_truth")
    pr, roc, best = port.combo_eval(g["A"], g["M1"], g["M2"], g["M3"], g["labels"], g["coeffs"])
    np.testing.assert_array_equal(pr, g["combo_aupr"])
    np.testing.assert_array_equal(roc, g["combo_auroc"])
    assert best == int(g["combo_best"])
    assert np.isnan(pr[0])  # the (1, 0, 0, 0) row is skipped


def test_eval_against_reference_build(port):
    """Random vectors with ties straight against MCPNet's kernels (where built)."""
    from oracle import oracle as O
    ref = O.ref()
    if ref is None:
        pytest.skip("reference kernels not built in this checkout")
    rng = np.random.default_rng(5)
    for _ in range(100):
        k = int(rng.integers(1, 9))
        pos = (rng.integers(0, 4 * k, int(rng.integers(0, 80))) / k).astype(np.float32)
        neg = (rng.integers(0, 4 * k, int(rng.integers(0, 80))) / k - 0.2).astype(np.float32)
        assert port.aupr_auroc(pos, neg) == ref.aupr_auroc(pos, neg)


def test_ap_mi_bit_exact(port, golden):
    """The AP MI restatement equals MCPNet's IntegralCumulativeHistogramKernel +
    AdaptivePartitionRankMIKernel2 bit for bit, given the ranks (which come
    from the oracle's rank transform: the reference's own lives in the absent
    splash module)."""
    g = golden("ap_mi")
    for name in g["names"]:
        R = port.ap_ranks(g[f"{name}_X"])
        assert np.array_equal(R, g[f"{name}_R"]), name
        mi = port.ap_mi(R)
        assert np.array_equal(mi.view(np.uint32), g[f"{name}_MI"].view(np.uint32)), name


def test_ap_ranks_ties_share_lowest(port):
    X = np.array([[0.5, 0.9, 0.5, 0.1, 0.9, -0.0, 0.0]], dtype=np.float32)
    assert port.ap_ranks(X).tolist() == [[2, 0, 2, 4, 0, 5, 5]]


def test_stouffer_clr_bit_exact(port, golden):
    """The restated Stouffer / CLR element transforms equal MCPNet's
    stouffer_vector_kernel / clr_vector_kernel given the same row statistics
    (the statistics themselves stand in for the absent splash
    GaussianParamsExclude1 and are not pinned)."""
    g = golden("stouffer")
    A = g["A"]
    for mode in ("all", "exclude_diagonal"):
        mean, sd = port.row_stats(A, mode)
        assert np.array_equal(mean, g[f"{mode}_mean"]) and np.array_equal(sd, g[f"{mode}_sd"])
        assert sd[5] == 0.0
        for clr, key in ((False, "stouffer"), (True, "clr")):
            got = port.transform_with_stats(A, mean, sd, clr)
            assert np.array_equal(got.view(np.uint32), g[f"{mode}_{key}"].view(np.uint32)), (mode, key)


def test_maxmins_tf_oracle(port, golden):
    """compute_maxmins_tfs restated on the oracle's masked max-min equals the
    composition of MCPNet's own mcp2_maxmin_kernel<float,true,true> bit for bit."""
    g = golden("tf_ensemble")
    got = port.maxmins_tf(g["A"], g["tfs"])
    for name, m in zip(("T", "M1", "M2", "M3"), got):
        assert np.array_equal(m.view(np.uint32), g[name].view(np.uint32)), name


def test_stouffer_tf_bit_exact(port, golden):
    """The restated TF Stouffer combine equals MCPNet's zscored_stouffer_kernel
    given the same z-scores; a constant row and a constant column give z = 0
    (the population statistics stand in for the absent splash StandardScore
    and are not pinned)."""
    g = golden("tf_ensemble")
    S = g["st_in"]
    stats = port.tf_stats(S)
    for got, key in zip(stats, ("st_rmean", "st_rsd", "st_cmean", "st_csd")):
        assert np.array_equal(got, g[key]), key
    assert stats[1][3] == 0.0 and stats[3][7] == 0.0
    out = port.stouffer_tf_with_stats(S, *stats)
    assert np.array_equal(out.view(np.uint32), g["st_out"].view(np.uint32))
    clr = port.stouffer_tf_with_stats(S, *stats, clr=True)  # the transform app's zscored_clr_kernel
    assert np.array_equal(clr.view(np.uint32), g["clr_out"].view(np.uint32))


def test_stouffer_tf_population_statistics(port):
    """Row and column statistics are the FP64 population mean / sd."""
    rng = np.random.default_rng(3)
    S = rng.random((7, 11)).astype(np.float32)
    rm, rs, cm, cs = port.tf_stats(S)
    S64 = S.astype(np.float64)
    np.testing.assert_array_equal(rm, S64.mean(1).astype(np.float32))
    np.testing.assert_allclose(rs, S64.std(1), rtol=1e-6)
    np.testing.assert_array_equal(cm, S64.mean(0).astype(np.float32))
    np.testing.assert_allclose(cs, S64.std(0), rtol=1e-6)


def test_tf_searches_oracle(port, golden):
    """The TF combo and TF-Stouffer coefficient searches over the TF truth rows."""
    g = golden("tf_ensemble")
    args = (g["T"], g["M1"], g["M2"], g["M3"], g["labels_tf"], g["coeffs"], "tf", g["row_gene"], g["col_tf"])
    pr, roc, best = port.combo_eval(*args)
    np.testing.assert_array_equal(pr, g["combo_aupr"])
    np.testing.assert_array_equal(roc, g["combo_auroc"])
    assert best == int(g["combo_best"])
    pr, roc, best = port.combo_stouffer_tf_eval(*args)
    np.testing.assert_array_equal(pr, g["st_aupr"])
    np.testing.assert_array_equal(roc, g["st_auroc"])
    assert best == int(g["st_best"])


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 1), (3, 2), (1000, 7), (100000, 3), (65536, 100)])
def test_shuffle_positions_match_reference_tuples(port, n, seed):
    """shuffle_truth (apps/pipeline/eval_mcpnet.cpp:214-224) shuffles (size_t, size_t, int)
    tuples; std::shuffle's swaps depend only on the length and the std::mt19937, so the
    shuffled positions used by the split evaluation give the same order."""
    a = port.shuffle_perm(n, seed)
    assert np.array_equal(a, port.shuffle_tuples_order(n, seed))
    assert np.array_equal(np.sort(a), np.arange(n))


def test_mask_entries_match_select_truth(port, golden):
    """The mask order (row-major labelled entries of the region) restated in numpy
    selects exactly the oracle's select_values2 vectors."""
    g = golden("eval_truth")
    A, L = g["A"], g["labels"]
    ti, ct = g["tf_idx"], g["col_tf"]
    for region, V, Lb, rg, c in (("lower", A, L, None, None), ("all", A, L, None, None),
                                  ("tf", A[ti], L[ti], ti, ct)):
        v, l = port.mask_entries(V, Lb, region, rg, c)
        pos, neg = port.select_truth(V, Lb, region, rg, c)
        assert np.array_equal(v[l == 1], pos) and np.array_equal(v[l == 0], neg), region


def test_split_aupr_composition_edges(port, golden):
    """A train part holding every entry reproduces the full AUPR and leaves an empty
    test part (AUPR 0); an empty train part has AUPR 0."""
    g = golden("eval_truth")
    A, L = g["A"], g["labels"]
    v, _ = port.mask_entries(A, L)
    full, tr, te = port.split_aupr(A, L, 2, [0, v.size])
    assert full == tuple(g["lower_ref"])[0]
    assert np.all(tr[:, 0] == 0.0) and np.all(te[:, 1] == 0.0)
    assert np.all(tr[:, 1] == full) and np.all(te[:, 0] == full)


@pytest.mark.parametrize("E", [0, 1, 2, 1000, 65535, 65536, 65537, 70001, 1 << 20])
def test_library_shuffle_equals_std_shuffle(built_lib, port, E):
    """mcpg_shuffle_positions (the split evaluation's shuffle; above 65,535 entries its draws
    run ahead of the swaps with prefetching) gives std::shuffle's order for every seed, and
    seed 0 keeps the mask order."""
    assert np.array_equal(built_lib.shuffle_positions(E, 0), np.arange(E, dtype=np.uint32))
    for seed in (1, 2, 99, 4000000007):
        got = built_lib.shuffle_positions(E, seed).astype(np.int64)
        assert np.array_equal(got, port.shuffle_perm(E, seed % (1 << 32)) if E else got), (E, seed)


def test_library_shuffle_rejects_bad_counts(built_lib):
    with pytest.raises(built_lib.MCPGError):
        built_lib.shuffle_positions(-1, 1)


@pytest.mark.parametrize("n", [1, 2, 7, 64, 150])
def test_widest_path_rows_equal_the_squaring_closure(port, n):
    """The widest-path rows (the sampled-row check of large closures) equal the
    repeated-squaring closure exactly, with ties, negative entries and a nonzero
    diagonal."""
    rng = np.random.default_rng(n + 17)
    A = (rng.integers(-3, 9, size=(n, n)) * 0.125).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, rng.integers(-2, 3, size=n) * 0.125)
    C, _ = port.closure(A)
    assert np.array_equal(port.widest_rows(A, np.arange(n)), C)


def test_dpi_rows_equal_the_full_filter(port):
    rng = np.random.default_rng(5)
    A = (rng.integers(0, 6, size=(90, 90)) * 0.2).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    for tol in (0.0, 0.1):
        out, mask, _ = port.dpi(A, tol)
        rows = np.array([0, 5, 89, 44])
        ro, rm, rr = port.dpi_rows(A, rows, tol)
        assert np.array_equal(ro.view(np.uint32), out[rows].view(np.uint32))
        assert np.array_equal(rm, mask[rows])
        assert rr == int((out[rows] != A[rows]).sum())


@pytest.mark.parametrize("n,frac,tol", [(60, 0.3, 0.1), (75, 0.1, 0.0), (64, 0.9, 0.5)])
def test_dpi_tf_on_tf_first_permutation(port, n, frac, tol):
    """The GPU's two-phase TF DPI decides on B = P A P^T with the t TFs first: a pair of
    one TF and one non-TF admits the intermediates y < t of B, any other pair all y; the
    x, z exclusion is B's diagonal.  Restated here in numpy and compared with the oracle's
    dpi_tf_kernel loop (dpi.hpp:74-110), which scans A's own order with its TF test."""
    rng = np.random.default_rng(n)
    A = (rng.integers(0, 9, size=(n, n)) * 0.125).astype(np.float32)  # ties
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    tfs = np.where(rng.random(n) < frac, np.float32(np.inf), np.float32(-np.inf))
    is_tf = tfs > 0
    perm = np.concatenate([np.flatnonzero(is_tf), np.flatnonzero(~is_tf)])
    t = int(is_tf.sum())
    B = A[perm][:, perm]
    tm = np.float32(1.0 / (1.0 - np.float64(np.float32(tol))))
    mask = np.zeros((n, n), dtype=np.uint8)
    for xp in range(n):
        for zp in range(n):
            x, z = perm[xp], perm[zp]
            if xp == zp:
                mask[x, z] = 1
                continue
            end = t if (xp < t) != (zp < t) else n
            ys = np.array([y for y in range(end) if y != xp and y != zp], dtype=np.int64)
            thr = np.float32(A[x, z] * tm)
            mask[x, z] = 1 if ys.size and np.minimum(B[xp, ys], B[zp, ys]).max() >= thr else 0
    _, om, _ = port.dpi_tf(A, tfs, tol)
    assert np.array_equal(mask, om)
