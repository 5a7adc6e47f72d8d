"""The semi-supervised split evaluation of the eval_mcpnet app on the GPU:
eval_aupr_mcp (train / test AUPRs over shuffled splits of the labelled
entries) and eval_combos over the same splits (coefficient row chosen on the
training entries), against the oracle's composition of the reference's loops
with the same std::shuffle.  AUPRs within 1e-12 (the GPU sums in another
order), chosen rows equal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("region", ["lower", "all", "tf"])
def test_split_aupr_vs_oracle(gpu, port, golden, region):
    import mcpnet_gb300 as M
    g = golden("eval_truth")
    A, L, ti, ct = g["A"], g["labels"], g["tf_idx"], g["col_tf"]
    if region == "tf":
        V, Lb, rg, c = A[ti], L[ti], ti, ct
    else:
        V, Lb, rg, c = A, L, None, None
    E = port.mask_entries(V, Lb, region, rg, c)[0].size
    tc = M.train_counts(E, tf=(region == "tf"))
    full, tr, te = gpu.split_aupr_dev(dev(V), dev(Lb), 4, tc, region, None if rg is None else dev(rg.astype(np.int32)),
                                      None if c is None else dev(c))
    wf, wtr, wte = port.split_aupr(V, Lb, 4, tc, region, rg, c)
    assert abs(full - wf) <= TOL
    assert tr.shape == wtr.shape and np.all(np.abs(tr - wtr) <= TOL) and np.all(np.abs(te - wte) <= TOL)
    assert abs(full - tuple(g[f"{region}_ref"])[0]) <= TOL  # the reference's AUPR of the whole mask
    hf, htr, hte = gpu.split_aupr(V, Lb, 4, tc, region, rg, c)
    assert hf == full and np.array_equal(htr, tr) and np.array_equal(hte, te)


def test_split_aupr_edges(gpu, port, golden):
    """Train counts 0 and all entries; no iterations; a count above the entries is an error."""
    import mcpnet_gb300 as M
    g = golden("eval_truth")
    A, L = g["A"], g["labels"]
    E = port.mask_entries(A, L)[0].size
    full, tr, te = gpu.split_aupr(A, L, 2, [0, E])
    assert np.all(tr[:, 0] == 0.0) and np.all(te[:, 1] == 0.0)
    assert np.all(np.abs(tr[:, 1] - full) <= TOL) and np.all(np.abs(te[:, 0] - full) <= TOL)
    f0, tr0, _ = gpu.split_aupr(A, L, 0, [5])
    assert abs(f0 - full) <= TOL and tr0.shape == (0, 1)
    with pytest.raises(M.MCPGError):
        gpu.split_aupr(A, L, 1, [E + 1])


def test_split_combo_eval_vs_oracle(gpu, port, golden):
    """Plain combos and the (diagonal-excluding) Stouffer combos; the oracle's
    composition gets the GPU's Stouffer matrices, whose statistics it checks
    elsewhere to an ulp."""
    import torch
    import mcpnet_gb300 as M
    g = golden("eval_truth")
    A, M1, M2, M3, L, cs = g["A"], g["M1"], g["M2"], g["M3"], g["labels"], g["coeffs"]
    E = port.mask_entries(A, L)[0].size
    tc = M.train_counts(E)
    res, best = gpu.split_combo_eval_dev(dev(A), dev(M1), dev(M2), dev(M3), dev(L), cs, 3, tc, "exclude_diagonal")
    n = A.shape[0]
    comb = torch.empty((n, n), device="cuda")
    st = torch.empty((n, n), device="cuda")
    smats = []
    for c in cs:
        gpu.combo_dev(dev(A), dev(M1), dev(M2), dev(M3), c, comb)
        gpu.transform_dev(comb, st)
        torch.cuda.synchronize()
        smats.append(st.cpu().numpy())
    wres, wbest = port.split_combo_eval(A, M1, M2, M3, L, cs, 3, tc, smats)
    assert np.array_equal(best, wbest)
    assert np.all(np.abs(res - wres) <= TOL)
    res2, best2 = gpu.split_combo_eval(A, M1, M2, M3, L, cs, 3, tc, "none")
    assert np.array_equal(best2[..., 0], wbest[..., 0]) and np.all(best2[..., 1] == 0)
    assert np.all(np.abs(res2[..., [0, 1, 4]] - wres[..., [0, 1, 4]]) <= TOL) and np.all(res2[..., [2, 3, 5]] == 0.0)


def test_split_combo_eval_tf(gpu, port, golden):
    """The TF ensemble's splits with the TF Stouffer transform."""
    import mcpnet_gb300 as M
    g = golden("tf_ensemble")
    T, M1, M2, M3, L, rg, ct, cs = (g[k] for k in ("T", "M1", "M2", "M3", "labels_tf", "row_gene", "col_tf",
                                                   "coeffs"))
    E = port.mask_entries(T, L, "tf", rg, ct)[0].size
    tc = M.train_counts(E, tf=True)
    res, best = gpu.split_combo_eval(T, M1, M2, M3, L, cs, 2, tc, "tf", "tf", rg, ct)
    smats = [gpu.transform_tf(gpu.combo(T, M1, M2, M3, c), "stouffer") for c in cs]
    wres, wbest = port.split_combo_eval(T, M1, M2, M3, L, cs, 2, tc, smats, "tf", rg, ct)
    assert np.array_equal(best, wbest)
    assert np.all(np.abs(res - wres) <= TOL)


def test_split_combo_eval_errors(gpu):
    import mcpnet_gb300 as M
    A = np.ones((4, 5), np.float32)
    L = np.zeros((4, 5), np.int8)
    with pytest.raises(M.MCPGError):  # square Stouffer on a rectangular matrix
        gpu.split_combo_eval(A, A, A, A, L, [0.25] * 4, 1, [1], "exclude_diagonal", "all")
    with pytest.raises(M.MCPGError):  # M1 missing with a non-zero coefficient
        gpu.split_combo_eval(A, None, None, None, L, [0.5, 0.5, 0, 0], 1, [1], "none", "all")
