"""Generate the golden fixtures in this folder from MCPNet's OWN kernels.

Runs the reference's hot-path headers compiled from the MCPNet source tree
(oracle/ref/ref_driver.cpp -> oracle/_ref/libmcpref.so; the tree is read from
$MCPNET_REF_ROOT, which must be set) on seeded synthetic inputs and
stores inputs and outputs together, so the fixtures need neither the
reference nor this script at test time.

    MCPNET_REF_ROOT=<MCPNet source tree> python tests/golden/make_golden.py

Fixtures (all float32 unless noted):
  mi_*.npz       X, W (reference weight rows), MI32 (reference --single MI),
                 MI64 (reference double MI, float64), bins, order
  mcp_*.npz      A (MI with diagonal 0), M2/M3/M4 (max-min products of
                 compute_mcp2/3/4), R2/R3/R4 (MCP ratios), M3s/R3s (mcp app's
                 symmetrised MCP3), DPI_out, DPI_mask (uint8), DPI_removed, tol
  maxmin_rect.npz  A (33 x 77), B (45 x 77) with negative entries, C = A (x) B
  dpi_ties.npz   a matrix with repeated values and zeros, DPI outputs at tol 0 and 0.1
  tf_90.npz      TF-restricted MCP / DPI / masked max-min outputs
  eval_cases.npz AUPR / AUROC of score vectors from the reference's aupr_kernel /
                 auroc_kernel (IT = float and IT = double, OT = double), incl.
                 ties, +-0, empty sides and both AUROC branches
  ap_mi.npz      adaptive-partitioning MI from the reference's own kernels
                 (IntegralCumulativeHistogramKernel + AdaptivePartitionRankMIKernel2)
                 on ranks of synthetic expression (with and without ties; tiny m)
  stouffer.npz   the reference's stouffer_vector_kernel / clr_vector_kernel on an MI
                 matrix with the oracle's row statistics (both statistics modes,
                 and a constant row whose deviation is 0)
  eval_truth.npz an MI matrix, its max-min products, int8 truth labels from the
                 synthetic GRN, TF rows, and AUPR / AUROC of each truth region
                 and of a coefficient table of combo scores
  tf_ensemble.npz  the TF ensemble on eval_truth's matrix and TFs: T, M1, M2, M3
                 of compute_maxmins_tfs from the reference's masked max-min
                 kernel; a t x n matrix with a constant row and column, its
                 (oracle) statistics and the reference's zscored_stouffer_kernel
                 and zscored_clr_kernel outputs; the combo and TF-Stouffer coefficient searches over the
                 TF truth rows

    python tests/golden/make_golden.py --only eval   # regenerate the eval fixtures only
    python tests/golden/make_golden.py --only tf     # the TF ensemble fixture only
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402


def synth(n, m, seed):
    import mcpnet_gb300 as M
    return M.synth_grn(n, m, seed=seed)


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["core", "eval", "ap", "stouffer", "tf"], default=None)
    args = ap.parse_args()
    if O.REF_ROOT is None:
        raise SystemExit("set MCPNET_REF_ROOT to the MCPNet source tree")
    O.build(with_ref=True)
    R = O.ref()
    if R is None:
        raise SystemExit("reference kernels not built (MCPNet sources not found)")
    if args.only in (None, "core"):
        core(R)
    if args.only in (None, "eval"):
        evaluation(R)
    if args.only in (None, "ap"):
        ap_mi(R)
    if args.only in (None, "stouffer"):
        stouffer(R)
    if args.only in (None, "tf"):
        tf_ensemble(R)
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


def core(R):

    # ---- MI ----
    for name, (n, m, seed, bins, order) in {
        "mi_37x211": (37, 211, 11, 10, 3),
        "mi_64x500": (64, 500, 12, 10, 3),
        "mi_3x7": (3, 7, 13, 10, 3),
        "mi_1x5": (1, 5, 14, 10, 3),
        "mi_20x64_b8k2": (20, 64, 15, 8, 2),
    }.items():
        X = synth(n, m, seed)
        W = R.bspline_weights(X, bins, order)
        MI32 = R.bspline_mi(X, bins, order)
        MI64 = R.bspline_mi(X.astype(np.float64), bins, order)
        np.savez_compressed(HERE / f"{name}.npz", X=X, W=W, MI32=MI32, MI64=MI64, bins=bins, order=order)

    # ---- MCP / DPI on an MI matrix ----
    for name, (n, m, seed) in {"mcp_70": (70, 300, 21), "mcp_130": (130, 200, 22)}.items():
        X = synth(n, m, seed)
        A = R.bspline_mi(X)
        np.fill_diagonal(A, 0.0)
        out = {"A": A}
        for pl in (2, 3, 4):
            M, Rt = R.mcp(A, pl)
            out[f"M{pl}"], out[f"R{pl}"] = M, Rt
        M3s, R3s = R.mcp(A, 3, symmetrize=True)
        out["M3s"], out["R3s"] = M3s, R3s
        tol = np.float32(0.1)
        o, mask, removed = R.dpi(A, tol)
        out.update(DPI_out=o, DPI_mask=mask, DPI_removed=np.int64(removed), tol=tol)
        np.savez_compressed(HERE / f"{name}.npz", **out)

    # ---- rectangular max-min with negative values ----
    rng = np.random.default_rng(31)
    A = rng.normal(size=(33, 77)).astype(np.float32)
    B = rng.normal(size=(45, 77)).astype(np.float32)
    np.savez_compressed(HERE / "maxmin_rect.npz", A=A, B=B, C=R.maxmin(A, B))

    # ---- DPI with ties and zeros ----
    v = rng.integers(0, 4, size=(40, 40)).astype(np.float32) * np.float32(0.25)
    T = np.maximum(v, v.T)
    np.fill_diagonal(T, 0.0)
    res = {"A": T}
    for tag, tol in (("t0", np.float32(0.0)), ("t1", np.float32(0.1))):
        o, mask, removed = R.dpi(T, tol)
        res.update({f"out_{tag}": o, f"mask_{tag}": mask, f"removed_{tag}": np.int64(removed), f"tol_{tag}": tol})
    np.savez_compressed(HERE / "dpi_ties.npz", **res)
    # ---- TF-restricted variants on an MI matrix ----
    X = synth(90, 250, 41)
    A = R.bspline_mi(X)
    np.fill_diagonal(A, 0.0)
    tfs = np.where(rng.random(90) < 0.2, np.float32(np.inf), np.float32(-np.inf)).astype(np.float32)
    tf = {"A": A, "tfs": tfs}
    for pl, transitions in ((2, (0, 1)), (3, (0, 1, 2)), (4, (0, 1, 2, 3))):
        for t in transitions:
            M, Rt = R.mcp_tf(A, tfs, pl, t)
            tf[f"M{pl}_t{t}"], tf[f"R{pl}_t{t}"] = M, Rt
    tol = np.float32(0.1)
    o, mask, removed = R.dpi_tf(A, tfs, tol)
    tf.update(DPI_out=o, DPI_mask=mask, DPI_removed=np.int64(removed), tol=tol)
    general = rng.normal(size=90).astype(np.float32)   # a general (non +-inf) mask
    tf["mask_general"] = general
    tf["MM_general"] = R.maxmin_masked(A, A, general)
    np.savez_compressed(HERE / "tf_90.npz", **tf)


def eval_cases(rng):
    """(pos, neg) float32 score vectors covering the curve code's branches."""
    q = lambda a, k: (np.floor(a * k) / k).astype(np.float32)
    c = []
    c.append((rng.random(200).astype(np.float32), (rng.random(3000) * 0.8).astype(np.float32)))  # P < N
    c.append((q(rng.random(150), 7), q(rng.random(400) * 0.9, 7)))                                # heavy ties
    c.append((rng.random(500).astype(np.float32), (rng.random(120) * 1.2).astype(np.float32)))    # P > N
    c.append((q(rng.random(50), 5), q(rng.random(50), 5)))                                        # P == N, ties
    c.append((np.zeros(0, np.float32), rng.random(10).astype(np.float32)))                        # no positives
    c.append((rng.random(10).astype(np.float32), np.zeros(0, np.float32)))                        # no negatives
    c.append((np.zeros(0, np.float32), np.zeros(0, np.float32)))                                  # nothing
    c.append((np.array([0.25], np.float32), np.array([0.25], np.float32)))                        # one tie
    c.append((np.array([-0.0, 1.0, -2.5, 0.0, 3.0], np.float32),                                  # +-0, negatives
              np.array([0.0, -0.0, -2.5, -3.0, 0.5, 1.0, 1.0], np.float32)))
    c.append((np.full(5, 0.5, np.float32), np.full(7, 0.5, np.float32)))                          # all equal
    c.append((rng.normal(0.3, 1.0, 1500).astype(np.float32), rng.normal(0.0, 1.0, 30000).astype(np.float32)))
    c.append((q(rng.random(12000), 1000), q(rng.random(3000), 1000)))                             # P > N, ties
    return c


def evaluation(R):
    rng = np.random.default_rng(77)
    ev = {}
    cases = eval_cases(rng)
    for k, (pos, neg) in enumerate(cases):
        ev[f"pos_{k}"], ev[f"neg_{k}"] = pos, neg
        ev[f"ref32_{k}"] = np.array(R.aupr_auroc(pos, neg, np.float32))
        ev[f"ref64_{k}"] = np.array(R.aupr_auroc(pos, neg, np.float64))
    ev["ncases"] = np.int64(len(cases))
    np.savez_compressed(HERE / "eval_cases.npz", **ev)

    # ---- a truth matrix on an MI network of a synthetic GRN ----
    import mcpnet_gb300 as M
    n = 90
    X, E = M.synth_grn(n, 300, seed=51, with_edges=True)
    A = R.bspline_mi(X)
    np.fill_diagonal(A, 0.0)
    Lb = np.full((n, n), -1, dtype=np.int8)
    unk = rng.random((n, n)) < 0.3
    Lb[~unk] = 0
    Lb = np.minimum(Lb, Lb.T)                       # symmetric, as a truth matrix
    Lb[E[:, 0], E[:, 1]] = 1
    Lb[E[:, 1], E[:, 0]] = 1
    np.fill_diagonal(Lb, -1)
    tf = rng.random(n) < 0.2
    tf_idx = np.nonzero(tf)[0].astype(np.int32)
    out = {"A": A, "labels": Lb, "tf_idx": tf_idx, "col_tf": tf.astype(np.uint8)}
    for region, V, L, rg, ct in (("lower", A, Lb, None, None), ("all", A, Lb, None, None),
                                  ("tf", A[tf_idx], Lb[tf_idx], tf_idx, tf.astype(np.uint8))):
        pos, neg = O.port().select_truth(V, L, region, rg, ct)
        out[f"{region}_pos"], out[f"{region}_neg"] = pos, neg
        out[f"{region}_ref"] = np.array(R.aupr_auroc(pos, neg, np.float32))
    M1, _ = R.mcp(A, 2)
    M2, _ = R.mcp(A, 3)
    M3, _ = R.mcp(A, 4)
    out.update(M1=M1, M2=M2, M3=M3)
    cs = np.array([[1, 0, 0, 0], [0.25, 0.25, 0.25, 0.25], [0, 1, 0, 0], [0.5, 0.5, 0, 0], [0, 0, 0, 1],
                   [0.1, 0.2, 0.3, 0.4], [0, 0.5, 0.5, 0]], dtype=np.float64)
    out["coeffs"] = cs
    pr = np.full(len(cs), np.nan)
    roc = np.full(len(cs), np.nan)
    best, top = 0, 0.0
    for i, c in enumerate(cs):
        if c[0] == 1 and not c[1:].any():
            continue
        S = O.port().combo(A, M1, M2, M3, c)
        pos, neg = O.port().select_truth(S, Lb, "lower")
        pr[i], roc[i] = R.aupr_auroc(pos, neg, np.float32)
        if pr[i] > top:
            top, best = pr[i], i
    out.update(combo_aupr=pr, combo_auroc=roc, combo_best=np.int64(best))
    np.savez_compressed(HERE / "eval_truth.npz", **out)


def ap_mi(R):
    import mcpnet_gb300 as M
    P = O.port()
    out = {}
    cases = {"g40x300": M.synth_grn(40, 300, seed=61), "g24x1000": M.synth_grn(24, 1000, seed=62),
             "g9x7": M.synth_grn(9, 7, seed=63), "g5x3": M.synth_grn(5, 3, seed=64),
             "g4x1": M.synth_grn(4, 1, seed=65), "g6x2": M.synth_grn(6, 2, seed=66),
             "ties15x80": (np.round(np.random.default_rng(67).random((15, 80)) * 6) / 6).astype(np.float32)}
    for name, X in cases.items():
        Rk = P.ap_ranks(X)
        out[f"{name}_X"] = X
        out[f"{name}_R"] = Rk.astype(np.int32)
        out[f"{name}_MI"] = R.ap_mi(Rk)
    out["names"] = np.array(sorted(cases))
    np.savez_compressed(HERE / "ap_mi.npz", **out)



def stouffer(R):
    P = O.port()
    with np.load(HERE / "mcp_70.npz") as z:
        A = z["A"].copy()
    A[5, :] = np.float32(0.25)  # a constant row: sd 0 -> its z-scores are 0
    out = {"A": A}
    for mode in ("all", "exclude_diagonal"):
        mean, sd = P.row_stats(A, mode)
        out[f"{mode}_mean"], out[f"{mode}_sd"] = mean, sd
        out[f"{mode}_stouffer"] = R.transform_with_stats(A, mean, sd, clr=False)
        out[f"{mode}_clr"] = R.transform_with_stats(A, mean, sd, clr=True)
    np.savez_compressed(HERE / "stouffer.npz", **out)

def tf_ensemble(R):
    P = O.port()
    with np.load(HERE / "eval_truth.npz") as z:
        A, labels, tf_idx, col_tf, cs = z["A"], z["labels"], z["tf_idx"], z["col_tf"], z["coeffs"]
    n = A.shape[0]
    tfs = np.full(n, -np.inf, dtype=np.float32)
    tfs[tf_idx] = np.inf
    T, M1, M2, M3 = R.maxmins_tf(A, tfs)
    out = {"A": A, "tfs": tfs, "T": T, "M1": M1, "M2": M2, "M3": M3}
    S = P.combo(T, M1, M2, M3, np.array([0.25, 0.25, 0.25, 0.25]))
    S[3, :] = np.float32(0.5)   # a constant row and a constant column: sd 0 -> z 0
    S[:, 7] = np.float32(0.5)
    rm, rs, cm, csd = P.tf_stats(S)
    _, zr, zc = P.stouffer_tf_with_stats(S, rm, rs, cm, csd, want_z=True)
    out.update(st_in=S, st_rmean=rm, st_rsd=rs, st_cmean=cm, st_csd=csd, st_out=R.zscored_stouffer(zr, zc),
               clr_out=R.zscored_clr(zr, zc))
    lab = np.ascontiguousarray(labels[tf_idx])
    out.update(labels_tf=lab, row_gene=tf_idx.astype(np.int32), col_tf=col_tf, coeffs=cs)
    pr, roc, best = R.combo_eval(T, M1, M2, M3, lab, cs, "tf", tf_idx, col_tf)
    out.update(combo_aupr=pr, combo_auroc=roc, combo_best=np.int64(best))
    pr, roc, best = R.combo_stouffer_tf_eval(T, M1, M2, M3, lab, cs, "tf", tf_idx, col_tf)
    out.update(st_aupr=pr, st_auroc=roc, st_best=np.int64(best))
    np.savez_compressed(HERE / "tf_ensemble.npz", **out)


if __name__ == "__main__":
    main()
