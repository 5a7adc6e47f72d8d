"""Parity at the benchmark configurations' own sizes, through the C ABI.

* 2,000 genes x 2,000 samples (the plain FP32 GPU pipeline): MI on sampled rows
  against the oracle's float and double MI, then the whole chain bit for bit on
  the GPU's MI -- diagonal 0, the max-min products M1 = A (x) A, M2 = A (x) M1,
  M3 = M1 (x) M1 with the MCP2/3/4 ratios, the mcp app's symmetrised MCP3, and
  the DPI filter (tolerance 0.1) with its mask and removed count.
* 20,000 x 2,000 (the bench workload, bf16f8 MI) and 32,768 x 4,096 (the large
  single-GPU run): the same chain plus the converged max-capacity closure, every
  output checked bit for bit on sampled rows (each row costs n^2 on the CPU:
  a product row from the full operands, a DPI row from the full matrix, a
  closure row by a widest-path search, which is independent of the squaring).
  At 32,768 x 4,096 also the MI accuracy of the bf16f8 and bf16x3 forms against
  FP64 on sampled gene pairs.
* 4,096 x 1,024 (the differentiation form): central finite differences
  (step 1e-3) of the FP32 GPU forward on 64 seeded entries of X, and the
  max-min / ratio part of the backward against the oracle.

Max-min, ratio, DPI and closure outputs are selections of input entries (or one
rounded division), so they must match bit for bit; the MI matches within the
tolerances of the MI tests (2e-5 bits for FP32, 1e-4 nats for the tensor-core
forms).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20260001
NATS = np.log(2.0)


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def sample_rows(n, k, seed):
    rng = np.random.default_rng(seed)
    s = set(rng.choice(n, size=k, replace=False).tolist()) | {0, 1, n // 2, n - 1}
    return np.array(sorted(s), dtype=np.int64)


def _free():
    import torch
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def test_c2_plain_fp32_chain_at_2000(gpu, port, built_lib):
    import torch
    n = m = 2000
    X = built_lib.synth_grn(n, m, seed=SEED)
    Xd = torch.from_numpy(X).cuda()
    Ad = torch.empty((n, n), dtype=torch.float32, device="cuda")
    gpu.bspline_mi_dev(Xd, Ad, 10, 3, "fp32")
    gpu.synchronize()
    MI = Ad.cpu().numpy()
    assert np.array_equal(MI, MI.T)

    # MI on three row slabs against the reference's float MI and the double MI
    W32 = port.bspline_weights(X)
    W64 = port.bspline_weights(X.astype(np.float64))
    for r0 in (0, n // 2 - 4, n - 8):
        ref32 = port.bspline_mi_rows(W32, m, r0, r0 + 8)
        ref64 = port.bspline_mi_rows(W64, m, r0, r0 + 8)
        assert np.abs(MI[r0:r0 + 8] - ref32).max() < 2e-5
        assert np.abs(MI[r0:r0 + 8] - ref64).max() < 2e-5
    del W32, W64

    # the chain, bit for bit, on the GPU's MI
    gpu.set_diagonal_dev(Ad, 0.0)
    A = Ad.cpu().numpy()
    assert np.all(np.diag(A) == 0)
    f32 = dict(dtype=torch.float32, device="cuda")
    M1, M2, M3, R2, R3, R4 = (torch.empty((n, n), **f32) for _ in range(6))
    gpu.maxmins_dev(Ad, M1, M2, M3, R2, R3, R4)
    for pl, (Mg, Rg) in zip((2, 3, 4), ((M1, R2), (M2, R3), (M3, R4))):
        Mo, Ro = port.mcp(A, pl)
        assert np.array_equal(bits(Mg.cpu().numpy()), bits(Mo)), f"MCP{pl} max-min"
        assert np.array_equal(bits(Rg.cpu().numpy()), bits(Ro)), f"MCP{pl} ratio"
    Ms, Rs = gpu.mcp(A, 3, symmetrize=True)
    Mso, Rso = port.mcp(A, 3, symmetrize=True)
    assert np.array_equal(bits(Ms), bits(Mso)) and np.array_equal(bits(Rs), bits(Rso))
    D = torch.empty((n, n), **f32)
    mask = torch.empty((n, n), dtype=torch.uint8, device="cuda")
    removed = gpu.dpi_dev(Ad, D, 0.1, mask)
    Do, mo, ro = port.dpi(A, 0.1)
    assert np.array_equal(bits(D.cpu().numpy()), bits(Do))
    assert np.array_equal(mask.cpu().numpy(), mo)
    assert removed == ro > 0
    del Xd, Ad, M1, M2, M3, R2, R3, R4, D, mask
    _free()


def _chain_sampled_rows(gpu, port, built_lib, n, m, precision, k_rows):
    """Runs MI -> diagonal 0 -> M1/M2/M3 + ratios -> DPI(0.1) -> TF DPI(0.1) -> closure
    on the GPU and checks every output on sampled rows against the oracle, bit for bit."""
    import torch
    X = built_lib.synth_grn(n, m, seed=SEED)
    f32 = dict(dtype=torch.float32, device="cuda")
    Ad = torch.empty((n, n), **f32)
    gpu.bspline_mi_dev(torch.from_numpy(X).cuda(), Ad, 10, 3, precision)
    gpu.set_diagonal_dev(Ad, 0.0)
    M1, M2, M3, R2, R3, R4 = (torch.empty((n, n), **f32) for _ in range(6))
    gpu.maxmins_dev(Ad, M1, M2, M3, R2, R3, R4)
    rows = sample_rows(n, k_rows, seed=n + m)
    ri = torch.from_numpy(rows).cuda()
    got = {k: v[ri].cpu().numpy() for k, v in (("M2", M2), ("M3", M3), ("R2", R2), ("R3", R3), ("R4", R4))}
    del M2, M3, R2, R3, R4
    A = Ad.cpu().numpy()
    M1h = M1.cpu().numpy()
    del M1
    _free()
    assert np.array_equal(A, A.T), "MI is stored symmetric"

    Ar, M1r = A[rows], M1h[rows]
    assert np.array_equal(bits(M1r), bits(port.maxmin(Ar, A))), "M1 = A (x) A"
    assert np.array_equal(bits(got["M2"]), bits(port.maxmin(Ar, M1h))), "M2 = A (x) M1"
    assert np.array_equal(bits(got["M3"]), bits(port.maxmin(M1r, M1h))), "M3 = M1 (x) M1"
    assert np.array_equal(bits(got["R2"]), bits(port.ratio(Ar, M1r))), "MCP2 ratio"
    assert np.array_equal(bits(got["R3"]), bits(port.ratio(Ar, got["M2"]))), "MCP3 ratio"
    assert np.array_equal(bits(got["R4"]), bits(port.ratio(Ar, got["M3"]))), "MCP4 ratio"
    del M1h

    D = torch.empty((n, n), **f32)
    mask = torch.empty((n, n), dtype=torch.uint8, device="cuda")
    removed = gpu.dpi_dev(Ad, D, 0.1, mask)
    Dr, maskr = D[ri].cpu().numpy(), mask[ri].cpu().numpy()
    assert removed == int((D != Ad).sum().item()), "removed count = changed entries"
    del D, mask
    _free()
    Do, mo, _ = port.dpi_rows(A, rows, 0.1)
    assert np.array_equal(bits(Dr), bits(Do)), "DPI output rows"
    assert np.array_equal(maskr, mo), "DPI mask rows"

    # TF DPI (dpi_tf_kernel) with a seeded set of n/16 TFs: at these sizes it runs in two
    # phases on the TF-first permutation of the matrix
    rng = np.random.default_rng(n + 1)
    tfs = np.full(n, -np.inf, dtype=np.float32)
    tfs[rng.choice(n, n // 16, replace=False)] = np.inf
    D = torch.empty((n, n), **f32)
    mask = torch.empty((n, n), dtype=torch.uint8, device="cuda")
    removed_tf = gpu.dpi_tf_dev(Ad, D, tfs, 0.1, mask)
    Dr, maskr = D[ri].cpu().numpy(), mask[ri].cpu().numpy()
    assert removed_tf == int((D != Ad).sum().item()), "TF DPI removed count = changed entries"
    del D, mask
    _free()
    Do, mo, _ = port.dpi_tf_rows(A, tfs, rows, 0.1)
    assert np.array_equal(bits(Dr), bits(Do)), "TF DPI output rows"
    assert np.array_equal(maskr, mo), "TF DPI mask rows"

    Cl = torch.empty((n, n), **f32)
    iters = gpu.closure_dev(Ad, Cl, 64)
    assert iters > 0
    Clr = Cl[ri].cpu().numpy()
    del Cl, Ad
    _free()
    assert np.array_equal(bits(Clr), bits(port.widest_rows(A, rows))), "closure rows"
    return X, A, rows, removed, iters


def test_c3_chain_sampled_rows_at_20000(gpu, port, built_lib):
    _chain_sampled_rows(gpu, port, built_lib, 20000, 2000, "bf16f8", 12)


def test_c5_chain_sampled_rows_and_mi_accuracy_at_32768(gpu, port, built_lib):
    import torch
    n, m = 32768, 4096
    X, A, rows, removed, iters = _chain_sampled_rows(gpu, port, built_lib, n, m, "bf16f8", 12)
    del A
    # MI accuracy vs FP64 on sampled pairs: rows S against 2,048 seeded columns T.
    # MI(i, j) depends only on genes i and j, so the oracle needs the weights of S u T only.
    S = rows[:8]
    T = np.setdiff1d(np.sort(np.random.default_rng(7).choice(n, 2048, replace=False)), S)
    genes = np.concatenate([S, T])
    W64 = port.bspline_weights(X[genes].astype(np.float64))
    ref = port.bspline_mi_rows(W64, m, 0, len(S))[:, len(S):]  # S x T
    del W64
    stats = pytest.importorskip("scipy.stats")
    f32 = dict(dtype=torch.float32, device="cuda")
    for form in ("bf16f8", "bf16x3"):
        MI = torch.empty((n, n), **f32)
        gpu.bspline_mi_dev(torch.from_numpy(X).cuda(), MI, 10, 3, form)
        got = MI[torch.from_numpy(S).cuda()][:, torch.from_numpy(T).cuda()].cpu().numpy().astype(np.float64)
        del MI
        _free()
        err_nats = float(np.abs(got - ref).max()) * NATS
        assert err_nats <= 1e-4, (form, err_nats)
        k = ref.size // 100
        a = set(np.argpartition(-ref.ravel(), k - 1)[:k].tolist())
        b = set(np.argpartition(-got.ravel(), k - 1)[:k].tolist())
        jac = len(a & b) / len(a | b)
        union = np.array(sorted(a | b))
        rho = float(stats.spearmanr(ref.ravel()[union], got.ravel()[union])[0])
        assert jac >= 0.95 and rho >= 0.99, (form, jac, rho)


def test_c4_gradient_finite_differences_and_maxmin_backward_at_4096(gpu, port, built_lib):
    """Central differences (step 1e-3) of the FP32 GPU forward of L = sum over a
    seeded 5 % of gene pairs of U(-1, 1) x MCP3 score, on 64 seeded entries of X:
    the median relative difference to the GPU gradient must stay within 5 % (the
    FP32 forward's own rounding at a 1e-3 step is a few percent; the loss is only
    piecewise smooth, since a max-min witness can switch inside the step).  Then
    the max-min / ratio part of the backward, dL/dA, against the oracle composed
    on the same float products, accumulated in double."""
    import torch
    rng = np.random.default_rng(20260004)
    n, m = 4096, 1024
    X = built_lib.synth_grn(n, m, seed=SEED)
    iu = np.triu_indices(n, 1)
    sel = rng.random(len(iu[0])) < 0.05
    pr, pc = iu[0][sel].astype(np.int64), iu[1][sel].astype(np.int64)
    coef = rng.uniform(-1, 1, int(sel.sum()))
    ri, ci, cf = (torch.from_numpy(v).cuda() for v in (pr, pc, coef))
    Xd = torch.from_numpy(X).cuda()
    L0, dX, dA = gpu.mcp3_loss_grad_dev(Xd, ri, ci, cf, witness="saved", return_dA=True)
    dX, dA = dX.cpu().numpy(), dA.cpu().numpy()

    rel = []
    for _ in range(64):
        g, s = int(rng.integers(n)), int(rng.integers(m))
        x = np.float32(X[g, s])
        xp, xm = np.float32(x + np.float32(1e-3)), np.float32(x - np.float32(1e-3))
        Xp = X.copy()
        Xp[g, s] = xp
        Lp = gpu.mcp3_loss_dev(torch.from_numpy(Xp).cuda(), ri, ci, cf)
        Xp[g, s] = xm
        Lm = gpu.mcp3_loss_dev(torch.from_numpy(Xp).cuda(), ri, ci, cf)
        fd = (Lp - Lm) / (float(xp) - float(xm))
        rel.append(abs(fd - float(dX[g, s])) / max(abs(fd), abs(float(dX[g, s])), 1e-12))
    rel = np.array(rel)
    assert np.median(rel) <= 0.05, np.sort(rel)

    # dL/dA through the ratio and both max-min products, against the oracle on the GPU's
    # float A, M1, M2 (bit-exact products), gradients accumulated in double
    f32 = dict(dtype=torch.float32, device="cuda")
    Ad = torch.empty((n, n), **f32)
    gpu.bspline_mi_dev(Xd, Ad, 10, 3, "fp32")
    gpu.set_diagonal_dev(Ad, 0.0)
    M1d, M2d = torch.empty((n, n), **f32), torch.empty((n, n), **f32)
    gpu.maxmin_dev(Ad, Ad, M1d)
    gpu.maxmin_dev(Ad, M1d, M2d)
    gpu.synchronize()
    A64, M1, M2 = (t.cpu().numpy().astype(np.float64) for t in (Ad, M1d, M2d))
    del Ad, M1d, M2d
    _free()
    c = np.zeros((n, n))
    np.add.at(c, (pr, pc), coef)
    dA_o, dM2, dM1 = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    port.ratio_bwd(A64, M2, c, dA_o, dM2)
    port.maxmin_bwd(A64, M1, M2, dM2, dA_o, dM1, want_witness=False)
    port.maxmin_bwd(A64, A64, M1, dM1, dA_o, dA_o, want_witness=False)
    np.fill_diagonal(dA_o, 0.0)
    scale = np.abs(dA_o).max()
    assert scale > 0
    assert np.abs(dA - dA_o).max() <= 1e-5 * scale
