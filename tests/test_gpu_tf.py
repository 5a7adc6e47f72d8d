"""TF-restricted variants on the GPU (masked max-min, compute_mcp{2,3,4}_tfs,
dpi_tf_kernel): bit-exact against the reference's golden fixtures and the
oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TRANSITIONS = ((2, (0, 1)), (3, (0, 1, 2)), (4, (0, 1, 2, 3)))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def test_tf_golden(gpu, golden):
    g = golden("tf_90")
    A, tfs = g["A"], g["tfs"]
    for pl, ts in TRANSITIONS:
        for t in ts:
            M, R = gpu.mcp_tf(A, tfs, pl, t)
            assert np.array_equal(bits(M), bits(g[f"M{pl}_t{t}"])), (pl, t)
            assert np.array_equal(bits(R), bits(g[f"R{pl}_t{t}"])), (pl, t)
    out, mask, removed = gpu.dpi_tf(A, tfs, float(g["tol"]), want_mask=True)
    assert np.array_equal(bits(out), bits(g["DPI_out"]))
    assert np.array_equal(mask, g["DPI_mask"])
    assert removed == int(g["DPI_removed"])
    assert np.array_equal(bits(gpu.maxmin_masked(A, A, g["mask_general"])), bits(g["MM_general"]))


def _tf_vector(rng, n, frac):
    return np.where(rng.random(n) < frac, np.float32(np.inf), np.float32(-np.inf)).astype(np.float32)


@pytest.mark.parametrize("n,frac", [(1, 1.0), (3, 0.5), (40, 0.0), (40, 1.0), (131, 0.1), (200, 0.3)])
def test_tf_vs_oracle(gpu, port, n, frac):
    rng = np.random.default_rng(n * 13 + int(frac * 10))
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    tfs = _tf_vector(rng, n, frac)
    if frac == 1.0 and n == 1:
        tfs[:] = np.inf
    for pl, ts in TRANSITIONS:
        for t in ts:
            M, R = gpu.mcp_tf(A, tfs, pl, t)
            Mo, Ro = port.mcp_tf(A, tfs, pl, t)
            assert np.array_equal(bits(M), bits(Mo)) and np.array_equal(bits(R), bits(Ro)), (pl, t)
    for tol in (0.0, 0.1):
        out, mask, removed = gpu.dpi_tf(A, tfs, tol, want_mask=True)
        oo, om, orem = port.dpi_tf(A, tfs, tol)
        assert np.array_equal(bits(out), bits(oo)) and np.array_equal(mask, om) and removed == orem


def test_masked_maxmin_general_and_rect(gpu, port):
    rng = np.random.default_rng(17)
    A = rng.normal(size=(70, 45)).astype(np.float32)
    B = rng.normal(size=(33, 45)).astype(np.float32)
    for mask in (rng.normal(size=45).astype(np.float32), _tf_vector(rng, 45, 0.3),
                 np.full(45, -np.inf, np.float32)):
        assert np.array_equal(bits(gpu.maxmin_masked(A, B, mask)), bits(port.maxmin_masked(A, B, mask)))


def test_tf_bad_transition(gpu, built_lib):
    A = np.zeros((4, 4), np.float32)
    tfs = np.array([np.inf, -np.inf, np.inf, -np.inf], np.float32)
    with pytest.raises(built_lib.MCPGError):
        gpu.mcp_tf(A, tfs, 2, 2)


def _mi_like(built_lib, gpu, n, m, seed):
    """An MI matrix (the DPI's real input) with diagonal 0."""
    X = built_lib.synth_grn(n, m, seed=seed)
    A = gpu.bspline_mi(X, 10, 3, "bf16f8")
    np.fill_diagonal(A, 0)
    return A


@pytest.mark.parametrize("n,frac", [(1100, 0.15), (1601, 0.3), (2100, 0.6)])
@pytest.mark.parametrize("tol", [0.0, 0.1, 0.5])
def test_two_phase_tf_dpi_on_mi_matrices(gpu, port, built_lib, n, frac, tol):
    """Above 1,024 genes with at least 128 TFs the TF DPI runs in two phases on the
    TF-first permutation of the matrix (a tiled max-min over the first min(512, t)
    intermediates, then an early-exit scan of each undecided pair to its own end):
    the same outputs, mask and removed count as the reference's dpi_tf_kernel loop.
    The TF counts put t below and above the first phase's 512 intermediates."""
    rng = np.random.default_rng(n + int(frac * 100))
    A = _mi_like(built_lib, gpu, n, 400, seed=n)
    tfs = _tf_vector(rng, n, frac)
    assert (tfs > 0).sum() >= 128
    out, mask, removed = gpu.dpi_tf(A, tfs, tol, want_mask=True)
    oo, om, orem = port.dpi_tf(A, tfs, tol)
    assert np.array_equal(bits(out), bits(oo))
    assert np.array_equal(mask, om)
    assert removed == orem


def test_two_phase_tf_dpi_ties_nonsymmetric_and_general_tf_values(gpu, port):
    """Many ties, a non-symmetric input, and a TF vector of arbitrary values (a gene
    is a TF when its value is > 0, as in the reference)."""
    rng = np.random.default_rng(35)
    n = 1300
    A = (rng.integers(0, 7, size=(n, n)) * 0.125).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    tfs = (rng.random(n) - 0.7).astype(np.float32)  # ~30 % positive, none infinite
    for M in (A, (rng.random((n, n)) ** 3).astype(np.float32)):
        out, mask, removed = gpu.dpi_tf(M, tfs, 0.1, want_mask=True)
        oo, om, orem = port.dpi_tf(M, tfs, 0.1)
        assert np.array_equal(bits(out), bits(oo)) and np.array_equal(mask, om) and removed == orem


def test_two_phase_tf_dpi_falls_back_when_most_outputs_stay_undecided(gpu, port):
    """tol = 0.999: almost nothing is deleted, the pending list overflows, and the
    product form rewrites every output."""
    rng = np.random.default_rng(36)
    n = 1200
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    tfs = _tf_vector(rng, n, 0.25)
    out, mask, removed = gpu.dpi_tf(A, tfs, 0.999, want_mask=True)
    oo, om, orem = port.dpi_tf(A, tfs, 0.999)
    assert np.array_equal(bits(out), bits(oo)) and np.array_equal(mask, om) and removed == orem
