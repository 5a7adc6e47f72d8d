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
