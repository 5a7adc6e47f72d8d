"""GPU DPI filter and max-capacity closure: bit-exact against the oracle and
the reference's golden fixtures."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("name", ["mcp_70", "mcp_130"])
def test_dpi_golden(gpu, golden, name):
    g = golden(name)
    out, mask, removed = gpu.dpi(g["A"], float(g["tol"]), want_mask=True)
    assert np.array_equal(bits(out), bits(g["DPI_out"]))
    assert np.array_equal(mask, g["DPI_mask"])
    assert removed == int(g["DPI_removed"])


def test_dpi_ties_golden(gpu, golden):
    g = golden("dpi_ties")
    for tag in ("t0", "t1"):
        out, mask, removed = gpu.dpi(g["A"], float(g[f"tol_{tag}"]), want_mask=True)
        assert np.array_equal(bits(out), bits(g[f"out_{tag}"]))
        assert np.array_equal(mask, g[f"mask_{tag}"])
        assert removed == int(g[f"removed_{tag}"])


@pytest.mark.parametrize("n", [1, 2, 3, 16, 17, 129, 257])
@pytest.mark.parametrize("tol", [0.0, 0.1, 0.5])
def test_dpi_vs_oracle(gpu, port, n, tol):
    rng = np.random.default_rng(n * 7 + int(tol * 10))
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    out, mask, removed = gpu.dpi(A, tol, want_mask=True)
    oo, om, orem = port.dpi(A, tol)
    assert np.array_equal(bits(out), bits(oo))
    assert np.array_equal(mask, om)
    assert removed == orem


def test_dpi_nonsymmetric_and_nonzero_diagonal(gpu, port):
    rng = np.random.default_rng(21)
    A = rng.random((150, 150)).astype(np.float32)  # not symmetric, diagonal kept
    out, mask, removed = gpu.dpi(A, 0.1, want_mask=True)
    oo, om, orem = port.dpi(A, 0.1)
    assert np.array_equal(bits(out), bits(oo)) and np.array_equal(mask, om) and removed == orem


@pytest.mark.parametrize("n", [1, 2, 40, 130, 300])
def test_closure_vs_oracle(gpu, port, n):
    rng = np.random.default_rng(n + 3)
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    out, it = gpu.closure(A)
    oo, oit = port.closure(A)
    assert it == oit
    assert np.array_equal(bits(out), bits(oo))


def test_closure_not_converged_reports(gpu, port, built_lib):
    rng = np.random.default_rng(4)
    n = 200
    # a path graph with increasing capacities needs several squarings
    A = np.zeros((n, n), np.float32)
    w = rng.random(n - 1).astype(np.float32) + 0.5
    idx = np.arange(n - 1)
    A[idx, idx + 1] = w
    A[idx + 1, idx] = w
    out, it = gpu.closure(A, max_iter=2)
    assert it == -1
    full, fit = gpu.closure(A)
    assert fit > 2
    assert np.array_equal(bits(full), bits(port.closure(A)[0]))


def _mi_like(built_lib, gpu, n, m, seed):
    """An MI matrix (the DPI's real input) with diagonal 0."""
    X = built_lib.synth_grn(n, m, seed=seed)
    A = gpu.bspline_mi(X, 10, 3, "bf16f8")
    np.fill_diagonal(A, 0)
    return A


@pytest.mark.parametrize("n", [1100, 1601, 2100])
@pytest.mark.parametrize("tol", [0.0, 0.1, 0.5])
def test_two_phase_dpi_on_mi_matrices(gpu, port, built_lib, n, tol):
    """Above 1,024 genes the DPI runs in two phases (a tiled max-min over the first
    512 intermediates, then an early-exit scan of the undecided outputs): the same
    outputs, mask and removed count as the reference's loop."""
    A = _mi_like(built_lib, gpu, n, 400, seed=n)
    out, mask, removed = gpu.dpi(A, tol, want_mask=True)
    oo, om, orem = port.dpi(A, tol)
    assert np.array_equal(bits(out), bits(oo))
    assert np.array_equal(mask, om)
    assert removed == orem


def test_two_phase_dpi_ties_and_nonsymmetric(gpu, port):
    rng = np.random.default_rng(33)
    n = 1300
    A = (rng.integers(0, 7, size=(n, n)) * 0.125).astype(np.float32)  # many ties
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    for M in (A, (rng.random((n, n)) ** 3).astype(np.float32)):  # the second one is not symmetric
        out, mask, removed = gpu.dpi(M, 0.1, want_mask=True)
        oo, om, orem = port.dpi(M, 0.1)
        assert np.array_equal(bits(out), bits(oo)) and np.array_equal(mask, om) and removed == orem


def test_two_phase_dpi_falls_back_when_most_outputs_stay_undecided(gpu, port):
    """tol = 0.999 raises every threshold 1000-fold: almost nothing is deleted, the
    pending list overflows, and the one-phase product gives the result instead."""
    rng = np.random.default_rng(34)
    n = 1200
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    out, mask, removed = gpu.dpi(A, 0.999, want_mask=True)
    oo, om, orem = port.dpi(A, 0.999)
    assert np.array_equal(bits(out), bits(oo)) and np.array_equal(mask, om) and removed == orem
