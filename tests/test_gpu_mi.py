"""GPU B-spline MI through the C ABI against the reference's golden fixtures
and the oracle.  Tolerances are stated in bits (the reference's unit; 1 bit =
ln 2 nats):
  * weights: bit-exact (same float operations as the reference)
  * FP32 MI vs the reference's --single MI and vs its double MI: 2e-5 bits
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MI_CASES = ["mi_37x211", "mi_64x500", "mi_3x7", "mi_1x5", "mi_20x64_b8k2"]
FP32_TOL_BITS = 2e-5


@pytest.mark.parametrize("name", MI_CASES)
def test_weights_bit_exact_golden(gpu, golden, name):
    g = golden(name)
    W, H = gpu.bspline_weights(g["X"], int(g["bins"]), int(g["order"]))
    assert np.array_equal(W[:, :-1].view(np.uint32), g["W"][:, :-1].view(np.uint32))
    np.testing.assert_allclose(H, g["W"][:, -1].astype(np.float64), rtol=0, atol=2e-6)
    np.testing.assert_allclose(W[:, -1], H.astype(np.float32))


@pytest.mark.parametrize("name", MI_CASES)
def test_mi_fp32_golden(gpu, golden, name):
    g = golden(name)
    MI, H = gpu.bspline_mi(g["X"], int(g["bins"]), int(g["order"]), "fp32", return_H=True)
    assert np.array_equal(MI, MI.T)
    np.testing.assert_allclose(MI, g["MI32"], rtol=0, atol=FP32_TOL_BITS)
    np.testing.assert_allclose(MI, g["MI64"], rtol=0, atol=FP32_TOL_BITS)


@pytest.mark.parametrize("n,m,bins,order", [(17, 129, 10, 3), (33, 1000, 10, 3), (70, 257, 10, 3),
                                            (19, 100, 7, 3), (12, 80, 12, 4), (25, 64, 5, 1), (9, 31, 2, 2)])
def test_mi_fp32_vs_oracle(gpu, port, built_lib, n, m, bins, order):
    X = built_lib.synth_grn(n, m, seed=n * 31 + m)
    MI = gpu.bspline_mi(X, bins, order, "fp32")
    ref64 = port.bspline_mi(X.astype(np.float64), bins, order)
    np.testing.assert_allclose(MI, ref64, rtol=0, atol=FP32_TOL_BITS)


def test_mi_constant_gene_and_ties(gpu, port):
    rng = np.random.default_rng(3)
    X = rng.random((20, 150)).astype(np.float32)
    X[4] = 0.5          # constant gene: scale = 1, offset = 0
    X[7, ::2] = 1.0     # many samples exactly on the right boundary
    X[9] = np.round(X[9] * 4) / 4  # knots hit exactly
    MI = gpu.bspline_mi(X, 10, 3, "fp32")
    np.testing.assert_allclose(MI, port.bspline_mi(X.astype(np.float64)), rtol=0, atol=FP32_TOL_BITS)


def test_mi_bad_args(gpu, built_lib):
    with pytest.raises(built_lib.MCPGError):
        gpu.bspline_mi(np.zeros((4, 8), np.float32), bins=3, order=4)
    with pytest.raises(built_lib.MCPGError):
        gpu.bspline_mi(np.zeros((4, 8), np.float32), bins=40, order=3)
