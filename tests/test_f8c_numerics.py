"""The FP8-corrected MI form (bf16f8) restated in numpy on the CPU: the
operand planes the weights kernel writes (BF16 hi * 2^8, E4M3 H8 = e4m3(16 hi),
E4M3 L8 = e4m3(4096 (w - hi)), from the reference's float weights), the joint
table they give in exact arithmetic, and its MI against the FP64 oracle.

This pins the numerical scheme independently of the tensor cores: the scales
multiply to 2^16 in every product, no E4M3 value saturates, and the scheme's
own error (the E4M3 rounding of the correction terms) is within the 1e-4-nats
bound with room for the FP32 accumulation the GPU adds.
"""
import numpy as np
import pytest

NATS = np.log(2.0)


def _round_to_grid(x, mant_bits, emin):
    """Round to nearest even onto a binary floating-point grid with `mant_bits`
    explicit mantissa bits and minimum normal exponent `emin` (subnormals kept)."""
    x = np.asarray(x, np.float64)
    a = np.abs(x)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    q = np.exp2(np.maximum(e, emin) - mant_bits)
    return np.sign(x) * np.round(a / q) * q  # np.round: half to even


def bf16(x):
    return _round_to_grid(x, 7, -126)


def e4m3(x):
    return _round_to_grid(x, 3, -6)


def _mi_from_joint(P, H, bins=10):
    n = H.size
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(P > 0, P * np.log2(P), 0.0)
    return H[:, None] + H[None, :] + t.reshape(n, bins, n, bins).sum(axis=(1, 3))


def test_grid_rounding_matches_known_values():
    assert bf16(1.0 + 2.0 ** -8) == 1.0          # tie to even
    assert bf16(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6
    assert e4m3(1.0625) == 1.0                    # 1 + 2^-4: tie to even
    assert e4m3(448.0) == 448.0 and e4m3(2.0 ** -9) == 2.0 ** -9  # largest finite, smallest subnormal
    assert e4m3(0.75 * 2.0 ** -9) == 2.0 ** -9


@pytest.mark.parametrize("n,m", [(60, 300), (40, 2000), (24, 64)])
def test_f8c_scheme_within_bound(port, built_lib, n, m):
    X = built_lib.synth_grn(n, m, seed=7000 + n + m)
    W = np.asarray(port.bspline_weights(X), np.float64)[:, :10 * m].reshape(n * 10, m)  # float weights
    hf = bf16(W)
    hi = hf * 256.0
    H8 = e4m3(16.0 * hf)
    L8 = e4m3(4096.0 * (W - hf))
    # no E4M3 value reaches the format's largest finite value (448): nothing saturates
    assert np.abs(H8).max() <= 16.0 and np.abs(L8).max() <= 8.0
    # 2^16 P = hi hi' + H8 L8' + L8 H8'  (exact in float64 at these sizes)
    P = (hi @ hi.T + H8 @ L8.T + L8 @ H8.T) / 65536.0 / m
    ref = port.bspline_mi(X.astype(np.float64))
    Wd = np.asarray(port.bspline_weights(X.astype(np.float64)), np.float64)
    H = Wd[:, -1]
    got = _mi_from_joint(P, H)
    iu = np.triu_indices(n, 1)
    err_nats = float(np.abs(got[iu] - ref[iu]).max()) * NATS
    bound = 1e-4 if m >= 200 else 3e-4   # nats; the scheme must leave half for the FP32 accumulation
    assert err_nats <= 0.5 * bound, err_nats
    # and the correction is what closes the gap: BF16 alone misses the bound at these sizes
    P1 = (hi @ hi.T) / 65536.0 / m
    err1 = float(np.abs(_mi_from_joint(P1, H)[iu] - ref[iu]).max()) * NATS
    assert err1 > 4 * err_nats
