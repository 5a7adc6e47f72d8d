"""compute_combo on the GPU takes a float-float path with a certified error
bound and falls back to the double formula only near float rounding
boundaries; the result must equal the reference's double computation
(the oracle, compiled without FMA contraction) bit for bit on every input."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COEFFS = [(0.25, 0.25, 0.25, 0.25), (0.1, 0.2, 0.3, 0.4), (1, 1, 1, 1), (0.5, -0.5, 0.3, 0.0),
          (1 / 3, 1 / 7, 0.0, 1.0), (-1.0, 1.0, 0.0, 0.0), (1e-8, 1.0, 0.0, 0.0), (0.0, 0.75, 0.25, 0.0),
          (1.0, 0.0, 0.0, 0.0), (0.0, 0.0, 0.0, 0.0), (3.0, -2.0, 1e-3, 7.5)]


def inputs(rng, shape):
    kind = rng.integers(0, 6, size=shape)
    u = rng.random(shape)
    x = np.where(kind == 0, u,                                   # uniform [0, 1)
        np.where(kind == 1, np.floor(u * 17) / 16,               # small dyadic values, many ties
        np.where(kind == 2, 1e-7 + u * 2e-7,                     # around FLT_EPSILON
        np.where(kind == 3, 0.0,                                 # zeros
        np.where(kind == 4, u * 1e30, -u))))).astype(np.float32)  # large, negative
    return x


@pytest.mark.parametrize("ci", range(len(COEFFS)))
def test_combo_bit_exact_stress(gpu, port, ci):
    import torch
    rng = np.random.default_rng(100 + ci)
    rows, cols = 1500, 1500
    mi, m1, m2, m3 = (inputs(rng, (rows, cols)) for _ in range(4))
    cs = np.array(COEFFS[ci], dtype=np.float64)
    want = port.combo(mi, m1, m2, m3, cs)
    d = lambda x: torch.from_numpy(x).cuda()
    out = torch.empty((rows, cols), device="cuda")
    gpu.combo_dev(d(mi), d(m1), d(m2), d(m3), cs, out)
    got = out.cpu().numpy()
    bad = got.view(np.uint32) != want.view(np.uint32)
    assert not bad.any(), (int(bad.sum()), got[bad][:5], want[bad][:5])
