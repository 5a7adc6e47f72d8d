"""Tensor-core (tcgen05) B-spline MI against the reference's double-precision
MI (golden fixtures) and the FP64 oracle.  Tolerances in bits (1 bit = ln 2
nats); the benchmark spec's bound is 1e-4 nats = 1.44e-4 bits:
  bf16x3 (hi+lo split) 2e-5 bits   fp16x3 2e-5 bits
  fp16 (single)        2e-4 bits   bf16 (single) 3e-3 bits (does not meet the bound)
  bf16f8 (BF16 hi*hi + E4M3 hi*lo + lo*hi correction) 1e-4 bits
The single-rounding forms carry one 16-bit rounding per weight, which only
averages out over many samples: below 200 samples their bound is 10x looser
(3x for bf16f8, whose residual is the E4M3 rounding of the correction terms).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"bf16x3": 2e-5, "fp16x3": 2e-5, "fp16": 2e-4, "bf16": 3e-3, "bf16f8": 1e-4}
SMALL_M = {"fp16": 10, "bf16": 10, "bf16f8": 3}


def tol_for(prec, m):
    return TOL[prec] * (SMALL_M.get(prec, 1) if m < 200 else 1)


MI_CASES = ["mi_37x211", "mi_64x500", "mi_3x7", "mi_1x5"]


@pytest.mark.parametrize("prec", ["bf16x3", "bf16", "fp16", "fp16x3", "bf16f8"])
@pytest.mark.parametrize("name", MI_CASES)
def test_mi_tc_golden(gpu, golden, name, prec):
    g = golden(name)
    MI = gpu.bspline_mi(g["X"], 10, 3, prec)
    assert np.array_equal(MI, MI.T)
    np.testing.assert_allclose(MI, g["MI64"], rtol=0, atol=tol_for(prec, g["X"].shape[1]))


@pytest.mark.parametrize("n,m", [(13, 64), (25, 65), (37, 300), (130, 1000), (251, 129)])
def test_mi_bf16x3_vs_oracle(gpu, port, built_lib, n, m):
    X = built_lib.synth_grn(n, m, seed=1000 + n + m)
    ref = port.bspline_mi(X.astype(np.float64))
    for prec in ("bf16x3", "fp16", "bf16f8"):
        MI = gpu.bspline_mi(X, 10, 3, prec)
        err = np.abs(MI - ref).max()
        assert err <= tol_for(prec, m), (prec, err)


def test_mi_tc_matches_fp32_path(gpu, built_lib):
    X = built_lib.synth_grn(300, 700, seed=77)
    a = gpu.bspline_mi(X, 10, 3, "fp32")
    b = gpu.bspline_mi(X, 10, 3, "bf16x3")
    assert np.abs(a - b).max() < 3e-5
    c = gpu.bspline_mi(X, 10, 3, "bf16f8")
    assert np.array_equal(c, c.T) and np.abs(a - c).max() < 1e-4


def test_mi_tc_unsupported_bins_report(gpu, built_lib):
    X = built_lib.synth_grn(20, 64, seed=3)
    with pytest.raises(built_lib.MCPGError) as e:
        gpu.bspline_mi(X, 8, 3, "bf16x3")
    assert e.value.status == built_lib.ERR_UNSUPPORTED


@pytest.mark.parametrize("prec", ["bf16x3", "bf16f8", "fp32"])
def test_host_slabbed_mi_equals_device_mi(gpu, built_lib, prec):
    """The host entry point computes in row slabs and copies finished slabs back
    while later ones compute; the result is bit-identical to one device call."""
    import torch
    n, m = 1000, 300
    X = built_lib.synth_grn(n, m, seed=55)
    host = gpu.bspline_mi(X, 10, 3, prec)
    Xd = torch.from_numpy(X).cuda()
    dev = torch.empty((n, n), device="cuda")
    gpu.bspline_mi_dev(Xd, dev, 10, 3, prec)
    gpu.synchronize()
    assert np.array_equal(host, dev.cpu().numpy())


@pytest.mark.parametrize("prec", ["bf16f8", "bf16x3"])
def test_one_sm_form_matches_pair_form(gpu, built_lib, tmp_path, prec):
    """The 1-SM kernel (MCPG_TC_FORM=1sm; also the fallback when no SM pair fits)
    gives the default 2-SM kernel's MI to FP32 rounding.  The form is chosen once
    per process, so the 1-SM run is a child process."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    X = built_lib.synth_grn(250, 400, seed=91)
    np.save(tmp_path / "x.npy", X)
    code = (f"import sys, numpy as np; sys.path.insert(0, {str(root)!r}); import mcpnet_gb300 as M; "
            f"X = np.load({str(tmp_path / 'x.npy')!r}); "
            f"np.save({str(tmp_path / 'one.npy')!r}, M.Handle(0).bspline_mi(X, 10, 3, {prec!r}))")
    r = subprocess.run([sys.executable, "-c", code], env=dict(os.environ, MCPG_TC_FORM="1sm"),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    one = np.load(tmp_path / "one.npy")
    pair = gpu.bspline_mi(X, 10, 3, prec)
    assert np.abs(one - pair).max() <= 2e-6


@pytest.mark.parametrize("prec", ["bf16f8", "bf16x3"])
def test_bounded_wait_runs_out_and_the_handle_recovers(gpu, built_lib, prec):
    """A device wait that runs out: the test hook gives the next tensor-core launch
    a 5 ms barrier-wait limit and starves its TMA producers, so the MMA issuer's
    first wait expires with no load or MMA in flight.  The call must return
    ERR_DEVICE_TIMEOUT with a message, and the next normal call on the same handle
    (which needs every SM's tensor memory again, so the starved launch must have
    freed it) must give the same bits as before."""
    import torch
    n, m = 300, 640
    X = torch.from_numpy(built_lib.synth_grn(n, m, seed=77)).cuda()
    ref = torch.empty((n, n), dtype=torch.float32, device="cuda")
    gpu.bspline_mi_dev(X, ref, 10, 3, prec)
    gpu.synchronize()
    out = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    gpu.test_tc_timeout(5_000_000, starve=True)
    with pytest.raises(built_lib.MCPGError) as e:
        gpu.bspline_mi_dev(X, out, 10, 3, prec)
    assert e.value.status == built_lib.ERR_DEVICE_TIMEOUT
    assert b"bounded barrier wait" in gpu._L.mcpg_last_error(gpu._h)
    again = torch.empty((n, n), dtype=torch.float32, device="cuda")
    gpu.bspline_mi_dev(X, again, 10, 3, prec)
    gpu.synchronize()
    assert torch.equal(again.view(torch.int32), ref.view(torch.int32))


def test_timeout_hook_argument_check(gpu, built_lib):
    assert gpu._L.mcpg_test_tc_timeout(gpu._h, 10, 1) == built_lib.ERR_ARG
    assert gpu._L.mcpg_test_tc_timeout(None, 5_000_000, 1) == built_lib.ERR_ARG
