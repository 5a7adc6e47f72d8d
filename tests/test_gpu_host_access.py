"""Host entry points that address the caller's host buffers in place (GB300:
the device reads pageable memory through the host page tables over
NVLink-C2C) give the same bits as the staged path and the device path, leave
an output's padding alone, populate an untouched output first, and stage an
input whose pages are not resident."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIRECT_IN, DIRECT_OUT = 1, 2


def device_mi(gpu, X, precision):
    import torch
    dX = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    n = X.shape[0]
    dMI = torch.empty((n, n), device="cuda")
    gpu.bspline_mi_dev(dX, dMI, 10, 3, precision)
    torch.cuda.synchronize()
    return dMI.cpu().numpy()


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("precision", ["bf16x3", "bf16f8", "fp32"])
@pytest.mark.parametrize("n", [600, 1000])
def test_pageable_in_place_matches_device(gpu, built_lib, precision, n):
    """1,000 genes take the staged path's row slabs (FP32) or its whole-matrix launch
    (tensor-core forms, whose packed tiles must give the device path's bits)."""
    X = built_lib.synth_grn(n, 700, seed=31)
    want = device_mi(gpu, X, precision)
    gpu.set_host_access("auto")
    got = gpu.bspline_mi(X, precision=precision)   # pageable X, fresh (untouched) np.empty output
    assert gpu.last_host_access() == DIRECT_IN | DIRECT_OUT
    assert same_bits(got, want)
    gpu.set_host_access("staged")
    try:
        staged = gpu.bspline_mi(X, precision=precision)
        assert gpu.last_host_access() == 0
    finally:
        gpu.set_host_access("auto")
    assert same_bits(staged, want)


def test_pinned_in_place(gpu, built_lib):
    import torch
    import mcpnet_gb300 as M
    n, m = 1000, 512
    X = built_lib.synth_grn(n, m, seed=32)
    want = device_mi(gpu, X, "bf16x3")
    Xp = torch.empty((n, m), dtype=torch.float32, pin_memory=True)
    Xp.numpy()[:] = X
    MIp = torch.empty((n, n), dtype=torch.float32, pin_memory=True)
    rc = M.lib().mcpg_bspline_mi(gpu._h, Xp.data_ptr(), n, m, m, 10, 3, M.PRECISIONS["bf16x3"], MIp.data_ptr(),
                                 n, None)
    assert rc == 0
    assert gpu.last_host_access() == DIRECT_IN | DIRECT_OUT
    assert same_bits(MIp.numpy(), want)


def test_padded_buffers_keep_their_padding(gpu, built_lib):
    """ldx > m and ldmi > n: the kernels read / write the caller's strided rows
    and never touch the padding columns."""
    import mcpnet_gb300 as M
    n, m, px, pm = 300, 257, 7, 5
    X = built_lib.synth_grn(n, m, seed=33)
    want = device_mi(gpu, X, "bf16x3")
    Xpad = np.full((n, m + px), np.nan, np.float32)
    Xpad[:, :m] = X
    MIpad = np.full((n, n + pm), 7.0, np.float32)
    rc = M.lib().mcpg_bspline_mi(gpu._h, Xpad.ctypes.data, n, m, m + px, 10, 3, M.PRECISIONS["bf16x3"],
                                 MIpad.ctypes.data, n + pm, None)
    assert rc == 0
    assert gpu.last_host_access() == DIRECT_IN | DIRECT_OUT
    assert same_bits(MIpad[:, :n], want)
    assert np.all(MIpad[:, n:] == 7.0)


def test_untouched_input_is_staged(gpu):
    """An input whose pages were never touched is not resident: it is staged
    (a first touch by the GPU would be a slow IOMMU fault)."""
    import mmap
    import mcpnet_gb300 as M
    n, m = 64, 4096
    buf = mmap.mmap(-1, n * m * 4)     # a fresh anonymous mapping: zero pages, none populated
    X = np.frombuffer(buf, dtype=np.float32).reshape(n, m)
    MI = np.empty((n, n), np.float32)
    rc = M.lib().mcpg_bspline_mi(gpu._h, X.ctypes.data, n, m, m, 10, 3, M.PRECISIONS["fp32"], MI.ctypes.data, n,
                                 None)
    assert rc == 0
    assert gpu.last_host_access() & DIRECT_IN == 0
    assert np.all(MI == device_mi(gpu, X, "fp32"))


def test_ap_mi_in_place(gpu, built_lib):
    X = built_lib.synth_grn(400, 300, seed=34)
    gpu.set_host_access("auto")
    got = gpu.ap_mi(X, noise=1e-5, seed=3)
    assert gpu.last_host_access() == DIRECT_IN | DIRECT_OUT
    gpu.set_host_access("staged")
    try:
        staged = gpu.ap_mi(X, noise=1e-5, seed=3)
    finally:
        gpu.set_host_access("auto")
    assert same_bits(got, staged)


def test_host_access_mode_checked(gpu):
    import mcpnet_gb300 as M
    assert M.lib().mcpg_set_host_access(gpu._h, 7) == M.ERR_ARG


def _both(gpu, fn):
    """fn() with in-place host access and with staged copies; returns both results and the in-place bits."""
    gpu.set_host_access("auto")
    a = fn()
    bits = gpu.last_host_access()
    gpu.set_host_access("staged")
    try:
        b = fn()
        assert gpu.last_host_access() == 0
    finally:
        gpu.set_host_access("auto")
    return a, b, bits


def _flat(x):
    if isinstance(x, dict):
        return _flat([x[k] for k in sorted(x)])
    if isinstance(x, (tuple, list)):
        out = []
        for y in x:
            out += _flat(y)
        return out
    return [x]


def _same(a, b):
    for x, y in zip(_flat(a), _flat(b)):
        if isinstance(x, np.ndarray):
            assert x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8))
        else:
            assert x == y


def test_host_entry_points_in_place(gpu, built_lib):
    """Every host entry point that writes its outputs in place gives the staged
    path's bits; outputs that are operands of later products (M1) stay staged."""
    n = 300
    X = built_lib.synth_grn(n, 200, seed=35)
    A = gpu.bspline_mi(X)
    np.fill_diagonal(A, 0)
    B = np.ascontiguousarray(A[:, ::-1])
    tfs = np.where(np.arange(n) % 7 == 0, np.inf, -np.inf).astype(np.float32)
    cases = {
        "maxmin": (lambda: gpu.maxmin(A, B), DIRECT_OUT),
        "ratio": (lambda: gpu.ratio(A, B), DIRECT_IN | DIRECT_OUT),
        "mcp3_sym": (lambda: gpu.mcp(A, 3, symmetrize=True), DIRECT_OUT),
        "mcp4": (lambda: gpu.mcp(A, 4), DIRECT_OUT),
        "dpi": (lambda: gpu.dpi(A, 0.1, want_mask=True), DIRECT_OUT),
        "closure": (lambda: gpu.closure(A), DIRECT_OUT),
        "maxmins": (lambda: gpu.maxmins(A), DIRECT_OUT),
        "maxmin_masked": (lambda: gpu.maxmin_masked(A, B, tfs), DIRECT_OUT),
        "mcp_tf": (lambda: gpu.mcp_tf(A, tfs, 4, 3), DIRECT_OUT),
        "maxmins_tf": (lambda: gpu.maxmins_tf(A, tfs), DIRECT_OUT),
        "dpi_tf": (lambda: gpu.dpi_tf(A, tfs, 0.1, want_mask=True), DIRECT_OUT),
        "transform": (lambda: gpu.transform(A), DIRECT_OUT),
        "stouffer_tf": (lambda: gpu.stouffer_tf(A[:40]), DIRECT_OUT),
        "combo": (lambda: gpu.combo(A, B, A, B, [0.25, 0.25, 0.25, 0.25]), DIRECT_IN | DIRECT_OUT),
    }
    for name, (fn, want_bits) in cases.items():
        a, b, bits = _both(gpu, fn)
        assert bits == want_bits, name
        _same(a, b)
