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


@pytest.mark.parametrize("precision", ["bf16x3", "fp32"])
def test_pageable_in_place_matches_device(gpu, built_lib, precision):
    X = built_lib.synth_grn(600, 700, seed=31)
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
