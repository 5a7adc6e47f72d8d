"""The no-allocation MI entry point, through the C ABI.

Some callers cannot call cudaMalloc (an application whose device memory is
owned by its own pool allocator, or a latency-critical loop that cannot take
cudaMalloc's implicit synchronisation); mcpg_bspline_mi_fp32_noalloc serves
them from a fixed 32 MiB device array.  It runs the same kernels on the same
weight-table layout as the handle's FP32 path, so its output must equal that
path's bit for bit.  This file is collected last on purpose, so that a run
stopping at the first failure has run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(built_lib, port):
    import torch
    L = built_lib.lib()
    n, m = 300, 700
    X_host = built_lib.synth_grn(n, m, seed=99)
    X = torch.from_numpy(X_host).cuda()
    h = built_lib.Handle(0)
    try:
        ref = torch.empty((n, n), dtype=torch.float32, device="cuda")
        h.bspline_mi_dev(X, ref, 10, 3, "fp32")
        h.synchronize()
        ref = ref.cpu().numpy()
        stream = torch.cuda.current_stream().cuda_stream
        for _ in range(2):  # two calls in a row share the static scratch
            out = torch.full((n, n), float("nan"), dtype=torch.float32, device="cuda")
            Hd = torch.empty(n, dtype=torch.float64, device="cuda")
            rc = L.mcpg_bspline_mi_fp32_noalloc(X.data_ptr(), n, m, m, 10, 3, out.data_ptr(), n, Hd.data_ptr(),
                                                stream)
            assert rc == built_lib.OK
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))
            # H may also be left to the scratch array
            out2 = torch.full((n, n), float("nan"), dtype=torch.float32, device="cuda")
            rc = L.mcpg_bspline_mi_fp32_noalloc(X.data_ptr(), n, m, m, 10, 3, out2.data_ptr(), n, None, stream)
            assert rc == built_lib.OK
            torch.cuda.synchronize()
            assert np.array_equal(out2.cpu().numpy().view(np.uint32), ref.view(np.uint32))
        # and against the oracle's FP64 MI (the handle path's own tolerance, in bits)
        ref64 = port.bspline_mi(X_host.astype(np.float64))
        assert np.abs(out2.cpu().numpy() - ref64).max() < 2e-5
    finally:
        h.close()


def test_noalloc_rejects_problems_beyond_its_scratch(built_lib):
    import torch
    L = built_lib.lib()
    X = torch.zeros((8, 8), dtype=torch.float32, device="cuda")
    out = torch.zeros((8, 8), dtype=torch.float32, device="cuda")
    # 5000 genes x 2000 samples needs 400 MB of weights: rejected before any device work
    rc = L.mcpg_bspline_mi_fp32_noalloc(X.data_ptr(), 5000, 2000, 2000, 10, 3, out.data_ptr(), 5000, None, 0)
    assert rc == built_lib.ERR_SCRATCH_LIMIT
    assert b"32 MiB" in L.mcpg_status_string(rc)
    assert L.mcpg_bspline_mi_fp32_noalloc(None, 8, 8, 8, 10, 3, out.data_ptr(), 8, None, 0) == built_lib.ERR_ARG
    # bin counts without a compiled kernel are argument errors, not CUDA errors
    for bins, order in ((1, 1), (13, 3)):
        rc = L.mcpg_bspline_mi_fp32_noalloc(X.data_ptr(), 8, 8, 8, bins, order, out.data_ptr(), 8, None, 0)
        assert rc == built_lib.ERR_ARG, (bins, rc)
