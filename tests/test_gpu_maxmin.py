"""GPU max-min products, MCP compositions, ratio: bit-exact against the oracle
and the reference's golden fixtures, through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("rows,cols,k", [(1, 1, 1), (2, 3, 1), (3, 2, 7), (17, 5, 16), (129, 131, 33),
                                         (200, 70, 300), (64, 300, 15), (5, 5, 0)])
def test_maxmin_rect(gpu, port, rows, cols, k):
    rng = np.random.default_rng(rows * 1000 + cols * 10 + k)
    A = rng.normal(size=(rows, k)).astype(np.float32)
    B = rng.normal(size=(cols, k)).astype(np.float32)
    assert np.array_equal(bits(gpu.maxmin(A, B)), bits(port.maxmin(A, B)))


@pytest.mark.parametrize("n", [1, 2, 3, 17, 128, 129, 300])
def test_maxmin_symmetric(gpu, port, n):
    rng = np.random.default_rng(n)
    A = rng.random((n, n)).astype(np.float32)
    C = gpu.maxmin(A)  # A (x) A: symmetric kernel path
    assert np.array_equal(bits(C), bits(port.maxmin(A)))
    assert np.array_equal(C, C.T)


def test_maxmin_golden_rect(gpu, golden):
    g = golden("maxmin_rect")
    assert np.array_equal(bits(gpu.maxmin(g["A"], g["B"])), bits(g["C"]))


def test_maxmin_ties_and_infinities(gpu, port):
    rng = np.random.default_rng(5)
    A = rng.integers(0, 3, size=(70, 41)).astype(np.float32)
    A[3, :] = -np.inf
    A[:, 7] = np.inf
    B = rng.integers(0, 3, size=(66, 41)).astype(np.float32)
    assert np.array_equal(bits(gpu.maxmin(A, B)), bits(port.maxmin(A, B)))


@pytest.mark.parametrize("name", ["mcp_70", "mcp_130"])
def test_mcp_golden(gpu, golden, name):
    g = golden(name)
    A = g["A"]
    for pl in (2, 3, 4):
        M, R = gpu.mcp(A, pl)
        assert np.array_equal(bits(M), bits(g[f"M{pl}"])), pl
        assert np.array_equal(bits(R), bits(g[f"R{pl}"])), pl
    M, R = gpu.mcp(A, 3, symmetrize=True)
    assert np.array_equal(bits(M), bits(g["M3s"])) and np.array_equal(bits(R), bits(g["R3s"]))


@pytest.mark.parametrize("n", [1, 5, 131, 260])
def test_mcp_vs_oracle(gpu, port, n):
    rng = np.random.default_rng(100 + n)
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    for pl in (2, 3, 4):
        M, R = gpu.mcp(A, pl)
        Mo, Ro = port.mcp(A, pl)
        assert np.array_equal(bits(M), bits(Mo)) and np.array_equal(bits(R), bits(Ro)), pl


def test_ratio_edges(gpu, port):
    rng = np.random.default_rng(9)
    A = rng.normal(size=(37, 53)).astype(np.float32)
    M = rng.normal(size=(37, 53)).astype(np.float32)
    A[0, :5] = [0, 1e-8, -1e-8, 0.5, 0.25]
    M[0, :5] = [0, 0.5, 0.5, 0, 1e-9]
    M[1, :3] = [np.inf, -np.inf, 1e-30]
    assert np.array_equal(bits(gpu.ratio(A, M)), bits(port.ratio(A, M)))


def test_device_entry_points_and_unaligned_ld(gpu, port):
    import torch
    rng = np.random.default_rng(11)
    n, k = 77, 45
    A = rng.random((n, k)).astype(np.float32)
    big = torch.zeros((n, k + 3), device="cuda", dtype=torch.float32)  # ld = 48 but view starts at column 1
    big[:, 1:k + 1] = torch.from_numpy(A).cuda()
    Av = big[:, 1:k + 1]                      # unaligned base, ld 48
    Cd = torch.empty((n, n), device="cuda", dtype=torch.float32)
    gpu.maxmin_dev(Av, Av, Cd)
    gpu.synchronize()
    assert np.array_equal(bits(Cd.cpu().numpy()), bits(port.maxmin(A)))


def test_bad_arguments_report_errors(gpu, built_lib):
    L, h = built_lib.lib(), gpu._h
    A = np.zeros((4, 4), np.float32)
    C = np.zeros((4, 4), np.float32)
    assert L.mcpg_maxmin(h, A.ctypes.data, 2, A.ctypes.data, 4, 4, 4, 4, C.ctypes.data, 4) == built_lib.ERR_ARG
    assert b"leading dimension" in L.mcpg_last_error(h)
    assert L.mcpg_mcp(h, A.ctypes.data, 4, 4, 5, 0, C.ctypes.data, 4, None, 4) == built_lib.ERR_ARG


def test_injected_allocation_failure_is_reported(built_lib):
    h = built_lib.Handle(0)
    try:
        h.fail_next_allocs(1)
        with pytest.raises(built_lib.MCPGError) as e:
            h.maxmin(np.ones((8, 8), np.float32))
        assert e.value.status == built_lib.ERR_OOM
        # the handle stays usable afterwards
        assert np.array_equal(h.maxmin(np.ones((8, 8), np.float32)), np.ones((8, 8), np.float32))
    finally:
        h.close()


@pytest.mark.parametrize("n", [3, 130, 257])
def test_maxmins_shared_m1_matches_oracle(gpu, port, n):
    import torch
    rng = np.random.default_rng(300 + n)
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    Ad = torch.from_numpy(A).cuda()
    outs = [torch.empty((n, n), device="cuda") for _ in range(6)]
    gpu.maxmins_dev(Ad, *outs)
    gpu.synchronize()
    M1, M2, M3, R2, R3, R4 = (o.cpu().numpy() for o in outs)
    for pl, M, R in ((2, M1, R2), (3, M2, R3), (4, M3, R4)):
        Mo, Ro = port.mcp(A, pl)
        assert np.array_equal(bits(M), bits(Mo)) and np.array_equal(bits(R), bits(Ro)), pl
    # ratios only (M1 in scratch)
    R3b = torch.empty((n, n), device="cuda")
    gpu.maxmins_dev(Ad, R3=R3b)
    gpu.synchronize()
    assert np.array_equal(bits(R3b.cpu().numpy()), bits(port.mcp(A, 3)[1]))


@pytest.mark.parametrize("cs", [(1.0, 0.0, 0.0, 0.0), (0.0, 1.0, 0.0, 0.0), (0.5, 0.25, 1.0, 0.0),
                                (0.1, 0.2, 0.3, 0.4), (0.0, 0.0, 0.0, 0.0)])
def test_combo_matches_oracle(gpu, port, cs):
    """compute_combo, the ensemble MCP score, bit-exact against the oracle's
    restatement (the reference routine itself needs the absent splash
    patterns, so this op is pinned only through the restatement)."""
    import torch
    rng = np.random.default_rng(int(sum(cs) * 100))
    n = 133
    A = rng.random((n, n)).astype(np.float32)
    A = np.maximum(A, A.T)
    np.fill_diagonal(A, 0)
    A[0, :5] = [1e-9, 0, 0.5, 0.25, 0.75]
    M1 = port.maxmin(A)
    M2 = port.maxmin(A, M1)
    M3 = port.maxmin(M1)
    ref = port.combo(A, M1, M2, M3, cs)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    out = torch.empty((n, n), device="cuda")
    gpu.combo_dev(t(A), t(M1), t(M2), t(M3), cs, out)
    gpu.synchronize()
    assert np.array_equal(bits(out.cpu().numpy()), bits(ref))
