"""CPU-only checks of the C ABI library: it loads, exports every symbol the
public header declares, rejects bad arguments without touching a GPU, and its
host-only synthetic generator is deterministic and well formed."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "mcpgpu.h").read_text()
    return sorted(set(re.findall(r"MCPG_API\s+[\w\s\*]+?\b(mcpg_\w+)\s*\(", text)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    assert "mcpg_bspline_mi" in syms and "mcpg_maxmin_dev" in syms and len(syms) >= 25


def test_library_exports_every_declared_symbol(built_lib):
    L = built_lib.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    bound = {name for name, _, _ in built_lib.ABI}
    assert set(declared_symbols()) == bound  # python binding covers the whole ABI


def test_null_handle_and_status_strings(built_lib):
    L = built_lib.lib()
    assert L.mcpg_version() >= 100
    assert L.mcpg_status_string(0) == b"ok"
    assert L.mcpg_status_string(-1) == b"invalid argument"
    assert L.mcpg_maxmin(None, None, 0, None, 0, 1, 1, 1, None, 1) == built_lib.ERR_ARG
    assert L.mcpg_bspline_mi_dev(None, None, 1, 1, 1, 10, 3, 0, None, 1, None) == built_lib.ERR_ARG
    assert L.mcpg_destroy(None) == 0
    assert L.mcpg_create(None, 0) == built_lib.ERR_ARG
    assert L.mcpg_last_error(None) == b"null handle"


def test_synth_deterministic_and_scaled(built_lib):
    X1 = built_lib.synth_grn(50, 80, seed=123)
    X2 = built_lib.synth_grn(50, 80, seed=123)
    X3 = built_lib.synth_grn(50, 80, seed=124)
    assert X1.dtype == np.float32 and X1.shape == (50, 80)
    assert np.array_equal(X1, X2) and not np.array_equal(X1, X3)
    assert np.all(X1 >= 0) and np.all(X1 <= 1)
    assert np.allclose(X1.min(1), 0) and np.allclose(X1.max(1), 1)


def test_synth_graph_is_a_dag_with_poisson2_indegree(built_lib):
    n = 4000
    _, E = built_lib.synth_grn(n, 2, seed=9, with_edges=True)
    assert E.shape[1] == 2 and len(E) > 0
    assert np.all(E[:, 0] != E[:, 1])
    indeg = np.bincount(E[:, 1], minlength=n)
    assert 1.8 < indeg.mean() < 2.2
    assert len({tuple(e) for e in E.tolist()}) == len(E)  # no duplicate parents
    # acyclic: Kahn's algorithm consumes every node
    out = [[] for _ in range(n)]
    for p, c in E:
        out[p].append(c)
    deg = indeg.copy()
    stack = [i for i in range(n) if deg[i] == 0]
    seen = 0
    while stack:
        u = stack.pop(); seen += 1
        for v in out[u]:
            deg[v] -= 1
            if deg[v] == 0:
                stack.append(v)
    assert seen == n


def test_synth_bad_args():
    import synthgrn
    L = synthgrn.lib()
    assert L.mcps_synth_grn(-1, 5, 1, None, 5, None, 0, None) == -1
    X = np.empty((2, 5), np.float32)
    assert L.mcps_synth_grn(2, 5, 1, X.ctypes.data, 4, None, 0, None) == -1


def test_synth_library_exports_its_header_and_stays_off_the_gpu_library():
    """The generator is its own host-only library: it exports what
    include/mcpsynth.h declares and links neither libmcpgpu.so nor CUDA."""
    import subprocess
    import synthgrn
    text = (ROOT / "include" / "mcpsynth.h").read_text()
    syms = sorted(set(re.findall(r"MCPS_API\s+[\w\s\*]+?\b(mcps_\w+)\s*\(", text)))
    assert syms == ["mcps_synth_grn"]
    L = synthgrn.lib()
    assert all(hasattr(L, s) for s in syms)
    deps = subprocess.run(["ldd", str(synthgrn.LIB_PATH)], capture_output=True, text=True).stdout
    assert "mcpgpu" not in deps and "libcuda" not in deps and "cudart" not in deps, deps
    # the GPU library no longer carries the generator
    assert "synth" not in (ROOT / "include" / "mcpgpu.h").read_text()


# SHA-256 of synth_grn(n, m, seed=20260001) (X bytes, edge bytes), recorded when the
# generator moved out of libmcpgpu.so into libmcpsynth.so: the move left the bytes unchanged.
# The values hold for x86-64 glibc; libm's tanh / log / cos may round differently elsewhere.
SYNTH_SHA256 = {
    (1000, 1000): ("bbb9414b057fbd6e43e7ec205fb69f59ba9989520674ce3362638cf02c1e063b",
                   "cda002529dedc28ea4b5e499b54b88cbea520d464b2216d7b45323a87381dc17"),
    (2000, 2000): ("6a4bf74fcb08753887d2b9df8acc095f47c598769a036f04cb7495f547e1b5d1",
                   "ecb7cb2cf710aa96fad4831e05f1bef97b654052c6db6d576b1ae2ffd0e4ff70"),
    (4096, 1024): ("9876fe3c0070a4658abb87ce08409a0b582b87d892cfe32821f2ab93e8ae582c",
                   "7dec94c30f6707a9f4d3a02159ee4a4db5afe2b76a3f82fb76398b903242587e"),
    (20000, 2000): ("d77d88235e0e47d8df98767710255804a58e63cc063d1ce2a9e37f5b6ff180d9",
                    "8138011b55693990a36729eb93f33b57d5dbde0c94754324aa118a2d8267b03f"),
}


@pytest.mark.parametrize("shape", sorted(SYNTH_SHA256))
def test_synth_bytes_unchanged(shape):
    import hashlib
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("checksums recorded with x86-64 glibc")
    import synthgrn
    X, E = synthgrn.synth_grn(*shape, seed=20260001, with_edges=True)
    assert (hashlib.sha256(X.tobytes()).hexdigest(), hashlib.sha256(E.tobytes()).hexdigest()) == SYNTH_SHA256[shape]


def test_no_cpu_fallback_without_gpu(built_lib):
    """On a machine without a GPU the library refuses to create a handle
    instead of computing on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(built_lib.MCPGError):
        built_lib.Handle(0)
