import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libmcpgpu.so")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        with np.load(GOLDEN / f"{name}.npz") as z:
            return {k: z[k] for k in z.files}
    return load


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    return O.port()


@pytest.fixture(scope="session")
def built_lib():
    """Build libmcpgpu.so in-tree if stale and return the package."""
    from mcpnet_gb300 import build as B
    B.build()
    import mcpnet_gb300 as M
    return M


@pytest.fixture(scope="session")
def gpu(built_lib):
    """A library handle on cuda:0 on torch's current stream (so tests that mix
    torch tensors with *_dev calls are ordered); GPU tests fail (not skip)
    without a GPU."""
    h = built_lib.Handle(0)
    import torch
    h.set_stream(torch.cuda.current_stream().cuda_stream)
    yield h
    h.close()
