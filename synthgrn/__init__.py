"""Seeded synthetic GRN expression: the input generator of every benchmark
configuration (host only).

``synth_grn(n, m, seed)`` returns n genes x m samples of float32 expression in
[0, 1] from a random sparse DAG (in-degree ~ Poisson(2), weights +-U(0.5, 1.5),
x_g = tanh(sum w x_parent) + N(0, 0.3^2), roots ~ N(0, 1), per-gene min-max
rescale), optionally with the DAG's edges as ground truth.

The generator is its own small C++ library, libmcpsynth.so (synth.cpp here,
declared in include/mcpsynth.h), with no CUDA dependency: a CPU-only run of
the reference path makes the same input bytes without loading the GPU
library.  ``build()`` compiles it in-tree (g++, OpenMP); it is rebuilt when
the source is newer than the library.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
INCLUDE = HERE.parent / "include"
LIB_DIR = HERE / "_lib"
LIB_PATH = LIB_DIR / "libmcpsynth.so"
SRC = HERE / "synth.cpp"
HDR = INCLUDE / "mcpsynth.h"

_lib = None


def build(force: bool = False) -> Path:
    """Compile libmcpsynth.so if it is missing or older than its sources."""
    stale = force or not LIB_PATH.exists() or max(SRC.stat().st_mtime, HDR.stat().st_mtime) > LIB_PATH.stat().st_mtime
    if stale:
        LIB_DIR.mkdir(exist_ok=True)
        # -ffp-contract=off: no FMA contraction, so x86-64 and aarch64 round the same operations
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden", "-fopenmp", "-ffp-contract=off",
               f"-I{INCLUDE}", str(SRC), "-o", str(LIB_PATH)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"libmcpsynth.so build failed\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        L.mcps_synth_grn.restype = C.c_int
        L.mcps_synth_grn.argtypes = [C.c_int64, C.c_int64, C.c_uint64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                     C.POINTER(C.c_int64)]
        _lib = L
    return _lib


def synth_grn(n: int, m: int, seed: int = 20260001, with_edges: bool = False):
    """Seeded synthetic GRN expression (n genes x m samples, float32 in [0, 1]);
    with_edges=True also returns the DAG as an (edges, 2) int32 array of
    (parent, child)."""
    X = np.empty((n, m), dtype=np.float32)
    ne = C.c_int64(0)
    rc = lib().mcps_synth_grn(n, m, seed, X.ctypes.data if X.size else None, max(m, 1), None, 0, C.byref(ne))
    if rc:
        raise ValueError(f"synth_grn({n}, {m}): bad arguments (status {rc})")
    if not with_edges:
        return X
    E = np.empty((max(ne.value, 1), 2), dtype=np.int32)
    rc = lib().mcps_synth_grn(n, 0, seed, None, 1, E.ctypes.data, ne.value, C.byref(ne))
    if rc:
        raise ValueError(f"synth_grn({n}, 0): bad arguments (status {rc})")
    return X, E[: ne.value]
