"""mcpnet_gb300 -- GB300 (sm_103a) implementation of MCPNet's compute core.

Python host mirror of the C ABI in include/mcpgpu.h (libmcpgpu.so, built
in-tree by ``python -m mcpnet_gb300.build``).  The operations mirror MCPNet's
helper-level calls (apps/pipeline/mcpnet_helper.hpp):

=====================  =====================================================
``bspline_mi``          compute_mi           (mcpnet_helper.hpp:56-99)
``bspline_weights``     Transform<BSplineWeightsKernel> (mcpnet_helper.hpp:67-80)
``maxmin``              InnerProduct<mcp2_maxmin_kernel> (filter/mcp.hpp:72-93)
``ratio``               compute_ratio        (mcpnet_helper.hpp:172-184)
``mcp``                 compute_mcp2/3/4     (mcpnet_helper.hpp:199-365)
``dpi``                 the dpi app's mask + apply (apps/filter/dpi.cpp:236-287)
``closure``             max-capacity closure by repeated squaring (no reference routine)
=====================  =====================================================

Host calls take and return numpy arrays (``float32``, C-contiguous rows);
``*_dev`` calls take torch CUDA tensors and run asynchronously on the handle's
stream.  There is no CPU fallback: without the built library or a GPU these
raise.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libmcpgpu.so"

OK, ERR_ARG, ERR_OOM, ERR_CUDA, ERR_NOT_CONVERGED, ERR_UNSUPPORTED, ERR_DEVICE_TIMEOUT = 0, -1, -2, -3, -4, -5, -6
ERR_SCRATCH_LIMIT = -7
PRECISIONS = {"fp32": 0, "bf16": 1, "bf16x3": 2, "fp16": 3, "fp16x3": 4, "bf16f8": 5}

# (name, restype, argtypes) of every exported symbol -- the full C ABI.
_i64, _f32p, _f64p, _vp = C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_double), C.c_void_p
ABI = [
    ("mcpg_version", C.c_int, []),
    ("mcpg_status_string", C.c_char_p, [C.c_int]),
    ("mcpg_create", C.c_int, [C.POINTER(_vp), C.c_int]),
    ("mcpg_destroy", C.c_int, [_vp]),
    ("mcpg_last_error", C.c_char_p, [_vp]),
    ("mcpg_set_stream", C.c_int, [_vp, _vp]),
    ("mcpg_synchronize", C.c_int, [_vp]),
    ("mcpg_kernel_launches", C.c_int64, [_vp]),
    ("mcpg_test_fail_allocs", C.c_int, [_vp, C.c_int]),
    ("mcpg_test_tc_timeout", C.c_int, [_vp, _i64, C.c_int]),
    ("mcpg_profile", C.c_int, [_vp, C.c_int]),
    ("mcpg_profile_report", C.c_int64, [_vp, C.c_char_p, C.c_int64]),
    ("mcpg_bspline_mi", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, C.c_int, _vp, _i64, _vp]),
    ("mcpg_bspline_mi_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, C.c_int, _vp, _i64, _vp]),
    ("mcpg_bspline_weights", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _vp]),
    ("mcpg_bspline_weights_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _vp]),
    ("mcpg_maxmin", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_maxmin_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_ratio", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_ratio_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_set_diagonal_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_float]),
    ("mcpg_mcp", C.c_int, [_vp, _vp, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
    ("mcpg_mcp_dev", C.c_int, [_vp, _vp, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
    ("mcpg_combo_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _vp, _i64]),
    ("mcpg_maxmins_dev", C.c_int, [_vp, _vp, _i64, _i64] + [_vp, _i64] * 6),
    ("mcpg_dpi", C.c_int, [_vp, _vp, _i64, _i64, C.c_float, _vp, _i64, _vp, C.POINTER(C.c_int64)]),
    ("mcpg_dpi_dev", C.c_int, [_vp, _vp, _i64, _i64, C.c_float, _vp, _i64, _vp, C.POINTER(C.c_int64)]),
    ("mcpg_closure", C.c_int, [_vp, _vp, _i64, _i64, C.c_int, _vp, _i64, C.POINTER(C.c_int)]),
    ("mcpg_maxmin_masked", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64]),
    ("mcpg_maxmin_masked_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64]),
    ("mcpg_mcp_tf", C.c_int, [_vp, _vp, _i64, _i64, _vp, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
    ("mcpg_mcp_tf_dev", C.c_int, [_vp, _vp, _i64, _i64, _vp, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
    ("mcpg_dpi_tf", C.c_int, [_vp, _vp, _i64, _i64, C.c_float, _vp, _vp, _i64, _vp, C.POINTER(C.c_int64)]),
    ("mcpg_dpi_tf_dev", C.c_int, [_vp, _vp, _i64, _i64, C.c_float, _vp, _vp, _i64, _vp, C.POINTER(C.c_int64)]),
    ("mcpg_closure_dev", C.c_int, [_vp, _vp, _i64, _i64, C.c_int, _vp, _i64, C.POINTER(C.c_int)]),
    ("mcpg_maxmin_witness", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp, _i64]),
    ("mcpg_maxmin_witness_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp, _i64]),
    ("mcpg_maxmin_bwd", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64,
                                  _vp, _i64, _vp, _i64]),
    ("mcpg_maxmin_bwd_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64,
                                      _vp, _i64, _vp, _i64]),
    ("mcpg_ratio_bwd_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64]),
    ("mcpg_bspline_mi_bwd", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
    ("mcpg_bspline_mi_bwd_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
    ("mcpg_bspline_mi_fp32_noalloc", C.c_int, [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp, _vp]),
    ("mcpg_aupr_auroc", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _vp]),
    ("mcpg_aupr_auroc_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _vp]),
    ("mcpg_eval_truth", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("mcpg_eval_truth_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64, C.c_int, _vp, _vp, _vp, _vp, _vp,
                                      _vp]),
    ("mcpg_select_truth_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64, C.c_int, _vp, _vp, _vp, _i64, _vp,
                                        _i64, _vp, _vp]),
    ("mcpg_combo_eval_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64,
                                      C.c_int, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
]
ABI += [
    ("mcpg_ap_ranks_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_float, C.c_uint64, _vp, _i64]),
    ("mcpg_ap_mi_ranks", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_ap_mi_ranks_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_ap_mi", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_float, C.c_uint64, _vp, _i64]),
    ("mcpg_ap_mi_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_float, C.c_uint64, _vp, _i64]),
]
ABI += [
    ("mcpg_maxmins", C.c_int, [_vp, _vp, _i64, _i64] + [_vp, _i64] * 6),
    ("mcpg_combo", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _vp, _i64]),
    ("mcpg_combo_eval", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64,
                                  C.c_int, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
]
ABI += [
    ("mcpg_row_stats_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, _vp, _vp]),
    ("mcpg_transform", C.c_int, [_vp, _vp, _i64, _i64, C.c_int, C.c_int, _vp, _i64]),
    ("mcpg_transform_dev", C.c_int, [_vp, _vp, _i64, _i64, C.c_int, C.c_int, _vp, _i64]),
    ("mcpg_combo_stouffer_eval_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _i64,
                                               C.c_int, _vp, _vp, _vp, _i64, C.c_int, _vp, _vp, _vp]),
]
ABI += [
    ("mcpg_combo_stouffer_eval", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _i64,
                                           C.c_int, _vp, _vp, _vp, _i64, C.c_int, _vp, _vp, _vp]),
]
ABI += [
    ("mcpg_maxmins_tf", C.c_int, [_vp, _vp, _i64, _i64, _vp] + [_vp, _i64] * 4),
    ("mcpg_maxmins_tf_dev", C.c_int, [_vp, _vp, _i64, _i64, _vp] + [_vp, _i64] * 4),
    ("mcpg_stouffer_tf", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_stouffer_tf_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64]),
    ("mcpg_stouffer_tf_stats_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _vp, _vp, _vp]),
    ("mcpg_transform_tf", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, _vp, _i64]),
    ("mcpg_transform_tf_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, C.c_int, _vp, _i64]),
    ("mcpg_combo_stouffer_tf_eval", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp,
                                              _i64, C.c_int, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    ("mcpg_combo_stouffer_tf_eval_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp,
                                                  _i64, C.c_int, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
]
ABI += [
    ("mcpg_set_host_access", C.c_int, [_vp, C.c_int]),
    ("mcpg_last_host_access", C.c_int, [_vp]),
]
ABI += [
    ("mcpg_shuffle_positions", C.c_int, [_vp, _i64, C.c_uint64]),
    ("mcpg_split_aupr", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64, C.c_int, _vp, _vp, _i64, _vp, _i64, _vp,
                                  _vp, _vp]),
    ("mcpg_split_aupr_dev", C.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _i64, C.c_int, _vp, _vp, _i64, _vp, _i64, _vp,
                                      _vp, _vp]),
    ("mcpg_split_combo_eval", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64,
                                        C.c_int, _vp, _vp, _vp, _i64, C.c_int, _i64, _vp, _i64, _vp, _vp]),
    ("mcpg_split_combo_eval_dev", C.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64,
                                            C.c_int, _vp, _vp, _vp, _i64, C.c_int, _i64, _vp, _i64, _vp, _vp]),
]
STOUFFER_MODES = {"none": -1, "all": 0, "exclude_diagonal": 1, "tf": 2}
HOST_ACCESS = {"auto": 0, "staged": 1}


def train_counts(entries: int, tf: bool = False):
    """The eval_mcpnet app's training sizes (apps/pipeline/eval_mcpnet.cpp:240-250): (size_t)(f * entries)
    for f = 0.005, 0.01, 0.02, 0.05, 0.1, and with TFs also 0.2, 0.3, 0.4, 0.5."""
    fr = [0.005, 0.01, 0.02, 0.05, 0.1] + ([0.2, 0.3, 0.4, 0.5] if tf else [])
    return np.array([int(f * float(entries)) for f in fr], dtype=np.int64)


def shuffle_positions(entries: int, seed: int) -> np.ndarray:
    """Iteration `seed`'s shuffled order of the eval_mcpnet app (shuffle_truth,
    apps/pipeline/eval_mcpnet.cpp:214-224) as mask positions (host only; seed 0 keeps the order)."""
    out = np.empty(max(int(entries), 0), dtype=np.uint32)
    rc = lib().mcpg_shuffle_positions(out.ctypes.data if out.size else None, int(entries), int(seed))
    if rc != 0:
        raise MCPGError(rc, f"shuffle_positions: bad count {entries}")
    return out


TRANSFORMS = {"stouffer": 0, "clr": 1}
ROW_STATS = {"all": 0, "exclude_diagonal": 1}
TRUTH_REGIONS = {"lower": 0, "all": 1, "tf": 2}
AP_NOISE = 1e-5  # the reference apps' tie-breaking noise amplitude (apps/correlation/mi.cpp:128-129)

_lib = None


class MCPGError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mcpgpu status {status}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """Load libmcpgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m mcpnet_gb300.build` "
                               "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in ABI:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _f32(a) -> np.ndarray:
    a = np.asarray(a, dtype=np.float32)
    return a if a.flags.c_contiguous else np.ascontiguousarray(a)


def synth_grn(n: int, m: int, seed: int = 20260001, with_edges: bool = False):
    """Seeded synthetic GRN expression (n genes x m samples, float32 in [0, 1]),
    from the host-only generator library (synthgrn, libmcpsynth.so)."""
    try:
        from synthgrn import synth_grn as _synth
    except ImportError:  # the package is used from outside the repository root
        sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
        from synthgrn import synth_grn as _synth
    return _synth(n, m, seed, with_edges)


class Handle:
    """One device, one stream.  Not thread-safe (as the C handle)."""

    def __init__(self, device: int = 0):
        self._L = lib()
        h = C.c_void_p()
        rc = self._L.mcpg_create(C.byref(h), device)
        if rc:
            raise MCPGError(rc, f"mcpg_create(device={device}) failed: "
                            f"{self._L.mcpg_status_string(rc).decode()}")
        self._h = h
        self.device = device

    # -- plumbing --
    def close(self):
        if getattr(self, "_h", None):
            self._L.mcpg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int, what: str):
        if rc:
            raise MCPGError(rc, f"{what}: {self._L.mcpg_last_error(self._h).decode()}")

    @property
    def kernel_launches(self) -> int:
        return int(self._L.mcpg_kernel_launches(self._h))

    def set_stream(self, stream_ptr: int):
        """Run this handle's work on an existing CUDA stream (e.g. torch's current
        stream, so *_dev calls are ordered with torch operations)."""
        self._check(self._L.mcpg_set_stream(self._h, stream_ptr), "set_stream")

    def synchronize(self):
        self._check(self._L.mcpg_synchronize(self._h), "synchronize")

    def profile(self, enable: bool = True):
        """Start (clearing) or stop per-kernel CUDA-event timing."""
        self._check(self._L.mcpg_profile(self._h, int(enable)), "profile")

    def profile_report(self) -> dict:
        import json
        need = self._L.mcpg_profile_report(self._h, None, 0)
        if need < 0:
            self._check(int(need), "profile_report")
        buf = C.create_string_buffer(int(need))
        self._L.mcpg_profile_report(self._h, buf, need)
        return json.loads(buf.value.decode())

    def fail_next_allocs(self, count: int):
        self._check(self._L.mcpg_test_fail_allocs(self._h, count), "test_fail_allocs")

    def test_tc_timeout(self, wait_ns: int, starve: bool = True):
        """Testing hook: the next tensor-core MI launch waits at most wait_ns per barrier
        wait, and with starve its producers issue no loads (the call then fails with
        ERR_DEVICE_TIMEOUT and the handle stays usable)."""
        self._check(self._L.mcpg_test_tc_timeout(self._h, int(wait_ns), int(bool(starve))), "test_tc_timeout")

    # -- host-buffer entry points --
    def bspline_mi(self, X, bins: int = 10, order: int = 3, precision: str = "fp32", return_H: bool = False):
        """All-pairs B-spline MI (bits) of the genes (rows) of X, from host memory.  precision:
        "fp32" (CUDA cores), "bf16f8" (BF16 hi*hi + E4M3 correction: the fastest form within
        1e-4 nats of FP64), "bf16x3" / "fp16x3" (16-bit hi+lo splits), "bf16" / "fp16" (single
        rounding).  With return_H, also the FP64 marginal entropies."""
        X = _f32(X)
        n, m = X.shape
        MI = np.empty((n, n), dtype=np.float32)
        H = np.empty(n, dtype=np.float64) if return_H else None
        self._check(self._L.mcpg_bspline_mi(self._h, _ptr(X), n, m, m, bins, order, PRECISIONS[precision],
                                             _ptr(MI), n, _ptr(H)), "bspline_mi")
        return (MI, H) if return_H else MI

    def bspline_weights(self, X, bins: int = 10, order: int = 3):
        X = _f32(X)
        n, m = X.shape
        W = np.empty((n, bins * m + 1), dtype=np.float32)
        H = np.empty(n, dtype=np.float64)
        self._check(self._L.mcpg_bspline_weights(self._h, _ptr(X), n, m, m, bins, order, _ptr(W), _ptr(H)),
                    "bspline_weights")
        return W, H

    def maxmin(self, A, B=None):
        A = _f32(A)
        same = B is None
        B = A if same else _f32(B)
        rows, k = A.shape
        cols = B.shape[0]
        if B.shape[1] != k:
            raise ValueError("maxmin: A and B need the same number of columns")
        Cm = np.empty((rows, cols), dtype=np.float32)
        self._check(self._L.mcpg_maxmin(self._h, _ptr(A), k, _ptr(B), k, rows, cols, k, _ptr(Cm), cols), "maxmin")
        return Cm

    def ratio(self, A, M):
        A, M = _f32(A), _f32(M)
        rows, cols = A.shape
        R = np.empty((rows, cols), dtype=np.float32)
        self._check(self._L.mcpg_ratio(self._h, _ptr(A), cols, _ptr(M), cols, rows, cols, _ptr(R), cols), "ratio")
        return R

    def mcp(self, A, path_len: int, symmetrize: bool = False, want_maxmin: bool = True, want_ratio: bool = True):
        A = _f32(A)
        n = A.shape[0]
        M = np.empty((n, n), dtype=np.float32) if want_maxmin else None
        R = np.empty((n, n), dtype=np.float32) if want_ratio else None
        self._check(self._L.mcpg_mcp(self._h, _ptr(A), n, n, path_len, int(symmetrize), _ptr(M), n, _ptr(R), n),
                    "mcp")
        return M, R

    def dpi(self, A, tol: float = 0.1, want_mask: bool = False):
        A = _f32(A)
        n = A.shape[0]
        out = np.empty((n, n), dtype=np.float32)
        mask = np.empty((n, n), dtype=np.uint8) if want_mask else None
        removed = C.c_int64(0)
        self._check(self._L.mcpg_dpi(self._h, _ptr(A), n, n, tol, _ptr(out), n, _ptr(mask), C.byref(removed)), "dpi")
        return out, mask, removed.value

    def maxmin_masked(self, A, B, mask):
        A = _f32(A)
        same = B is None
        B = A if same else _f32(B)
        mask = _f32(mask)
        rows, k = A.shape
        cols = B.shape[0]
        Cm = np.empty((rows, cols), dtype=np.float32)
        self._check(self._L.mcpg_maxmin_masked(self._h, _ptr(A), k, _ptr(B), k, rows, cols, k, _ptr(mask),
                                                _ptr(Cm), cols), "maxmin_masked")
        return Cm

    def mcp_tf(self, A, tfs, path_len: int, transition: int):
        """compute_mcp{2,3,4}_tfs: returns (maxmin, ratio), each t x n."""
        A = _f32(A)
        tfs = _f32(tfs)
        n = A.shape[0]
        t = int((tfs > 0).sum())
        M = np.empty((t, n), dtype=np.float32)
        R = np.empty((t, n), dtype=np.float32)
        self._check(self._L.mcpg_mcp_tf(self._h, _ptr(A), n, n, _ptr(tfs), path_len, transition, _ptr(M), n,
                                         _ptr(R), n), "mcp_tf")
        return M, R

    def maxmins_tf(self, A, tfs):
        """compute_maxmins_tfs: returns (T, M1, M2, M3), each t x n (T = the TF rows of A)."""
        A = _f32(A)
        tfs = _f32(tfs)
        n = A.shape[0]
        t = int((tfs > 0).sum())
        outs = [np.empty((t, n), dtype=np.float32) for _ in range(4)]
        args = []
        for o in outs:
            args += [_ptr(o), n]
        self._check(self._L.mcpg_maxmins_tf(self._h, _ptr(A), n, n, _ptr(tfs), *args), "maxmins_tf")
        return tuple(outs)

    def maxmins_tf_dev(self, A, tfs, T=None, M1=None, M2=None, M3=None):
        """compute_maxmins_tfs into t x n CUDA tensors (each optional); tfs is a host array."""
        tfs = _f32(tfs)
        n = A.shape[0]
        args = []
        for o in (T, M1, M2, M3):
            args += [self._dp(o), self._ld(o) if o is not None else n]
        self._check(self._L.mcpg_maxmins_tf_dev(self._h, self._dp(A), n, self._ld(A), _ptr(tfs), *args),
                    "maxmins_tf_dev")

    def dpi_tf(self, A, tfs, tol: float = 0.1, want_mask: bool = False):
        A = _f32(A)
        tfs = _f32(tfs)
        n = A.shape[0]
        out = np.empty((n, n), dtype=np.float32)
        mask = np.empty((n, n), dtype=np.uint8) if want_mask else None
        removed = C.c_int64(0)
        self._check(self._L.mcpg_dpi_tf(self._h, _ptr(A), n, n, tol, _ptr(tfs), _ptr(out), n, _ptr(mask),
                                         C.byref(removed)), "dpi_tf")
        return out, mask, removed.value

    def closure(self, A, max_iter: int = 64):
        A = _f32(A)
        n = A.shape[0]
        out = np.empty((n, n), dtype=np.float32)
        it = C.c_int(0)
        rc = self._L.mcpg_closure(self._h, _ptr(A), n, n, max_iter, _ptr(out), n, C.byref(it))
        if rc == ERR_NOT_CONVERGED:
            return out, -1
        self._check(rc, "closure")
        return out, it.value

    # -- device entry points (torch CUDA tensors, float32, row-major, stride(1) == 1) --
    @staticmethod
    def _dp(t):
        return None if t is None else t.data_ptr()

    @staticmethod
    def _ld(t):
        if t.dim() != 2 or t.stride(1) != 1:
            raise ValueError("device matrices must be 2-D with unit column stride")
        return t.stride(0)

    def bspline_mi_dev(self, X, MI, bins=10, order=3, precision="fp32", H=None):
        n, m = X.shape
        self._check(self._L.mcpg_bspline_mi_dev(self._h, self._dp(X), n, m, self._ld(X), bins, order,
                                                 PRECISIONS[precision], self._dp(MI), self._ld(MI), self._dp(H)),
                    "bspline_mi_dev")

    def maxmin_dev(self, A, B, Cm):
        rows, k = A.shape
        self._check(self._L.mcpg_maxmin_dev(self._h, self._dp(A), self._ld(A), self._dp(B), self._ld(B), rows,
                                             B.shape[0], k, self._dp(Cm), self._ld(Cm)), "maxmin_dev")

    def ratio_dev(self, A, M, R):
        rows, cols = A.shape
        self._check(self._L.mcpg_ratio_dev(self._h, self._dp(A), self._ld(A), self._dp(M), self._ld(M), rows, cols,
                                            self._dp(R), self._ld(R)), "ratio_dev")

    def maxmin_witness_dev(self, A, B, Cm, K):
        rows, k = A.shape
        self._check(self._L.mcpg_maxmin_witness_dev(self._h, self._dp(A), self._ld(A), self._dp(B), self._ld(B),
                                                     rows, B.shape[0], k, self._dp(Cm), self._ld(Cm), self._dp(K),
                                                     self._ld(K)), "maxmin_witness_dev")

    def maxmin_bwd_dev(self, A, B, Cm, dC, K, dA, dB):
        """Accumulate the adjoint of Cm = A (x) B into dA, dB (K: saved witness or None)."""
        rows, k = A.shape
        self._check(self._L.mcpg_maxmin_bwd_dev(
            self._h, self._dp(A), self._ld(A), self._dp(B), self._ld(B), rows, B.shape[0], k,
            self._dp(Cm), self._ld(Cm) if Cm is not None else 0, self._dp(dC), self._ld(dC),
            self._dp(K), self._ld(K) if K is not None else 0, self._dp(dA), self._ld(dA), self._dp(dB),
            self._ld(dB)), "maxmin_bwd_dev")

    def ratio_bwd_dev(self, A, M, dR, dA, dM):
        rows, cols = A.shape
        self._check(self._L.mcpg_ratio_bwd_dev(self._h, self._dp(A), self._ld(A), self._dp(M), self._ld(M), rows, cols,
                                                self._dp(dR), self._ld(dR), self._dp(dA), self._ld(dA), self._dp(dM),
                                                self._ld(dM)), "ratio_bwd_dev")

    def bspline_mi_bwd_dev(self, X, G, dX, bins=10, order=3):
        n, m = X.shape
        self._check(self._L.mcpg_bspline_mi_bwd_dev(self._h, self._dp(X), n, m, self._ld(X), bins, order,
                                                     self._dp(G), self._ld(G), self._dp(dX), self._ld(dX)),
                    "bspline_mi_bwd_dev")

    def maxmin_witness(self, A, B=None):
        A = _f32(A)
        B = A if B is None else _f32(B)
        rows, k = A.shape
        cols = B.shape[0]
        Cm = np.empty((rows, cols), dtype=np.float32)
        K = np.empty((rows, cols), dtype=np.int32)
        self._check(self._L.mcpg_maxmin_witness(self._h, _ptr(A), k, _ptr(B), k, rows, cols, k, _ptr(Cm), cols,
                                                 _ptr(K), cols), "maxmin_witness")
        return Cm, K

    def bspline_mi_bwd(self, X, G, bins=10, order=3):
        X, G = _f32(X), _f32(G)
        n, m = X.shape
        dX = np.empty((n, m), dtype=np.float32)
        self._check(self._L.mcpg_bspline_mi_bwd(self._h, _ptr(X), n, m, m, bins, order, _ptr(G), n, _ptr(dX), m),
                    "bspline_mi_bwd")
        return dX

    def mcp3_loss_dev(self, X, rows_idx, cols_idx, coef, bins=10, order=3, precision="fp32"):
        """Forward only: L = sum_e coef[e] * R[rows_idx[e], cols_idx[e]] (FP64 sum of the FP32 scores)."""
        import torch
        n, m = X.shape
        self.set_stream(torch.cuda.current_stream(X.device).cuda_stream)  # order with the torch ops below
        f32 = dict(dtype=torch.float32, device=X.device)
        A = torch.empty((n, n), **f32)
        self.bspline_mi_dev(X, A, bins, order, precision)
        self.set_diagonal_dev(A, 0.0)
        R = torch.empty((n, n), **f32)
        self.mcp_dev(A, 3, M=None, R=R)
        return float((coef.to(torch.float64) * R[rows_idx, cols_idx].to(torch.float64)).sum().item())

    def mcp3_loss_grad_dev(self, X, rows_idx, cols_idx, coef, witness: str = "auto", bins=10, order=3,
                           return_dA: bool = False):
        """Differentiation form of the pipeline (torch CUDA tensors): with
        A = MI(X) (FP32, diagonal 0), M1 = A (x) A, M2 = A (x) M1, R = ratio(A, M2),
        L = sum_e coef[e] * R[rows_idx[e], cols_idx[e]]; returns (L, dL/dX).
        witness: "saved" keeps int32 argmax indices of both products, "recompute"
        finds them again from the products, "auto" saves them when the two
        n x n int32 arrays take under a quarter of the free device memory."""
        import torch
        n, m = X.shape
        dev = X.device
        self.set_stream(torch.cuda.current_stream(dev).cuda_stream)  # order with the torch ops below
        f32 = dict(dtype=torch.float32, device=dev)
        if witness == "auto":
            free, _ = torch.cuda.mem_get_info(dev)
            witness = "saved" if 2 * n * n * 4 < free // 4 else "recompute"
        MI = torch.empty((n, n), **f32)
        self.bspline_mi_dev(X, MI, bins, order, "fp32")
        A = MI
        self.set_diagonal_dev(A, 0.0)
        M1, M2, R = (torch.empty((n, n), **f32) for _ in range(3))
        K1 = K2 = None
        if witness == "saved":
            K1 = torch.empty((n, n), dtype=torch.int32, device=dev)
            K2 = torch.empty((n, n), dtype=torch.int32, device=dev)
            self.maxmin_witness_dev(A, A, M1, K1)
            self.maxmin_witness_dev(A, M1, M2, K2)
        else:
            self.maxmin_dev(A, A, M1)
            self.maxmin_dev(A, M1, M2)
        self.ratio_dev(A, M2, R)
        L = (coef.to(torch.float64) * R[rows_idx, cols_idx].to(torch.float64)).sum()
        dR = torch.zeros((n, n), **f32)
        dR.index_put_((rows_idx, cols_idx), coef.to(torch.float32), accumulate=True)
        dA, dM2, dM1 = (torch.zeros((n, n), **f32) for _ in range(3))
        self.ratio_bwd_dev(A, M2, dR, dA, dM2)
        self.maxmin_bwd_dev(A, M1, M2, dM2, K2, dA, dM1)
        self.maxmin_bwd_dev(A, A, M1, dM1, K1, dA, dA)
        dA.fill_diagonal_(0.0)  # the diagonal reset cuts the gradient to MI_ii
        dX = torch.empty((n, m), **f32)
        self.bspline_mi_bwd_dev(X, dA, dX, bins, order)
        if return_dA:
            return float(L.item()), dX, dA
        return float(L.item()), dX

    def set_diagonal_dev(self, A, value: float):
        self._check(self._L.mcpg_set_diagonal_dev(self._h, self._dp(A), A.shape[0], A.shape[1], self._ld(A), value),
                    "set_diagonal_dev")

    def mcp_dev(self, A, path_len, M=None, R=None, symmetrize=False):
        n = A.shape[0]
        self._check(self._L.mcpg_mcp_dev(self._h, self._dp(A), n, self._ld(A), path_len, int(symmetrize),
                                          self._dp(M), self._ld(M) if M is not None else n,
                                          self._dp(R), self._ld(R) if R is not None else n), "mcp_dev")

    def maxmins_dev(self, A, M1=None, M2=None, M3=None, R2=None, R3=None, R4=None):
        """compute_maxmins with the MCP2/3/4 ratios fused (torch CUDA tensors, all optional)."""
        n = A.shape[0]
        args = []
        for t in (M1, M2, M3, R2, R3, R4):
            args += [self._dp(t), self._ld(t) if t is not None else n]
        self._check(self._L.mcpg_maxmins_dev(self._h, self._dp(A), n, self._ld(A), *args), "maxmins_dev")

    def mcp_tf_dev(self, A, tfs, path_len: int, transition: int, M=None, R=None):
        """compute_mcp{2,3,4}_tfs into t x n CUDA tensors (each optional); tfs is a host array."""
        tfs = _f32(tfs)
        n = A.shape[0]
        self._check(self._L.mcpg_mcp_tf_dev(self._h, self._dp(A), n, self._ld(A), _ptr(tfs), path_len, transition,
                                             self._dp(M), self._ld(M) if M is not None else n, self._dp(R),
                                             self._ld(R) if R is not None else n), "mcp_tf_dev")

    def dpi_tf_dev(self, A, out, tfs, tol: float = 0.1, mask=None):
        """dpi_tf_kernel + mask on CUDA tensors; returns the removed count."""
        tfs = _f32(tfs)
        n = A.shape[0]
        removed = C.c_int64(0)
        self._check(self._L.mcpg_dpi_tf_dev(self._h, self._dp(A), n, self._ld(A), tol, _ptr(tfs), self._dp(out),
                                             self._ld(out), self._dp(mask), C.byref(removed)), "dpi_tf_dev")
        return removed.value

    def combo_dev(self, mi, M1, M2, M3, coeffs, out):
        """compute_combo: out = mi / (c0 mi + c1 M1 + c2 M2 + c3 M3) (torch CUDA tensors; Mk may be None when ck == 0)."""
        cs = np.ascontiguousarray(coeffs, dtype=np.float64)
        rows, cols = mi.shape
        ld = lambda t: self._ld(t) if t is not None else cols
        self._check(self._L.mcpg_combo_dev(self._h, self._dp(mi), self._ld(mi), self._dp(M1), ld(M1), self._dp(M2),
                                            ld(M2), self._dp(M3), ld(M3), rows, cols, cs.ctypes.data, self._dp(out),
                                            self._ld(out)), "combo_dev")

    # ---- adaptive-partitioning MI ----
    def ap_mi(self, X, noise: float = 0.0, seed: int = 1):
        """compute_ap_mi: (noise) -> descending ranks -> AP MI, n x n float32 (bits)."""
        X = _f32(X)
        n, m = X.shape
        MI = np.empty((n, n), dtype=np.float32)
        self._check(self._L.mcpg_ap_mi(self._h, _ptr(X), n, m, m, noise, seed, _ptr(MI), n), "ap_mi")
        return MI

    def ap_mi_ranks(self, R):
        """AP MI from integer ranks in [0, m) (n x m)."""
        R = np.ascontiguousarray(R, dtype=np.int32)
        n, m = R.shape
        MI = np.empty((n, n), dtype=np.float32)
        self._check(self._L.mcpg_ap_mi_ranks(self._h, _ptr(R), n, m, m, _ptr(MI), n), "ap_mi_ranks")
        return MI

    def ap_ranks_dev(self, X, R, noise: float = 0.0, seed: int = 1):
        n, m = X.shape
        self._check(self._L.mcpg_ap_ranks_dev(self._h, self._dp(X), n, m, self._ld(X), noise, seed, self._dp(R),
                                               self._ld(R)), "ap_ranks_dev")

    def ap_mi_dev(self, X, MI, noise: float = 0.0, seed: int = 1):
        n, m = X.shape
        self._check(self._L.mcpg_ap_mi_dev(self._h, self._dp(X), n, m, self._ld(X), noise, seed, self._dp(MI),
                                            self._ld(MI)), "ap_mi_dev")

    def ap_mi_ranks_dev(self, R, MI):
        n, m = R.shape
        self._check(self._L.mcpg_ap_mi_ranks_dev(self._h, self._dp(R), n, m, self._ld(R), self._dp(MI),
                                                  self._ld(MI)), "ap_mi_ranks_dev")

    def maxmins(self, A, want=("M1", "M2", "M3", "R2", "R3", "R4")):
        """compute_maxmins with the MCP2/3/4 ratios: dict of the requested n x n outputs."""
        A = _f32(A)
        n = A.shape[0]
        names = ("M1", "M2", "M3", "R2", "R3", "R4")
        out = {k: np.empty((n, n), dtype=np.float32) for k in names if k in want}
        args = []
        for k in names:
            args += [_ptr(out.get(k)), n]
        self._check(self._L.mcpg_maxmins(self._h, _ptr(A), n, n, *args), "maxmins")
        return out

    def combo(self, mi, M1, M2, M3, coeffs):
        """compute_combo on host matrices (Mk may be None when its coefficient is 0)."""
        mi = _f32(mi)
        rows, cols = mi.shape
        cs = np.ascontiguousarray(coeffs, dtype=np.float64)
        keep = [None if x is None else _f32(x) for x in (M1, M2, M3)]
        out = np.empty((rows, cols), dtype=np.float32)
        self._check(self._L.mcpg_combo(self._h, _ptr(mi), cols, _ptr(keep[0]), cols, _ptr(keep[1]), cols,
                                        _ptr(keep[2]), cols, rows, cols, cs.ctypes.data, _ptr(out), cols), "combo")
        return out

    def combo_eval(self, mi, M1, M2, M3, labels, coeffs, region="lower", row_gene=None, col_tf=None):
        """Host form of combo_eval_dev: (aupr ndarray, auroc ndarray, best row)."""
        mi = _f32(mi)
        rows, cols = mi.shape
        keep = [None if x is None else _f32(x) for x in (M1, M2, M3)]
        labels = np.ascontiguousarray(labels, dtype=np.int8)
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        rg = None if row_gene is None else np.ascontiguousarray(row_gene, dtype=np.int32)
        ct = None if col_tf is None else np.ascontiguousarray(col_tf, dtype=np.uint8)
        a = np.empty(cs.shape[0], dtype=np.float64)
        b = np.empty(cs.shape[0], dtype=np.float64)
        best = C.c_int64(0)
        self._check(self._L.mcpg_combo_eval(self._h, _ptr(mi), cols, _ptr(keep[0]), cols, _ptr(keep[1]), cols,
                                             _ptr(keep[2]), cols, rows, cols, _ptr(labels), cols,
                                             TRUTH_REGIONS[region], _ptr(rg), _ptr(ct), cs.ctypes.data, cs.shape[0],
                                             _ptr(a), _ptr(b), C.byref(best)), "combo_eval")
        return a, b, best.value

    # ---- Stouffer / CLR ----
    def transform(self, A, kind="stouffer", stats="exclude_diagonal"):
        """compute_stouffer (or CLR) of an n x n host matrix."""
        A = _f32(A)
        n = A.shape[0]
        out = np.empty((n, n), dtype=np.float32)
        self._check(self._L.mcpg_transform(self._h, _ptr(A), n, n, TRANSFORMS[kind], ROW_STATS[stats], _ptr(out), n),
                    "transform")
        return out

    def transform_dev(self, A, out, kind="stouffer", stats="exclude_diagonal"):
        n = A.shape[0]
        self._check(self._L.mcpg_transform_dev(self._h, self._dp(A), n, self._ld(A), TRANSFORMS[kind],
                                                ROW_STATS[stats], self._dp(out), self._ld(out)), "transform_dev")

    def set_host_access(self, mode="auto"):
        """'auto': host entry points address pageable / pinned host buffers in place where the device can;
        'staged': always copy through device scratch."""
        self._check(self._L.mcpg_set_host_access(self._h, HOST_ACCESS[mode]), "set_host_access")

    def last_host_access(self) -> int:
        """MCPG_HOST_DIRECT_* bits (1 input, 2 output) of the last host MI call."""
        return int(self._L.mcpg_last_host_access(self._h))

    def stouffer_tf(self, A):
        """compute_stouffer_tf of a t x n host matrix."""
        A = _f32(A)
        rows, cols = A.shape
        out = np.empty((rows, cols), dtype=np.float32)
        self._check(self._L.mcpg_stouffer_tf(self._h, _ptr(A), rows, cols, cols, _ptr(out), cols), "stouffer_tf")
        return out

    def transform_tf(self, A, kind="stouffer"):
        """The transform app's TF form (row and column z-scores; Stouffer or CLR) of a t x n host matrix."""
        A = _f32(A)
        rows, cols = A.shape
        out = np.empty((rows, cols), dtype=np.float32)
        self._check(self._L.mcpg_transform_tf(self._h, _ptr(A), rows, cols, cols, TRANSFORMS[kind], _ptr(out), cols),
                    "transform_tf")
        return out

    def transform_tf_dev(self, A, out, kind="stouffer"):
        rows, cols = A.shape
        self._check(self._L.mcpg_transform_tf_dev(self._h, self._dp(A), rows, cols, self._ld(A), TRANSFORMS[kind],
                                                   self._dp(out), self._ld(out)), "transform_tf_dev")

    def stouffer_tf_dev(self, A, out):
        rows, cols = A.shape
        self._check(self._L.mcpg_stouffer_tf_dev(self._h, self._dp(A), rows, cols, self._ld(A), self._dp(out),
                                                  self._ld(out)), "stouffer_tf_dev")

    # ---- semi-supervised split evaluation (eval_mcpnet) ----
    def split_aupr(self, values, labels, iterations, train_counts, region="lower", row_gene=None, col_tf=None):
        """eval_aupr_mcp on host arrays: (full AUPR, train[iters, parts], test[iters, parts])."""
        values = _f32(values)
        labels = np.ascontiguousarray(labels, dtype=np.int8)
        rows, cols = values.shape
        tc = np.ascontiguousarray(train_counts, dtype=np.int64)
        rg = None if row_gene is None else np.ascontiguousarray(row_gene, dtype=np.int32)
        ct = None if col_tf is None else np.ascontiguousarray(col_tf, dtype=np.uint8)
        full = C.c_double(0)
        tr = np.zeros((iterations, tc.size))
        te = np.zeros((iterations, tc.size))
        self._check(self._L.mcpg_split_aupr(self._h, _ptr(values), rows, cols, cols, _ptr(labels), cols,
                                             TRUTH_REGIONS[region], _ptr(rg), _ptr(ct), iterations, _ptr(tc), tc.size,
                                             C.byref(full), _ptr(tr), _ptr(te)), "split_aupr")
        return full.value, tr, te

    def split_aupr_dev(self, values, labels, iterations, train_counts, region="lower", row_gene=None, col_tf=None):
        """As split_aupr for CUDA tensors (values float32, labels int8, row_gene int32, col_tf uint8)."""
        rows, cols = values.shape
        tc = np.ascontiguousarray(train_counts, dtype=np.int64)
        full = C.c_double(0)
        tr = np.zeros((iterations, tc.size))
        te = np.zeros((iterations, tc.size))
        self._check(self._L.mcpg_split_aupr_dev(self._h, self._dp(values), rows, cols, self._ld(values),
                                                 self._dp(labels), self._ld(labels), TRUTH_REGIONS[region],
                                                 self._dp(row_gene), self._dp(col_tf), iterations, _ptr(tc), tc.size,
                                                 C.byref(full), _ptr(tr), _ptr(te)), "split_aupr_dev")
        return full.value, tr, te

    def split_combo_eval(self, mi, M1, M2, M3, labels, coeffs, iterations, train_counts, stouffer="none",
                         region="lower", row_gene=None, col_tf=None):
        """eval_combos over the shuffled splits on host arrays: (results[iters, parts, 6], best[iters, parts, 2])."""
        mi = _f32(mi)
        rows, cols = mi.shape
        keep = [None if x is None else _f32(x) for x in (M1, M2, M3)]
        labels = np.ascontiguousarray(labels, dtype=np.int8)
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        tc = np.ascontiguousarray(train_counts, dtype=np.int64)
        rg = None if row_gene is None else np.ascontiguousarray(row_gene, dtype=np.int32)
        ct = None if col_tf is None else np.ascontiguousarray(col_tf, dtype=np.uint8)
        res = np.zeros((iterations, tc.size, 6))
        best = np.zeros((iterations, tc.size, 2), dtype=np.int64)
        self._check(self._L.mcpg_split_combo_eval(
            self._h, _ptr(mi), cols, _ptr(keep[0]), cols, _ptr(keep[1]), cols, _ptr(keep[2]), cols, rows, cols,
            _ptr(labels), cols, TRUTH_REGIONS[region], _ptr(rg), _ptr(ct), cs.ctypes.data, cs.shape[0],
            STOUFFER_MODES[stouffer], iterations, _ptr(tc), tc.size, _ptr(res), _ptr(best)), "split_combo_eval")
        return res, best

    def split_combo_eval_dev(self, mi, M1, M2, M3, labels, coeffs, iterations, train_counts, stouffer="none",
                             region="lower", row_gene=None, col_tf=None):
        """As split_combo_eval for CUDA tensors."""
        rows, cols = mi.shape
        ld = lambda t: self._ld(t) if t is not None else cols
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        tc = np.ascontiguousarray(train_counts, dtype=np.int64)
        res = np.zeros((iterations, tc.size, 6))
        best = np.zeros((iterations, tc.size, 2), dtype=np.int64)
        self._check(self._L.mcpg_split_combo_eval_dev(
            self._h, self._dp(mi), self._ld(mi), self._dp(M1), ld(M1), self._dp(M2), ld(M2), self._dp(M3), ld(M3),
            rows, cols, self._dp(labels), self._ld(labels), TRUTH_REGIONS[region], self._dp(row_gene),
            self._dp(col_tf), cs.ctypes.data, cs.shape[0], STOUFFER_MODES[stouffer], iterations, _ptr(tc), tc.size,
            _ptr(res), _ptr(best)), "split_combo_eval_dev")
        return res, best

    def stouffer_tf_stats_dev(self, A):
        """The statistics of stouffer_tf_dev: (row_mean, row_sd, col_mean, col_sd) float32 CUDA tensors."""
        import torch
        rows, cols = A.shape
        r = [torch.empty(rows, dtype=torch.float32, device=A.device) for _ in range(2)]
        c = [torch.empty(cols, dtype=torch.float32, device=A.device) for _ in range(2)]
        self._check(self._L.mcpg_stouffer_tf_stats_dev(self._h, self._dp(A), rows, cols, self._ld(A), self._dp(r[0]),
                                                        self._dp(r[1]), self._dp(c[0]), self._dp(c[1])),
                    "stouffer_tf_stats_dev")
        return r[0], r[1], c[0], c[1]

    def combo_stouffer_tf_eval(self, mi, M1, M2, M3, labels, coeffs, region="tf", row_gene=None, col_tf=None):
        """Host form of the TF Stouffer coefficient search: (aupr, auroc, best row)."""
        mi = _f32(mi)
        rows, cols = mi.shape
        keep = [None if x is None else _f32(x) for x in (M1, M2, M3)]
        labels = np.ascontiguousarray(labels, dtype=np.int8)
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        rg = None if row_gene is None else np.ascontiguousarray(row_gene, dtype=np.int32)
        ct = None if col_tf is None else np.ascontiguousarray(col_tf, dtype=np.uint8)
        a = np.empty(cs.shape[0], dtype=np.float64)
        b = np.empty(cs.shape[0], dtype=np.float64)
        best = C.c_int64(0)
        self._check(self._L.mcpg_combo_stouffer_tf_eval(
            self._h, _ptr(mi), cols, _ptr(keep[0]), cols, _ptr(keep[1]), cols, _ptr(keep[2]), cols, rows, cols,
            _ptr(labels), cols, TRUTH_REGIONS[region], _ptr(rg), _ptr(ct), cs.ctypes.data, cs.shape[0], _ptr(a),
            _ptr(b), C.byref(best)), "combo_stouffer_tf_eval")
        return a, b, best.value

    def combo_stouffer_tf_eval_dev(self, mi, M1, M2, M3, labels, coeffs, region="tf", row_gene=None, col_tf=None):
        """The TF Stouffer coefficient search on CUDA tensors: (aupr, auroc, best row)."""
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        rows, cols = mi.shape
        ld = lambda t: self._ld(t) if t is not None else cols
        a = np.empty(cs.shape[0], dtype=np.float64)
        b = np.empty(cs.shape[0], dtype=np.float64)
        best = C.c_int64(0)
        self._check(self._L.mcpg_combo_stouffer_tf_eval_dev(
            self._h, self._dp(mi), self._ld(mi), self._dp(M1), ld(M1), self._dp(M2), ld(M2), self._dp(M3), ld(M3),
            rows, cols, self._dp(labels), self._ld(labels), TRUTH_REGIONS[region], self._dp(row_gene),
            self._dp(col_tf), cs.ctypes.data, cs.shape[0], _ptr(a), _ptr(b), C.byref(best)),
            "combo_stouffer_tf_eval_dev")
        return a, b, best.value

    def row_stats_dev(self, A, mean, sd, stats="exclude_diagonal"):
        rows, cols = A.shape
        self._check(self._L.mcpg_row_stats_dev(self._h, self._dp(A), rows, cols, self._ld(A), ROW_STATS[stats],
                                                self._dp(mean), self._dp(sd)), "row_stats_dev")

    def combo_stouffer_eval_dev(self, mi, M1, M2, M3, labels, coeffs, region="lower", row_gene=None, col_tf=None,
                                stats="exclude_diagonal"):
        """The Stouffer half of the ensemble coefficient search: (aupr, auroc, best row)."""
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        n = mi.shape[0]
        ld = lambda t: self._ld(t) if t is not None else n
        a = np.empty(cs.shape[0], dtype=np.float64)
        b = np.empty(cs.shape[0], dtype=np.float64)
        best = C.c_int64(0)
        self._check(self._L.mcpg_combo_stouffer_eval_dev(
            self._h, self._dp(mi), self._ld(mi), self._dp(M1), ld(M1), self._dp(M2), ld(M2), self._dp(M3), ld(M3), n,
            self._dp(labels), self._ld(labels), TRUTH_REGIONS[region], self._dp(row_gene), self._dp(col_tf),
            cs.ctypes.data, cs.shape[0], ROW_STATS[stats], _ptr(a), _ptr(b), C.byref(best)), "combo_stouffer_eval_dev")
        return a, b, best.value

    # ---- gold-standard evaluation ----
    def aupr_auroc(self, pos, neg):
        """AUPR and AUROC of positive / negative score vectors (aupr_kernel / auroc_kernel)."""
        pos, neg = _f32(pos).ravel(), _f32(neg).ravel()
        a, b = C.c_double(0), C.c_double(0)
        self._check(self._L.mcpg_aupr_auroc(self._h, _ptr(pos), pos.size, _ptr(neg), neg.size, C.byref(a),
                                             C.byref(b)), "aupr_auroc")
        return a.value, b.value

    def aupr_auroc_dev(self, pos, neg):
        """As aupr_auroc, for contiguous 1-D float32 CUDA tensors."""
        a, b = C.c_double(0), C.c_double(0)
        self._check(self._L.mcpg_aupr_auroc_dev(self._h, self._dp(pos), pos.numel(), self._dp(neg), neg.numel(),
                                                 C.byref(a), C.byref(b)), "aupr_auroc_dev")
        return a.value, b.value

    def eval_truth(self, values, labels, region="lower", row_gene=None, col_tf=None):
        """compute_aupr_auroc over a host score matrix and int8 label matrix.

        Returns (aupr, auroc, n_pos, n_neg)."""
        values = _f32(values)
        labels = np.ascontiguousarray(labels, dtype=np.int8)
        rows, cols = values.shape
        if labels.shape != values.shape:
            raise ValueError("labels must have the shape of values")
        rg = None if row_gene is None else np.ascontiguousarray(row_gene, dtype=np.int32)
        ct = None if col_tf is None else np.ascontiguousarray(col_tf, dtype=np.uint8)
        a, b, npos, nneg = C.c_double(0), C.c_double(0), C.c_int64(0), C.c_int64(0)
        self._check(self._L.mcpg_eval_truth(self._h, _ptr(values), rows, cols, cols, _ptr(labels), cols,
                                             TRUTH_REGIONS[region], _ptr(rg), _ptr(ct), C.byref(a), C.byref(b),
                                             C.byref(npos), C.byref(nneg)), "eval_truth")
        return a.value, b.value, npos.value, nneg.value

    def eval_truth_dev(self, values, labels, region="lower", row_gene=None, col_tf=None):
        """As eval_truth for CUDA tensors (values float32, labels int8, row_gene int32, col_tf uint8)."""
        rows, cols = values.shape
        a, b, npos, nneg = C.c_double(0), C.c_double(0), C.c_int64(0), C.c_int64(0)
        self._check(self._L.mcpg_eval_truth_dev(self._h, self._dp(values), rows, cols, self._ld(values),
                                                 self._dp(labels), self._ld(labels), TRUTH_REGIONS[region],
                                                 self._dp(row_gene), self._dp(col_tf), C.byref(a), C.byref(b),
                                                 C.byref(npos), C.byref(nneg)), "eval_truth_dev")
        return a.value, b.value, npos.value, nneg.value

    def select_truth_dev(self, values, labels, region="lower", row_gene=None, col_tf=None):
        """select_values2: (pos, neg) float32 CUDA tensors in row-major order."""
        import torch
        rows, cols = values.shape
        npos, nneg = C.c_int64(0), C.c_int64(0)
        args = (self._h, self._dp(values), rows, cols, self._ld(values), self._dp(labels), self._ld(labels),
                TRUTH_REGIONS[region], self._dp(row_gene), self._dp(col_tf))
        self._check(self._L.mcpg_select_truth_dev(*args, None, 0, None, 0, C.byref(npos), C.byref(nneg)),
                    "select_truth_dev")
        pos = torch.empty(npos.value, dtype=torch.float32, device=values.device)
        neg = torch.empty(nneg.value, dtype=torch.float32, device=values.device)
        self._check(self._L.mcpg_select_truth_dev(*args, self._dp(pos), pos.numel(), self._dp(neg), neg.numel(),
                                                   C.byref(npos), C.byref(nneg)), "select_truth_dev")
        return pos, neg

    def combo_eval_dev(self, mi, M1, M2, M3, labels, coeffs, region="lower", row_gene=None, col_tf=None):
        """Ensemble coefficient search: per coefficient row the AUPR / AUROC of compute_combo at the
        labelled entries.  Returns (aupr ndarray, auroc ndarray, best row)."""
        cs = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64).reshape(-1, 4))
        rows, cols = mi.shape
        ld = lambda t: self._ld(t) if t is not None else cols
        a = np.empty(cs.shape[0], dtype=np.float64)
        b = np.empty(cs.shape[0], dtype=np.float64)
        best = C.c_int64(0)
        self._check(self._L.mcpg_combo_eval_dev(self._h, self._dp(mi), self._ld(mi), self._dp(M1), ld(M1),
                                                 self._dp(M2), ld(M2), self._dp(M3), ld(M3), rows, cols,
                                                 self._dp(labels), self._ld(labels), TRUTH_REGIONS[region],
                                                 self._dp(row_gene), self._dp(col_tf), cs.ctypes.data, cs.shape[0],
                                                 _ptr(a), _ptr(b), C.byref(best)), "combo_eval_dev")
        return a, b, best.value

    def dpi_dev(self, A, out, tol=0.1, mask=None):
        n = A.shape[0]
        removed = C.c_int64(0)
        self._check(self._L.mcpg_dpi_dev(self._h, self._dp(A), n, self._ld(A), tol, self._dp(out), self._ld(out),
                                          self._dp(mask), C.byref(removed)), "dpi_dev")
        return removed.value

    def closure_dev(self, A, out, max_iter=64):
        n = A.shape[0]
        it = C.c_int(0)
        rc = self._L.mcpg_closure_dev(self._h, self._dp(A), n, self._ld(A), max_iter, self._dp(out), self._ld(out),
                                      C.byref(it))
        if rc == ERR_NOT_CONVERGED:
            return -1
        self._check(rc, "closure_dev")
        return it.value
