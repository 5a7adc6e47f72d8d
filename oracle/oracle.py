"""ctypes access to the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two libraries:
  * ``port()``  -- oracle/_build/libmcporacle.so, the C restatement of the
    reference arithmetic (oracle/mcp_oracle_impl.h); builds anywhere.
  * ``ref()``   -- oracle/_ref/libmcpref.so, MCPNet's own kernels compiled from
    the reference headers (oracle/ref/ref_driver.cpp); exists only where the
    reference sources were present at build time.  ``None`` otherwise.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this module.  The product (mcpnet_gb300, libmcpgpu.so) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libmcporacle.so"
REF_LIB = HERE / "_ref" / "libmcpref.so"
REF_FAST_LIB = HERE / "_ref" / "libmcpref_fastmath.so"
# MCPNet source tree for the reference build; unset = no reference build (the restatement still builds)
REF_ROOT = Path(os.environ["MCPNET_REF_ROOT"]) if os.environ.get("MCPNET_REF_ROOT") else None

_i64, _vp = C.c_int64, C.c_void_p


def build(with_ref: bool | None = None) -> None:
    """make the oracle (and the reference build when the reference tree exists)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if with_ref is None:
        with_ref = REF_ROOT is not None and (REF_ROOT / "include" / "mcp").is_dir()
    if with_ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", "ref-fast", f"REF_ROOT={REF_ROOT}"], check=True)


def _bind(L, sfx: str, prefix: str):
    sig = {
        "bspline_weights": (None, [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp]),
        "bspline_mi": (None, [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64]),
        "bspline_mi_from_weights": (None, [_vp, _i64, _i64, C.c_int, _vp, _i64]),
        "bspline_mi_rows": (None, [_vp, _i64, _i64, C.c_int, _i64, _i64, _vp, _i64]),
        "maxmin": (None, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64]),
        "ratio": (None, [_vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64]),
        "max_transpose": (None, [_vp, _i64, _i64, _vp, _i64]),
        "dpi": (C.c_int64, [_vp, _i64, _i64, C.c_double, _vp, _i64, _vp]),
        "closure": (C.c_int, [_vp, _i64, _i64, _vp, _i64, C.c_int]),
        "dpi_rows": (C.c_int64, [_vp, _i64, _i64, C.c_double, _vp, _i64, _vp, _i64, _vp]),
        "widest_rows": (None, [_vp, _i64, _i64, _vp, _i64, _vp, _i64]),
        "maxmin_masked": (None, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, f"{prefix}{name}_{sfx}", None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    for name, res, args in (
        ("mi_bwd", None, [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp, _i64]),
        ("maxmin_bwd", None, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64,
                              _vp]),
        ("ratio_bwd", None, [_vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64]),
    ):
        f = getattr(L, f"{prefix}{name}_{sfx}", None)
        if f is not None:
            f.restype = res
            f.argtypes = args
    f = getattr(L, f"{prefix}dpi_tf_{sfx}", None)
    if f is not None:
        f.restype = C.c_int64
        f.argtypes = [_vp, _i64, _i64, C.c_float if sfx == "f32" else C.c_double, _vp, _vp, _i64, _vp]
    f = getattr(L, f"{prefix}dpi_tf_rows_{sfx}", None)
    if f is not None:
        f.restype = C.c_int64
        f.argtypes = [_vp, _i64, _i64, C.c_float if sfx == "f32" else C.c_double, _vp, _vp, _i64, _vp, _i64, _vp]


class _TfCompositions:
    """The reference's TF-restricted helpers restated on top of maxmin /
    maxmin_masked / ratio: compute_mcp{2,3,4}_tfs
    (apps/pipeline/mcpnet_helper.hpp:209-243, 281-333, 367-434)."""

    @staticmethod
    def tf_rows(A, tfs):
        return np.ascontiguousarray(A[np.asarray(tfs) > 0])

    def mcp_tf(self, A, tfs, path_len, transition):
        A = np.ascontiguousarray(A, dtype=np.float32)
        tfs = np.ascontiguousarray(tfs, dtype=np.float32)
        tg = self.tf_rows(A, tfs)
        mm = lambda X, Y, masked: self.maxmin_masked(X, Y, tfs) if masked else self.maxmin(X, Y)
        if path_len == 2:      # compute_maxmin1_tfs
            assert transition in (0, 1)
            M = mm(tg, A, transition == 1)
        elif path_len == 3:    # compute_maxmin2_tfs
            assert transition in (0, 1, 2)
            M1 = mm(A, A, transition == 2)
            M = mm(tg, M1, transition in (1, 2))
        else:                  # compute_maxmin3_tfs
            assert transition in (0, 1, 2, 3)
            M1 = mm(A, A, transition == 3)
            M2 = mm(tg, A, transition != 0)
            M = mm(M2, M1, transition in (2, 3))
        return M, self.ratio(tg, M)

    def maxmins_tf(self, A, tfs):
        """compute_maxmins_tfs (apps/pipeline/mcpnet_helper.hpp:470-505): (T, M1, M2, M3)."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        tfs = np.ascontiguousarray(tfs, dtype=np.float32)
        tg = self.tf_rows(A, tfs)
        M1 = self.maxmin_masked(tg, A, tfs)             # ttg
        M2 = self.maxmin_masked(M1, A, tfs)             # tttg
        M3 = self.maxmin_masked(M1, self.maxmin_masked(A, A, tfs), tfs)  # ttttg
        return tg, M1, M2, M3


class _EvalCompositions:
    """compute_aupr_auroc and the ensemble coefficient search composed from
    the selection, combo and curve routines of the concrete oracle."""

    REGIONS = {"lower": 0, "all": 1, "tf": 2}

    def eval_truth(self, values, labels, region="lower", row_gene=None, col_tf=None):
        """compute_aupr_auroc (apps/pipeline/mcpnet_helper.hpp:1050-1071)."""
        pos, neg = self.select_truth(values, labels, region, row_gene, col_tf)
        a, b = self.aupr_auroc(pos, neg)
        return a, b, pos.size, neg.size

    def combo_eval(self, mi, M1, M2, M3, labels, coeffs, region="lower", row_gene=None, col_tf=None):
        """The coefficient loop of apps/pipeline/mcpnet.cpp:575-616."""
        cs = np.asarray(coeffs, dtype=np.float64).reshape(-1, 4)
        pr = np.full(cs.shape[0], np.nan)
        roc = np.full(cs.shape[0], np.nan)
        best, top = 0, 0.0
        for i, c in enumerate(cs):
            if c[0] == 1 and c[1] == 0 and c[2] == 0 and c[3] == 0:
                continue
            R = port().combo(mi, M1, M2, M3, c)
            pr[i], roc[i], _, _ = self.eval_truth(R, labels, region, row_gene, col_tf)
            if pr[i] > top:
                top, best = pr[i], i
        return pr, roc, best

    @staticmethod
    def mask_entries(values, labels, region="lower", row_gene=None, col_tf=None):
        """The labelled entries (label 0 or 1) of the region in row-major order -- the reference's
        mask order (select_lower_triangle; select_from_list, whose mask is sorted by row and column,
        apps/pipeline/mcpnet_helper.hpp:818-826; select_tfs_from_mat) -- as (scores, labels)."""
        V = np.asarray(values)
        L = np.asarray(labels)
        rows, cols = L.shape
        i = np.arange(rows)[:, None]
        j = np.arange(cols)[None, :]
        keep = (L == 0) | (L == 1)
        if region == "lower":
            keep &= j < i
        elif region == "tf":
            g = np.asarray(row_gene, dtype=np.int64)[:, None]
            keep &= (j != g) & ~((g > j) & (np.asarray(col_tf)[None, :] != 0))
        idx = np.flatnonzero(keep)
        return np.ascontiguousarray(V.reshape(rows, -1)[:, :cols].ravel()[idx]), L.ravel()[idx]

    def _aupr_of(self, v, l):
        return self.aupr_auroc(v[l == 1], v[l == 0])[0]

    def split_aupr(self, values, labels, iterations, train_counts, region="lower", row_gene=None, col_tf=None):
        """eval_aupr_mcp (apps/pipeline/eval_mcpnet.cpp:227-301): (full, train[iters, parts], test[iters, parts])."""
        v, l = self.mask_entries(values, labels, region, row_gene, col_tf)
        full = self._aupr_of(v, l)
        tr = np.zeros((iterations, len(train_counts)))
        te = np.zeros_like(tr)
        for i in range(1, iterations + 1):
            perm = port().shuffle_perm(v.size, i)
            for jx, k in enumerate(train_counts):
                a, b = perm[:k], perm[k:]
                tr[i - 1, jx] = self._aupr_of(v[a], l[a])
                te[i - 1, jx] = self._aupr_of(v[b], l[b])
        return full, tr, te

    def split_combo_eval(self, mi, M1, M2, M3, labels, coeffs, iterations, train_counts, stouffer_mats=None,
                         region="lower", row_gene=None, col_tf=None):
        """eval_combos over the shuffled splits (apps/pipeline/eval_mcpnet.cpp:319-462, 814-893):
        results[iters, parts, 6] (train, test, Stouffer train, Stouffer test, full, Stouffer full) and
        best[iters, parts, 2].  stouffer_mats: the Stouffer transform of every row's combo matrix, or None."""
        cs = np.asarray(coeffs, dtype=np.float64).reshape(-1, 4)
        P = port()
        _, lab = self.mask_entries(mi, labels, region, row_gene, col_tf)
        ent = [self.mask_entries(P.combo(mi, M1, M2, M3, c), labels, region, row_gene, col_tf)[0] for c in cs]
        st = None if stouffer_mats is None else \
            [self.mask_entries(S, labels, region, row_gene, col_tf)[0] for S in stouffer_mats]
        full_p = [self._aupr_of(e, lab) for e in ent]
        full_s = [self._aupr_of(e, lab) for e in st] if st is not None else None
        skip = [c[0] == 1 and c[1] == 0 and c[2] == 0 and c[3] == 0 for c in cs]
        res = np.zeros((iterations, len(train_counts), 6))
        best = np.zeros((iterations, len(train_counts), 2), dtype=np.int64)
        for i in range(1, iterations + 1):
            perm = P.shuffle_perm(lab.size, i)
            for jx, k in enumerate(train_counts):
                tr, te = perm[:k], perm[k:]
                mp = ms = 0.0
                co = sco = 0
                for c in range(len(cs)):
                    if skip[c]:
                        continue
                    a = self._aupr_of(ent[c][tr], lab[tr])
                    if a > mp:
                        mp, co = a, c
                    if st is not None:
                        a = self._aupr_of(st[c][tr], lab[tr])
                        if a > ms:
                            ms, sco = a, c
                r = res[i - 1, jx]
                r[0], r[1], r[4] = mp, self._aupr_of(ent[co][te], lab[te]), full_p[co]
                if st is not None:
                    r[2], r[3], r[5] = ms, self._aupr_of(st[sco][te], lab[te]), full_s[sco]
                best[i - 1, jx] = (co, sco)
        return res, best

    def combo_stouffer_tf_eval(self, mi, M1, M2, M3, labels, coeffs, region="tf", row_gene=None, col_tf=None):
        """The TF Stouffer half of the loop (apps/pipeline/mcpnet.cpp:622-661 with --tf-input)."""
        cs = np.asarray(coeffs, dtype=np.float64).reshape(-1, 4)
        pr = np.full(cs.shape[0], np.nan)
        roc = np.full(cs.shape[0], np.nan)
        best, top = 0, 0.0
        for i, c in enumerate(cs):
            if c[0] == 1 and c[1] == 0 and c[2] == 0 and c[3] == 0:
                continue
            R = port().stouffer_tf(port().combo(mi, M1, M2, M3, c))
            pr[i], roc[i], _, _ = self.eval_truth(R, labels, region, row_gene, col_tf)
            if pr[i] > top:
                top, best = pr[i], i
        return pr, roc, best


class _Port(_TfCompositions, _EvalCompositions):
    """The C restatement (float and double)."""

    def __init__(self, path: Path):
        self.L = C.CDLL(str(path))
        for sfx in ("f32", "f64"):
            _bind(self.L, sfx, "orc_")
        self.L.orc_num_threads.restype = C.c_int
        for name in ("orc_aupr", "orc_auroc"):
            f = getattr(self.L, name)
            f.restype = C.c_double
            f.argtypes = [_vp, _i64, _vp, _i64]
        self.L.orc_select_truth.argtypes = [_vp, _i64, _i64, _i64, _vp, _i64, C.c_int, _vp, _vp, _vp, _vp, _vp,
                                            _vp]
        self.L.orc_ranks_desc.argtypes = [_vp, _i64, _i64, _i64, _vp]
        self.L.orc_row_stats.argtypes = [_vp, _i64, _i64, _i64, C.c_int, _vp, _vp]
        self.L.orc_transform.argtypes = [_vp, _i64, _i64, _vp, _vp, C.c_int, _vp, _i64]
        self.L.orc_shuffle_u32.argtypes = [_vp, _i64, C.c_uint32]
        self.L.orc_shuffle_tuples.argtypes = [_i64, C.c_uint32, _vp]
        self.L.orc_row_stats_pop.argtypes = [_vp, _i64, _i64, _i64, _vp, _vp]
        self.L.orc_col_stats.argtypes = [_vp, _i64, _i64, _i64, _vp, _vp]
        self.L.orc_stouffer_tf.argtypes = [_vp, _i64, _i64, _i64, _vp, _vp, _vp, _vp, C.c_int, _vp, _i64, _vp, _vp]
        self.L.orc_ap_mi.argtypes = [_vp, _i64, _i64, _vp, _i64]

    @staticmethod
    def _dt(a):
        return "f32" if a.dtype == np.float32 else "f64"

    def threads(self) -> int:
        return int(self.L.orc_num_threads())

    def bspline_weights(self, X, bins=10, order=3):
        X = np.ascontiguousarray(X)
        n, m = X.shape
        W = np.empty((n, bins * m + 1), dtype=X.dtype)
        getattr(self.L, f"orc_bspline_weights_{self._dt(X)}")(X.ctypes.data, n, m, m, bins, order, W.ctypes.data)
        return W

    def bspline_mi(self, X, bins=10, order=3):
        X = np.ascontiguousarray(X)
        n, m = X.shape
        MI = np.empty((n, n), dtype=X.dtype)
        getattr(self.L, f"orc_bspline_mi_{self._dt(X)}")(X.ctypes.data, n, m, m, bins, order, MI.ctypes.data, n)
        return MI

    def bspline_mi_from_weights(self, W, m, bins=10):
        W = np.ascontiguousarray(W)
        n = W.shape[0]
        MI = np.empty((n, n), dtype=W.dtype)
        getattr(self.L, f"orc_bspline_mi_from_weights_{self._dt(W)}")(W.ctypes.data, n, m, bins, MI.ctypes.data, n)
        return MI

    def bspline_mi_rows(self, W, m, r0, r1, bins=10):
        W = np.ascontiguousarray(W)
        n = W.shape[0]
        out = np.empty((r1 - r0, n), dtype=W.dtype)
        getattr(self.L, f"orc_bspline_mi_rows_{self._dt(W)}")(W.ctypes.data, n, m, bins, r0, r1, out.ctypes.data, n)
        return out

    def maxmin(self, A, B=None):
        A = np.ascontiguousarray(A)
        B = A if B is None else np.ascontiguousarray(B)
        rows, k = A.shape
        cols = B.shape[0]
        Cm = np.empty((rows, cols), dtype=A.dtype)
        getattr(self.L, f"orc_maxmin_{self._dt(A)}")(A.ctypes.data, k, B.ctypes.data, k, rows, cols, k,
                                                     Cm.ctypes.data, cols)
        return Cm

    def ratio(self, A, M):
        A, M = np.ascontiguousarray(A), np.ascontiguousarray(M)
        rows, cols = A.shape
        R = np.empty_like(A)
        getattr(self.L, f"orc_ratio_{self._dt(A)}")(A.ctypes.data, cols, M.ctypes.data, cols, rows, cols,
                                                    R.ctypes.data, cols)
        return R

    def max_transpose(self, M):
        M = np.ascontiguousarray(M)
        n = M.shape[0]
        out = np.empty_like(M)
        getattr(self.L, f"orc_max_transpose_{self._dt(M)}")(M.ctypes.data, n, n, out.ctypes.data, n)
        return out

    def combo(self, mi, M1, M2, M3, cs):
        mi = np.ascontiguousarray(mi)
        rows, cols = mi.shape
        cs = np.ascontiguousarray(cs, dtype=np.float64)
        ptr = lambda x: None if x is None else np.ascontiguousarray(x, dtype=mi.dtype).ctypes.data
        keep = [None if x is None else np.ascontiguousarray(x, dtype=mi.dtype) for x in (M1, M2, M3)]
        out = np.empty_like(mi)
        f = getattr(self.L, f"orc_combo_{self._dt(mi)}")
        f.argtypes = [_vp] * 4 + [_i64, _i64, _i64, _vp, _vp, _i64]
        f(mi.ctypes.data, *(None if k is None else k.ctypes.data for k in keep), rows, cols, cols, cs.ctypes.data,
          out.ctypes.data, cols)
        return out

    def dpi(self, A, tol=0.1):
        """tol is the float tolerance of `dpi --single`; the multiplier uses (double)tol."""
        A = np.ascontiguousarray(A)
        n = A.shape[0]
        out = np.empty_like(A)
        mask = np.empty((n, n), dtype=np.uint8)
        t = float(np.float32(tol)) if A.dtype == np.float32 else float(tol)
        removed = getattr(self.L, f"orc_dpi_{self._dt(A)}")(A.ctypes.data, n, n, t, out.ctypes.data, n,
                                                            mask.ctypes.data)
        return out, mask, int(removed)

    def dpi_rows(self, A, rows, tol=0.1):
        """Rows `rows` of dpi(A, tol): (out rows, mask rows, removed count of those rows)."""
        A = np.ascontiguousarray(A)
        n = A.shape[0]
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        out = np.empty((rows.size, n), dtype=A.dtype)
        mask = np.empty((rows.size, n), dtype=np.uint8)
        t = float(np.float32(tol)) if A.dtype == np.float32 else float(tol)
        removed = getattr(self.L, f"orc_dpi_rows_{self._dt(A)}")(A.ctypes.data, n, n, t, rows.ctypes.data, rows.size,
                                                                 out.ctypes.data, n, mask.ctypes.data)
        return out, mask, int(removed)

    def widest_rows(self, A, rows):
        """Rows `rows` of the maximum-capacity closure of a symmetric A, by widest-path search."""
        A = np.ascontiguousarray(A)
        n = A.shape[0]
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        out = np.empty((rows.size, n), dtype=A.dtype)
        getattr(self.L, f"orc_widest_rows_{self._dt(A)}")(A.ctypes.data, n, n, rows.ctypes.data, rows.size,
                                                          out.ctypes.data, n)
        return out

    def maxmin_masked(self, A, B, mask):
        A = np.ascontiguousarray(A)
        B = A if B is None else np.ascontiguousarray(B)
        mask = np.ascontiguousarray(mask, dtype=A.dtype)
        rows, k = A.shape
        cols = B.shape[0]
        Cm = np.empty((rows, cols), dtype=A.dtype)
        getattr(self.L, f"orc_maxmin_masked_{self._dt(A)}")(A.ctypes.data, k, B.ctypes.data, k, rows, cols, k,
                                                            mask.ctypes.data, Cm.ctypes.data, cols)
        return Cm

    def dpi_tf(self, A, tfs, tol=0.1):
        A = np.ascontiguousarray(A)
        tfs = np.ascontiguousarray(tfs, dtype=A.dtype)
        n = A.shape[0]
        out = np.empty_like(A)
        mask = np.empty((n, n), dtype=np.uint8)
        removed = getattr(self.L, f"orc_dpi_tf_{self._dt(A)}")(A.ctypes.data, n, n, tol, tfs.ctypes.data,
                                                               out.ctypes.data, n, mask.ctypes.data)
        return out, mask, int(removed)

    def dpi_tf_rows(self, A, tfs, rows, tol=0.1):
        """Rows `rows` of dpi_tf(A, tfs, tol): (out rows, mask rows, removed count of those rows)."""
        A = np.ascontiguousarray(A)
        tfs = np.ascontiguousarray(tfs, dtype=A.dtype)
        n = A.shape[0]
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        out = np.empty((rows.size, n), dtype=A.dtype)
        mask = np.empty((rows.size, n), dtype=np.uint8)
        removed = getattr(self.L, f"orc_dpi_tf_rows_{self._dt(A)}")(A.ctypes.data, n, n, tol, tfs.ctypes.data,
                                                                    rows.ctypes.data, rows.size, out.ctypes.data, n,
                                                                    mask.ctypes.data)
        return out, mask, int(removed)

    # -- adjoints (this build's definitions; see mcp_oracle_impl.h) --
    def mi_bwd(self, X, G, bins=10, order=3):
        X = np.ascontiguousarray(X)
        G = np.ascontiguousarray(G, dtype=X.dtype)
        n, m = X.shape
        dX = np.zeros_like(X)
        getattr(self.L, f"orc_mi_bwd_{self._dt(X)}")(X.ctypes.data, n, m, m, bins, order, G.ctypes.data, n,
                                                     dX.ctypes.data, m)
        return dX

    def maxmin_bwd(self, A, B, Cm, dC, dA, dB, want_witness=True):
        """Accumulates into dA, dB (may be the same array); returns the witnesses
        (None with want_witness=False, which scans only the entries with a gradient)."""
        A, B, Cm, dC = (np.ascontiguousarray(x) for x in (A, B, Cm, dC))
        rows, k = A.shape
        cols = B.shape[0]
        K = np.empty((rows, cols), dtype=np.int32) if want_witness else None
        getattr(self.L, f"orc_maxmin_bwd_{self._dt(A)}")(A.ctypes.data, k, B.ctypes.data, k, rows, cols, k,
                                                         Cm.ctypes.data, cols, dC.ctypes.data, cols, dA.ctypes.data,
                                                         dA.shape[1], dB.ctypes.data, dB.shape[1],
                                                         None if K is None else K.ctypes.data)
        return K

    def ratio_bwd(self, A, M, dR, dA, dM):
        A, M, dR = (np.ascontiguousarray(x) for x in (A, M, dR))
        rows, cols = A.shape
        getattr(self.L, f"orc_ratio_bwd_{self._dt(A)}")(A.ctypes.data, cols, M.ctypes.data, cols, rows, cols,
                                                        dR.ctypes.data, cols, dA.ctypes.data, cols, dM.ctypes.data,
                                                        cols)

    def aupr_auroc(self, pos, neg):
        """aupr_kernel / auroc_kernel::operator()(pos, count, neg, count), sums in double."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).ravel()
        neg = np.ascontiguousarray(neg, dtype=np.float64).ravel()
        return (float(self.L.orc_aupr(pos.ctypes.data, pos.size, neg.ctypes.data, neg.size)),
                float(self.L.orc_auroc(pos.ctypes.data, pos.size, neg.ctypes.data, neg.size)))

    STATS = {"all": 0, "exclude_diagonal": 1}

    def row_stats(self, A, mode="exclude_diagonal"):
        """FP64 row mean / unbiased sd rounded to float (stands in for GaussianParamsExclude1)."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        rows, cols = A.shape
        mean = np.empty(rows, np.float32)
        sd = np.empty(rows, np.float32)
        self.L.orc_row_stats(A.ctypes.data, rows, cols, cols, self.STATS[mode], mean.ctypes.data, sd.ctypes.data)
        return mean, sd

    def transform_with_stats(self, A, mean, sd, clr=False):
        """stouffer_vector_kernel / clr_vector_kernel restated, given the row statistics."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        n = A.shape[0]
        mean = np.ascontiguousarray(mean, dtype=np.float32)
        sd = np.ascontiguousarray(sd, dtype=np.float32)
        out = np.empty_like(A)
        self.L.orc_transform(A.ctypes.data, n, n, mean.ctypes.data, sd.ctypes.data, int(clr), out.ctypes.data, n)
        return out

    def transform(self, A, clr=False, mode="exclude_diagonal"):
        mean, sd = self.row_stats(A, mode)
        return self.transform_with_stats(A, mean, sd, clr)

    def shuffle_perm(self, n, seed):
        """shuffle_truth's order of n mask entries for `seed` (std::shuffle, std::mt19937) as positions."""
        a = np.empty(n, dtype=np.uint32)
        self.L.orc_shuffle_u32(a.ctypes.data, n, seed)
        return a.astype(np.int64)

    def shuffle_tuples_order(self, n, seed):
        """The same shuffle applied to the reference's (size_t, size_t, int) mask tuples."""
        out = np.empty(n, dtype=np.int64)
        self.L.orc_shuffle_tuples(n, seed, out.ctypes.data)
        return out

    def tf_stats(self, A):
        """Population row and column statistics of a t x n matrix, FP64 rounded to float (stand in for
        StandardScore<T,T,false>): (row_mean, row_sd, col_mean, col_sd)."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        rows, cols = A.shape
        rm, rs = np.empty(rows, np.float32), np.empty(rows, np.float32)
        cm, cs = np.empty(cols, np.float32), np.empty(cols, np.float32)
        self.L.orc_row_stats_pop(A.ctypes.data, rows, cols, cols, rm.ctypes.data, rs.ctypes.data)
        self.L.orc_col_stats(A.ctypes.data, rows, cols, cols, cm.ctypes.data, cs.ctypes.data)
        return rm, rs, cm, cs

    def stouffer_tf_with_stats(self, A, rmean, rsd, cmean, csd, want_z=False, clr=False):
        """compute_stouffer_tf given the statistics (clr: the transform app's zscored_clr_kernel); with
        want_z also the row / column z-score matrices."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        rows, cols = A.shape
        f = lambda v: np.ascontiguousarray(v, dtype=np.float32)
        rmean, rsd, cmean, csd = f(rmean), f(rsd), f(cmean), f(csd)
        out = np.empty_like(A)
        zr = np.empty_like(A) if want_z else None
        zc = np.empty_like(A) if want_z else None
        self.L.orc_stouffer_tf(A.ctypes.data, rows, cols, cols, rmean.ctypes.data, rsd.ctypes.data, cmean.ctypes.data,
                               csd.ctypes.data, int(clr), out.ctypes.data, cols, None if zr is None else zr.ctypes.data,
                               None if zc is None else zc.ctypes.data)
        return (out, zr, zc) if want_z else out

    def stouffer_tf(self, A, clr=False):
        return self.stouffer_tf_with_stats(A, *self.tf_stats(A), clr=clr)

    def ap_ranks(self, X):
        """Descending ranks per gene, ties sharing the lowest rank (int64, n x m)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        n, m = X.shape
        R = np.empty((n, m), dtype=np.int64)
        self.L.orc_ranks_desc(X.ctypes.data, n, m, m, R.ctypes.data)
        return R

    def ap_mi(self, R):
        """AP MI (AdaptivePartitionRankMIKernel2, symmetric) from integer ranks, float32."""
        R = np.ascontiguousarray(R, dtype=np.int64)
        n, m = R.shape
        out = np.empty((n, n), dtype=np.float32)
        self.L.orc_ap_mi(R.ctypes.data, n, m, out.ctypes.data, n)
        return out

    def select_truth(self, values, labels, region="lower", row_gene=None, col_tf=None):
        """select_lower_triangle / select_tfs_from_mat + select_values2: (pos, neg) float32, row-major."""
        V = np.ascontiguousarray(values, dtype=np.float32)
        Lb = np.ascontiguousarray(labels, dtype=np.int8)
        rows, cols = V.shape
        rg = None if row_gene is None else np.ascontiguousarray(row_gene, dtype=np.int32)
        ct = None if col_tf is None else np.ascontiguousarray(col_tf, dtype=np.uint8)
        pos = np.empty(rows * cols + 1, dtype=np.float32)
        neg = np.empty(rows * cols + 1, dtype=np.float32)
        npos, nneg = C.c_int64(0), C.c_int64(0)
        ptr = lambda a: None if a is None else a.ctypes.data
        self.L.orc_select_truth(V.ctypes.data, rows, cols, cols, Lb.ctypes.data, cols, self.REGIONS[region], ptr(rg),
                                ptr(ct), pos.ctypes.data, C.byref(npos), neg.ctypes.data, C.byref(nneg))
        return pos[:npos.value].copy(), neg[:nneg.value].copy()

    def closure(self, A, max_iter=64):
        A = np.ascontiguousarray(A)
        n = A.shape[0]
        out = np.empty_like(A)
        it = getattr(self.L, f"orc_closure_{self._dt(A)}")(A.ctypes.data, n, n, out.ctypes.data, n, max_iter)
        return out, int(it)

    # -- the reference's composite helpers, restated on top of the kernels --
    def mcp(self, A, path_len, symmetrize=False):
        """compute_mcp2/3/4 (apps/pipeline/mcpnet_helper.hpp:199-365); symmetrize as apps/filter/mcp.cpp:463-476."""
        M1 = self.maxmin(A)
        if path_len == 2:
            M = M1
        elif path_len == 3:
            M = self.maxmin(A, M1)
            if symmetrize:
                M = self.max_transpose(M)
        elif path_len == 4:
            M = self.maxmin(M1)
        else:
            raise ValueError(path_len)
        return M, self.ratio(A, M)


class _Ref(_TfCompositions, _EvalCompositions):
    """MCPNet's own kernels driven over whole matrices (float, plus f64 MI)."""

    def __init__(self, path: Path):
        L = C.CDLL(str(path))
        L.ref_bspline_weights_f32.argtypes = [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp]
        L.ref_bspline_weights_f64.argtypes = [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp]
        L.ref_bspline_mi_f32.argtypes = [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp]
        L.ref_bspline_mi_f64.argtypes = [_vp, _i64, _i64, _i64, C.c_int, C.c_int, _vp, _i64, _vp]
        L.ref_maxmin_f32.argtypes = [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64]
        L.ref_maxmin_symm_f32.argtypes = [_vp, _i64, _i64, _vp, _i64]
        L.ref_ratio_f32.argtypes = [_vp, _i64, _vp, _i64, _i64, _i64, _vp, _i64]
        L.ref_max_transpose_f32.argtypes = [_vp, _i64, _i64, _vp, _i64]
        L.ref_dpi_f32.argtypes = [_vp, _i64, _i64, C.c_float, _vp, _i64, _vp]
        L.ref_dpi_f32.restype = C.c_int64
        L.ref_bspline_mi_rows_f32.argtypes = [_vp, _i64, _i64, C.c_int, _i64, _i64, _vp, _i64]
        L.ref_maxmin_masked_f32.argtypes = [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64]
        L.ref_dpi_tf_f32.argtypes = [_vp, _i64, _i64, C.c_float, _vp, _vp, _i64, _vp]
        L.ref_dpi_tf_f32.restype = C.c_int64
        L.ref_aupr_auroc_f32.argtypes = [_vp, _i64, _vp, _i64, _vp]
        L.ref_ap_mi_f32.argtypes = [_vp, _i64, _i64, _vp, _i64]
        L.ref_transform_f32.argtypes = [_vp, _i64, _i64, _vp, _vp, C.c_int, _vp, _i64]
        L.ref_zscored_stouffer_f32.argtypes = [_vp, _vp, _i64, _i64, _vp]
        L.ref_zscored_clr_f32.argtypes = [_vp, _vp, _i64, _i64, _vp]
        L.ref_aupr_auroc_f64.argtypes = [_vp, _i64, _vp, _i64, _vp]
        self.L = L

    def aupr_auroc(self, pos, neg, dtype=np.float32):
        """MCPNet's aupr_kernel / auroc_kernel with IT = dtype, OT = double."""
        pos = np.ascontiguousarray(pos, dtype=dtype).ravel()
        neg = np.ascontiguousarray(neg, dtype=dtype).ravel()
        out = np.zeros(2, dtype=np.float64)
        f = self.L.ref_aupr_auroc_f32 if dtype == np.float32 else self.L.ref_aupr_auroc_f64
        f(pos.ctypes.data, pos.size, neg.ctypes.data, neg.size, out.ctypes.data)
        return float(out[0]), float(out[1])

    def transform_with_stats(self, A, mean, sd, clr=False):
        """MCPNet's stouffer_vector_kernel / clr_vector_kernel with the given row statistics."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        n = A.shape[0]
        mean = np.ascontiguousarray(mean, dtype=np.float32)
        sd = np.ascontiguousarray(sd, dtype=np.float32)
        out = np.empty_like(A)
        self.L.ref_transform_f32(A.ctypes.data, n, n, mean.ctypes.data, sd.ctypes.data, int(clr), out.ctypes.data, n)
        return out

    def zscored_stouffer(self, zi, zj):
        """MCPNet's zscored_stouffer_kernel on row-aligned row / column z-score matrices."""
        zi = np.ascontiguousarray(zi, dtype=np.float32)
        zj = np.ascontiguousarray(zj, dtype=np.float32)
        rows, cols = zi.shape
        out = np.empty_like(zi)
        self.L.ref_zscored_stouffer_f32(zi.ctypes.data, zj.ctypes.data, rows, cols, out.ctypes.data)
        return out

    def zscored_clr(self, zi, zj):
        """MCPNet's zscored_clr_kernel on row-aligned row / column z-score matrices."""
        zi = np.ascontiguousarray(zi, dtype=np.float32)
        zj = np.ascontiguousarray(zj, dtype=np.float32)
        rows, cols = zi.shape
        out = np.empty_like(zi)
        self.L.ref_zscored_clr_f32(zi.ctypes.data, zj.ctypes.data, rows, cols, out.ctypes.data)
        return out

    def ap_mi(self, R):
        """MCPNet's IntegralCumulativeHistogramKernel + AdaptivePartitionRankMIKernel2 on given ranks."""
        R = np.ascontiguousarray(R, dtype=np.int64)
        n, m = R.shape
        out = np.empty((n, n), dtype=np.float32)
        self.L.ref_ap_mi_f32(R.ctypes.data, n, m, out.ctypes.data, n)
        return out

    def select_truth(self, values, labels, region="lower", row_gene=None, col_tf=None):
        """The selection loops are app code (not compiled here): the restatement stands in."""
        return port().select_truth(values, labels, region, row_gene, col_tf)

    def maxmin_masked(self, A, B, mask):
        A = np.ascontiguousarray(A, dtype=np.float32)
        B = A if B is None else np.ascontiguousarray(B, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.float32)
        rows, k = A.shape
        cols = B.shape[0]
        Cm = np.empty((rows, cols), dtype=np.float32)
        self.L.ref_maxmin_masked_f32(A.ctypes.data, k, B.ctypes.data, k, rows, cols, k, mask.ctypes.data,
                                     Cm.ctypes.data, cols)
        return Cm

    def dpi_tf(self, A, tfs, tol=0.1):
        A = np.ascontiguousarray(A, dtype=np.float32)
        tfs = np.ascontiguousarray(tfs, dtype=np.float32)
        n = A.shape[0]
        out = np.empty_like(A)
        mask = np.empty((n, n), dtype=np.uint8)
        removed = self.L.ref_dpi_tf_f32(A.ctypes.data, n, n, tol, tfs.ctypes.data, out.ctypes.data, n,
                                        mask.ctypes.data)
        return out, mask, int(removed)

    def bspline_mi_rows(self, W, m, r0, r1, bins=10):
        W = np.ascontiguousarray(W, dtype=np.float32)
        n = W.shape[0]
        out = np.empty((r1 - r0, n), dtype=np.float32)
        self.L.ref_bspline_mi_rows_f32(W.ctypes.data, n, m, bins, r0, r1, out.ctypes.data, n)
        return out

    def threads(self) -> int:
        return port().threads()

    def bspline_weights(self, X, bins=10, order=3):
        X = np.ascontiguousarray(X)
        n, m = X.shape
        W = np.empty((n, bins * m + 1), dtype=X.dtype)
        f = self.L.ref_bspline_weights_f32 if X.dtype == np.float32 else self.L.ref_bspline_weights_f64
        f(X.ctypes.data, n, m, m, bins, order, W.ctypes.data)
        return W

    def bspline_mi(self, X, bins=10, order=3):
        X = np.ascontiguousarray(X)
        n, m = X.shape
        MI = np.empty((n, n), dtype=X.dtype)
        f = self.L.ref_bspline_mi_f32 if X.dtype == np.float32 else self.L.ref_bspline_mi_f64
        f(X.ctypes.data, n, m, m, bins, order, MI.ctypes.data, n, None)
        return MI

    def maxmin(self, A, B=None):
        A = np.ascontiguousarray(A, dtype=np.float32)
        rows, k = A.shape
        if B is None:
            Cm = np.empty((rows, rows), dtype=np.float32)
            self.L.ref_maxmin_symm_f32(A.ctypes.data, k, rows, Cm.ctypes.data, rows)
            return Cm
        B = np.ascontiguousarray(B, dtype=np.float32)
        cols = B.shape[0]
        Cm = np.empty((rows, cols), dtype=np.float32)
        self.L.ref_maxmin_f32(A.ctypes.data, k, B.ctypes.data, k, rows, cols, k, Cm.ctypes.data, cols)
        return Cm

    def ratio(self, A, M):
        A, M = np.ascontiguousarray(A, dtype=np.float32), np.ascontiguousarray(M, dtype=np.float32)
        rows, cols = A.shape
        R = np.empty_like(A)
        self.L.ref_ratio_f32(A.ctypes.data, cols, M.ctypes.data, cols, rows, cols, R.ctypes.data, cols)
        return R

    def max_transpose(self, M):
        M = np.ascontiguousarray(M, dtype=np.float32)
        n = M.shape[0]
        out = np.empty_like(M)
        self.L.ref_max_transpose_f32(M.ctypes.data, n, n, out.ctypes.data, n)
        return out

    def dpi(self, A, tol=0.1):
        A = np.ascontiguousarray(A, dtype=np.float32)
        n = A.shape[0]
        out = np.empty_like(A)
        mask = np.empty((n, n), dtype=np.uint8)
        removed = self.L.ref_dpi_f32(A.ctypes.data, n, n, tol, out.ctypes.data, n, mask.ctypes.data)
        return out, mask, int(removed)

    def mcp(self, A, path_len, symmetrize=False):
        M1 = self.maxmin(A)
        if path_len == 2:
            M = M1
        elif path_len == 3:
            M = self.maxmin(A, M1)
            if symmetrize:
                M = self.max_transpose(M)
        else:
            M = self.maxmin(M1)
        return M, self.ratio(A, M)


_port = None
_ref = {}


def port() -> _Port:
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build(with_ref=False)
        _port = _Port(PORT_LIB)
    return _port


def ref(fast_math: bool = False):
    """MCPNet's own kernels, or None when they were not built here."""
    path = REF_FAST_LIB if fast_math else REF_LIB
    if path not in _ref:
        try:
            _ref[path] = _Ref(path) if path.exists() else None
        except OSError:  # built for another machine
            _ref[path] = None
    return _ref[path]
