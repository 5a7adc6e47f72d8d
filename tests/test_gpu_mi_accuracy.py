"""MI accuracy report against the FP64 oracle (the reference's templates with
T = double): max-abs error in bits and nats, and top-1% edge-rank agreement
(Jaccard of the top-1% edge sets, Spearman of the two score lists over their
union), for every tensor-core form and the FP32 CUDA-core path.

* 1,000 genes x 1,000 samples, the whole matrix: the top 1% of the 499,500
  unordered pairs;
* 20,000 genes x 2,000 samples (the bench workload), 16 sampled rows
  (10,000..10,015 against all genes): the top 1% of each row, averaged.

The forms that meet the 1e-4-nats bound must also keep the top-1% edges
(Jaccard >= 0.98); the single-rounding forms are reported.  With
MCPG_ACCURACY_OUT set, the figures are written there as JSON.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMS = ["fp32", "bf16x3", "bf16f8", "fp16x3", "fp16", "bf16"]
BOUNDED = {"fp32", "bf16x3", "bf16f8", "fp16x3"}
NATS = np.log(2.0)
_report = {}


def _agreement(ref, got):
    """Jaccard of the top-k sets (k = 1% of the entries) and Spearman over their union."""
    stats = pytest.importorskip("scipy.stats")
    k = max(1, ref.size // 100)
    a = np.argpartition(-ref, k - 1)[:k]
    b = np.argpartition(-got, k - 1)[:k]
    sa, sb = set(a.tolist()), set(b.tolist())
    union = np.array(sorted(sa | sb))
    jac = len(sa & sb) / len(sa | sb)
    rho = float(stats.spearmanr(ref[union], got[union])[0])
    return jac, rho


def _record(case, form, err_bits, jac, rho):
    _report.setdefault(case, {})[form] = {"max_abs_bits": err_bits, "max_abs_nats": err_bits * NATS,
                                          "top1_jaccard": jac, "top1_spearman": rho}
    out = os.environ.get("MCPG_ACCURACY_OUT")
    if out:
        with open(out, "w") as f:
            json.dump(_report, f, indent=1)


def _check(form, err_bits, jac):
    if form in BOUNDED:
        assert err_bits * NATS <= 1e-4, (form, err_bits)
        assert jac >= 0.98, (form, jac)


@pytest.fixture(scope="module")
def full_1000(port, built_lib):
    X = built_lib.synth_grn(1000, 1000, seed=20260001)
    return X, port.bspline_mi(X.astype(np.float64))


@pytest.mark.parametrize("form", FORMS)
def test_accuracy_full_matrix_1000(gpu, full_1000, form):
    X, ref = full_1000
    got = gpu.bspline_mi(X, 10, 3, form).astype(np.float64)
    iu = np.triu_indices(X.shape[0], 1)
    err = float(np.abs(got[iu] - ref[iu]).max())
    jac, rho = _agreement(ref[iu], got[iu])
    _record("1000x1000 (all pairs)", form, err, jac, rho)
    _check(form, err, jac)


@pytest.fixture(scope="module")
def rows_20000(port, built_lib):
    n, m, r0, r1 = 20000, 2000, 10000, 10016
    X = built_lib.synth_grn(n, m, seed=20260001)
    W = port.bspline_weights(X.astype(np.float64))
    return X, port.bspline_mi_rows(W, m, r0, r1), (r0, r1)


@pytest.mark.parametrize("form", FORMS)
def test_accuracy_rows_20000(gpu, rows_20000, form):
    import torch
    X, ref, (r0, r1) = rows_20000
    n = X.shape[0]
    MI = torch.empty((n, n), device="cuda")
    gpu.bspline_mi_dev(torch.from_numpy(X).cuda(), MI, 10, 3, form)
    gpu.synchronize()
    got = MI[r0:r1].cpu().numpy().astype(np.float64)
    del MI
    errs, jacs, rhos = [], [], []
    for r in range(r1 - r0):
        keep = np.arange(n) != r0 + r
        errs.append(np.abs(got[r, keep] - ref[r, keep]).max())
        j, s = _agreement(ref[r, keep], got[r, keep])
        jacs.append(j)
        rhos.append(s)
    err, jac, rho = float(max(errs)), float(np.mean(jacs)), float(np.mean(rhos))
    _record("20000x2000 (rows 10000..10015, per-row top 1%)", form, err, jac, rho)
    _check(form, err, jac)
