"""The C++ host program (mcpgpu_cli), the reference-style drop-in for the
`mi` / `mcp` / `dpi` / `mcpnet` apps: file formats on CPU, the GPU methods
against the oracle on a GPU."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "mcpnet_gb300" / "_lib" / "mcpgpu_cli"


def write_exp(path, X, names=None):
    n, m = X.shape
    names = names or [f"g{i}" for i in range(n)]
    with open(path, "w") as f:
        f.write("Id\tAlias\t" + "\t".join(f"s{j}" for j in range(m)) + "\n")
        for i in range(n):
            f.write(f"{names[i]}\t---\t" + "\t".join(repr(float(v)) for v in X[i]) + "\n")


def read_exp(path):
    lines = Path(path).read_text().splitlines()
    return np.array([[float(v) for v in l.split("\t")[2:]] for l in lines[1:]], dtype=np.float32)


def read_bin(path):
    d = np.fromfile(path, dtype=np.int64, count=2)
    return np.fromfile(path, dtype=np.float32, offset=16).reshape(d)


def run(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=600)


def test_convert_round_trip(built_lib, tmp_path):
    X = built_lib.synth_grn(9, 13, seed=2)
    write_exp(tmp_path / "x.exp", X)
    r = run("convert", "-i", tmp_path / "x.exp", "-o", tmp_path / "x.bin")
    assert r.returncode == 0, r.stderr
    assert np.array_equal(read_bin(tmp_path / "x.bin"), X)
    r = run("convert", "-i", tmp_path / "x.bin", "-o", tmp_path / "y.exp")
    assert r.returncode == 0 and np.array_equal(read_exp(tmp_path / "y.exp"), X)


def test_text_io_round_trip_exact(built_lib, tmp_path):
    """EXP / CSV text written in parallel blocks (9 significant digits) reads back to the
    same float bits, through the program and through a double; CRLF lines, blank lines and
    a leading '+' parse; a row with the wrong number of values is reported."""
    rng = np.random.default_rng(3)
    X = rng.standard_normal((301, 257)).astype(np.float32) * np.float32(1e3)
    X[0, :6] = [0.0, -0.0, 1e-40, 3.4028235e38, -1.1754944e-38, np.float32(1) / 3]
    with open(tmp_path / "x.bin", "wb") as f:
        np.array(X.shape, dtype=np.int64).tofile(f)
        X.tofile(f)
    for ext in ("exp", "csv"):
        r = run("convert", "-i", tmp_path / "x.bin", "-o", tmp_path / f"y.{ext}")
        assert r.returncode == 0, r.stderr
        r = run("convert", "-i", tmp_path / f"y.{ext}", "-o", tmp_path / f"z_{ext}.bin")
        assert r.returncode == 0, r.stderr
        assert np.array_equal(read_bin(tmp_path / f"z_{ext}.bin").view(np.uint32), X.view(np.uint32)), ext
    assert np.array_equal(read_exp(tmp_path / "y.exp"), X)
    (tmp_path / "w.exp").write_text("Id\tAlias\ta\tb\r\n\r\ng0\t---\t+1.5\t2e-3\r\ng1\t---\t-0\t7\n")
    r = run("convert", "-i", tmp_path / "w.exp", "-o", tmp_path / "w.bin")
    assert r.returncode == 0, r.stderr
    assert np.array_equal(read_bin(tmp_path / "w.bin"), np.array([[1.5, 2e-3], [-0.0, 7]], np.float32))
    (tmp_path / "bad.exp").write_text("Id\tAlias\ta\tb\ng0\t---\t1\t2\ng1\t---\t3\n")
    r = run("convert", "-i", tmp_path / "bad.exp", "-o", tmp_path / "bad.bin")
    assert r.returncode != 0 and "row g1" in r.stderr and "wrong number of values" in r.stderr


def test_bad_usage_reports(built_lib, tmp_path):
    assert run("mi").returncode != 0
    r = run("frobnicate", "-i", tmp_path / "none.exp", "-o", tmp_path / "o.exp")
    assert r.returncode != 0 and "cannot open" in r.stderr
    # auc_pr_roc needs a score matrix and exactly one truth source (checked before any GPU work)
    r = run("auc_pr_roc", "-i", tmp_path / "s.exp")
    assert r.returncode != 0 and "exactly one of -g" in r.stderr
    r = run("auc_pr_roc", "-i", tmp_path / "s.exp", "-g", tmp_path / "t.txt", "-x", tmp_path / "t.exp")
    assert r.returncode != 0 and "exactly one of -g" in r.stderr
    r = run("auc_pr_roc", "-g", tmp_path / "t.txt")
    assert r.returncode != 0 and "needs -i" in r.stderr


@pytest.mark.gpu
def test_cli_pipeline_matches_oracle(built_lib, port, tmp_path):
    X = built_lib.synth_grn(60, 200, seed=8)
    write_exp(tmp_path / "x.exp", X)
    r = run("mcpnet", "-i", tmp_path / "x.exp", "-o", tmp_path / "out", "--mi-method", "0", "-m", "1", "2", "3")
    assert r.returncode == 0, r.stderr
    mi = read_exp(tmp_path / "out_bs.mi.exp")  # written after the diagonal reset, as mcpnet.cpp:299-356
    want = port.bspline_mi(X.astype(np.float64))
    np.fill_diagonal(want, 0)
    np.testing.assert_allclose(mi, want, rtol=0, atol=2e-5)
    assert not np.diag(mi).any()
    A = mi.copy()
    for k, pl in ((2, 2), (3, 3), (4, 4)):
        got = read_exp(tmp_path / f"out_bs.mcp{k}.exp")
        assert np.array_equal(got, port.mcp(A, pl)[1])
    r = run("dpi", "-i", tmp_path / "out_bs.mi.exp", "-o", tmp_path / "dpi.exp", "-l", "0.1")
    assert r.returncode == 0 and "Mask removing" in r.stdout
    assert np.array_equal(read_exp(tmp_path / "dpi.exp"), port.dpi(A, 0.1)[0])
    r = run("mcp", "-i", tmp_path / "out_bs.mi.exp", "-o", tmp_path / "m3.exp", "-m", "2", "--diagonal", "0",
            "-x", tmp_path / "mm3.exp")
    assert r.returncode == 0
    M, R = port.mcp(A, 3, symmetrize=True)
    assert np.array_equal(read_exp(tmp_path / "m3.exp"), R) and np.array_equal(read_exp(tmp_path / "mm3.exp"), M)


def read_text_matrix(path, sep):
    lines = Path(path).read_text().splitlines()
    skip = 2 if lines[0].split(sep)[1] == "Alias" else 1
    return np.array([[float(v) for v in l.split(sep)[skip:]] for l in lines[1:]], dtype=np.float32)


def test_csv_round_trip(built_lib, tmp_path):
    X = built_lib.synth_grn(7, 11, seed=3)
    write_exp(tmp_path / "x.exp", X)
    r = run("convert", "-i", tmp_path / "x.exp", "-o", tmp_path / "x.csv")
    assert r.returncode == 0, r.stderr
    assert np.array_equal(read_text_matrix(tmp_path / "x.csv", ","), X)
    # a CSV without the Alias column reads too
    with open(tmp_path / "y.csv", "w") as f:
        f.write("Id," + ",".join(f"s{j}" for j in range(11)) + "\n")
        for i in range(7):
            f.write(f"g{i}," + ",".join(repr(float(v)) for v in X[i]) + "\n")
    r = run("convert", "-i", tmp_path / "y.csv", "-o", tmp_path / "y.exp")
    assert r.returncode == 0, r.stderr
    assert np.array_equal(read_exp(tmp_path / "y.exp"), X)


@pytest.mark.gpu
@pytest.mark.parametrize("method,prec", [("2", "bf16x3"), ("6", "bf16f8")])
def test_cli_tensor_core_mi(built_lib, gpu, tmp_path, method, prec):
    """`mi -m 2` / `-m 6`: the tensor-core B-spline forms, the same matrix as the library call."""
    X = built_lib.synth_grn(40, 300, seed=13)
    write_exp(tmp_path / "x.exp", X)
    r = run("mi", "-i", tmp_path / "x.exp", "-o", tmp_path / "mi.exp", "-m", method)
    assert r.returncode == 0, r.stderr
    want = gpu.bspline_mi(read_exp(tmp_path / "x.exp"), 10, 3, prec)
    np.fill_diagonal(want, 0.0)
    got = read_exp(tmp_path / "mi.exp")
    np.fill_diagonal(got, 0.0)
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_cli_ap_mi(built_lib, gpu, tmp_path):
    """`mi -m 1` (the reference's default): seeded U[0, 1e-5) noise, ranks, AP MI."""
    X = built_lib.synth_grn(50, 300, seed=12)
    write_exp(tmp_path / "x.exp", X)
    r = run("mi", "-i", tmp_path / "x.exp", "-o", tmp_path / "ap.exp", "--seed", "5")
    assert r.returncode == 0, r.stderr
    got = read_exp(tmp_path / "ap.exp")
    X32 = read_exp(tmp_path / "x.exp")
    assert np.array_equal(got, gpu.ap_mi(X32, noise=1e-5, seed=5))


@pytest.mark.gpu
def test_cli_ensemble_eval(built_lib, port, tmp_path):
    """mcpnet --mi-input -m 2 4 -f coeffs --eval -g truth: AUPRs and the chosen
    combo against the oracle's composition of the reference's loop."""
    n = 70
    X, E = built_lib.synth_grn(n, 250, seed=14, with_edges=True)
    A = port.bspline_mi(X)
    np.fill_diagonal(A, 0)
    names = [f"g{i}" for i in range(n)]
    write_exp(tmp_path / "mi.exp", A, names)
    rng = np.random.default_rng(2)
    L = np.full((n, n), -1, np.int8)
    with open(tmp_path / "truth.txt", "w") as f:
        for s, t in E:
            f.write(f"g{s}\tg{t}\t1\n")
            L[s, t] = 1
        for _ in range(600):
            s, t = rng.integers(0, n, 2)
            if s != t and L[s, t] == -1:
                f.write(f"g{s}\tg{t}\t0\n")
                L[s, t] = 0
    cs = np.array([[0.25, 0.25, 0.25, 0.25], [1, 0, 0, 0], [0.5, 0.5, 0, 0], [0, 0, 0.5, 0.5]])
    np.savetxt(tmp_path / "coeffs.txt", cs)
    r = run("mcpnet", "-i", tmp_path / "mi.exp", "-o", tmp_path / "o", "--mi-input", "-m", "1", "4", "-f",
            tmp_path / "coeffs.txt", "--eval", "-g", tmp_path / "truth.txt")
    assert r.returncode == 0, r.stderr
    M = port.maxmin(A, A)
    M2 = port.maxmin(A, M)
    M3 = port.maxmin(M, M)
    pr, roc, best = port.combo_eval(A, M, M2, M3, L, cs, region="all")
    lines = [l for l in r.stdout.splitlines() if l.startswith("Computed,Combo AUPR")]
    got = [float(l.split()[2].split(",")[0]) for l in lines]
    want = [p for p in pr if p == p]
    assert len(got) == len(want) and np.allclose(got, want, rtol=0, atol=1e-11)
    tag = "_".join(f"{c:.3f}" for c in cs[best])
    chosen = read_exp(tmp_path / f"o_inmi.mcp_{tag}.exp")
    assert np.array_equal(chosen, port.combo(A, M, M2, M3, cs[best]))
    st = [l for l in r.stdout.splitlines() if l.startswith("Computed,Combo Stouffer AUPR")]
    assert len(st) == len(want)
    sbest = [l for l in r.stdout.splitlines() if l.startswith("Computed,MAX Combo AND Stouffer")][0]
    stag = sbest.split("(")[1].split(")")[0]
    assert (tmp_path / f"o_inmi.mcpst_{stag}.exp").exists()
    mcp2 = [l for l in r.stdout.splitlines() if l.startswith("Computed,auprroc,mcp2,")][0].split(",")
    a, b, _, _ = port.eval_truth(port.mcp(A, 2)[1], L, "all")
    assert abs(float(mcp2[3]) - a) <= 1e-11 and abs(float(mcp2[4]) - b) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("truth", ["matrix", "list"])
def test_cli_tf_input(built_lib, port, tmp_path, truth):
    """mcpnet --tf-input: TF rows only, compute_mcp{2,3,4}_tfs with transitions
    1 / 2 / 3, the TF ensemble and its TF Stouffer search, the truth reduced to
    TF sources -- against the oracle's composition of the reference's steps."""
    n = 64
    X, E = built_lib.synth_grn(n, 240, seed=21, with_edges=True)
    A = port.bspline_mi(X)
    np.fill_diagonal(A, 0)
    names = [f"g{i}" for i in range(n)]
    write_exp(tmp_path / "mi.exp", A, names)
    tf_rows = np.array([i for i in range(n) if i % 5 == 1 or i in (0, 2)], np.int32)
    with open(tmp_path / "tfs.txt", "w") as f:
        f.write("  missing_gene \n")
        for i in tf_rows:
            f.write(f" g{i}\t\n")
    tfs = np.full(n, -np.inf, np.float32)
    tfs[tf_rows] = np.inf
    col_tf = (tfs > 0).astype(np.uint8)
    rng = np.random.default_rng(4)
    L = np.full((n, n), -1, np.int8)
    for s, t in E:
        L[s, t] = L[t, s] = 1
    for _ in range(900):
        s, t = rng.integers(0, n, 2)
        if s != t and L[s, t] == -1:
            L[s, t] = L[t, s] = 0
    if truth == "matrix":
        write_exp(tmp_path / "truth.exp", L.astype(np.float32), names)
        targs = ["-x", tmp_path / "truth.exp"]
        Lt, region, rg, ct = L[tf_rows], "tf", tf_rows, col_tf
    else:
        with open(tmp_path / "truth.txt", "w") as f:
            for s in range(n):
                for t in range(n):
                    if L[s, t] in (0, 1):
                        f.write(f"g{s}\tg{t}\t{L[s, t]}\n")
        targs = ["-g", tmp_path / "truth.txt"]
        Lt = L[tf_rows].copy()
        Lt[np.arange(len(tf_rows)), tf_rows] = -1
        region, rg, ct = "all", None, None
    cs = np.array([[0.25, 0.25, 0.25, 0.25], [0.5, 0.5, 0, 0], [0, 1, 0, 0], [0.2, 0.3, 0.1, 0.4]])
    np.savetxt(tmp_path / "coeffs.txt", cs)
    r = run("mcpnet", "-i", tmp_path / "mi.exp", "-o", tmp_path / "o", "--mi-input", "--tf-input",
            tmp_path / "tfs.txt", "-m", "1", "2", "3", "4", "-f", tmp_path / "coeffs.txt", "--eval", *targs)
    assert r.returncode == 0, r.stderr
    out = lambda name: read_exp(tmp_path / f"o_tf_inmi.{name}.exp")
    header = (tmp_path / "o_tf_inmi.mcp2.exp").read_text().splitlines()
    assert [l.split("\t")[0] for l in header[1:]] == [f"g{i}" for i in tf_rows]
    for k in (2, 3, 4):
        M, R = port.mcp_tf(A, tfs, k, k - 1)
        assert np.array_equal(out(f"mcp{k}"), R), k
        line = [l for l in r.stdout.splitlines() if l.startswith(f"Computed,auprroc,mcp{k},")][0].split(",")
        a, b, _, _ = port.eval_truth(R, Lt, region, rg, ct)
        assert abs(float(line[3]) - a) <= 1e-11 and abs(float(line[4]) - b) <= 1e-11
    T, M1, M2, M3 = port.maxmins_tf(A, tfs)
    pr, roc, best = port.combo_eval(T, M1, M2, M3, Lt, cs, region, rg, ct)
    got = [float(l.split()[2].split(",")[0]) for l in r.stdout.splitlines() if l.startswith("Computed,Combo AUPR")]
    assert np.allclose(got, pr, rtol=0, atol=1e-11)
    tag = "_".join(f"{c:.3f}" for c in cs[best])
    assert np.array_equal(out(f"mcp_{tag}"), port.combo(T, M1, M2, M3, cs[best]))
    spr, sroc, sbest = port.combo_stouffer_tf_eval(T, M1, M2, M3, Lt, cs, region, rg, ct)
    got = [float(l.split()[3].split(",")[0]) for l in r.stdout.splitlines()
           if l.startswith("Computed,Combo Stouffer AUPR")]
    assert np.allclose(got, spr, rtol=0, atol=1e-6)  # statistics to an ulp: AUPR close, not equal
    stag = [l for l in r.stdout.splitlines() if l.startswith("Computed,MAX Combo AND Stouffer")][0]
    stag = stag.split("(")[1].split(")")[0]
    st = out(f"mcpst_{stag}")
    want = port.stouffer_tf(port.combo(T, M1, M2, M3, np.array([float(v) for v in stag.split("_")])))
    np.testing.assert_allclose(st, want, rtol=1e-5, atol=1e-5)


def test_cli_tf_input_without_tfs(built_lib, tmp_path):
    """A TF file naming no gene stops mcpnet with the reference's message."""
    A = np.eye(4, dtype=np.float32)
    write_exp(tmp_path / "mi.exp", A)
    (tmp_path / "tfs.txt").write_text("nothing\n")
    r = run("mcpnet", "-i", tmp_path / "mi.exp", "-o", tmp_path / "o", "--mi-input", "--tf-input",
            tmp_path / "tfs.txt")
    assert r.returncode != 0 and "no transcription factors" in r.stderr


@pytest.mark.gpu
def test_cli_mcp_dpi_tf_and_partials(built_lib, port, tmp_path):
    """mcp -f / dpi -f keep TF rows (compute_mcp{2,3,4}_tfs; dpi_tf_kernel over all
    pairs), the mcp app's default transition -1 (0 for MCP2 / MCP3, 1 for MCP4), and
    mcp -m 5: ratio(input, first (x) second)."""
    n = 48
    X = built_lib.synth_grn(n, 200, seed=23)
    A = port.bspline_mi(X)
    np.fill_diagonal(A, 0)
    names = [f"g{i}" for i in range(n)]
    write_exp(tmp_path / "mi.exp", A, names)
    tf_rows = [i for i in range(n) if i % 4 == 3]
    (tmp_path / "tfs.txt").write_text("".join(f"g{i}\n" for i in tf_rows))
    tfs = np.full(n, -np.inf, np.float32)
    tfs[tf_rows] = np.inf
    for method, tr, want_tr in ((1, None, 0), (2, None, 0), (3, None, 1), (3, 2, 2), (1, 1, 1)):
        extra = [] if tr is None else ["--tf-gene-transition", tr]
        r = run("mcp", "-i", tmp_path / "mi.exp", "-o", tmp_path / "m.exp", "-m", method, "-f", tmp_path / "tfs.txt",
                "-x", tmp_path / "mm.exp", *extra)
        assert r.returncode == 0, r.stderr
        M, R = port.mcp_tf(A, tfs, method + 1, want_tr)
        assert np.array_equal(read_exp(tmp_path / "m.exp"), R), (method, tr)
        assert np.array_equal(read_exp(tmp_path / "mm.exp"), M), (method, tr)
        rows = [l.split("\t")[0] for l in (tmp_path / "m.exp").read_text().splitlines()[1:]]
        assert rows == [f"g{i}" for i in tf_rows]
    r = run("dpi", "-i", tmp_path / "mi.exp", "-o", tmp_path / "d.exp", "-l", "0.1", "-f", tmp_path / "tfs.txt")
    assert r.returncode == 0, r.stderr
    out, _, removed = port.dpi_tf(A, tfs, 0.1)
    assert np.array_equal(read_exp(tmp_path / "d.exp"), out[tf_rows])
    assert f"Mask removing {removed} elements" in r.stdout
    rng = np.random.default_rng(5)
    F1 = rng.random((n, 30)).astype(np.float32)
    F2 = rng.random((n, 30)).astype(np.float32)
    write_exp(tmp_path / "f1.exp", F1, names)
    write_exp(tmp_path / "f2.exp", F2, names)
    r = run("mcp", "-i", tmp_path / "mi.exp", "-o", tmp_path / "p.exp", "-m", "5", "--first", tmp_path / "f1.exp",
            "--second", tmp_path / "f2.exp", "-x", tmp_path / "pm.exp", "--clamped")
    assert r.returncode == 0, r.stderr
    MM = port.maxmin(F1, F2)
    assert np.array_equal(read_exp(tmp_path / "pm.exp"), MM)
    assert np.array_equal(read_exp(tmp_path / "p.exp"), port.ratio(A, MM))


@pytest.mark.gpu
def test_cli_transform(built_lib, port, tmp_path):
    """transform -m 1 / 2: CLR / Stouffer of the square matrix (the GPU's statistics
    are within an ulp of the oracle's, so the values agree to float rounding), and
    with -f the TF form, equal bit for bit to the library's own call."""
    n = 40
    X = built_lib.synth_grn(n, 150, seed=24)
    A = port.bspline_mi(X)
    np.fill_diagonal(A, 0)
    names = [f"g{i}" for i in range(n)]
    write_exp(tmp_path / "mi.exp", A, names)
    tf_rows = [1, 5, 6, 22, 39]
    (tmp_path / "tfs.txt").write_text("".join(f"g{i}\n" for i in tf_rows))
    import mcpnet_gb300 as M
    h = M.Handle(0)
    try:
        for method, kind in ((1, "clr"), (2, "stouffer")):
            r = run("transform", "-i", tmp_path / "mi.exp", "-o", tmp_path / "t.exp", "-m", method)
            assert r.returncode == 0, r.stderr
            got = read_exp(tmp_path / "t.exp")
            assert np.array_equal(got, h.transform(A, kind))
            np.testing.assert_allclose(got, port.transform(A, clr=(kind == "clr")), rtol=1e-5, atol=1e-5)
            r = run("transform", "-i", tmp_path / "mi.exp", "-o", tmp_path / "tf.exp", "-m", method, "-f",
                    tmp_path / "tfs.txt")
            assert r.returncode == 0, r.stderr
            got = read_exp(tmp_path / "tf.exp")
            assert np.array_equal(got, h.transform_tf(A[tf_rows], kind))
            np.testing.assert_allclose(got, port.stouffer_tf(A[tf_rows], clr=(kind == "clr")), rtol=1e-5, atol=1e-5)
    finally:
        h.close()


def _stats(vals, i):
    """eval_mcpnet's per-part min / max / mean (sum / (i - 1)) / stdev over i iterations."""
    v = np.asarray(vals, dtype=np.float64)[:i]
    mean = v.sum() / i
    return v.min(), v.max(), v.sum() / (i - 1), np.sqrt(i / (i - 1) * ((v * v).sum() / i - mean * mean))


def _stat_lines(out, what):
    got = {}
    for l in out.splitlines():
        if l.startswith(f"AUPR {what} "):
            head, val, dec, it, _ = l.split(",")
            # the first block for a tag (MI's, before the MCPs' blocks with the same tag)
            got.setdefault((head[len(f"AUPR {what} "):], int(dec.split()[1]), int(it.split()[1])), float(val))
    return got


@pytest.mark.gpu
def test_cli_eval_mcpnet(built_lib, port, tmp_path):
    """eval_mcpnet --mi-file -x truth -m 1 4 5: the split AUPR summaries of MI and MCP2
    against the oracle's composition of eval_aupr_mcp, and the ensemble summary
    against the library's split coefficient search."""
    import mcpnet_gb300 as M
    n, iters = 60, 10
    X, E = built_lib.synth_grn(n, 220, seed=25, with_edges=True)
    A = port.bspline_mi(X)
    np.fill_diagonal(A, 0)
    names = [f"g{i}" for i in range(n)]
    write_exp(tmp_path / "mi.exp", A, names)
    L = np.zeros((n, n), np.int8)
    for s, t in E:
        L[s, t] = L[t, s] = 1
    write_exp(tmp_path / "truth.exp", L.astype(np.float32), names)
    cs = np.array([[0.25, 0.25, 0.25, 0.25], [0.5, 0.5, 0, 0], [0, 0.5, 0.25, 0.25]])
    np.savetxt(tmp_path / "coeffs.txt", cs)
    r = run("eval_mcpnet", "--mi-file", tmp_path / "mi.exp", "-x", tmp_path / "truth.exp", "-m", "1", "4", "5",
            "-f", tmp_path / "coeffs.txt", "--iterations", iters)
    assert r.returncode == 0, r.stderr
    Am = A.copy()
    E_ = port.mask_entries(Am, L)[0].size
    tc = M.train_counts(E_)
    heads = [l for l in r.stdout.splitlines() if l.startswith("AUPR full,")]
    assert len(heads) == 2
    for head, V in zip(heads, (Am, port.mcp(Am, 2)[1])):
        full, tr, te = port.split_aupr(V, L, iters, tc)
        assert abs(float(head.split(",")[1]) - full) <= 1e-11
    got = _stat_lines(r.stdout, "full")
    full, tr, te = port.split_aupr(Am, L, iters, tc)
    for j in range(len(tc)):
        for what, arr in (("train", tr[:, j]), ("test", te[:, j])):
            want = _stats(arr, iters)
            for name, w in zip(("min", "max", "mean", "stdev"), want):
                assert abs(got[(f"{what} {name}", j, iters)] - w) <= 1e-9 * max(1.0, abs(w)), (what, name, j)
    h = M.Handle(0)
    try:
        M1 = port.maxmin(Am, Am)
        res, _ = h.split_combo_eval(Am, M1, port.maxmin(Am, M1), port.maxmin(M1, M1), L, cs, iters, tc,
                                    "exclude_diagonal")
    finally:
        h.close()
    st = _stat_lines(r.stdout, "stouffer full")
    for j in range(len(tc)):
        want = _stats(res[:, j, 2], iters)
        assert abs(st[("train min", j, iters)] - want[0]) <= 1e-11
        assert abs(st[("train max", j, iters)] - want[1]) <= 1e-11
        want = _stats(res[:, j, 4], iters)
        full_lines = {k: v for k, v in got.items() if k[0].startswith("full ")}
        assert abs(full_lines[("full min", j, iters)] - want[0]) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("truth", ["matrix", "list"])
def test_cli_auc_pr_roc(built_lib, port, tmp_path, truth):
    """auc_pr_roc: AUPR / AUROC of a score matrix against a truth matrix (below the
    diagonal) or list (the listed pairs), as the oracle's compute_aupr_auroc."""
    n = 50
    X, E = built_lib.synth_grn(n, 180, seed=26, with_edges=True)
    A = port.bspline_mi(X)
    names = [f"g{i}" for i in range(n)]
    write_exp(tmp_path / "s.exp", A, names)
    L = np.zeros((n, n), np.int8)
    for s_, t in E:
        L[s_, t] = L[t, s_] = 1
    if truth == "matrix":
        write_exp(tmp_path / "t.exp", L.astype(np.float32), names)
        targ, region, Lw = ["-x", tmp_path / "t.exp"], "lower", L
    else:
        Lw = np.full((n, n), -1, np.int8)
        with open(tmp_path / "t.txt", "w") as f:
            for i in range(n):
                for j in range(n):
                    if i != j and (i + j) % 3 == 0:
                        f.write(f"g{i}\tg{j}\t{L[i, j]}\n")
                        Lw[i, j] = L[i, j]
        targ, region = ["-g", tmp_path / "t.txt"], "all"
    r = run("auc_pr_roc", "-i", tmp_path / "s.exp", *targ)
    assert r.returncode == 0, r.stderr
    got = {l.split(",")[1].split()[0]: float(l.split(",")[1].split()[1]) for l in r.stdout.splitlines()
           if l.startswith("Computed,au")}
    a, b, _, _ = port.eval_truth(read_exp(tmp_path / "s.exp"), Lw, region)
    assert abs(got["aupr"] - a) <= 1e-11 and abs(got["auroc"] - b) <= 1e-11
