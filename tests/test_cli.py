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


def test_bad_usage_reports(built_lib, tmp_path):
    assert run("mi").returncode != 0
    r = run("frobnicate", "-i", tmp_path / "none.exp", "-o", tmp_path / "o.exp")
    assert r.returncode != 0 and "cannot open" in r.stderr


@pytest.mark.gpu
def test_cli_pipeline_matches_oracle(built_lib, port, tmp_path):
    X = built_lib.synth_grn(60, 200, seed=8)
    write_exp(tmp_path / "x.exp", X)
    r = run("mcpnet", "-i", tmp_path / "x.exp", "-o", tmp_path / "out", "--mi-method", "0", "-m", "1", "2", "3")
    assert r.returncode == 0, r.stderr
    mi = read_exp(tmp_path / "out_bs.mi.exp")
    np.testing.assert_allclose(mi, port.bspline_mi(X.astype(np.float64)), rtol=0, atol=2e-5)
    A = mi.copy()
    np.fill_diagonal(A, 0)
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
