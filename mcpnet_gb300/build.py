"""In-tree build of libmcpgpu.so (CUDA kernels + C ABI) for sm_103a.

Every translation unit compiles in parallel (one nvcc / g++ process each) into
mcpnet_gb300/_build/, then links into mcpnet_gb300/_lib/libmcpgpu.so with the
CUDA runtime linked statically.  No cmake; runs on x86_64 and aarch64 hosts.

    python -m mcpnet_gb300.build          # build if stale
    python -m mcpnet_gb300.build --force  # rebuild everything
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libmcpgpu.so"
APPS = PKG / "apps"
CLI = LIBDIR / "mcpgpu_cli"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmcpgpu.so")
    return cand


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
               f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-fopenmp", "-ffp-contract=off",
               f"-I{INCLUDE}", f"-I{_cuda_home() / 'include'}", "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and link libmcpgpu.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    todo = [s for s in srcs if force or _stale(BUILD / (s.name + ".o"), [s, *hdrs])]
    jobs = max(1, min(len(todo), os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(lambda s: _compile(s, verbose), todo))
    objs = [BUILD / (s.name + ".o") for s in srcs]
    if force or todo or _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    cli_src = APPS / "mcpgpu_cli.cpp"
    if cli_src.exists() and (force or _stale(CLI, [cli_src, LIB, *_headers()])):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", f"-I{INCLUDE}", str(cli_src), "-o", str(CLI), f"-L{LIBDIR}",
               "-lmcpgpu", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed\n{r.stdout}\n{r.stderr}")
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
