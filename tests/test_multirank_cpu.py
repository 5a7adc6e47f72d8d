"""The N > 1 launch path of bench.py on CPU: replicas with gloo, max-over-ranks
timing, rank 0 alone prints (the reference arm), others exit cleanly."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    v = bench.reduce_max(float(rank + 1) * 10.0, world)
    q.put((rank, v))
    dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 20.0), (1, 20.0)]


def test_reference_arm_under_torchrun_two_ranks(tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29613", str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--genes", "300", "--samples", "100",
           "--ref-seconds", "0.2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")


def test_reference_arm_never_maps_the_gpu_library():
    """The reference arm times the CPU path only: its process maps the oracle and
    the host-only input generator, never libmcpgpu.so."""
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import bench\n"
        "bench.main(['--impl', 'reference', '--genes', '200', '--samples', '100', '--steps', '1', '--warmup', '3',"
        " '--ref-seconds', '0.05'])\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPS', 'libmcpgpu' in maps, 'libmcpsynth' in maps, 'mcpnet_gb300' in sys.modules)\n" % str(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=str(ROOT),
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("MAPS")][0]
    assert line == "MAPS False True False", line
