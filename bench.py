#!/usr/bin/env python
"""Benchmark of the MCPNet compute core on GB300.

Metric (one JSON line on rank 0):
  "MI gene-pairs/s + max-min Gop/s at n=20k: BF16-TC vs FP32 GPU, MI err<=1e-4"

Workload (default): seeded synthetic GRN expression, 20,000 genes x 2,000
samples, B-spline MI with 10 bins and spline order 3.
  * ``value``  -- B-spline MI gene pairs per second (n(n-1)/2 per step), one
    step = scale + weights + tensor-core contraction with the fused entropy
    epilogue (default form bf16f8: BF16 hi*hi plus the E4M3 hi*lo + lo*hi
    correction; ``mi_forms`` times bf16x3 beside it), inputs resident in HBM,
    timed with CUDA events on the library's
    stream; W >= 3 untimed warm-up steps.  Working set (X 160 MB, weights
    1.6 GB, MI 1.6 GB) is larger than the 129 MB L2, so no flush is needed.
  * ``e2e``    -- the same metric through the host C ABI (mcpg_bspline_mi with
    pinned host buffers: host->device copy of X and device->host copy of MI
    inside the timed region).
  * ``maxmin`` -- the FP32 max-min product A (x) M1 (the second product of
    MCP3, a full n^3 non-symmetric product) in Gop/s (2 ops per triple), and
    the MCP2 stage (symmetric A (x) A with the ratio fused) in ms.
  * ``mi_fp32``-- the plain FP32 CUDA-core MI on the same input, and the
    tensor-core speed-up over it.
  * ``cpu_baseline`` -- the CPU oracle (a restatement of the reference's
    OpenMP loops) on a bounded row slab of the same workload, all host cores.

``--impl reference`` times the reference's CPU implementation of the path (the
oracle's restatement on this host; the compiled reference where it was built
for this machine) on bounded samples, and prints the same metric.

Multi-GPU (``torchrun --nproc-per-node N``): the path has no exchange step on
one node's replicas; every rank runs the same workload on its own GPU
("replicas only"), and value sums the ranks' work over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MI gene-pairs/s + max-min Gop/s at n=20k: BF16-TC vs FP32 GPU, MI err≤1e-4"
UNIT = "gene-pairs/s"


# ---------------------------------------------------------------- helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def reduce_max(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- CPU legs
class CpuMiSampler:
    """Times the reference's CPU MI (OpenMP over rows, float) on a row slab of
    the n x m workload.  Uses MCPNet's own kernels where they were compiled for
    this machine (oracle/_ref), else the oracle's restatement of them."""

    def __init__(self, n: int, m: int, seed: int):
        from oracle import oracle as O
        from synthgrn import synth_grn  # host-only generator: the GPU library is never loaded here
        self.n, self.m = n, m
        R = O.ref()
        self.kind = "reference" if R is not None else "port"
        self.impl = R if R is not None else O.port()
        X = synth_grn(n, m, seed=seed)
        self.W = self.impl.bspline_weights(X)
        self.threads = O.port().threads()

    def run(self, target_s: float):
        t0 = time.perf_counter()
        self.impl.bspline_mi_rows(self.W, self.m, 0, 1)
        per_row = max(time.perf_counter() - t0, 1e-4)
        rows = int(max(1, min(self.n, target_s / per_row)))
        t0 = time.perf_counter()
        self.impl.bspline_mi_rows(self.W, self.m, 0, rows)
        dt = time.perf_counter() - t0
        pairs = rows * self.n
        return pairs / dt, {"rows": rows, "pairs": pairs, "seconds": dt, "threads": self.threads}

    def describe(self, info) -> str:
        src = ("MCPNet's BSplineMIKernel compiled from the reference sources" if self.kind == "reference"
               else "the reference's loops restated in oracle/")
        return (f"MI of rows 0..{info['rows']} x all {self.n} genes ({info['pairs']} pairs), m={self.m}, float, "
                f"{info['seconds']:.1f} s, OpenMP over rows; {src}")


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    sampler = CpuMiSampler(args.genes, args.samples, args.seed)
    vals = []
    info = {}
    for i in range(args.warmup + args.steps):
        v, info = sampler.run(args.ref_seconds)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, "fp32-cpu"),
        "ms_per_step": info["seconds"] * 1e3,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["threads"], "kind": sampler.kind,
                         "sample": sampler.describe(info) + " (per step)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# (kernel, precision, genes, samples, bins, order) -> (DRAM bytes per launch, how it was measured)
MEASURED_TRAFFIC = {
    ("mi_tc", "bf16f8", 20000, 2000, 10, 3): (
        42.33e9 + 1.61e9, "ncu dram__bytes_read.sum + dram__bytes_write.sum, one full-size launch, one pass"),
}


def workload_config(args, precision):
    return {"workload": f"bspline-mi {args.genes} genes x {args.samples} samples, {args.bins} bins, order "
                        f"{args.order}, {precision}; max-min products at n={args.genes}",
            "genes": args.genes, "samples": args.samples, "bins": args.bins, "order": args.order,
            "precision": precision, "seed": args.seed, "parallelism": "replicas",
            "l2": "inputs larger than L2 (weights and MI matrices >> 129 MB); no flush"}


# ---------------------------------------------------------------- GPU arm
def gpu_arm(args, ws, rank, local):
    import torch
    import mcpnet_gb300 as M

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, m = args.genes, args.samples
    pairs = n * (n - 1) // 2
    X_host = M.synth_grn(n, m, seed=args.seed)
    X = torch.from_numpy(X_host).to(dev)
    MI = torch.empty((n, n), dtype=torch.float32, device=dev)
    h = M.Handle(local)
    stream = torch.cuda.current_stream(dev)
    h.set_stream(stream.cuda_stream)

    def mi_step(prec):
        h.bspline_mi_dev(X, MI, args.bins, args.order, prec)

    # ---- warm-up ----
    for _ in range(args.warmup):
        mi_step(args.precision)
    torch.cuda.synchronize(dev)

    # ---- timed MI (value) ----
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = h.kernel_launches
    h.profile(True)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for a, b in evs:
        a.record(stream)
        mi_step(args.precision)
        b.record(stream)
    torch.cuda.synchronize(dev)
    barrier(ws)
    wall = time.perf_counter() - t0
    prof = h.profile_report()
    h.profile(False)
    launches = h.kernel_launches - launches0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    dev_s = sum(step_ms) / 1e3
    dev_s_max = reduce_max(dev_s, ws)
    value = ws * pairs * args.steps / dev_s_max
    clk = clocks.stop()

    # dominant kernel of the MI step and its roofline
    kname = "mi_fp32" if args.precision == "fp32" else "mi_tc"
    kern = prof.get(kname, {"launches": 0, "ms": float("nan")})
    k_ms = kern["ms"] / max(kern["launches"], 1)
    flops = 2.0 * args.bins * args.bins * m * pairs  # algorithmic: 2 b^2 m per unordered pair
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    props = torch.cuda.get_device_properties(dev)
    sms = props.multi_processor_count
    f_max = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    if args.precision == "fp32":
        peak_tf = sms * 128 * 2 * f_max / 1e12
        peak_src = f"FP32 FMA peak = {sms} SMs x 128 lanes x 2 x {f_max/1e6:.0f} MHz (computed)"
        bound = "fp32-alu"
    else:
        peak_tf = float(peaks.get("bf16_tflops", 1900.0))
        peak_src = "MEASURED_PEAKS.json bf16_tflops (burst, of measured)" if "bf16_tflops" in peaks \
            else "fallback 1.9 PFLOP/s"
        bound = "tensor"
    achieved_tf = flops / (k_ms / 1e3) / 1e12
    # DRAM bytes of one launch from an ncu capture of this exact workload (dram__bytes_read.sum +
    # dram__bytes_write.sum, a one-pass capture of the full-size launch); other workloads: null
    traffic = MEASURED_TRAFFIC.get((kname, args.precision, n, m, args.bins, args.order))
    roofline = {"bound": bound, "kernel": kname, "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                "frac": achieved_tf / peak_tf, "traffic": traffic[0] if traffic else None,
                "traffic_source": traffic[1] if traffic else None, "peak_source": peak_src,
                "kernel_ms": k_ms, "algorithmic_flop_per_launch": flops,
                "note": "achieved counts 2*b^2*m flops per unordered gene pair; the FP8-corrected form "
                        "(bf16f8) issues them once in BF16 and twice in FP8 (twice the BF16 rate: the time of "
                        "2x BF16), the BF16 hi+lo split (bf16x3) 3x in BF16"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        # operand types of the contraction (FP32 accumulation in every tensor-core form)
        "dtype": {"bf16f8": "bf16+e4m3"}.get(args.precision, "bf16" if args.precision.startswith("bf16") else
                                             ("f16" if args.precision.startswith("fp16") else "f32")),
        "data": "synthetic (seeded SEM GRN, in-degree ~ Poisson(2), weights +-U(0.5,1.5))",
        "config": workload_config(args, args.precision),
        "clocks": clk, "gpu_launches": launches, "roofline": roofline,
        "kernel_profile": prof, "wall_s": wall, "sms": sms,
    }

    # ---- plain FP32 GPU MI on the same input ----
    MI32 = None
    if args.precision != "fp32" and not args.no_fp32:
        mi_step("fp32")
        torch.cuda.synchronize(dev)
        MI_tc = None
        ts = []
        for _ in range(args.fp32_steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            mi_step("fp32")
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        MI32 = MI.clone()
        mi_step(args.precision)
        torch.cuda.synchronize(dev)
        diff = float((MI - MI32).abs().max().item())
        f_ms = float(np.mean(ts))
        line["mi_fp32"] = {"ms": f_ms, "pairs_per_s": pairs / (f_ms / 1e3),
                           "speedup_tc_vs_fp32": f_ms / (dev_s / args.steps * 1e3),
                           "max_abs_diff_vs_tc_bits": diff}

    # ---- the other tensor-core forms on the same input (step time, max |diff| vs the FP32 MI) ----
    others = [p for p in args.compare.split(",") if p in M.PRECISIONS and p not in (args.precision, "fp32")]
    if args.precision != "fp32" and others:
        line["mi_forms"] = {}
        for prec in others:
            for _ in range(2):
                mi_step(prec)
            torch.cuda.synchronize(dev)
            ts = []
            for _ in range(3):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                mi_step(prec)
                b.record(stream)
                b.synchronize()
                ts.append(a.elapsed_time(b))
            o_ms = float(np.mean(ts))
            rec = {"ms_per_step": o_ms, "pairs_per_s": pairs / (o_ms / 1e3)}
            if MI32 is not None:
                rec["max_abs_diff_vs_fp32_bits"] = float((MI - MI32).abs().max().item())
            line["mi_forms"][prec] = rec
        MI32 = None

    # ---- max-min products ----
    if not args.no_maxmin:
        A = MI
        h.set_diagonal_dev(A, 0.0)
        M1 = torch.empty_like(A)
        R = torch.empty_like(A)
        C = torch.empty_like(A)
        h.maxmin_dev(A, A, M1)  # symmetric A (x) A
        torch.cuda.synchronize(dev)
        # A (x) M1: full non-symmetric product (MCP3's second product)
        h.profile(True)
        ts = []
        for _ in range(args.maxmin_steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            h.maxmin_dev(A, M1, C)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        mm_prof = h.profile_report()
        h.profile(False)
        mm_ms = float(np.mean(ts))
        ops = 2.0 * n * n * n
        gops = ops / (mm_ms / 1e3) / 1e9
        alu_peak = sms * 128 * f_max / 1e9
        med = clk.get("sm_mhz") or None
        line["maxmin"] = {"gops": gops, "ms": mm_ms, "n": n, "product": "A (x) M1, full n^3",
                          "alu_peak_gops_at_max_clock": alu_peak,
                          "frac_alu_peak_at_max_clock": gops / alu_peak,
                          "alu_peak_note": f"{sms} SMs x 128 lanes x {f_max/1e6:.0f} MHz, 1 FP32 op/lane/clk; "
                                           "algorithmic 2 ops (min, max) per triple",
                          "kernel_profile": mm_prof}
        if med:
            line["maxmin"]["frac_alu_peak_at_median_clock"] = gops / (sms * 128 * med * 1e6 / 1e9)
        # MCP2 stage: symmetric A (x) A with the ratio fused
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        h.mcp_dev(A, 2, M=None, R=R)
        b.record(stream)
        b.synchronize()
        line["maxmin"]["mcp2_ms"] = a.elapsed_time(b)
        # the DPI filter (tolerance 0.1) and the converged max-capacity closure on the same MI
        Dm = torch.empty((n, n), dtype=torch.uint8, device=dev)
        h.dpi_dev(A, C, 0.1, Dm)  # untimed: scratch
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        removed = h.dpi_dev(A, C, 0.1, Dm)
        b.record(stream)
        b.synchronize()
        dpi_ms = a.elapsed_time(b)
        line["maxmin"]["dpi"] = {"ms": dpi_ms, "tol": 0.1, "removed": removed,
                                 "one_phase_equivalent_gops": 2.0 * 0.5 * n ** 3 / (dpi_ms / 1e3) / 1e9,
                                 "note": "two phases: the tiled max-min over the first 512 intermediates, then an "
                                         "early-exit scan of the outputs it left undecided"}
        del Dm
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        iters = h.closure_dev(A, C, 64)
        b.record(stream)
        b.synchronize()
        cl_ms = a.elapsed_time(b)
        line["maxmin"]["closure"] = {"ms": cl_ms, "squarings": iters,
                                     "frac_alu_peak_at_max_clock": 2.0 * 0.5 * n ** 3 * max(iters, 1) / (cl_ms / 1e3)
                                     / (alu_peak * 1e9)}
        del M1, R, C

    # ---- end to end through the host C ABI ----
    if not args.no_e2e:
        Xp = torch.empty((n, m), dtype=torch.float32, pin_memory=True)
        Xp.numpy()[:] = X_host
        MIp = torch.empty((n, n), dtype=torch.float32, pin_memory=True)
        xa, ma = Xp.numpy(), MIp.numpy()
        import ctypes as C
        L = M.lib()
        pr = M.PRECISIONS[args.precision]

        def host_call():
            rc = L.mcpg_bspline_mi(h._h, xa.ctypes.data, n, m, m, args.bins, args.order, pr, ma.ctypes.data, n, None)
            if rc:
                raise M.MCPGError(rc, L.mcpg_last_error(h._h).decode())
        host_call()
        barrier(ws)
        ts = []
        for _ in range(args.e2e_steps):
            t0 = time.perf_counter()
            host_call()
            ts.append(time.perf_counter() - t0)
        e_s = reduce_max(float(np.mean(ts)), ws)
        access = int(L.mcpg_last_host_access(h._h))
        line["e2e"] = {"value": ws * pairs / e_s, "unit": UNIT, "h2d_bytes_per_step": n * m * 4,
                       "d2h_bytes_per_step": n * n * 4, "ms_per_step": e_s * 1e3,
                       "api": "mcpg_bspline_mi (host buffers, pinned)",
                       "transfer": ("in place over NVLink-C2C: the kernels read X from and write MI to the host "
                                    "buffers" if access == 3 else "staged copies (slab-overlapped device-to-host)"),
                       "host_access_bits": access}
        # the same call on pageable buffers (what MCPNet's aligned_matrix holds), output pages touched
        xg, mg = np.array(X_host, dtype=np.float32), np.zeros((n, n), np.float32)
        pg = lambda: L.mcpg_bspline_mi(h._h, xg.ctypes.data, n, m, m, args.bins, args.order, pr, mg.ctypes.data, n,
                                       None)
        assert pg() == 0
        tp = []
        for _ in range(args.e2e_steps):
            t0 = time.perf_counter()
            assert pg() == 0
            tp.append(time.perf_counter() - t0)
        p_s = reduce_max(float(np.mean(tp)), ws)
        line["e2e_pageable"] = {"value": ws * pairs / p_s, "unit": UNIT, "ms_per_step": p_s * 1e3,
                                "host_access_bits": int(L.mcpg_last_host_access(h._h))}
        del xg, mg

    # ---- CPU baseline (rank 0, N = 1 only) ----
    if rank == 0 and ws == 1 and not args.no_cpu:
        sampler = CpuMiSampler(n, m, args.seed)
        v, info = sampler.run(args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": info["threads"], "kind": sampler.kind,
                                "sample": sampler.describe(info)}
    h.close()

    # ---- the large single-GPU configuration, once (N = 1 only; not part of `value`) ----
    if ws == 1 and not args.no_large:
        sub = argparse.Namespace(**vars(args))
        sub.genes, sub.samples, sub.mi_method = 32768, 4096, "bspline"
        sub.no_eval, sub.closure, sub.split_iters, sub.no_cpu = True, False, 0, True
        sub.tfs = 2048
        pl = pipeline_run(sub, local)
        line["large_pipeline"] = {
            "workload": "32768 genes x 4096 samples: B-spline MI (%s), diagonal 0, MCP2/3/4 (M1 shared, ratios "
                        "fused), DPI(0.1), TF MCP2/3/4, TF products and TF DPI(0.1) with 2048 seeded TFs; "
                        "each stage timed once with CUDA events" % args.precision,
            "stage_s": pl["stage_s"], "wall_s": pl["wall_s"], "stages": pl["stages"], "clocks": pl["clocks"]}
    if rank == 0:
        print(json.dumps(line), flush=True)


def pipeline_arm(args, ws, rank, local):
    line = pipeline_run(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def pipeline_run(args, local):
    """The whole MCPNet compute core once, stage by stage (the large single-GPU
    configuration: 32,768 genes x 4,096 samples by default): B-spline MI
    (tensor cores), diagonal reset, the three max-min products with the
    MCP2/3/4 ratios fused (M1 shared), the DPI filter, optionally the
    max-capacity closure, then the gold-standard evaluation (AUPR / AUROC of
    the MI and MCP2 networks against the synthetic GRN's edges, every other
    pair a negative) and the ensemble coefficient search over a 35-row
    coefficient grid, plain and Stouffer-transformed.  Returns one JSON object with per-stage
    times and roofline fractions, and the reference CPU path's time on the host cores
    extrapolated from timed row slabs."""
    import torch
    import mcpnet_gb300 as M

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, m, b = args.genes, args.samples, args.bins
    X = torch.from_numpy(M.synth_grn(n, m, seed=args.seed)).to(dev)
    h = M.Handle(local)
    stream = torch.cuda.current_stream(dev)
    h.set_stream(stream.cuda_stream)
    f32 = dict(dtype=torch.float32, device=dev)
    A = torch.empty((n, n), **f32)
    R2, R3, R4, D = (torch.empty((n, n), **f32) for _ in range(4))
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fmax = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    tc_peak = float(peaks.get("bf16_tflops", 1900.0)) * 1e12
    hbm = float(peaks.get("hbm_gbs", 6800.0)) * 1e9
    alu_peak = sms * 128 * fmax

    def timed(fn):
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        e.record(stream)
        e.synchronize()
        return a.elapsed_time(e) / 1e3

    # warm-up on a small problem (module load, workspace)
    Xs = X[:256].contiguous()
    As = torch.empty((256, 256), **f32)
    mi_fn = ((lambda src, dst: h.ap_mi_dev(src, dst, noise=1e-5, seed=args.seed)) if args.mi_method == "ap" else
             (lambda src, dst: h.bspline_mi_dev(src, dst, b, args.order, args.precision)))
    mi_fn(Xs, As)
    h.set_diagonal_dev(As, 0.0)
    h.maxmins_dev(As, R2=torch.empty_like(As))
    torch.cuda.synchronize(dev)

    clocks = ClockSampler(local)
    clocks.start()
    h.profile(True)
    st = {}
    t_all0 = time.perf_counter()
    st["mi"] = timed(lambda: mi_fn(X, A))
    st["diagonal"] = timed(lambda: h.set_diagonal_dev(A, 0.0))
    if args.no_eval:
        st["mcp234"] = timed(lambda: h.maxmins_dev(A, R2=R2, R3=R3, R4=R4))
    else:  # the ensemble search below needs the three products too
        M1, M2, M3 = (torch.empty((n, n), **f32) for _ in range(3))
        st["mcp234"] = timed(lambda: h.maxmins_dev(A, M1, M2, M3, R2=R2, R3=R3, R4=R4))
    removed = [0]
    st["dpi"] = timed(lambda: removed.__setitem__(0, h.dpi_dev(A, D, 0.1)))
    ev = {}
    if not args.no_eval:
        # gold standard: the synthetic GRN's edges are positives, every other pair a negative
        _, E = M.synth_grn(n, 1, seed=args.seed, with_edges=True)
        Lb = torch.zeros((n, n), dtype=torch.int8, device=dev)
        Ed = torch.from_numpy(E.astype(np.int64)).to(dev)
        Lb[Ed[:, 0], Ed[:, 1]] = 1
        Lb[Ed[:, 1], Ed[:, 0]] = 1
        coeffs = np.array([(a, b_, c, 4 - a - b_ - c) for a in range(5) for b_ in range(5 - a)
                           for c in range(5 - a - b_)], dtype=np.float64) / 4.0  # 35 rows, step 0.25
        r = [None]
        h.eval_truth_dev(A, Lb)  # untimed: grows the evaluation workspace to this size
        h.combo_eval_dev(A, M1, M2, M3, Lb, coeffs[1:2])
        st["eval_mi"] = timed(lambda: r.__setitem__(0, h.eval_truth_dev(A, Lb)))
        ev["mi"] = r[0]
        st["eval_mcp2"] = timed(lambda: r.__setitem__(0, h.eval_truth_dev(R2, Lb)))
        ev["mcp2"] = r[0]
        st["combo_search"] = timed(lambda: r.__setitem__(0, h.combo_eval_dev(A, M1, M2, M3, Lb, coeffs)))
        ev["combo"] = r[0]
        h.combo_stouffer_eval_dev(A, M1, M2, M3, Lb, coeffs[1:2])  # untimed: workspace
        st["combo_stouffer_search"] = timed(
            lambda: r.__setitem__(0, h.combo_stouffer_eval_dev(A, M1, M2, M3, Lb, coeffs)))
        ev["combo_stouffer"] = r[0]
        ev["coeffs"] = coeffs
        if args.split_iters > 0:
            # the eval_mcpnet app's semi-supervised evaluation: shuffled train / test splits
            entries = ev["mi"][2] + ev["mi"][3]
            tcs = M.train_counts(entries)
            h.split_aupr_dev(R2, Lb, 1, tcs[:1])  # untimed: workspace
            st["split_aupr_mcp2"] = timed(lambda: r.__setitem__(0, h.split_aupr_dev(R2, Lb, args.split_iters, tcs)))
            ev["split_aupr"] = r[0]
            st["split_combo_stouffer"] = timed(lambda: r.__setitem__(0, h.split_combo_eval_dev(
                A, M1, M2, M3, Lb, coeffs, args.split_iters, tcs, "exclude_diagonal")))
            ev["split_combo"] = r[0]
            ev["split_entries"] = entries
    tfst = {}
    if args.tfs > 0:
        # --tf-input: a seeded set of TF genes (the synthetic GRN has no TF annotation)
        t = min(args.tfs, n)
        tf_idx = np.sort(np.random.default_rng(args.seed + 7).choice(n, size=t, replace=False)).astype(np.int32)
        tfs = np.full(n, -np.inf, np.float32)
        tfs[tf_idx] = np.inf
        Rt = [torch.empty((t, n), **f32) for _ in range(3)]
        Tm, M1t, M2t, M3t = (torch.empty((t, n), **f32) for _ in range(4))
        tf_stages = {
            "mcp_tf": lambda: [h.mcp_tf_dev(A, tfs, k, k - 1, R=Rt[k - 2]) for k in (2, 3, 4)],
            "maxmins_tf": lambda: h.maxmins_tf_dev(A, tfs, Tm, M1t, M2t, M3t),
            "dpi_tf": lambda: tfst.__setitem__("removed", h.dpi_tf_dev(A, D, tfs, 0.1)),
        }
        if not args.no_eval:
            rows_d = torch.from_numpy(tf_idx).to(dev)
            Lt = Lb[rows_d.long()].contiguous()
            ct = torch.from_numpy((tfs > 0).astype(np.uint8)).to(dev)
            tf_stages["tf_eval_mcp2"] = lambda: tfst.__setitem__("mcp2", h.eval_truth_dev(Rt[0], Lt, "tf", rows_d, ct))
            tf_stages["tf_combo_search"] = lambda: tfst.__setitem__(
                "combo", h.combo_eval_dev(Tm, M1t, M2t, M3t, Lt, coeffs, "tf", rows_d, ct))
            tf_stages["tf_combo_stouffer_search"] = lambda: tfst.__setitem__(
                "combo_stouffer", h.combo_stouffer_tf_eval_dev(Tm, M1t, M2t, M3t, Lt, coeffs, "tf", rows_d, ct))
        for key, fn in tf_stages.items():
            fn()  # untimed: grows this stage's workspace
            st[key] = timed(fn)
        tfst["t"] = t
    iters = None
    if args.closure:
        Cl = torch.empty((n, n), **f32)
        it = [0]
        st["closure"] = timed(lambda: it.__setitem__(0, h.closure_dev(A, Cl, 64)))
        iters = it[0]
        del Cl
    wall = time.perf_counter() - t_all0
    prof = h.profile_report()
    h.profile(False)
    clk = clocks.stop()

    pairs = n * (n - 1) // 2
    mi_flops = 2.0 * b * b * m * pairs
    w_ms = prof.get("bspline_weights_f8", prof.get("bspline_weights16", {})).get("ms", float("nan"))
    tc_ms = prof.get("mi_tc", {}).get("ms", float("nan"))
    ldw = -(-m // 64) * 64
    w_bytes = n * m * 4 + 2 * n * b * ldw * 2
    mm_ms = st["mcp234"] * 1e3
    # executed min/max work: M1 and M3 symmetric (n^3 / 2 triples each), M2 full (n^3)
    mm_ops_exec = 2.0 * (0.5 + 1.0 + 0.5) * n ** 3
    stages = {}
    if args.mi_method == "ap":
        stages["ap_mi"] = {"ms": st["mi"] * 1e3, "pairs_per_s": n * (n + 1) / 2 / st["mi"],
                           "kernels": {k: v for k, v in prof.items() if k.startswith("ap_")}}
    else:
        stages["bspline_weights"] = {"ms": w_ms, "GB/s": w_bytes / (w_ms / 1e3) / 1e9,
                                     "frac_hbm": w_bytes / (w_ms / 1e3) / hbm}
        stages["mi_tc"] = {"ms": tc_ms, "TFLOP/s_algorithmic": mi_flops / (tc_ms / 1e3) / 1e12,
                           "frac_tensor_algorithmic": mi_flops / (tc_ms / 1e3) / tc_peak,
                           # BF16-equivalent issued work: x3 for the 16-bit split, x2 for bf16f8
                           # (one BF16 pass + an E4M3 pass of twice the flops at twice the rate)
                           "frac_tensor_issued": {"bf16x3": 3.0, "fp16x3": 3.0, "bf16f8": 2.0, "bf16": 1.0,
                                                  "fp16": 1.0}.get(args.precision, 0.0)
                           * mi_flops * (128 / 120) / (tc_ms / 1e3) / tc_peak}
    stages["maxmin_M1_M2_M3_with_ratios"] = {"ms": mm_ms, "Gop/s_executed": mm_ops_exec / (mm_ms / 1e3) / 1e9,
                                             "frac_alu_peak": mm_ops_exec / (mm_ms / 1e3) / alu_peak}
    dpi_ms = st["dpi"] * 1e3
    stages["dpi"] = {"ms": dpi_ms, "removed": removed[0],
                     "frac_alu_peak": 2.0 * 0.5 * n ** 3 / (dpi_ms / 1e3) / alu_peak}
    if args.closure:
        cl_ms = st["closure"] * 1e3
        stages["closure"] = {"ms": cl_ms, "iterations": iters,
                             "frac_alu_peak": 2.0 * 0.5 * n ** 3 * iters / (cl_ms / 1e3) / alu_peak}
    if not args.no_eval:
        npos, nneg = ev["mi"][2], ev["mi"][3]
        lower = n * (n - 1) // 2
        # labels read by the count, gather and rank passes over the lower triangle; every
        # negative's and positive's score read once
        ev_bytes = 3 * lower + 4 * (npos + nneg)
        for key in ("eval_mi", "eval_mcp2"):
            e_ms = st[key] * 1e3
            stages[key] = {"ms": e_ms, "aupr": ev[key[5:]][0], "auroc": ev[key[5:]][1], "n_pos": npos,
                           "n_neg": nneg, "GB/s": ev_bytes / (e_ms / 1e3) / 1e9,
                           "frac_hbm": ev_bytes / (e_ms / 1e3) / hbm}
        for key in ("combo_search", "combo_stouffer_search"):
            pr, roc, best = ev["combo" if key == "combo_search" else "combo_stouffer"]
            stages[key] = {"ms": st[key] * 1e3, "rows": len(ev["coeffs"]),
                           "ms_per_row": st[key] * 1e3 / (len(ev["coeffs"]) - 1),
                           "best_row": int(best), "best_coeffs": ev["coeffs"][best].tolist(),
                           "best_aupr": float(pr[best]), "best_auroc": float(roc[best])}
    if args.tfs > 0:
        t = tfst["t"]
        # executed triples: MCP2 T(x)A; MCP3 A(x)A (symmetric) + T(x)M1; MCP4 A(x)A + T(x)A + M2(x)M1
        # (every masked product runs over the t TF columns)
        tri = {"mcp_tf": n * n * t + 4.0 * t * t * n, "maxmins_tf": 0.5 * n * n * t + 3.0 * t * t * n,
               "dpi_tf": 0.5 * n ** 3 + 0.5 * n * n * t}
        for key in ("mcp_tf", "maxmins_tf", "dpi_tf"):
            ms_ = st[key] * 1e3
            stages[key] = {"ms": ms_, "tfs": t, "Gop/s_executed": 2 * tri[key] / (ms_ / 1e3) / 1e9,
                           "frac_alu_peak": 2 * tri[key] / (ms_ / 1e3) / alu_peak}
        stages["dpi_tf"]["removed"] = tfst["removed"]
        if not args.no_eval:
            stages["tf_eval_mcp2"] = {"ms": st["tf_eval_mcp2"] * 1e3, "aupr": tfst["mcp2"][0],
                                      "auroc": tfst["mcp2"][1], "n_pos": tfst["mcp2"][2], "n_neg": tfst["mcp2"][3]}
            for key, k in (("tf_combo_search", "combo"), ("tf_combo_stouffer_search", "combo_stouffer")):
                pr, roc, best = tfst[k]
                stages[key] = {"ms": st[key] * 1e3, "rows": len(coeffs),
                               "ms_per_row": st[key] * 1e3 / (len(coeffs) - 1), "best_row": int(best),
                               "best_coeffs": coeffs[best].tolist(), "best_aupr": float(pr[best]),
                               "best_auroc": float(roc[best])}
    if not args.no_eval and args.split_iters > 0:
        k = args.split_iters
        full, tr, te = ev["split_aupr"]
        stages["split_aupr_mcp2"] = {"ms": st["split_aupr_mcp2"] * 1e3, "iterations": k, "parts": int(tr.shape[1]),
                                     "entries": int(ev["split_entries"]),
                                     "ms_per_iteration": st["split_aupr_mcp2"] * 1e3 / k, "full_aupr": full,
                                     "train_aupr_mean": tr.mean(0).tolist(), "test_aupr_mean": te.mean(0).tolist()}
        res, best = ev["split_combo"]
        stages["split_combo_stouffer"] = {"ms": st["split_combo_stouffer"] * 1e3, "iterations": k,
                                          "rows": len(coeffs), "ms_per_iteration": st["split_combo_stouffer"] * 1e3 / k,
                                          "test_aupr_mean": res[..., 1].mean(0).tolist(),
                                          "stouffer_test_aupr_mean": res[..., 3].mean(0).tolist()}
    line = {"mode": "pipeline", "genes": n, "samples": m, "mi_method": args.mi_method, "precision": args.precision,
            "stage_s": st, "wall_s": wall, "stages": stages, "closure_iterations": iters, "clocks": clk,
            "kernel_profile": prof, "sms": sms}
    if not args.no_cpu:
        sampler = CpuMiSampler(min(n, args.cpu_genes), m, args.seed)
        v, info = sampler.run(args.cpu_seconds / 2)
        from oracle import oracle as O
        P = O.port()
        Ah = A.cpu().numpy()
        t0 = time.perf_counter()
        P.maxmin(Ah[:1], Ah)
        per_row = max(time.perf_counter() - t0, 1e-4)
        rows = int(max(1, min(n, (args.cpu_seconds / 2) / per_row)))
        t0 = time.perf_counter()
        P.maxmin(Ah[:rows], Ah)
        mm_row_s = (time.perf_counter() - t0) / rows
        cpu_mi_s = pairs / v
        cpu_mm_s = mm_row_s * n * (0.5 + 1.0 + 0.5 + 0.5)  # M1, M2, M3 as the reference's SYMM patterns + DPI bound
        cpu_ev_s = None
        if not args.no_eval:
            # compute_aupr_auroc on a row slab of the lower triangle, scaled by entries
            Lh = Lb.cpu().numpy()
            er = min(n, 4096)
            t0 = time.perf_counter()
            P.eval_truth(Ah[:er], Lh[:er], "lower")
            cpu_ev_s = (time.perf_counter() - t0) * (n * (n - 1) / 2) / (er * (er - 1) / 2)
        line["cpu_baseline"] = {"kind": sampler.kind, "cores": info["threads"],
                                "mi_s_extrapolated": cpu_mi_s, "maxmin_dpi_s_extrapolated": cpu_mm_s,
                                "eval_one_matrix_s_extrapolated": cpu_ev_s,
                                "total_s_extrapolated": cpu_mi_s + cpu_mm_s,
                                "sample": f"MI {sampler.describe(info)}; max-min rows 0..{rows} x {n} x {n} "
                                          f"({mm_row_s:.3f} s/row); DPI counted as one symmetric product "
                                          "(an upper bound: the reference's DPI scan exits early)"}
    h.close()
    return line


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mcpgpu", choices=["mcpgpu", "reference"])
    ap.add_argument("--genes", type=int, default=20000)
    ap.add_argument("--samples", type=int, default=2000)
    ap.add_argument("--bins", type=int, default=10)
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--precision", default="bf16f8", choices=["fp32", "bf16", "bf16x3", "fp16", "fp16x3", "bf16f8"])
    ap.add_argument("--compare", default="bf16x3",
                    help="comma-separated tensor-core forms timed beside the headline one on the same input "
                         "('' for none)")
    ap.add_argument("--mi-method", default="bspline", choices=["bspline", "ap"],
                    help="with --pipeline: B-spline MI (default) or adaptive-partitioning MI (U[0,1e-5) noise)")
    ap.add_argument("--seed", type=int, default=20260001)
    ap.add_argument("--fp32-steps", type=int, default=2)
    ap.add_argument("--maxmin-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-maxmin", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the one-off 32,768 x 4,096 pipeline leg of the default run")
    ap.add_argument("--pipeline", action="store_true",
                    help="run the whole compute core once, stage by stage (defaults to 32768 x 4096)")
    ap.add_argument("--closure", action="store_true", help="with --pipeline: add the max-capacity closure")
    ap.add_argument("--split-iters", type=int, default=0,
                    help="with --pipeline: add the eval_mcpnet split evaluation (MCP2 split AUPRs and the Stouffer "
                         "split coefficient search) over this many shuffles")
    ap.add_argument("--tfs", type=int, default=0,
                    help="with --pipeline: add the --tf-input stages (TF MCP2/3/4, TF max-min products, TF DPI, "
                         "TF evaluation and searches) for this many seeded TF genes")
    ap.add_argument("--no-eval", action="store_true",
                    help="with --pipeline: skip the gold-standard evaluation and the ensemble coefficient search")
    ap.add_argument("--cpu-genes", type=int, default=8192,
                    help="with --pipeline: genes of the CPU MI sample (its weights are built on the host)")
    args = ap.parse_args(argv)
    if args.pipeline and "--genes" not in (argv or sys.argv):
        args.genes, args.samples = 32768, 4096
    if args.warmup < 3:
        args.warmup = 3  # timing rule: at least 3 warm-up steps
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")
    try:
        if args.impl == "reference":
            reference_arm(args, ws, rank)
        elif args.pipeline:
            pipeline_arm(args, ws, rank, local)
        else:
            gpu_arm(args, ws, rank, local)
    finally:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
