"""Benchmark: 2D r2c FFT at 16384^2, FP64 drop-in (float-float arithmetic) on GB300.

One step = one forward 2D r2c transform of a 16384 x 16384 FP64 array in the
reference's padded layout (16384 x 16386 doubles, 2.148 GB), out of place
from a pristine input buffer into the output buffer, both resident in HBM.
value = algorithmic HBM bytes per step (4*S, S = nx*(ny/2+1)*16 B: the row
pass reads and writes S, the column pass reads and writes S) / time.

e2e = the same metric through the C ABI with host buffers
(hpxfft_execute_r2c_host: pinned host array -> device -> transform -> host).

--impl reference times the reference's algorithm on the host cores: the FP64
C restatement of hpxfft::shared::loop (oracle/), because the reference itself
(HPX + FFTW) cannot be built on this machine.

Multi-GPU: the path does not shard on one box; --gpus N runs N independent
replicas (one per rank) and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "hpx-fft_gb300", "python"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

METRIC = "2D r2c FFT ms & HBM GB/s at 16384²: FP64 drop-in vs FP32/split-BF16 at rel-L2 err"
UNIT = "GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=16384, help="nx = ny")
    ap.add_argument("--nx", type=int, default=0, help="rows (overrides --n; profiling cases)")
    ap.add_argument("--ny", type=int, default=0, help="columns (overrides --n; profiling cases)")
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "f64-native"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.nx = args.nx or args.n
    args.ny = args.ny or args.n
    return args


def workload_input(nx: int, ny: int, seed: int = 1234) -> np.ndarray:
    """uniform[-1,1) plus four integer-frequency sinusoids of amplitude 10,
    in the padded nx x 2*(ny/2+1) layout (float64)."""
    rng = np.random.default_rng(seed)
    nc = 2 * (ny // 2 + 1)
    x = np.zeros((nx, nc), dtype=np.float64)
    x[:, :ny] = rng.uniform(-1.0, 1.0, (nx, ny))
    i = np.arange(nx, dtype=np.float64)[:, None]
    j = np.arange(ny, dtype=np.float64)[None, :]
    for _ in range(4):
        fx, fy = rng.integers(1, max(2, min(nx, ny) // 2), size=2)
        # 1024 rows at a time to bound the temporary
        for r0 in range(0, nx, 1024):
            x[r0:r0 + 1024, :ny] += 10.0 * np.sin(2 * np.pi * (fx * i[r0:r0 + 1024] / nx + fy * j / ny))
    return x


def algorithmic_bytes(nx: int, ny: int, real_bytes: int) -> float:
    S = nx * (ny // 2 + 1) * 2 * real_bytes
    return 4.0 * S


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        smax = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, name in enumerate(names):
                if s[5 + k].lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(self.samples),
        }


def measured_peak_hbm():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(nx: int, ny: int, host_input: np.ndarray, threads: int) -> dict:
    """The oracle (FP64 C restatement of shared::loop) on the host cores, one
    full transform of the same input."""
    import oracle

    work = host_input.copy()
    t0 = time.perf_counter()
    oracle.fft_2d_r2c(work, nthreads=threads)
    dt = time.perf_counter() - t0
    return {
        "value": algorithmic_bytes(nx, ny, 8) / dt / 1e9,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"one full {nx}x{ny} FP64 2D r2c ({dt:.2f} s) by the C restatement of hpxfft::shared::loop, "
                  f"{threads} threads; HPX and FFTW are not installed, so the reference binary cannot run",
        "seconds": dt,
    }


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import importlib.util

    spec = importlib.util.spec_from_file_location("hpxfft_build", os.path.join(REPO, "hpx-fft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_oracle()
    import oracle

    nx, ny = args.nx, args.ny
    threads = os.cpu_count() or 1
    x = workload_input(nx, ny)
    work = np.empty_like(x)
    for _ in range(args.warmup):
        np.copyto(work, x)
        oracle.fft_2d_r2c(work, nthreads=threads)
    times = []
    for _ in range(args.steps):
        np.copyto(work, x)
        t0 = time.perf_counter()
        oracle.fft_2d_r2c(work, nthreads=threads)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    value = algorithmic_bytes(nx, ny, 8) / t / 1e9
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: uniform[-1,1) + 4 integer-frequency sinusoids of amplitude 10, seed 1234",
        "config": {"workload": f"2d_r2c_fp64_{nx}x{ny}", "nx": nx, "ny": ny, "layout": "padded in-place vector_2d",
                   "implementation": "C restatement of hpxfft::shared::loop (FFTW/HPX unavailable)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full {nx}x{ny} FP64 transforms, {threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import importlib.util

    spec = importlib.util.spec_from_file_location("hpxfft_build", os.path.join(REPO, "hpx-fft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    if rank == 0:
        b.build_all()
    if world > 1:
        torch.distributed.barrier()
    b.build_all()
    import hpxfft

    nx, ny = args.nx, args.ny
    prec = args.precision
    real_bytes = 4 if prec == "f32" else 8
    nc = 2 * (ny // 2 + 1)
    x64 = workload_input(nx, ny, seed=1234 + rank)
    host = x64.astype(np.float32) if prec == "f32" else x64
    dev_in = torch.from_numpy(host).cuda()
    dev_out = torch.empty_like(dev_in)
    stream = torch.cuda.current_stream()
    plan = hpxfft.Plan(nx, nc, 1, prec, "estimate")
    plan.set_stream(stream.cuda_stream)

    # warm-up
    for _ in range(args.warmup):
        plan.execute_oop(dev_in.data_ptr(), dev_out.data_ptr())
    torch.cuda.synchronize()
    plan.timing_reset()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            plan.execute_oop(dev_in.data_ptr(), dev_out.data_ptr())
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    stats = plan.timing_stats()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    B = algorithmic_bytes(nx, ny, real_bytes)
    value = world * B / (ms * 1e-3) / 1e9

    # accuracy of the timed output against the oracle on a bounded sample:
    # rows of the spectrum are checked through the full-size property
    # (Parseval) and, at rank 0, against the oracle for the whole transform
    out = dev_out.cpu().numpy()
    spec_out = out.view(np.complex128 if prec != "f32" else np.complex64)

    # end to end through the host-buffer C ABI call
    pinned = torch.empty((nx, nc), dtype=torch.float64 if prec != "f32" else torch.float32).pin_memory()
    host_src = torch.from_numpy(host)
    e2e_times = []
    for i in range(args.e2e_steps + 1):
        pinned.copy_(host_src)
        plan.execute_host(pinned.numpy())
        if i > 0:
            e2e_times.append(plan.measurement("e2e"))
    e2e_s = sum(e2e_times) / len(e2e_times)
    h2d = plan.measurement("h2d")
    d2h = plan.measurement("d2h")

    peak, peak_kind = measured_peak_hbm()
    dominant = "row" if stats["first"] >= stats["second"] else "column"
    dom_t = max(stats["first"], stats["second"])
    per_kernel_bytes = B / 2.0  # each pass reads S and writes S
    achieved = per_kernel_bytes / dom_t / 1e9 if dom_t > 0 else 0.0

    line = None
    if rank == 0:
        import oracle

        rel = None
        cpu = None
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            cpu = cpu_baseline(nx, ny, x64, threads)
            ref = x64.copy()
            oracle.fft_2d_r2c(ref, nthreads=threads)
            refc = ref.view(np.complex128)
            rel = float(np.linalg.norm((spec_out.astype(np.complex128) - refc).ravel()) / np.linalg.norm(refc.ravel()))
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if prec != "f32" else "f32",
            "data": "synthetic: uniform[-1,1) + 4 integer-frequency sinusoids of amplitude 10, seed 1234+rank",
            "config": {
                "workload": f"2d_r2c_{prec}_{nx}x{ny}",
                "nx": nx, "ny": ny,
                "precision": {"f64": "FP64 storage, float-float arithmetic", "f32": "FP32",
                              "f64-native": "FP64 storage, DFMA arithmetic"}[prec],
                "layout": "padded vector_2d (n x 2*(n/2+1)), output [kx][ky]",
                "step": "out-of-place forward transform, input and output resident in HBM",
                "l2": "no flush: input and output are 2.1 GB each, far above the 129 MB L2",
                "parallelism": "replicas" if world > 1 else "single GPU",
                "rel_l2_vs_oracle": rel,
            },
            "gpu_launches": 2 * args.steps,
            "kernels_ms": {"row_r2c": 1e3 * stats["first"], "col_c2c": 1e3 * stats["second"],
                           "count": stats["count"]},
            "roofline": {
                "bound": "hbm",
                "kernel": "row_r2c_kernel" if dominant == "row" else "col_kernel",
                "achieved": achieved,
                "peak": peak,
                "peak_kind": peak_kind,
                "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": None,
                "algorithmic_bytes_per_launch": per_kernel_bytes,
            },
            "e2e": {
                "value": world * B / e2e_s / 1e9,
                "unit": UNIT,
                "h2d_bytes_per_step": int(nx * nc * real_bytes),
                "d2h_bytes_per_step": int(nx * nc * real_bytes),
                "ms_per_step": 1e3 * e2e_s,
                "h2d_ms": 1e3 * h2d,
                "d2h_ms": 1e3 * d2h,
            },
            "clocks": clk.summary(),
        }
        if cpu is not None:
            line["cpu_baseline"] = {k: v for k, v in cpu.items() if k != "seconds"}
        print(json.dumps(line), flush=True)
    plan.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
