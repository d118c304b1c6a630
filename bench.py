"""Benchmark: 2D r2c FFT at 16384^2, FP64 drop-in (float-float arithmetic) on GB300.

One step = one forward 2D r2c transform of a 16384 x 16384 FP64 array in the
reference's padded layout (16384 x 16386 doubles, 2.148 GB), out of place
from a pristine input buffer into the output buffer, both resident in HBM.
value = algorithmic HBM bytes per step (4*S, S = nx*(ny/2+1)*16 B: the row
pass reads and writes S, the column pass reads and writes S) / time.

e2e = the same metric through the C ABI with host buffers
(hpxfft_execute_r2c_host on a page-locked host array: chunked copies over
the host link overlapped with the kernels, timed from before the first byte
leaves the host to after the last byte lands back).

--impl reference times the reference's algorithm on the host cores: the FP64
C restatement of hpxfft::shared::loop (oracle/), because the reference itself
(HPX + FFTW) cannot be built on this machine.

Multi-GPU: the path does not shard on one box; --gpus N runs N independent
replicas (one per rank) and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import math
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
NOMINAL_HBM_GBS = 7900.0  # GB300 HBM3e, nominal
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
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "bf16x3", "f64-native"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the FP32 / batch / backward sections")
    ap.add_argument("--batch-only", action="store_true", help="only the uneven FP32 batch (profiling)")
    ap.add_argument("--scale-only", action="store_true", help="only the 32768^2 FP64 section (profiling)")
    ap.add_argument("--prime-only", action="store_true",
                    help="only the prime-length transforms beside cuFFT (profiling; --nx/--ny set the size)")
    ap.add_argument("--batch-count", type=int, default=1024)
    ap.add_argument("--batch-flag", default="measure", choices=["estimate", "measure"])
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


def workload_name(nx: int, ny: int, prec: str = "f64") -> str:
    """The workload label both arms print (same transform, size and input)."""
    return f"2d_r2c_{prec}_{nx}x{ny}"


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


def pocketfft_context(nx: int, ny: int, host_input: np.ndarray, threads: int):
    """scipy.fft.rfft2 (pocketfft, FP64) of the same input on the same host
    cores: a production CPU FFT beside the restatement, since FFTW (the
    reference's FFT library) is not installed.  Context only, timed outside
    every timed region; None when scipy is missing or the run fails."""
    try:
        import scipy.fft

        x = np.ascontiguousarray(host_input[:, :ny])
        t0 = time.perf_counter()
        out = scipy.fft.rfft2(x, workers=threads)
        dt = time.perf_counter() - t0
        del out, x
    except Exception:
        return None
    return {
        "value": algorithmic_bytes(nx, ny, 8) / dt / 1e9,
        "unit": UNIT,
        "cores": threads,
        "sample": f"one {nx}x{ny} FP64 scipy.fft.rfft2 ({dt:.2f} s, workers={threads}): pocketfft standing in "
                  f"for FFTW, which is not installed",
    }


def _cpulist(text: str) -> set:
    cpus = set()
    for part in text.strip().split(","):
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        elif part:
            cpus.add(int(part))
    return cpus


def gpu_local_cpus(torch, dev: int):
    """(NUMA node, this process's CPUs on it) of the host memory next to GPU
    `dev`, from sysfs; (None, None) when unknown."""
    try:
        p = torch.cuda.get_device_properties(dev)
        bus = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            node = int(f.read())
        if node < 0:
            return None, None
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            cpus = _cpulist(f.read()) & os.sched_getaffinity(0)
        return node, (cpus or None)
    except Exception:
        return None, None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def replica_max_ms(ms: float, world: int) -> float:
    """The slowest replica's step time (max over ranks): with N independent
    replicas the whole-job rate is N x one replica's bytes over this time."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


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
        "config": {"workload": workload_name(nx, ny), "nx": nx, "ny": ny, "layout": "padded in-place vector_2d",
                   "implementation": "C restatement of hpxfft::shared::loop (FFTW/HPX unavailable)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full {nx}x{ny} FP64 transforms, {threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    pocket = pocketfft_context(nx, ny, x, threads)
    if pocket is not None:
        line["cpu_pocketfft"] = pocket
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
    f32 = prec in ("f32", "bf16x3")
    real_bytes = 4 if f32 else 8
    nc = 2 * (ny // 2 + 1)
    x64 = workload_input(nx, ny, seed=1234 + rank)
    host = x64.astype(np.float32) if f32 else x64
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
    ms = replica_max_ms(ms, world)
    B = algorithmic_bytes(nx, ny, real_bytes)
    value = world * B / (ms * 1e-3) / 1e9

    # accuracy of the timed output against the oracle on a bounded sample:
    # rows of the spectrum are checked through the full-size property
    # (Parseval) and, at rank 0, against the oracle for the whole transform
    out = dev_out.cpu().numpy()
    spec_out = out.view(np.complex64 if f32 else np.complex128)

    # end to end through the host-buffer C ABI call, on a page-locked buffer
    # allocated and filled by this thread while it runs on the CPUs of the
    # GPU's own NUMA node (the buffer's pages land in the memory next to the
    # GPU instead of crossing to the other node on every transfer)
    numa_node, local_cpus = gpu_local_cpus(torch, local)
    saved_affinity = os.sched_getaffinity(0)
    if local_cpus:
        os.sched_setaffinity(0, local_cpus)
    try:
        pinned = torch.empty((nx, nc), dtype=torch.float32 if f32 else torch.float64).pin_memory()
        host_src = torch.from_numpy(host)
        e2e_times = []
        for i in range(args.e2e_steps + 1):
            pinned.copy_(host_src)
            plan.execute_host(pinned.numpy())
            if i > 0:
                e2e_times.append(plan.measurement("e2e"))
    finally:
        os.sched_setaffinity(0, saved_affinity)
    e2e_s = sum(e2e_times) / len(e2e_times)
    h2d = plan.measurement("h2d")
    d2h = plan.measurement("d2h")
    zero_copy = plan.measurement("host_zero_copy") == 1.0
    pipelined = plan.measurement("host_pipelined") == 1.0

    peak, peak_kind = measured_peak_hbm()
    # per launch: every kernel of the step reads S and writes S (B / 2)
    steps = int(plan.measurement("column_steps"))
    kernels = {"row_r2c_kernel": stats["first"]}
    if steps == 2:
        step_kernel = {"bf16x3": "colstep_tc_kernel", "f64": "colstep_warp_kernel",
                       "f32": "colstep_direct_kernel"}.get(prec, "colstep_kernel")
        kernels[f"{step_kernel} (A)"] = plan.measurement("mean_col_step_a")
        kernels[f"{step_kernel} (B)"] = plan.measurement("mean_col_step_b")
    else:
        kernels["col_kernel"] = stats["second"]
    dominant = max(kernels, key=kernels.get)
    traffic = profiled_traffic(prec, nx, ny, dominant)
    # DRAM bytes of the whole step from the committed per-kernel ncu traffic
    # (None unless every kernel of the step was captured)
    step_traffic = [profiled_traffic(prec, nx, ny, k) for k in kernels]
    step_dram = sum(step_traffic) if step_traffic and all(t is not None for t in step_traffic) else None
    dom_t = kernels[dominant]
    per_kernel_bytes = B / 2.0
    achieved = per_kernel_bytes / dom_t / 1e9 if dom_t > 0 else 0.0

    line = None
    if rank == 0:
        import oracle

        rel = None
        cpu = None
        oracle_ref = None
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            cpu = cpu_baseline(nx, ny, x64, threads)
            pocket = pocketfft_context(nx, ny, x64, threads)
            ref = x64.copy()
            oracle.fft_2d_r2c(ref, nthreads=threads)
            refc = ref.view(np.complex128)
            rel = float(np.linalg.norm((spec_out.astype(np.complex128) - refc).ravel()) / np.linalg.norm(refc.ravel()))
            oracle_ref = refc
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
            "dtype": "f32" if f32 else "f64",
            "data": "synthetic: uniform[-1,1) + 4 integer-frequency sinusoids of amplitude 10, seed 1234+rank",
            "config": {
                "workload": workload_name(nx, ny, prec),
                "nx": nx, "ny": ny,
                "precision": {"f64": "FP64 storage, float-float arithmetic", "f32": "FP32",
                              "bf16x3": "FP32 storage, split-BF16 tensor-core column stage",
                              "f64-native": "FP64 storage, DFMA arithmetic"}[prec],
                "layout": "padded vector_2d (n x 2*(n/2+1)), output [kx][ky]",
                "step": "out-of-place forward transform, input and output resident in HBM",
                "l2": ("no flush: input and output are %.2f GB each, above the 129 MB L2" % (nx * nc * real_bytes / 1e9)
                       if nx * nc * real_bytes > 129e6 else "no flush: arrays smaller than L2, numbers are L2-warm"),
                "parallelism": "replicas" if world > 1 else "single GPU",
                "rel_l2_vs_oracle": rel,
            },
            "gpu_launches": (1 + steps) * args.steps,
            "kernels_ms": dict({k: 1e3 * v for k, v in kernels.items()}, count=stats["count"]),
            "gflops": world * 2.5 * nx * ny * math.log2(nx * ny) / (ms * 1e-3) / 1e9,
            "frac_of_nominal_hbm": value / NOMINAL_HBM_GBS,
            "roofline": {
                "bound": "hbm",
                "kernel": dominant,
                "achieved": achieved,
                "peak": peak,
                "peak_kind": peak_kind,
                "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": traffic,
                "traffic_source": "profiles/dram_traffic_%s_%d.md (ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                  "scaled to a full launch)" % (prec, nx) if traffic else None,
                "algorithmic_bytes_per_launch": per_kernel_bytes,
                # the step as a whole: 2 S / t (one read and one write of the
                # array; a two-pass design reaches at most half the peak on
                # this count) and the DRAM bytes ncu measured for its kernels
                "step_2s_gbps": value / 2.0,
                "step_2s_frac": value / 2.0 / peak,
                "step_dram_gbps": world * step_dram / (ms * 1e-3) / 1e9 if step_dram else None,
                "step_dram_frac": world * step_dram / (ms * 1e-3) / 1e9 / peak if step_dram else None,
            },
            "e2e": {
                "value": world * B / e2e_s / 1e9,
                "unit": UNIT,
                "h2d_bytes_per_step": int(nx * nc * real_bytes),
                "d2h_bytes_per_step": int(nx * nc * real_bytes),
                "ms_per_step": 1e3 * e2e_s,
                # every timed end-to-end step (the value is their mean; a
                # step disturbed by the host shows here)
                "ms_steps": [round(1e3 * t, 3) for t in e2e_times],
                "ms_median": 1e3 * statistics.median(e2e_times),
                "h2d_ms": 1e3 * h2d,
                "d2h_ms": 1e3 * d2h,
                "host_numa_node": numa_node,
                "host_path": ("pipelined: 8 strided host-to-device copies (one per group of column-step-A rows) "
                              "overlapped with the row and step-A kernels, 8 device-to-host copies overlapped with "
                              "step B" if pipelined else
                              "zero-copy: the row pass reads and the last column step writes the page-locked host "
                              "buffer over the host link" if zero_copy else "staged through a device buffer"),
            },
            "clocks": clk.summary(),
        }
        if cpu is not None:
            line["cpu_baseline"] = {k: v for k, v in cpu.items() if k != "seconds"}
            if pocket is not None:
                line["cpu_pocketfft"] = pocket
        if not args.no_extras and world == 1:
            line["extras"] = extras(torch, hpxfft, args, x64, oracle_ref if cpu is not None else None, peak)
        print(json.dumps(line), flush=True)
    plan.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def _time_steps(torch, stream, fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def profiled_traffic(prec, nx, ny, label):
    """DRAM bytes per launch of kernel `label` from the committed ncu summary
    for this precision and size (None when there is none)."""
    if nx != ny:
        return None
    path = os.path.join(REPO, "profiles", f"dram_traffic_{prec}_{nx}.md")
    if not os.path.exists(path):
        return None
    name = label.split(" ")[0]
    step = {"(A)": "(step A)", "(B)": "(step B)"}.get(label.split(" ")[-1]) if " " in label else None
    col = None
    for line in open(path):
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if col is None:
            col = next((i for i, c in enumerate(cells) if c.startswith("traffic per")), None)
            continue
        if len(cells) <= col or not cells[0].startswith("`" + name):
            continue
        if step and step not in cells[0]:
            continue
        try:
            return float(cells[col])
        except ValueError:
            return None
    return None


def batch_workload(torch, hpxfft, stream, count, flag, steps, warm, peak):
    """`count` FP32 instances, nx and ny drawn independently from the
    2^k, 3*2^k, 5*2^k sizes between 256 and 4096 (seeded), uniform[-1,1)
    per-instance data, one persistent graph-replayed launch per step."""
    sizes = [256, 384, 512, 640, 768, 1024, 1536, 2048, 2560, 3072, 4096]
    rng = np.random.default_rng(1024)
    shapes = [(int(rng.choice(sizes)), int(rng.choice(sizes))) for _ in range(count)]
    with hpxfft.Batch([a for a, _ in shapes], [2 * (b // 2 + 1) for _, b in shapes], "f32", flag) as bt:
        arena = torch.zeros(bt.arena_bytes // 4, dtype=torch.float32, device="cuda")
        src = torch.empty_like(arena)
        for i, ((r, c), off) in enumerate(zip(shapes, bt.offsets)):
            g = torch.Generator(device="cuda")
            g.manual_seed(7919 * i + 1)
            w = 2 * (c // 2 + 1)
            src[off // 4: off // 4 + r * w].view(r, w)[:, :c] = torch.rand((r, c), generator=g, device="cuda") * 2 - 1
        arena.copy_(src)
        del src
        bt.set_stream(stream.cuda_stream)
        ms = _time_steps(torch, stream, lambda: bt.execute(arena.data_ptr()), steps, warm)
        bt.synchronize()
        Bb = bt.measurement("algorithmic_bytes")
        res = {"ms": ms, "value": Bb / (ms * 1e-3) / 1e9, "unit": "GB/s",
               "frac_of_measured_hbm": Bb / (ms * 1e-3) / 1e9 / peak,
               "instances": count, "items": bt.measurement("items"),
               "tuned": {"flag": flag, "lag": bt.measurement("lag"), "ctas_per_sm": bt.measurement("ctas_per_sm"),
                         "plan_s": bt.measurement("plan")},
               "launches_per_step": 1, "cuda_graph": True,
               "note": "in place, so steps after the first transform the previous output"}
    del arena
    return res


def _rel_to_oracle(got, oracle_ref):
    d = got.astype(np.complex128) - oracle_ref
    return float(np.linalg.norm(d.ravel()) / np.linalg.norm(oracle_ref.ravel())), float(np.abs(d).max())


def cufft_side(torch, stream, x64, nx, ny, steps, warm, oracle_ref, peak):
    """cuFFT (through torch.fft.rfft2, out of place, unpadded input) on the
    same input in FP64 and FP32: a GPU library timed beside the product for
    context, never called by it.  value uses the same 4 S bytes as the
    product's lines."""
    res = {"library": f"cuFFT via torch.fft.rfft2 (torch {torch.__version__})"}
    for prec, dt, rb in (("f64", torch.float64, 8), ("f32", torch.float32, 4)):
        x = torch.from_numpy(np.ascontiguousarray(x64[:, :ny], dtype=np.float64 if rb == 8 else np.float32)).cuda()
        holder = {}

        def step():
            holder["y"] = torch.fft.rfft2(x)

        ms = _time_steps(torch, stream, step, steps, warm)
        B = algorithmic_bytes(nx, ny, rb)
        sec = {"ms": ms, "value": B / (ms * 1e-3) / 1e9, "unit": "GB/s", "frac_of_measured_hbm": B / (ms * 1e-3) / 1e9 / peak}
        if oracle_ref is not None:
            sec["rel_l2_vs_fp64_oracle"], sec["max_abs_err_vs_fp64_oracle"] = _rel_to_oracle(
                holder["y"].cpu().numpy(), oracle_ref)
        res[prec] = sec
        del x, holder
        torch.cuda.empty_cache()
    return res


def prime_sizes(torch, hpxfft, stream, steps, warm, peak, nx=16381, ny=16382):
    """16381 x 16382 (16381 and ny/2 = 8191 prime): Bluestein's convolution
    on both passes, FP64 (float-float) and FP32, beside cuFFT on the same
    input.  The error reference is cuFFT's FP64 output (the oracle's O(p^2)
    radix-p step is too slow at this size); value uses the same 4 S bytes."""
    nc = 2 * (ny // 2 + 1)
    g = torch.Generator(device="cuda")
    g.manual_seed(16381)
    x = torch.rand((nx, ny), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    ref = torch.fft.rfft2(x)
    res = {"workload": f"2d_r2c_{nx}x{ny}", "cufft": {}}
    for prec, dt, rb in (("f64", torch.float64, 8), ("f32", torch.float32, 4)):
        B = algorithmic_bytes(nx, ny, rb)
        xin = torch.zeros((nx, nc), dtype=dt, device="cuda")
        xin[:, :ny] = x.to(dt)
        xout = torch.empty_like(xin)
        with hpxfft.Plan(nx, nc, 1, prec, "estimate") as p:
            p.set_stream(stream.cuda_stream)
            ms = _time_steps(torch, stream, lambda: p.execute_oop(xin.data_ptr(), xout.data_ptr()), steps, warm)
            p.synchronize()
            got = torch.view_as_complex(xout.view(nx, nc // 2, 2).to(torch.float64))
            res[prec] = {"ms": ms, "value": B / (ms * 1e-3) / 1e9, "unit": "GB/s",
                         "frac_of_measured_hbm": B / (ms * 1e-3) / 1e9 / peak,
                         "bluestein_rows": p.measurement("bluestein_rows"),
                         "bluestein_columns": p.measurement("bluestein_columns"),
                         "rel_l2_vs_cufft_f64": float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))}
        del xin, xout, got
        xs = x.to(dt)
        holder = {}

        def step():
            holder["y"] = torch.fft.rfft2(xs)

        ms = _time_steps(torch, stream, step, steps, warm)
        res["cufft"][prec] = {"ms": ms, "value": B / (ms * 1e-3) / 1e9, "unit": "GB/s"}
        del xs, holder
        torch.cuda.empty_cache()
    del x, ref
    torch.cuda.empty_cache()
    return res


def scale_32768(torch, hpxfft, stream, warm, peak, n=32768):
    """The scale configuration's second size: the FP64 drop-in at 32768^2
    (8.6 GB in, 8.6 GB out), input uniform[-1,1) plus four integer-frequency
    sinusoids of amplitude 10 generated on the device (seeded), error
    against the oracle on the host cores."""
    import oracle

    nc = 2 * (n // 2 + 1)
    g = torch.Generator(device="cuda")
    g.manual_seed(32768)
    xin = torch.zeros((n, nc), dtype=torch.float64, device="cuda")
    xin[:, :n] = torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    rng = np.random.default_rng(32768)
    i = torch.arange(n, device="cuda", dtype=torch.float64)[:, None]
    j = torch.arange(n, device="cuda", dtype=torch.float64)[None, :]
    for _ in range(4):
        fx, fy = (int(v) for v in rng.integers(1, n // 2, size=2))
        for r0 in range(0, n, 4096):  # bounded temporaries
            xin[r0:r0 + 4096, :n] += 10.0 * torch.sin(2 * math.pi * ((fx * i[r0:r0 + 4096]) % n / n + (fy * j) % n / n))
    xout = torch.empty_like(xin)
    B = algorithmic_bytes(n, n, 8)
    with hpxfft.Plan(n, nc, 1, "f64", "estimate") as p:
        p.set_stream(stream.cuda_stream)
        ms = _time_steps(torch, stream, lambda: p.execute_oop(xin.data_ptr(), xout.data_ptr()), 3, warm)
        p.timing_reset()
        p.execute_oop(xin.data_ptr(), xout.data_ptr())
        st = p.timing_stats()
        p.synchronize()
    res = {"workload": workload_name(n, n), "ms": ms, "value": B / (ms * 1e-3) / 1e9, "unit": "GB/s",
           "frac_of_measured_hbm": B / (ms * 1e-3) / 1e9 / peak,
           "rows_ms": 1e3 * st["first"], "columns_ms": 1e3 * st["second"],
           "input": "uniform[-1,1) + 4 integer-frequency sinusoids of amplitude 10, generated on the device"}
    host = xin.cpu().numpy()
    got = xout.cpu().numpy().view(np.complex128)
    del xin, xout, i, j
    torch.cuda.empty_cache()
    oracle.fft_2d_r2c(host, nthreads=os.cpu_count() or 1)
    ref = host.view(np.complex128)
    num = den = mx = 0.0
    for r0 in range(0, n, 2048):  # chunked: no full-size temporaries
        d = got[r0:r0 + 2048] - ref[r0:r0 + 2048]
        num += float(np.vdot(d, d).real)
        den += float(np.vdot(ref[r0:r0 + 2048], ref[r0:r0 + 2048]).real)
        mx = max(mx, float(np.abs(d).max()))
    res["rel_l2_vs_fp64_oracle"], res["max_abs_err_vs_fp64_oracle"] = math.sqrt(num / den), mx
    return res


def extras(torch, hpxfft, args, x64, oracle_ref, peak):
    """The other workloads of this path, measured in the same run:
    FP32 at the same size (precision), 1024 uneven FP32 transforms in one
    persistent graph-replayed launch (batching), the adjoint on 64 FP32
    2048^2 arrays (differentiation), a shape with prime lengths
    (Bluestein's convolution on both passes), and the FP64 drop-in at 32768^2
    (the scale configuration's second size)."""
    out = {}
    stream = torch.cuda.current_stream()
    nx, ny = args.nx, args.ny
    nc = 2 * (ny // 2 + 1)
    steps, warm = max(3, args.steps), max(3, args.warmup)

    # the FP64 transform with native DFMA arithmetic instead of float-float
    # (HPXFFT_PREC_F64_NATIVE, runtime-planned kernels): the alternative the
    # float-float design is measured against
    xin = torch.from_numpy(x64).cuda()
    xout = torch.empty_like(xin)
    with hpxfft.Plan(nx, nc, 1, "f64-native", "estimate") as pn:
        pn.set_stream(stream.cuda_stream)
        ms = _time_steps(torch, stream, lambda: pn.execute_oop(xin.data_ptr(), xout.data_ptr()), 3, 1)
        pn.synchronize()
        B = algorithmic_bytes(nx, ny, 8)
        sec = {"workload": workload_name(nx, ny, "f64-native"), "ms": ms, "value": B / (ms * 1e-3) / 1e9,
               "unit": "GB/s", "frac_of_measured_hbm": B / (ms * 1e-3) / 1e9 / peak}
        if oracle_ref is not None:
            sec["rel_l2_vs_fp64_oracle"], sec["max_abs_err_vs_fp64_oracle"] = _rel_to_oracle(
                xout.cpu().numpy().view(np.complex128), oracle_ref)
        out["precision_f64_native"] = sec
    del xin, xout
    torch.cuda.empty_cache()
    out["cufft_side_comparison"] = cufft_side(torch, stream, x64, nx, ny, steps, warm, oracle_ref, peak)
    try:
        out["pipe_peaks"] = hpxfft.pipe_peaks()
    except Exception as exc:  # the measurement is context, not part of the step
        out["pipe_peaks"] = {"error": str(exc)}

    # precision: FP32 in and out (CUDA cores, and with the split-BF16 tensor-core
    # column stage), error against the FP64 oracle
    x32 = torch.from_numpy(x64.astype(np.float32)).cuda()
    y32 = torch.empty_like(x32)
    for prec in ("f32", "bf16x3"):
        if prec == "bf16x3" and (nx < 1024 or nx > 65536 or nx & (nx - 1)):
            continue
        with hpxfft.Plan(nx, nc, 1, prec, "estimate") as p32:
            p32.set_stream(stream.cuda_stream)
            ms = _time_steps(torch, stream, lambda: p32.execute_oop(x32.data_ptr(), y32.data_ptr()), steps, warm)
            p32.synchronize()
            B = algorithmic_bytes(nx, ny, 4)
            sec = {"workload": workload_name(nx, ny, prec), "ms": ms, "value": B / (ms * 1e-3) / 1e9, "unit": "GB/s",
                   "frac_of_measured_hbm": B / (ms * 1e-3) / 1e9 / peak}
            if prec == "bf16x3":
                sec["tensor_core_stage"] = ("first radix-16 pass of both column steps, tcgen05 kind::f16, 3-term "
                                            "BF16 split, FP32 accumulate; FP32 rows (the plan's rule: the "
                                            "tensor-core row measured slower)")
            if oracle_ref is not None:
                sec["rel_l2_vs_fp64_oracle"], sec["max_abs_err_vs_fp64_oracle"] = _rel_to_oracle(
                    y32.cpu().numpy().view(np.complex64), oracle_ref)
            out[f"precision_{prec}"] = sec
    del x32, y32

    out["prime_sizes"] = prime_sizes(torch, hpxfft, stream, steps, warm, peak)
    out["scale_32768_f64"] = scale_32768(torch, hpxfft, stream, warm, peak)

    # batching: 1024 uneven FP32 instances; "measure": the plan step times
    # queue orders once and caches the winner
    out["batch_1024_uneven_f32"] = batch_workload(torch, hpxfft, stream, 1024, "measure", steps, warm, peak)

    # differentiation: adjoint of the r2c on 64 FP32 2048^2 arrays
    nb, n = 64, 2048
    g = torch.Generator(device="cuda")
    g.manual_seed(64)
    buf = torch.rand((nb, n, 2 * (n // 2 + 1)), generator=g, device="cuda")
    with hpxfft.Plan(n, 2 * (n // 2 + 1), nb, "f32", "estimate") as pb:
        pb.set_stream(stream.cuda_stream)
        ms = _time_steps(torch, stream, lambda: pb.backward_device(buf.data_ptr()), steps, warm)
        Bd = nb * algorithmic_bytes(n, n, 4)
        out["backward_64x2048_f32"] = {"ms": ms, "value": Bd / (ms * 1e-3) / 1e9, "unit": "GB/s",
                                       "frac_of_measured_hbm": Bd / (ms * 1e-3) / 1e9 / peak}
    del buf
    return out


def run_batch_only(args):
    """The uneven FP32 batch alone, one JSON line (profiling the batch kernel
    on fewer instances: --batch-count, --batch-flag estimate)."""
    import importlib.util

    import torch

    torch.cuda.set_device(0)
    spec = importlib.util.spec_from_file_location("hpxfft_build", os.path.join(REPO, "hpx-fft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_all()
    import hpxfft

    peak, _ = measured_peak_hbm()
    res = batch_workload(torch, hpxfft, torch.cuda.current_stream(), args.batch_count, args.batch_flag,
                         args.steps, max(3, args.warmup), peak)
    res["workload"] = f"batch_{args.batch_count}_uneven_f32"
    print(json.dumps(res), flush=True)
    return 0


def run_scale_only(args):
    """The 32768^2 FP64 section alone, one JSON line."""
    import importlib.util

    import torch

    torch.cuda.set_device(0)
    spec = importlib.util.spec_from_file_location("hpxfft_build", os.path.join(REPO, "hpx-fft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_all()
    import hpxfft

    peak, _ = measured_peak_hbm()
    print(json.dumps(scale_32768(torch, hpxfft, torch.cuda.current_stream(), max(3, args.warmup), peak)), flush=True)
    return 0


def run_prime_only(args):
    """The prime-length section alone, one JSON line (profiling the
    Bluestein path; --nx/--ny other than the 16384^2 default set the size)."""
    import importlib.util

    import torch

    torch.cuda.set_device(0)
    spec = importlib.util.spec_from_file_location("hpxfft_build", os.path.join(REPO, "hpx-fft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_all()
    import hpxfft

    peak, _ = measured_peak_hbm()
    nx, ny = (args.nx, args.ny) if (args.nx, args.ny) != (16384, 16384) else (16381, 16382)
    res = prime_sizes(torch, hpxfft, torch.cuda.current_stream(), args.steps, max(3, args.warmup), peak, nx, ny)
    print(json.dumps(res), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.batch_only:
        return run_batch_only(args)
    if args.prime_only:
        return run_prime_only(args)
    if args.scale_only:
        return run_scale_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
