"""Build the CUDA library (sm_103a) and the CPU oracle in tree.

libhpxfft_gb300.so  <- hpx-fft_gb300/csrc/*.cu   (nvcc, one TU per compute type, in parallel)
libhpxfft_oracle.so <- oracle/hpxfft_oracle.c      (gcc; test infrastructure only)

Outputs go to `_build/` folders next to the sources (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD = os.path.join(PKG_DIR, "_build")
LIB = os.path.join(BUILD, "libhpxfft_gb300.so")
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libhpxfft_oracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]
SOURCES = [
    "kernels_ff_rows.cu",
    "kernels_ff_cols.cu",
    "kernels_f32_rows.cu",
    "kernels_f32_cols.cu",
    "kernels_f64.cu",
    "kernels_tc_cols.cu",
    "twiddles.cu",
    "bluestein.cu",
    "plan.cu",
    "batch.cu",
    "pipe_peaks.cu",
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(REPO, "include", "hpxfft_gb300.h"))
    nvcc = _nvcc()
    objs = []
    cmds = []
    for name in SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src, *headers]):
            cmds.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj])
    if not cmds and os.path.exists(LIB) and _newer(LIB, objs):
        return LIB
    with ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        for _ in ex.map(_run, cmds):
            pass
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle(force: bool = False) -> str:
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE_DIR, "hpxfft_oracle.c")
    hdr = os.path.join(ORACLE_DIR, "hpxfft_oracle.h")
    if not force and _newer(ORACLE_LIB, [src, hdr, __file__]):
        return ORACLE_LIB
    cc = shutil.which("gcc") or "cc"
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-O2", "-std=c11", "-D_GNU_SOURCE", "-shared", "-fPIC", "-pthread", "-o", tmp, src, "-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


CPP_PROGRAMS = {
    # the drop-in C++ API: the reference's tests and its shared-loop driver
    "test_dropin": os.path.join(REPO, "tests", "cpp", "test_dropin.cpp"),
    "test_dropin_host": os.path.join(REPO, "tests", "cpp", "test_dropin_host.cpp"),
    "hpxfft_gpu_shared_loop": os.path.join(PKG_DIR, "examples", "shared_loop_2d.cpp"),
}


def build_cpp(force: bool = False) -> dict:
    """C++ programs against the drop-in headers, linked to the library."""
    cxx = shutil.which("g++") or "c++"
    inc = [f"-I{os.path.join(REPO, 'include')}", f"-I{os.path.join(PKG_DIR, 'include')}"]
    hdrs = []
    for root, _, files in os.walk(os.path.join(PKG_DIR, "include")):
        hdrs += [os.path.join(root, f) for f in files]
    out = {}
    cmds = []
    for name, src in CPP_PROGRAMS.items():
        exe = os.path.join(BUILD, name)
        out[name] = exe
        if not force and _newer(exe, [src, LIB, *hdrs]):
            continue
        cmds.append([cxx, "-std=c++17", "-O2", *inc, "-o", exe, src, f"-L{BUILD}", "-lhpxfft_gb300",
                     f"-Wl,-rpath,{BUILD}"])
    with ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        for _ in ex.map(_run, cmds):
            pass
    return out


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()
    build_cpp(force)


def resource_report(pattern: str | None = None) -> str:
    """Registers, spills and static shared memory of every kernel and
    non-inlined device function, as ptxas reports them (-Xptxas -v), grouped
    by function name: a markdown table, then one row per instance whose
    demangled name matches the regular expression `pattern`.  Compiles into
    a temporary folder; the library build is untouched."""
    import re
    import tempfile
    from collections import defaultdict

    nvcc = _nvcc()
    kernel_sources = [s for s in SOURCES if s.startswith("kernels_") or s in ("batch.cu", "bluestein.cu")]
    with tempfile.TemporaryDirectory() as tmp:
        cmds = [[nvcc, *ARCH, *NVCC_FLAGS, "-Xptxas", "-v", "-c", os.path.join(CSRC, s), "-o",
                 os.path.join(tmp, s + ".o")] for s in kernel_sources]

        def run(cmd):
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stderr}")
            return r.stderr

        with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
            logs = list(ex.map(run, cmds))
    funcs = {}
    cur = None
    for line in "\n".join(logs).splitlines():
        m = re.search(r"Function properties for (\S+)", line)
        if m:
            cur = funcs.setdefault(m.group(1), {"regs": 0, "spill": 0, "stack": 0, "smem": 0})
            continue
        m = re.search(r"(\d+) bytes stack frame, (\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m and cur is not None:
            cur["stack"] = int(m.group(1))
            cur["spill"] = int(m.group(2)) + int(m.group(3))
            continue
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            cur = funcs.setdefault(m.group(1), {"regs": 0, "spill": 0, "stack": 0, "smem": 0})
            continue
        m = re.search(r"Used (\d+) registers.*?(?:(\d+) bytes smem)?,", line)
        if m and cur is not None:
            cur["regs"] = int(m.group(1))
            s = re.search(r"(\d+) bytes smem", line)
            cur["smem"] = int(s.group(1)) if s else 0
    names = list(funcs)
    filt = shutil.which("c++filt")
    if filt:
        out = subprocess.run([filt], input="\n".join(names), capture_output=True, text=True).stdout.splitlines()
        if len(out) == len(names):
            names = out
    groups = defaultdict(list)
    for pretty, rec in zip(names, funcs.values()):
        base = pretty.split("(")[0]
        base = re.sub(r"^void ", "", base).split("<")[0].split("::")[-1]
        groups[base].append((pretty, rec))
    rows = ["| function | instances | registers (min-max) | static smem B (max) | stack B (max) | spill B (max) |",
            "|---|---|---|---|---|---|"]
    for base in sorted(groups):
        recs = [r for _, r in groups[base]]
        regs = [r["regs"] for r in recs]
        rows.append(f"| `{base}` | {len(recs)} | {min(regs)}-{max(regs)} | {max(r['smem'] for r in recs)} | "
                    f"{max(r['stack'] for r in recs)} | {max(r['spill'] for r in recs)} |")
    spilled = [(p, r) for b in groups for p, r in groups[b] if r["spill"]]
    rows.append("")
    rows.append(f"{len(funcs)} functions; {len(spilled)} with spills.")
    if spilled:
        # instances whose compiled length (third template argument, or the
        # batch bodies' first) is 0 choose their radices at plan time
        where = defaultdict(list)
        for p, r in spilled:
            base = re.sub(r"^void ", "", p.split("(")[0]).split("<")[0].split("::")[-1]
            runtime = re.search(r", 0, 0>", p) is not None
            where[(base, "runtime-planned (compiled length 0)" if runtime else "compiled shapes")].append(r["spill"])
        rows += ["", "| function | instances | which | spill B (min-max) |", "|---|---|---|---|"]
        for (base, kind), v in sorted(where.items()):
            rows.append(f"| `{base}` | {len(v)} | {kind} | {min(v)}-{max(v)} |")
    if pattern:
        rows += ["", "| instance | registers | static smem B | stack B | spill B |", "|---|---|---|---|---|"]
        for b in sorted(groups):
            for p, r in groups[b]:
                if re.search(pattern, p):
                    name = p.replace("hpxfft_gpu::", "").replace("void ", "")
                    rows.append(f"| `{name[:150]}` | {r['regs']} | {r['smem']} | {r['stack']} | {r['spill']} |")
    return "\n".join(rows)


if __name__ == "__main__":
    if "--resources" in sys.argv:
        i = sys.argv.index("--resources")
        print(resource_report(sys.argv[i + 1] if i + 1 < len(sys.argv) else None))
        sys.exit(0)
    build_all(force="--force" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
