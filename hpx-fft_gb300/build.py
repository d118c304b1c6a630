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
    "plan.cu",
    "batch.cu",
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


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
