"""CPU-only checks: the C ABI library loads and exports its header, and links
from plain C99; argument and size validation that never touches the GPU (2D,
3D and batch plans, the planner's size limits, the C++ drop-in classes, the
CLI driver); per-thread error messages; the wisdom file; no fallback when
the library is absent; the float-float conversions compiled for the host;
and the Python mirror of vector_2d."""
import ctypes
import os
import re
import shutil
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "hpxfft_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^HPXFFT_API[^(]*?\b(hpxfft_[a-z0-9_]+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = gpu_lib._capi.load()
    names = declared_symbols()
    assert len(names) >= 16
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(gpu_lib._capi.SIGNATURES)


def test_status_strings_and_flags(gpu_lib):
    lib = gpu_lib._capi.load()
    assert lib.hpxfft_status_string(0) == b"ok"
    assert lib.hpxfft_status_string(7) == b"file I/O error"
    for f in (b"estimate", b"measure", b"patient", b"exhaustive"):
        assert lib.hpxfft_plan_flag_valid(f) == 1
    for f in (b"", b"Estimate", b"fast", None):
        assert lib.hpxfft_plan_flag_valid(f) == 0


def test_plan_argument_errors_before_any_device_call(gpu_lib):
    # string_to_fftw_plan_flag throws std::invalid_argument (adapter_fftw.hpp:42)
    with pytest.raises(gpu_lib.HpxFftInvalidArgument, match="plan flag"):
        gpu_lib.Plan(4, 6, 1, "f64", "wisdom")
    with pytest.raises(gpu_lib.HpxFftError) as e:
        gpu_lib.Plan(4, 5, 1, "f64", "estimate")  # odd n_col: ny must be even (loop.cpp:164-165)
    assert e.value.status == gpu_lib._capi.HPXFFT_ERR_UNSUPPORTED_SIZE
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        gpu_lib.Plan(0, 6, 1, "f64", "estimate")
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        gpu_lib.Plan(4, 6, 1, "f16", "estimate")
    lib = gpu_lib._capi.load()
    h = ctypes.c_void_p()
    assert lib.hpxfft_plan_create(None, 4, 6, 1, 0, b"estimate") == gpu_lib._capi.HPXFFT_ERR_INVALID_ARG
    assert lib.hpxfft_plan_create(ctypes.byref(h), 4, 6, 0, 0, b"estimate") == gpu_lib._capi.HPXFFT_ERR_INVALID_ARG
    assert lib.hpxfft_plan_destroy(None) == gpu_lib._capi.HPXFFT_ERR_STATE
    assert lib.hpxfft_execute_r2c(None, None) == gpu_lib._capi.HPXFFT_ERR_STATE


def test_plan3d_argument_errors_before_any_device_call(gpu_lib):
    capi = gpu_lib._capi
    with pytest.raises(gpu_lib.HpxFftInvalidArgument, match="plan flag"):
        gpu_lib.Plan3D(4, 4, 6, 1, "f64", "wisdom")
    with pytest.raises(gpu_lib.HpxFftError) as e:
        gpu_lib.Plan3D(4, 4, 5, 1, "f64", "estimate")  # odd n_col
    assert e.value.status == capi.HPXFFT_ERR_UNSUPPORTED_SIZE
    with pytest.raises(gpu_lib.HpxFftError) as e:
        gpu_lib.Plan3D(256, 4, 6, 256, "f64", "estimate")  # n0 * batch > 65535
    assert e.value.status == capi.HPXFFT_ERR_UNSUPPORTED_SIZE
    for dims in ((0, 4, 6, 1), (4, 0, 6, 1), (4, 4, 6, 0)):
        with pytest.raises(gpu_lib.HpxFftInvalidArgument):
            gpu_lib.Plan3D(*dims, "f64", "estimate")
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        gpu_lib.Plan3D(4, 4, 6, 1, "f16", "estimate")
    lib = capi.load()
    h = ctypes.c_void_p()
    v = ctypes.c_double()
    n = ctypes.c_size_t()
    assert lib.hpxfft_plan3d_create(None, 4, 4, 6, 1, 0, b"estimate") == capi.HPXFFT_ERR_INVALID_ARG
    assert lib.hpxfft_plan3d_create(ctypes.byref(h), 4, 4, 6, 1, 0, b"wisdom") == capi.HPXFFT_ERR_INVALID_ARG
    assert h.value is None  # a failed create leaves the handle null
    assert lib.hpxfft_plan3d_destroy(None) == capi.HPXFFT_ERR_STATE
    assert lib.hpxfft_plan3d_set_stream(None, None) == capi.HPXFFT_ERR_STATE
    assert lib.hpxfft_execute3d_r2c(None, None) == capi.HPXFFT_ERR_STATE
    assert lib.hpxfft_plan3d_buffer_bytes(None, ctypes.byref(n)) == capi.HPXFFT_ERR_INVALID_ARG
    assert lib.hpxfft_plan3d_get_measurement(None, b"total", ctypes.byref(v)) == capi.HPXFFT_ERR_INVALID_ARG


@pytest.fixture(scope="module")
def ffhost(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("ff") / "ffhost.so"
    src = os.path.join(REPO, "tests", "cpp", "ff_host_check.cpp")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(out), src], check=True)
    lib = ctypes.CDLL(str(out))
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def test_float_float_round_trip(ffhost):
    rng = np.random.default_rng(11)
    x = rng.standard_normal(50000)
    y = np.zeros_like(x)
    for E in (-70, -3, 0, 1, 40):
        xs = x * 2.0**E
        ffhost.ff_roundtrip(_dp(xs), _dp(y), xs.size, E)
        assert np.max(np.abs(y - xs) / np.abs(xs)) <= 2.0**-47


def test_float_float_special_values(ffhost):
    x = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 2.0**-1074, 1.5, -3.25])
    y = np.zeros_like(x)
    ffhost.ff_roundtrip(_dp(x), _dp(y), x.size, 0)
    assert y[0] == 0 and y[1] == 0 and np.signbit(y[1])
    assert y[2] == np.inf and y[3] == -np.inf and np.isnan(y[4])
    assert y[5] == 0.0  # subnormal doubles flush (far below 2^-126 of any block scale)
    assert y[6] == 1.5 and y[7] == -3.25


def test_float_float_pair_to_double(ffhost):
    """Pairs with |lo| <= ulp(hi)/2, including powers of two with a negative
    lo (the one-bit renormalisation) and zero lo, against the exact sum."""
    rng = np.random.default_rng(13)
    n = 40000
    hi = rng.standard_normal(n).astype(np.float32)
    hi[:2000] = np.float32(2.0) ** rng.integers(-20, 20, 2000).astype(np.float32)
    ulp = np.spacing(np.abs(hi)).astype(np.float64)
    lo = (rng.uniform(-0.5, 0.5, n) * ulp).astype(np.float32)
    lo[:1000] = -np.abs(lo[:1000])
    lo[-1000:] = 0
    y = np.zeros(n)
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    for E in (-60, 0, 37):
        ffhost.ff_pair_to_double(fp(hi), fp(lo), _dp(y), n, E)
        exact = (hi.astype(np.float64) + lo.astype(np.float64)) * 2.0**E
        assert np.max(np.abs(y - exact) / np.abs(exact)) <= 2.0**-52


def test_float_float_arithmetic(ffhost):
    rng = np.random.default_rng(12)
    a, b = rng.standard_normal(20000), rng.standard_normal(20000)
    y = np.zeros_like(a)
    for op, f in ((0, np.add), (1, np.subtract), (2, np.multiply)):
        ffhost.ff_binop(_dp(a), _dp(b), _dp(y), a.size, op)
        scale = np.abs(a) + np.abs(b) if op < 2 else np.abs(a * b)
        assert np.max(np.abs(y - f(a, b)) / scale) < 2.0**-45


def test_vector_2d_mirror(gpu_lib):
    # test/src/test_vector_2d.cpp:6-33
    v2 = gpu_lib.util.vector_2d
    vec = v2(3, 3, 4.0)
    assert vec.n_row() == 3 and vec.n_col() == 3 and vec(0, 0) == 4.0 and vec(2, 2) == 4.0 and vec.size() == 9
    with pytest.raises(RuntimeError):
        v2(3, 3, 1.0).at(3, 3)
    # like the reference (vector_2d.hpp:218-221), at() bounds the flat index
    # i * n_col + j only: (0, 3) is element 3, i.e. (1, 0)
    vec[1, 0] = 7.0
    assert vec.at(0, 3) == 7.0
    with pytest.raises(RuntimeError):
        vec.at(2, 3)
    assert v2(2, 2, 5.0) == v2(2, 2, 5.0)
    assert not (v2(2, 2, 5.0) == v2(2, 2, 6.0))
    moved = v2(2, 4, 1.0)
    data = moved.take()
    assert data.shape == (2, 4) and moved.size() == 0


def test_distributed_comm_flag_is_validated(gpu_lib):
    v = gpu_lib.util.vector_2d(4, 6, 0.0)
    with pytest.raises(gpu_lib.HpxFftInvalidArgument, match="scatter or all_to_all"):
        gpu_lib.distributed.loop().initialize(v, "broadcast", "estimate")


def test_wisdom_file_round_trip_and_corrupt_files(gpu_lib, tmp_path):
    """The tuned-plan cache file (host only): batch entries and 2D plan
    choices; import then export gives the same entries, sorted by key; a
    corrupt file is rejected whole and
    merges nothing; unopenable paths raise the I/O status, like
    loop::write_plans_to_file's std::runtime_error (core/src/shared/loop.cpp:197-201)."""
    from hpxfft import batch as hb

    capi = gpu_lib._capi
    head = "hpxfft-gb300-wisdom 2\n"
    batch_entries = ["p2;512x642*3 16 3", "p2;256x514*8;384x258*8 8 2", "p0;64x66*1 0 1"]
    # 2D plan choices: columns (1 cluster, 2 steps), ff_pairs, tc_vectors, tc_rows
    plan_entries = ["2d;p0;16384x16386;b1;full;sm103 2 1 0 0", "2d;p3;4096x4098;b1;full;sm103 2 0 512 1"]
    good = tmp_path / "good.txt"
    good.write_text(head + "\n".join(batch_entries + plan_entries) + "\n")
    out = tmp_path / "out.txt"
    expected = sorted(batch_entries) + sorted(plan_entries)

    def exported():
        hb.wisdom_export(str(out))
        lines = out.read_text().splitlines()
        assert lines[0] == head.strip()
        return lines[1:]

    hb.wisdom_forget()
    try:
        assert exported() == []
        hb.wisdom_import(str(good))
        assert exported() == expected
        # a version-1 file (batch entries only) still imports
        v1 = tmp_path / "v1.txt"
        v1.write_text("hpxfft-gb300-wisdom 1\n" + batch_entries[0] + "\n")
        hb.wisdom_import(str(v1))
        assert exported() == expected
        corrupt = {
            "header": "not wisdom\n",
            "version": "hpxfft-gb300-wisdom 3\n",
            "2d entry in a version-1 file": "hpxfft-gb300-wisdom 1\n" + plan_entries[0] + "\n",
            "2d columns": head + "2d;p0;8x10;b1;full;sm103 3 1 0 0\n",
            "2d vectors": head + "2d;p3;8x10;b1;full;sm103 2 1 128 1\n",
            "2d too few": head + "2d;p0;8x10;b1;full;sm103 2 1 0\n",
            "lag range": head + "k 5000 2\n",
            "negative lag": head + "k -1 2\n",
            "ctas low": head + "k 8 0\n",
            "ctas high": head + "k 8 9\n",
            "truncated": head + "k1 8 2\nk2 8",
            "not a number": head + "k eight 2\n",
            "trailing junk": head + "k1 8 2\njunk\n",
        }
        for name, text in corrupt.items():
            bad = tmp_path / "bad.txt"
            bad.write_text(text)
            with pytest.raises(gpu_lib.HpxFftInvalidArgument):
                hb.wisdom_import(str(bad))
            assert exported() == expected, name
        empty = tmp_path / "empty.txt"
        empty.write_text(head)
        hb.wisdom_import(str(empty))
        assert exported() == expected
        for call in (lambda: hb.wisdom_import(str(tmp_path / "missing.txt")),
                     lambda: hb.wisdom_export(str(tmp_path))):
            with pytest.raises(gpu_lib.HpxFftError) as e:
                call()
            assert e.value.status == capi.HPXFFT_ERR_IO
    finally:
        hb.wisdom_forget()


def test_last_error_is_per_thread(gpu_lib):
    """hpxfft_last_error reports the calling thread's own failure while
    another thread fails differently in between (one host thread per handle,
    handles used concurrently)."""
    import threading

    lib = gpu_lib._capi.load()
    cases = [((4, 6, 1, 0, b"wisdom"), b"plan flag"), ((4, 5, 1, 0, b"estimate"), b"n_col must be")]
    start = threading.Barrier(len(cases))
    wrong = []

    def worker(args, expect):
        h = ctypes.c_void_p()
        start.wait()
        for _ in range(2000):
            assert lib.hpxfft_plan_create(ctypes.byref(h), *args) != gpu_lib._capi.HPXFFT_OK
            if expect not in lib.hpxfft_last_error():
                wrong.append(expect)

    threads = [threading.Thread(target=worker, args=c) for c in cases]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not wrong, wrong[:3]


def test_cpp_dropin_host_side(gpu_lib, build_mod, tmp_path):
    """What the C++ drop-in classes decide before a plan touches the device
    (exception types, unknown measurement keys, vector_2d ownership),
    compiled against the drop-in headers; runs without a GPU."""
    exe = build_mod.build_cpp()["test_dropin_host"]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all host-side drop-in checks passed" in r.stdout


def test_planner_size_limits_before_any_device_call(gpu_lib):
    """The planner's size boundary, decided on the host: shapes it cannot run
    return UNSUPPORTED_SIZE before the first CUDA call; shapes it plans get
    past planning (OK with a GPU, the CUDA status without one).  The direct
    kernels take prime factors up to 13 with rows of up to 8192 complex
    values per CTA on a cluster of up to 4 and columns of up to 4096 (FP64)
    or 8192 (FP32) per CTA on a cluster of up to 16; power-of-two columns
    beyond that take the two-kernel pass, every other length Bluestein's
    convolution or (long smooth rows) the column kernels on a transposed
    copy.  Rejected: odd ny, split-BF16 n_row outside the powers of two in
    [1024, 65536] or rows outside the direct kernels, and n_row above 2^21
    with rows outside the direct kernels."""
    capi = gpu_lib._capi
    lib = capi.load()
    F64, F32, BF = capi.PREC_F64, capi.PREC_F32, capi.PREC_BF16X3
    F64_NATIVE = capi.PREC_F64_NATIVE

    def status(n_row, ny, prec):
        h = ctypes.c_void_p()
        rc = lib.hpxfft_plan_create(ctypes.byref(h), n_row, 2 * (ny // 2 + 1), 1, prec, b"estimate")
        if rc == capi.HPXFFT_OK:
            lib.hpxfft_plan_destroy(h)
        return rc

    planned = [(4, 2, F64), (13, 26, F64), (4, 2 * 13 * 13, F64), (4, 32768, F64), (4, 65536, F64),
               (4, 65536, F32), (65536, 6, F64), (131072, 6, F32), (6, 2 * 3 * 5 * 7 * 11, F32),
               (1024, 6, BF), (65536, 6, BF),
               # longer than one CTA: split over C CTAs, the length divisible by C^2
               (5005, 6, F32), (3 * 4096, 6, F64), (4, 2 * 5005, F64), (4, 2 * 3 * 8192, F64),
               # Bluestein, the two-kernel pass alone, rows on a transposed copy
               (4, 34, F64), (17, 6, F64), (4, 2 * 19, F32), (23, 6, F32), (4, 131072, F32), (4, 131072, F64),
               (131072, 6, F64), (262144, 6, F32), (5005, 6, F64), (2 * 5005, 6, F64), (2 * 5005, 6, F32),
               (4, 2 * 9009, F64), (4, 4 * 9009, F32), (17, 34, F64_NATIVE), (1 << 21, 34, F32)]
    rejected = [(512, 6, BF), (1000, 6, BF), (3072, 6, BF), (131072, 6, BF), (1024, 34, BF),
                ((1 << 21) + 1, 34, F64), (1 << 22, 2 * 3 * 5 * 7 * 11 * 13 * 3, F32)]
    for shape in planned:
        assert status(*shape) != capi.HPXFFT_ERR_UNSUPPORTED_SIZE, shape
    for shape in rejected:
        assert status(*shape) == capi.HPXFFT_ERR_UNSUPPORTED_SIZE, shape


def test_every_entry_point_fails_loudly_without_the_library(tmp_path):
    """No CPU fallback: with the native library absent, each public entry
    point raises instead of computing anything (fresh interpreter, so no
    library is loaded yet)."""
    code = f"""
import sys
sys.path.insert(0, {os.path.join(REPO, 'hpx-fft_gb300', 'python')!r})
import hpxfft
hpxfft._capi.LIB_PATH = {str(tmp_path / 'absent' / 'libhpxfft_gb300.so')!r}
calls = {{
    "Plan": lambda: hpxfft.Plan(4, 6),
    "Plan3D": lambda: hpxfft.Plan3D(4, 4, 6),
    "Batch": lambda: hpxfft.Batch([8], [10], "f32"),
    "shared.loop": lambda: hpxfft.shared.loop().initialize(hpxfft.util.vector_2d(4, 6, 0.0), "estimate"),
    "plan_flag_valid": lambda: hpxfft.plan.plan_flag_valid("estimate"),
    "wisdom_forget": lambda: hpxfft.batch.wisdom_forget(),
}}
for name, call in calls.items():
    try:
        call()
    except OSError as e:
        assert "no CPU fallback" in str(e), (name, e)
    else:
        raise SystemExit(name + " ran without the library")
print("all raised")
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "all raised" in r.stdout, r.stdout + r.stderr


def test_cli_driver_rejects_bad_options_without_a_gpu(gpu_lib, build_mod, tmp_path):
    """hpxfft_gpu_shared_loop: an unknown option exits 2; a bad --plan ends
    the process with the std::invalid_argument of string_to_fftw_plan_flag
    (core/include/hpxfft/util/adapter_fftw.hpp:42) uncaught, as the
    reference's driver does (examples/hpxfft/shared_loop_2d.cpp:46); no
    output files are written in either case."""
    exe = build_mod.build_cpp()["hpxfft_gpu_shared_loop"]
    r = subprocess.run([exe, "--nx=4", "--threads=8"], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 2 and "unknown option --threads" in r.stderr
    r = subprocess.run([exe, "--nx", "4", "--ny", "6", "--plan=fastest"], capture_output=True, text=True,
                       timeout=60, cwd=tmp_path)
    assert r.returncode != 0 and "Invalid FFTW plan flag string" in r.stderr
    assert not (tmp_path / "runtimes").exists() and not (tmp_path / "plans").exists()


def test_c_abi_from_plain_c(gpu_lib, tmp_path):
    """The header compiles as strict C99 and a C program links the library
    and gets the host-side statuses: what a cgo / JNI / N-API binding needs."""
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("gcc not available")
    lib_dir = os.path.dirname(gpu_lib._capi.LIB_PATH)
    exe = tmp_path / "abi_host_check"
    src = os.path.join(REPO, "tests", "c", "abi_host_check.c")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{os.path.join(REPO, 'include')}",
                    "-o", str(exe), src, f"-L{lib_dir}", "-lhpxfft_gb300", f"-Wl,-rpath,{lib_dir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all C ABI host checks passed" in r.stdout


def test_batch_argument_errors_before_any_device_call(gpu_lib):
    """The batch plan rejects bad flags, shapes and precisions on the host."""
    capi = gpu_lib._capi
    invalid = [([8], [10], "f32", "fast"), ([], [], "f32"), ([8], [10], "bf16x3"), ([8, 8], [10], "f32")]
    for args in invalid:
        with pytest.raises(gpu_lib.HpxFftInvalidArgument):
            gpu_lib.Batch(*args)
    unsupported = [([8, 17], [10, 10], "f32"),  # 17 rows: a prime above 13
                   ([16384], [10], "f32"),      # a column must fit one CTA
                   ([8], [9], "f32")]           # odd n_col
    for args in unsupported:
        with pytest.raises(gpu_lib.HpxFftError) as e:
            gpu_lib.Batch(*args)
        assert e.value.status == capi.HPXFFT_ERR_UNSUPPORTED_SIZE, args
