"""hpxfft_execute_r2c_noalloc: the forward FP64 transform for callers that
cannot allocate device memory (their own pool holds it all, or they must not
trigger the device-wide synchronisation a cudaMalloc/cudaFree can cause).

It keeps its twiddle tables in a 1 MiB static device array instead of
plan-owned allocations, so its output is checked against the plan entry point
(hpxfft_execute_r2c_oop) on the same input, within the FP64 bar used by the
other tests (relative L2 <= 1e-12), for several calls in a row that share and
rewrite that array.  This file sorts last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _padded_input(torch, n_row, ny, seed):
    rng = np.random.default_rng(seed)
    host = np.zeros((n_row, 2 * (ny // 2 + 1)), dtype=np.float64)
    host[:, :ny] = rng.uniform(-1.0, 1.0, (n_row, ny))
    return torch.from_numpy(host).cuda()


def _with_plan(hpxfft, torch, x):
    n_row, n_col = x.shape
    out = torch.empty_like(x)
    with hpxfft.Plan(n_row, n_col, 1, "f64", "estimate") as plan:
        plan.set_stream(torch.cuda.current_stream().cuda_stream)
        plan.execute_oop(x.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
    return out


def _no_alloc(lib, torch, x):
    n_row, n_col = x.shape
    out = torch.empty_like(x)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.hpxfft_execute_r2c_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), n_row,
                                        n_col, stream)
    assert rc == 0, lib.hpxfft_last_error().decode()
    torch.cuda.synchronize()
    return out


def _rel_l2(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_no_alloc_matches_plan_entry_point(gpu_lib, cuda):
    lib = gpu_lib._capi.load()
    # consecutive calls with different shapes share (and rewrite) the static
    # scratch; the last one is the largest shape the scratch holds
    shapes = [(512, 1024), (96, 160), (512, 1024), (4096, 4096), (16384, 16384)]
    for seed, (n_row, ny) in enumerate(shapes):
        x = _padded_input(cuda, n_row, ny, seed)
        expected = _with_plan(gpu_lib, cuda, x)
        got = _no_alloc(lib, cuda, x)
        assert _rel_l2(got, expected) <= 1e-12, (n_row, ny)
        del x, expected, got


def test_no_alloc_in_place_and_twice_in_a_row(gpu_lib, cuda):
    lib = gpu_lib._capi.load()
    x = _padded_input(cuda, 256, 384, 7)
    expected = _with_plan(gpu_lib, cuda, x)
    stream = ctypes.c_void_p(cuda.cuda.current_stream().cuda_stream)
    for _ in range(2):
        y = x.clone()
        rc = lib.hpxfft_execute_r2c_noalloc(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(y.data_ptr()), 256,
                                            386, stream)
        assert rc == 0, lib.hpxfft_last_error().decode()
        cuda.cuda.synchronize()
        assert _rel_l2(y, expected) <= 1e-12


def test_no_alloc_rejects_sizes_beyond_its_scratch(gpu_lib, cuda):
    lib = gpu_lib._capi.load()
    buf = cuda.zeros(16, dtype=cuda.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    for n_row, n_col in ((16385, 6), (4, 16386 + 2)):
        rc = lib.hpxfft_execute_r2c_noalloc(p, p, n_row, n_col, None)
        assert rc == gpu_lib._capi.HPXFFT_ERR_UNSUPPORTED_SIZE
        assert b"16384" in lib.hpxfft_last_error()


def test_no_alloc_leaves_device_memory_untouched_after_first_call(gpu_lib, cuda):
    """After the first call on the device (the set-up call, which may load
    code), a call of another shape changes the device's free memory by
    nothing: the entry point allocates no device memory.  Both shapes have
    power-of-two lengths, whose kernels use no per-thread local memory.
    Inputs and outputs are allocated before the free memory is read."""
    lib = gpu_lib._capi.load()
    first = _padded_input(cuda, 1024, 2048, 11)
    second = _padded_input(cuda, 2048, 512, 12)
    out_first, out_second = cuda.empty_like(first), cuda.empty_like(second)
    stream = ctypes.c_void_p(cuda.cuda.current_stream().cuda_stream)

    def call(x, out):
        rc = lib.hpxfft_execute_r2c_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                            x.shape[0], x.shape[1], stream)
        assert rc == 0, lib.hpxfft_last_error().decode()
        cuda.cuda.synchronize()

    call(first, out_first)
    free_before, _ = cuda.cuda.mem_get_info()
    call(second, out_second)
    free_after, _ = cuda.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    assert _rel_l2(out_second, _with_plan(gpu_lib, cuda, second)) <= 1e-12
