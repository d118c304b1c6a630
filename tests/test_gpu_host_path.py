"""Host-buffer entry point (GPU): hpxfft_execute_r2c_host on page-locked
memory either overlaps chunked copies with the kernels (two-step column
plans of one array) or reads and writes the host buffer directly from the
kernels; on pageable memory it stages through a device buffer.  Every path
gives the bits of the device-buffer path.  Also: power-of-two sizes plan
compile-time chains."""
import numpy as np
import pytest

from gpu_helpers import padded, run_device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32", "bf16x3"])
@pytest.mark.parametrize("nx,ny", [(1024, 256), (8192, 64), (2048, 96)])
def test_pinned_and_pageable_match_device(gpu_lib, cuda, prec, nx, ny):
    torch = cuda
    dt = np.float32 if prec != "f64" else np.float64
    x = padded(np.random.default_rng(nx + ny).uniform(-1, 1, (nx, ny)), dt)
    nc = x.shape[1]
    with gpu_lib.Plan(nx, nc, 1, prec, "estimate") as plan:
        ref = run_device(torch, plan, x)
        pageable = x.copy()
        plan.execute_host(pageable)
        assert plan.measurement("host_zero_copy") == 0.0
        pinned_t = torch.from_numpy(x.copy()).pin_memory()
        pinned = pinned_t.numpy()
        plan.execute_host(pinned)
        assert plan.measurement("host_zero_copy") + plan.measurement("host_pipelined") == 1.0
        assert plan.measurement("e2e") > 0.0
    assert np.array_equal(pageable, ref), prec
    assert np.array_equal(pinned, ref), prec


@pytest.mark.parametrize("prec,nx,ny", [("f64", 16384, 1024), ("f64", 8192, 4096), ("f32", 8192, 2048),
                                        ("bf16x3", 4096, 1024)])
def test_pipelined_host_path_matches_device_path(gpu_lib, cuda, prec, nx, ny):
    """Chunked copies overlapped with the kernels: same bits as the device
    path, twice in a row on the same plan (the second reuses the copy
    streams and events)."""
    torch = cuda
    dt = np.float32 if prec != "f64" else np.float64
    x = padded(np.random.default_rng(nx * 3 + ny).uniform(-1, 1, (nx, ny)), dt)
    with gpu_lib.Plan(nx, x.shape[1], 1, prec, "estimate") as plan:
        ref = run_device(torch, plan, x)
        pinned_t = torch.from_numpy(x.copy()).pin_memory()
        for _ in range(2):
            pinned_t.copy_(torch.from_numpy(x))
            pinned = pinned_t.numpy()
            plan.execute_host(pinned)
            assert plan.measurement("host_pipelined") == 1.0, (prec, nx, ny)
            assert plan.measurement("h2d") > 0.0 and plan.measurement("e2e") > 0.0
            assert np.array_equal(pinned, ref), (prec, nx, ny)


def test_pinned_batch(gpu_lib, cuda):
    torch = cuda
    xs = np.stack([padded(np.random.default_rng(i).uniform(-1, 1, (8192, 40))) for i in range(3)])
    with gpu_lib.Plan(8192, 42, 3, "f64", "estimate") as plan:
        ref = run_device(torch, plan, xs)
        pinned = torch.from_numpy(xs.copy()).pin_memory().numpy()
        plan.execute_host(pinned)
        assert plan.measurement("host_zero_copy") == 1.0
    assert np.array_equal(pinned, ref)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_power_of_two_sizes_use_compiled_chains(gpu_lib, cuda, tmp_path, prec):
    for n in (256, 1024, 4096, 16384):
        path = tmp_path / f"plan_{prec}_{n}.txt"
        with gpu_lib.Plan(n, 2 * (n // 2 + 1), 1, prec, "estimate") as plan:
            plan.write_plan(path)
        text = path.read_text()
        assert "chain=runtime" not in text, (prec, n, text)
