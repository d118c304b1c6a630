"""Split-BF16 tensor-core precision (HPXFFT_PREC_BF16X3) vs the FP64 oracle (GPU).

The first radix-16 stage of both column steps runs as a tcgen05 matmul with
three-way BF16 splits of data and DFT matrix; everything else is FP32.  The
bar is the FP32 one: relative L2 <= 2e-6 against the FP64 oracle on the
FP32-rounded input.
"""
import numpy as np
import pytest

from gpu_helpers import padded, rel_l2, run_device, to_complex

pytestmark = pytest.mark.gpu
TOL = 2e-6


def oracle_fwd(oracle, x):
    p = oracle.padded(np.asarray(x, dtype=np.float64))
    oracle.fft_2d_r2c(p, nthreads=16)
    return oracle.spectrum(p)


def forward(hpxfft, torch, x, prec="bf16x3"):
    nx, ny = x.shape
    with hpxfft.Plan(nx, 2 * (ny // 2 + 1), 1, prec, "estimate") as plan:
        out = run_device(torch, plan, padded(x, np.float32))
        plan.synchronize()
    return to_complex(out)


# every tensor-core step length: nx = N1 * N2, N2 = 2^floor(log2(nx)/2)
SHAPES = [(1024, 96), (2048, 50), (4096, 130), (8192, 64), (16384, 18), (32768, 10), (65536, 6)]


@pytest.mark.parametrize("nx,ny", SHAPES)
def test_tensor_core_columns_vs_oracle(gpu_lib, cuda, oracle_lib, nx, ny):
    x = np.random.default_rng(nx + ny).uniform(-1, 1, (nx, ny)).astype(np.float32)
    got = forward(gpu_lib, cuda, x)
    ref = oracle_fwd(oracle_lib, x.astype(np.float64))
    err = rel_l2(got, ref)
    assert err <= TOL, (nx, ny, err)
    # different rounding from the all-FP32 path: the tensor-core stage ran
    assert not np.array_equal(got, forward(gpu_lib, cuda, x, "f32"))


def test_ragged_strips_and_sparse_columns(gpu_lib, cuda, oracle_lib):
    """Column counts that leave most of the last strip empty, and impulses
    that excite single DFT-matrix entries."""
    rng = np.random.default_rng(5)
    for nx, ny in ((1024, 2), (4096, 252), (2048, 130)):
        x = np.zeros((nx, ny), dtype=np.float32)
        idx = rng.integers(0, nx * ny, 40)
        x.ravel()[idx] = rng.uniform(-4, 4, 40).astype(np.float32)
        got = forward(gpu_lib, cuda, x)
        assert rel_l2(got, oracle_fwd(oracle_lib, x.astype(np.float64))) <= TOL, (nx, ny)


def test_headline_16384_squared(gpu_lib, cuda, oracle_lib):
    """16384^2, uniform[-1,1): relative L2 and max-abs against the FP64 oracle."""
    x = np.random.default_rng(3).uniform(-1, 1, (16384, 16384)).astype(np.float32)
    got = forward(gpu_lib, cuda, x)
    ref = oracle_fwd(oracle_lib, x.astype(np.float64))
    err = rel_l2(got, ref)
    max_abs = float(np.max(np.abs(got - ref)))
    print(f"bf16x3 16384^2: rel_l2={err:.3e} max_abs={max_abs:.3e} (|X| max {np.max(np.abs(ref)):.3e})")
    assert err <= TOL, err


def test_inverse_and_adjoint(gpu_lib, cuda, oracle_lib):
    rng = np.random.default_rng(77)
    nx, ny = 4096, 96
    x = rng.uniform(-1, 1, (nx, ny)).astype(np.float32)
    with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, "bf16x3", "estimate") as plan:
        spec = run_device(cuda, plan, padded(x, np.float32), "forward")
        back = run_device(cuda, plan, spec, "c2r")
        assert rel_l2(back[:, :ny] / (nx * ny), x) <= 1e-6
        g = rng.standard_normal((nx, ny // 2 + 1)) + 1j * rng.standard_normal((nx, ny // 2 + 1))
        buf = np.ascontiguousarray(g).view(np.float64).copy()
        ref = oracle_lib.fft_2d_r2c_adjoint(buf.copy())
        got = run_device(cuda, plan, buf.astype(np.float32), "backward")
        plan.synchronize()
    assert rel_l2(got[:, :ny], ref[:, :ny]) <= TOL


def test_plan_description_and_batch(gpu_lib, cuda, oracle_lib, tmp_path):
    rng = np.random.default_rng(9)
    xs = rng.uniform(-1, 1, (3, 2048, 40)).astype(np.float32)
    host = np.stack([padded(x, np.float32) for x in xs])
    with gpu_lib.Plan(2048, 42, 3, "bf16x3", "estimate") as plan:
        out = to_complex(run_device(cuda, plan, host))
        plan.write_plan(tmp_path / "plan.txt")
    text = (tmp_path / "plan.txt").read_text()
    assert "bf16x3-tcgen05" in text and "c2c-stepA" in text
    for i in range(3):
        assert rel_l2(out[i], oracle_fwd(oracle_lib, xs[i].astype(np.float64))) <= TOL


def test_unsupported_row_counts(gpu_lib, cuda):
    for n_row in (512, 3072, 131072, 1000):
        with pytest.raises(gpu_lib.HpxFftError) as e:
            gpu_lib.Plan(n_row, 18, 1, "bf16x3", "estimate")
        assert e.value.status == gpu_lib._capi.HPXFFT_ERR_UNSUPPORTED_SIZE


@pytest.mark.parametrize("nx,ny", [(1024, 96), (16384, 18), (65536, 6)])
def test_half_occupancy_variant(gpu_lib, cuda, oracle_lib, monkeypatch, nx, ny):
    """512 vectors per CTA (2 CTAs per SM) instead of the default 256."""
    monkeypatch.setenv("HPXFFT_TC_VECTORS", "512")
    x = np.random.default_rng(nx - ny).uniform(-1, 1, (nx, ny)).astype(np.float32)
    got = forward(gpu_lib, cuda, x)
    assert rel_l2(got, oracle_fwd(oracle_lib, x.astype(np.float64))) <= TOL, (nx, ny)


# every compiled tensor-core row shape: M = ny / 2 in 128 .. 8192
@pytest.mark.parametrize("ny", [256, 512, 1024, 2048, 4096, 8192, 16384])
def test_tensor_core_rows_vs_oracle(gpu_lib, cuda, oracle_lib, tmp_path, monkeypatch, ny):
    """Tensor-core rows, which the plan takes when asked (the rule keeps
    FP32 rows, measured faster)."""
    monkeypatch.setenv("HPXFFT_TC_ROWS", "1")
    nx = 1024
    with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, "bf16x3", "estimate") as plan:
        plan.write_plan(tmp_path / "plan.txt")
    first = (tmp_path / "plan.txt").read_text().split("GPU c2c")[0]
    assert "bf16x3-tcgen05" in first, first
    x = np.random.default_rng(ny).uniform(-1, 1, (nx, ny)).astype(np.float32)
    got = forward(gpu_lib, cuda, x)
    assert rel_l2(got, oracle_fwd(oracle_lib, x.astype(np.float64))) <= TOL, ny
    # the c2r rows of the inverse stay FP32 on the same plan shape
    with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, "bf16x3", "estimate") as plan:
        spec = run_device(cuda, plan, padded(x, np.float32), "forward")
        back = run_device(cuda, plan, spec, "c2r")
    assert rel_l2(back[:, :ny] / (nx * ny), x) <= 1e-6
