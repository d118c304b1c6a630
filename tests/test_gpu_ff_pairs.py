"""FP64 forward transform with float-float pairs between its kernels (GPU).

The row kernel hands its output to column step A, and A to step B, as raw
(hi, lo) float pairs with one scale exponent per row / per block; only the
input and the final output are doubles.  These tests compare that pipeline
with the double-format one (HPXFFT_FF_PAIRS=0) and with the oracle, with
inputs whose rows span very different exponents.
"""
import numpy as np
import pytest

from gpu_helpers import padded, rel_l2, run_device, to_complex

pytestmark = pytest.mark.gpu


def oracle_fwd(oracle, x):
    p = oracle.padded(np.asarray(x, dtype=np.float64))
    oracle.fft_2d_r2c(p, nthreads=16)
    return oracle.spectrum(p)


def forward(hpxfft, torch, host, batch=1):
    nx, nc = host.shape[-2:]
    with hpxfft.Plan(nx, nc, batch, "f64", "estimate") as plan:
        out = run_device(torch, plan, host)
    return to_complex(out)


def plan_text(hpxfft, nx, ny, path):
    with hpxfft.Plan(nx, 2 * (ny // 2 + 1), 1, "f64", "estimate") as plan:
        plan.write_plan(path)
    return path.read_text()


@pytest.mark.parametrize("nx,ny", [(8192, 64), (16384, 40), (32768, 12), (8192, 1536)])
def test_pairs_match_double_format_and_oracle(gpu_lib, cuda, oracle_lib, monkeypatch, tmp_path, nx, ny):
    assert "float-float pairs between kernels" in plan_text(gpu_lib, nx, ny, tmp_path / "pairs.txt")
    x = np.random.default_rng(nx + ny).uniform(-1, 1, (nx, ny))
    got = forward(gpu_lib, cuda, padded(x))
    monkeypatch.setenv("HPXFFT_FF_PAIRS", "0")
    assert "float-float pairs" not in plan_text(gpu_lib, nx, ny, tmp_path / "doubles.txt")
    ref_dbl = forward(gpu_lib, cuda, padded(x))
    assert rel_l2(got, ref_dbl) <= 5e-14  # both carry float-float rounding (~1e-14)
    assert rel_l2(got, oracle_fwd(oracle_lib, x)) <= 1e-12


def test_rows_of_very_different_scales(gpu_lib, cuda, oracle_lib):
    """Row exponents from -300 to +300, zero rows, and columns mixing them."""
    rng = np.random.default_rng(17)
    nx, ny = 8192, 96
    x = rng.uniform(-1, 1, (nx, ny))
    scale = 2.0 ** rng.choice([-300, -40, 0, 25, 300], nx)
    scale[rng.integers(0, nx, 100)] = 0.0
    x *= scale[:, None]
    got = forward(gpu_lib, cuda, padded(x))
    assert np.isfinite(got).all()
    ref = oracle_fwd(oracle_lib, x)
    assert rel_l2(got, ref) <= 1e-12
    # the small rows alone: their own transform must survive the mixing
    small = np.where(scale[:, None] <= 2.0**-40, x, 0.0)
    got_s = forward(gpu_lib, cuda, padded(small))
    assert rel_l2(got_s, oracle_fwd(oracle_lib, small)) <= 1e-12


@pytest.mark.parametrize("e", [-1000, -500, 500, 1000])
def test_extreme_uniform_exponents(gpu_lib, cuda, oracle_lib, e):
    x = np.random.default_rng(abs(e)).uniform(-1, 1, (8192, 64)) * 2.0**e
    got = forward(gpu_lib, cuda, padded(x))
    assert np.isfinite(got).all()
    # compare at unit scale: squares of 2^1000 overflow the norm
    assert rel_l2(got * 2.0**-e, oracle_fwd(oracle_lib, x) * 2.0**-e) <= 1e-12


def test_all_zero_input(gpu_lib, cuda):
    got = forward(gpu_lib, cuda, padded(np.zeros((8192, 32))))
    assert not np.any(got)


def test_batch_oop_and_host_path(gpu_lib, cuda, oracle_lib):
    torch = cuda
    rng = np.random.default_rng(23)
    xs = rng.uniform(-1, 1, (3, 8192, 50)) * np.array([1.0, 2.0**-200, 2.0**200])[:, None, None]
    host = np.stack([padded(x) for x in xs])
    with gpu_lib.Plan(8192, 52, 3, "f64", "estimate") as plan:
        dev_in = torch.from_numpy(host.copy()).cuda()
        dev_out = torch.empty_like(dev_in)
        plan.set_stream(torch.cuda.current_stream().cuda_stream)
        plan.execute_oop(dev_in.data_ptr(), dev_out.data_ptr())
        torch.cuda.synchronize()
        oop = to_complex(dev_out.cpu().numpy())
        assert np.array_equal(dev_in.cpu().numpy(), host)  # input untouched
        pinned = torch.from_numpy(host.copy()).pin_memory().numpy()
        plan.set_stream(None)
        plan.execute_host(pinned)
        assert np.array_equal(to_complex(pinned), oop)
    for i in range(3):
        assert rel_l2(oop[i], oracle_fwd(oracle_lib, xs[i])) <= 1e-12


@pytest.mark.parametrize("row16", ["1", "0"])
def test_ff_rows_radix16_and_radix8_chains(gpu_lib, cuda, oracle_lib, monkeypatch, row16):
    """Rows of 8192 float-float pairs run the radix-16 chain by default and
    the radix-8 one with HPXFFT_FF_ROW16=0: both against the oracle, on the
    device path and the chunked host path."""
    monkeypatch.setenv("HPXFFT_FF_ROW16", row16)
    rng = np.random.default_rng(16)
    for nx in (24, 8192):  # single-kernel columns; the two-step pass and the pipelined host path
        x = rng.uniform(-1, 1, (nx, 16384))
        host = padded(x)
        ref = oracle_lib.fft_2d_r2c(host.copy(), nthreads=16)
        with gpu_lib.Plan(nx, host.shape[1], 1, "f64", "estimate") as plan:
            got = run_device(cuda, plan, host.copy())
            assert rel_l2(got, ref) <= 1e-12, (row16, nx)
            pinned = cuda.from_numpy(host.copy()).pin_memory()
            out = plan.execute_host(pinned.numpy())
            assert rel_l2(out, ref) <= 1e-12, (row16, nx, "host")


@pytest.mark.parametrize("halves", ["1", "0"])
def test_ff_rows_of_16384_pairs_halves_and_cluster(gpu_lib, cuda, oracle_lib, monkeypatch, halves):
    """Rows of 32768 reals: by default two kernels (the halves' DFTs, then
    the radix-2 combination with the split), with HPXFFT_FF_ROW_HALVES=0 the
    two-CTA cluster kernel; against the oracle with the single-kernel column
    pass (a buffer of their own), the two-step pass (the column scratch, pair
    exchange) and the host-buffer path."""
    monkeypatch.setenv("HPXFFT_FF_ROW_HALVES", halves)
    rng = np.random.default_rng(32)
    for nx in (24, 4096):
        x = rng.uniform(-1, 1, (nx, 32768))
        x[:, ::7] += 3.0
        host = padded(x)
        ref = oracle_lib.fft_2d_r2c(host.copy(), nthreads=16)
        with gpu_lib.Plan(nx, host.shape[1], 1, "f64", "estimate") as plan:
            got = run_device(cuda, plan, host.copy())
            assert rel_l2(got, ref) <= 1e-12, (halves, nx)
            out = plan.execute_host(host.copy())
            assert rel_l2(out, ref) <= 1e-12, (halves, nx, "host")


def test_ff_rows_of_16384_pairs_batch_and_slab(gpu_lib, cuda, oracle_lib):
    """The half-row path with a batch of two (per-item strides of the
    half-row buffer, its exponents and the output) and as the rows-only pass
    of a two-rank slab decomposition (doubles out, then the slab's own
    column pass), against the oracle."""
    rng = np.random.default_rng(3232)
    nx, ny = 24, 32768
    xs = rng.uniform(-1, 1, (2, nx, ny))
    host = np.stack([padded(x) for x in xs])
    with gpu_lib.Plan(nx, host.shape[-1], 2, "f64", "estimate") as plan:
        got = run_device(cuda, plan, host.copy())
    for b in range(2):
        ref = oracle_lib.fft_2d_r2c(host[b].copy(), nthreads=16)
        assert rel_l2(got[b], ref) <= 1e-12, b
    import test_gpu_slab

    x = padded(xs[0])
    out, _ = test_gpu_slab.run_emulated(gpu_lib, cuda, x, 2, "f64")
    ref = oracle_lib.fft_2d_r2c(x.copy(), nthreads=16)
    assert rel_l2(out.view(np.complex128), ref.view(np.complex128)) <= 1e-12
