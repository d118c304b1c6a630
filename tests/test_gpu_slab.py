"""Slab decomposition kernels (hpxfft_slab_*) on one GPU (GPU).

P ranks are emulated in one process on one device: each rank's local phases
run through its own slab object, one after another on one stream, and the
exchanges between the phases are plain device copies (tile d of rank s's
send buffer into tile s of rank d's receive buffer), so no kernel waits on
another.  The stacked local results must equal the oracle's full transform:
FP64 <= 1e-12, FP32 and split-BF16 <= 2e-6 relative L2.  Shapes include
dcy not divisible by P (zero-padded last tile), P = 1, and inputs with
energy at every kx.
"""
import numpy as np
import pytest

from gpu_helpers import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"f64": 1e-12, "f32": 2e-6, "bf16x3": 2e-6}


def run_emulated(gpu_lib, torch, x_full, P, prec):
    nx, n_col = x_full.shape
    nxl = nx // P
    tdt = torch.float64 if prec == "f64" else torch.float32
    slabs = [gpu_lib.plan.Slab(nxl, n_col, P, r, prec, "estimate") for r in range(P)]
    try:
        tb = slabs[0].tile_bytes
        vals = [torch.from_numpy(np.ascontiguousarray(x_full[r * nxl:(r + 1) * nxl])).to(tdt).cuda() for r in range(P)]
        send = [torch.empty(P * tb, dtype=torch.uint8, device="cuda") for _ in range(P)]
        recv = [torch.empty(P * tb, dtype=torch.uint8, device="cuda") for _ in range(P)]
        stream = torch.cuda.current_stream().cuda_stream
        for s in slabs:
            s.set_stream(stream)

        def exchange(src, dst):
            for s_ in range(P):
                for d in range(P):
                    dst[d][s_ * tb:(s_ + 1) * tb].copy_(src[s_][d * tb:(d + 1) * tb])

        for r in range(P):
            slabs[r].rows(vals[r].data_ptr(), send[r].data_ptr())
        exchange(send, recv)
        for r in range(P):
            slabs[r].columns(recv[r].data_ptr())
        exchange(recv, send)  # send now holds the second exchange's result
        for r in range(P):
            slabs[r].finish(send[r].data_ptr(), vals[r].data_ptr())
        for s in slabs:
            s.synchronize()
        torch.cuda.synchronize()
        meas = {k: slabs[0].measurement(k) for k in ("first_fftw", "first_split", "second_fftw", "second_trans")}
        out = np.concatenate([v.cpu().numpy() for v in vals]).astype(np.float64)
    finally:
        for s in slabs:
            s.close()
    return out, meas


def full_input(nx, ny, seed, f32=False):
    rng = np.random.default_rng(seed)
    x = np.zeros((nx, 2 * (ny // 2 + 1)))
    x[:, :ny] = rng.uniform(-1, 1, (nx, ny))
    i, j = np.arange(nx)[:, None], np.arange(ny)[None, :]
    x[:, :ny] += 3.0 * np.sin(2 * np.pi * (5 * i / nx + 7 * j / ny))
    if f32:
        x = x.astype(np.float32).astype(np.float64)
    return x


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_slab_kernels_match_oracle(gpu_lib, cuda, oracle_lib, prec):
    for nx, ny, P in ((8, 12, 2), (12, 20, 3), (64, 96, 2), (64, 96, 4), (96, 160, 3), (1024, 1024, 4),
                      (256, 4096, 8), (2048, 64, 2), (16, 30, 1),
                      # primes above 13: Bluestein in the local rows and the column slab
                      (34, 38, 2), (51, 46, 3)):
        x = full_input(nx, ny, nx + ny + P, prec != "f64")
        got, meas = run_emulated(gpu_lib, cuda, x, P, prec)
        ref = oracle_lib.fft_2d_r2c(x.copy(), nthreads=8)
        err = rel_l2(got.view(np.complex128), ref.view(np.complex128))
        assert err <= TOL[prec], (prec, nx, ny, P, err)
        assert all(v >= 0 for v in meas.values())


def test_slab_4096_squared_fp64_two_ranks(gpu_lib, cuda, oracle_lib):
    x = full_input(4096, 4096, 4242)
    got, _ = run_emulated(gpu_lib, cuda, x, 2, "f64")
    ref = oracle_lib.fft_2d_r2c(x.copy(), nthreads=16)
    assert rel_l2(got.view(np.complex128), ref.view(np.complex128)) <= 1e-12


def test_slab_split_bf16_columns(gpu_lib, cuda, oracle_lib):
    """Split-BF16: FP32 rows, tensor-core column steps on the column slab."""
    x = full_input(2048, 512, 99, f32=True)
    got, _ = run_emulated(gpu_lib, cuda, x, 4, "bf16x3")
    ref = oracle_lib.fft_2d_r2c(x.copy(), nthreads=8)
    assert rel_l2(got.view(np.complex128), ref.view(np.complex128)) <= 2e-6


def test_slab_argument_errors(gpu_lib, cuda):
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        gpu_lib.plan.Slab(4, 10, 2, 2, "f64")  # rank >= n_ranks
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        gpu_lib.plan.Slab(4, 10, 2, 0, "f64", "fast")
    with pytest.raises(gpu_lib.HpxFftError) as e:
        gpu_lib.plan.Slab(4, 11, 2, 0, "f64")  # odd n_col
    assert e.value.status == gpu_lib._capi.HPXFFT_ERR_UNSUPPORTED_SIZE
