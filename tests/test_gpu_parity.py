"""CUDA path vs the CPU oracle on the same seeded inputs (GPU).

Tolerances (relative L2 over all nx*(ny/2+1) outputs):
  f64 (float-float arithmetic)  <= 1e-12   the drop-in bar against FP64 FFTW
  f64-native (DFMA)             <= 1e-13
  f32                           <= 2e-6    against the FP64 oracle
"""
import json
import os

import numpy as np
import pytest

from gpu_helpers import padded, rel_l2, run_device, to_complex

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = {"f64": 1e-12, "f64-native": 1e-13, "f32": 2e-6}


def forward(hpxfft, torch, x, precision, batch=1):
    nx, ny = x.shape[-2:]
    dt = np.float32 if precision == "f32" else np.float64
    host = np.stack([padded(xx, dt) for xx in x.reshape(-1, nx, ny)]) if batch > 1 else padded(x, dt)
    with hpxfft.Plan(nx, 2 * (ny // 2 + 1), batch, precision, "estimate") as plan:
        out = run_device(torch, plan, host)
    return to_complex(out)


def oracle_fwd(oracle, x):
    p = oracle.padded(np.asarray(x, dtype=np.float64))
    oracle.fft_2d_r2c(p, nthreads=8)
    return oracle.spectrum(p)


def test_kat_4x6_all_precisions(gpu_lib, cuda):
    kat = json.load(open(os.path.join(GOLDEN, "kat_4x6.json")))
    expected = np.array(kat["expected"])
    for prec in ("f64", "f64-native", "f32"):
        dt = np.float32 if prec == "f32" else np.float64
        v = np.array(kat["input_rows"], dtype=dt)
        with gpu_lib.Plan(4, 6, 1, prec, "estimate") as plan:
            out = run_device(cuda, plan, v)
        assert np.array_equal(out, expected.astype(dt)), (prec, out)


SMALL = [(1, 2), (2, 4), (3, 6), (4, 4), (5, 10), (8, 8), (6, 12), (16, 30), (20, 24), (12, 40),
         (7, 14), (8, 14), (11, 22), (13, 26), (21, 44), (77, 130), (143, 182),
         (64, 128), (96, 160), (128, 256), (256, 256), (384, 640), (640, 384), (1, 1024), (1024, 2)]


@pytest.mark.parametrize("prec", ["f64", "f64-native", "f32"])
def test_small_and_ragged_shapes(gpu_lib, cuda, oracle_lib, prec):
    rng = np.random.default_rng(101)
    for nx, ny in SMALL:
        x = rng.uniform(0, 1, (nx, ny))
        got = forward(gpu_lib, cuda, x.astype(np.float32) if prec == "f32" else x, prec)
        ref = oracle_fwd(oracle_lib, x.astype(np.float32).astype(np.float64) if prec == "f32" else x)
        err = rel_l2(got, ref)
        assert err <= TOL[prec], (prec, nx, ny, err)


def test_golden_rfft2_fixtures(gpu_lib, cuda):
    data = np.load(os.path.join(GOLDEN, "rfft2_small.npz"))
    for key in data.files:
        if not key.startswith("x_"):
            continue
        x, X = data[key], data["X_" + key[2:]]
        assert rel_l2(forward(gpu_lib, cuda, x, "f64"), X) <= 1e-12, key


# shapes that exercise the thread-block-cluster paths: row transforms split
# over 2 CTAs (ny = 32768 in float-float) and column strips over 2..16 CTAs
CLUSTER_SHAPES = [(4096, 16), (8192, 8), (16384, 6), (32768, 4), (3, 32768), (2, 65536)]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_cluster_split_transforms(gpu_lib, cuda, oracle_lib, prec):
    rng = np.random.default_rng(202)
    for nx, ny in CLUSTER_SHAPES:
        if prec == "f64" and ny > 32768:
            continue
        x = rng.uniform(-1, 1, (nx, ny))
        xin = x.astype(np.float32) if prec == "f32" else x
        got = forward(gpu_lib, cuda, xin, prec)
        ref = oracle_fwd(oracle_lib, xin.astype(np.float64))
        assert rel_l2(got, ref) <= TOL[prec], (prec, nx, ny)


@pytest.mark.parametrize("strategy", ["cluster", "steps"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_column_strategies(gpu_lib, cuda, oracle_lib, monkeypatch, strategy, prec):
    """Both column passes: one cluster-split kernel, or two four-step kernels through scratch."""
    monkeypatch.setenv("HPXFFT_COLUMNS", strategy)
    rng = np.random.default_rng(303)
    for nx, ny in ((1024, 40), (4096, 64), (8192, 36), (16384, 18), (32768, 10)):
        x = rng.uniform(-1, 1, (nx, ny))
        xin = x.astype(np.float32) if prec == "f32" else x
        got = forward(gpu_lib, cuda, xin, prec)
        assert rel_l2(got, oracle_fwd(oracle_lib, xin.astype(np.float64))) <= TOL[prec], (strategy, nx, ny)
        # the inverse runs the same column pass backwards
        spec = np.ascontiguousarray(got).view(np.float32 if prec == "f32" else np.float64)
        with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, prec, "estimate") as plan:
            back = run_device(cuda, plan, spec, "c2r")
        assert rel_l2(back[:, :ny] / (nx * ny), xin) <= (1e-6 if prec == "f32" else 1e-13)


def test_4096_squared_fp64_config_vs_oracle(gpu_lib, cuda, oracle_lib):
    """4096^2 FP64, values uniform[0,1) from a seed: the small drop-in config."""
    x = np.random.default_rng(1).uniform(0, 1, (4096, 4096))
    err = rel_l2(forward(gpu_lib, cuda, x, "f64"), oracle_fwd(oracle_lib, x))
    assert err <= 1e-12, err


def sinusoid_input(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, n))
    i = np.arange(n)[:, None]
    j = np.arange(n)[None, :]
    for _ in range(4):
        fx, fy = rng.integers(1, n // 2, size=2)
        x += 10.0 * np.sin(2 * np.pi * (fx * i / n + fy * j / n))
    return x


def test_16384_squared_fp64_vs_oracle(gpu_lib, cuda, oracle_lib):
    """The headline size: uniform[-1,1) + four sinusoids of amplitude 10."""
    x = sinusoid_input(16384, 7)
    got = forward(gpu_lib, cuda, x, "f64")
    ref = oracle_fwd(oracle_lib, x)
    err = rel_l2(got, ref)
    assert err <= 1e-12, err


def test_16384_squared_fp32_vs_fp64_oracle(gpu_lib, cuda, oracle_lib):
    """The precision configuration's FP32 path at 16384^2, uniform[-1,1)
    input, against the FP64 oracle of the same (float-representable) input:
    relative L2 <= 2e-6, and the max-abs error stays a small multiple of
    float rounding at the largest |X|."""
    x = np.random.default_rng(3).uniform(-1, 1, (16384, 16384)).astype(np.float32)
    got = forward(gpu_lib, cuda, x, "f32")
    ref = oracle_fwd(oracle_lib, x.astype(np.float64))
    err = rel_l2(got, ref)
    assert err <= 2e-6, err
    max_abs = float(np.max(np.abs(got.astype(np.complex128) - ref)))
    assert max_abs <= 64 * np.finfo(np.float32).eps * float(np.max(np.abs(ref))), max_abs


def test_ramp_closed_form_large(gpu_lib, cuda):
    """Ramp x[i][j] = j at 8192 x 16384: known answer without an oracle run."""
    nx, ny = 8192, 16384
    x = np.tile(np.arange(ny, dtype=np.float64), (nx, 1))
    got = forward(gpu_lib, cuda, x, "f64")
    X = np.zeros((nx, ny // 2 + 1), dtype=np.complex128)
    X[0, 0] = nx * ny * (ny - 1) / 2
    k = np.arange(1, ny // 2 + 1)
    X[0, 1:] = nx * ny / (np.exp(-2j * np.pi * k / ny) - 1)
    assert rel_l2(got, X) <= 1e-12


def test_linearity_and_parseval(gpu_lib, cuda):
    rng = np.random.default_rng(33)
    nx, ny = 2048, 4096
    a, b = rng.uniform(-1, 1, (nx, ny)), rng.uniform(-1, 1, (nx, ny))
    A, B = forward(gpu_lib, cuda, a, "f64"), forward(gpu_lib, cuda, b, "f64")
    C = forward(gpu_lib, cuda, 2.0 * a - 3.0 * b, "f64")
    assert rel_l2(C, 2.0 * A - 3.0 * B) <= 1e-13
    # Parseval over the half spectrum: interior columns count twice
    w = np.full(ny // 2 + 1, 2.0)
    w[0] = w[-1] = 1.0
    energy = np.sum(w * np.abs(A) ** 2) / (nx * ny)
    assert abs(energy - np.sum(a * a)) <= 1e-12 * np.sum(a * a)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_shift_theorem_and_exact_sinusoid_peaks(gpu_lib, cuda, prec):
    """Oracle-free checks, the same helpers and shapes that
    test_oracle.py::test_spectral_properties pins on the oracle: a circular
    shift multiplies each bin by its exact phase, and integer-frequency
    sinusoids give their exact sparse half spectrum."""
    import spectral_properties as sp

    tol = 1e-12 if prec == "f64" else 2e-6

    def fwd(x):
        return forward(gpu_lib, cuda, x, prec)

    for nx, ny in ((77, 130), (96, 160), (256, 512), (2048, 4096)):
        a = np.random.default_rng(nx * 7 + ny).uniform(-1, 1, (nx, ny))
        assert sp.shift_error(fwd, a, nx // 3 + 1, -(ny // 5) - 1) <= tol, (nx, ny)
        x, X = sp.pure_sinusoids(nx, ny, 4, nx + ny)
        assert sp.rel_l2(fwd(x), X) <= tol, (nx, ny)


def test_batch_of_equal_transforms(gpu_lib, cuda, oracle_lib):
    rng = np.random.default_rng(44)
    xs = rng.uniform(-1, 1, (5, 96, 80))
    got = forward(gpu_lib, cuda, xs, "f64", batch=5)
    for i in range(5):
        assert rel_l2(got[i], oracle_fwd(oracle_lib, xs[i])) <= 1e-12


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_c2r_round_trip(gpu_lib, cuda, prec):
    rng = np.random.default_rng(55)
    for nx, ny in ((4, 4), (48, 60), (512, 1024), (4096, 64)):
        x = rng.uniform(-1, 1, (nx, ny))
        dt = np.float32 if prec == "f32" else np.float64
        with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, prec, "estimate") as plan:
            spec = run_device(cuda, plan, padded(x, dt), "forward")
            back = run_device(cuda, plan, spec, "c2r")
        assert rel_l2(back[:, :ny] / (nx * ny), x) <= (1e-13 if prec == "f64" else 1e-6)
        assert not back[:, ny:].any()


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_backward_matches_oracle_adjoint(gpu_lib, cuda, oracle_lib, prec):
    rng = np.random.default_rng(66)
    for nx, ny in ((4, 4), (6, 10), (64, 96), (2048, 256)):
        g = rng.standard_normal((nx, ny // 2 + 1)) + 1j * rng.standard_normal((nx, ny // 2 + 1))
        buf = np.ascontiguousarray(g).view(np.float64).copy()
        ref = oracle_lib.fft_2d_r2c_adjoint(buf.copy())
        dt = np.float32 if prec == "f32" else np.float64
        with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, prec, "estimate") as plan:
            got = run_device(cuda, plan, buf.astype(dt), "backward")
        tol = 1e-12 if prec == "f64" else 2e-6
        assert rel_l2(got[:, :ny], ref[:, :ny]) <= tol, (nx, ny)


def test_split_bf16_rejects_sizes_outside_the_direct_kernels(gpu_lib, cuda):
    """Primes above 13 take Bluestein's convolution in FP64 and FP32
    (test_gpu_bluestein.py); split-BF16 keeps the direct kernels' sizes."""
    for n_row, n_col in ((1024, 36), (17, 16), (1024 * 17, 8)):
        with pytest.raises(gpu_lib.HpxFftError) as e:
            gpu_lib.Plan(n_row, n_col, 1, "bf16x3", "estimate")
        assert e.value.status == gpu_lib._capi.HPXFFT_ERR_UNSUPPORTED_SIZE


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_every_compiled_row_shape(gpu_lib, cuda, oracle_lib, prec):
    """Row lengths M = 128 .. 8192 (the compiled row chains, with the last
    pass fused into the packed-real split where its radix allows), 39 rows so
    packed row groups are ragged."""
    rng = np.random.default_rng(39)
    for ny in (256, 512, 1024, 2048, 4096, 8192, 16384):
        x = rng.uniform(-1, 1, (39, ny))
        got = forward(gpu_lib, cuda, x.astype(np.float32) if prec == "f32" else x, prec)
        ref = oracle_fwd(oracle_lib, x.astype(np.float32).astype(np.float64) if prec == "f32" else x)
        assert rel_l2(got, ref) <= TOL[prec], (prec, ny)
