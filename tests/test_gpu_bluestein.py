"""Sizes outside the direct kernels (GPU) against the oracle.

FFTW, which the reference calls for both passes, takes any n_row and any
even ny (core/src/shared/loop.cpp:163-182, core/src/util/adapter_fftw.cpp:
6-34).  Here three paths cover what the direct kernels do not:
  - Bluestein's convolution through power-of-two column plans, for a length
    with a prime factor above 13 (columns: n_row; rows: ny/2);
  - the row pass as a column pass on a transposed copy, for rows longer than
    a CTA cluster holds (ny/2 = 3 * 2^14, 2^17);
  - the two-kernel column pass alone, for power-of-two columns longer than a
    cluster holds (n_row = 2^17, 2^18).
The oracle (a mixed-radix restatement whose generic radix-p step is an
O(p^2) DFT, so any length) checks the forward transform, the c2r and the
adjoint.  The largest case, 4099 x 8198 (both lengths prime), is checked
against numpy's pocketfft instead, which runs it in seconds.

Tolerances (relative L2): f64 (float-float) and f64-native (DFMA) <= 1e-12; f32 <= 2e-6
against the FP64 oracle on FP32-representable inputs.
"""
import numpy as np
import pytest

from gpu_helpers import padded, rel_l2, run_device

pytestmark = pytest.mark.gpu
TOL = {"f64": 1e-12, "f64-native": 1e-12, "f32": 2e-6}

# (n_row, ny, Bluestein M for rows, Bluestein M for columns, rows transposed)
SHAPES = [
    (17, 34, 64, 64, 1),            # both lengths prime
    (1, 38, 64, 0, 1),              # one row of ny/2 = 19
    (1009, 64, 0, 2048, 0),         # prime columns, direct rows
    (64, 2 * 1031, 4096, 0, 1),     # prime rows, direct columns
    (97, 2 * 89, 256, 256, 1),
    (2 * 3 * 1009, 40, 0, 16384, 0),  # a large prime factor in a composite length
    (3, 2 * 8191, 16384, 0, 1),     # the Mersenne prime 8191 along rows
    (8, 2 * 3 * 16384, 0, 0, 1),    # rows of 3 * 2^14 complex values: transposed, no Bluestein
    (4, 2 * 131072, 0, 0, 1),       # rows of 2^17 complex values: transposed, two-kernel columns
    (131072, 6, 0, 0, 0),           # 2^17 columns: the two-kernel pass alone
    (3 * 65536, 6, 0, 524288, 0),   # smooth but longer than a cluster holds: Bluestein
]


def forward(gpu_lib, cuda, x, prec, batch=1, flag="estimate"):
    nx, ny = x.shape[-2:]
    dt = np.float32 if prec == "f32" else np.float64
    host = np.zeros(x.shape[:-1] + (2 * (ny // 2 + 1),), dtype=dt)
    host[..., :ny] = x
    with gpu_lib.Plan(nx, host.shape[-1], batch, prec, flag) as plan:
        out = run_device(cuda, plan, host)
        paths = tuple(plan.measurement(k) for k in ("bluestein_rows", "bluestein_columns", "transposed_rows"))
    return out.astype(np.float64), paths


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_forward_matches_oracle(gpu_lib, cuda, oracle_lib, prec):
    rng = np.random.default_rng(1009)
    for nx, ny, mr, mc, tr in SHAPES:
        x = rng.uniform(-1, 1, (nx, ny))
        if prec == "f32":
            x = x.astype(np.float32).astype(np.float64)
        got, paths = forward(gpu_lib, cuda, x, prec)
        assert paths == (mr, mc, tr), (nx, ny, paths)
        ref = oracle_lib.fft_2d_r2c(padded(x), nthreads=16)
        err = rel_l2(got, ref)
        assert err <= TOL[prec], (prec, nx, ny, err)


def test_power_of_two_columns_beyond_a_cluster_f32(gpu_lib, cuda, oracle_lib):
    rng = np.random.default_rng(262144)
    x = rng.uniform(-1, 1, (262144, 6)).astype(np.float32).astype(np.float64)
    got, paths = forward(gpu_lib, cuda, x, "f32")
    assert paths == (0, 0, 0)
    assert rel_l2(got, oracle_lib.fft_2d_r2c(padded(x), nthreads=16)) <= 2e-6


def test_native_fp64_arithmetic(gpu_lib, cuda, oracle_lib):
    rng = np.random.default_rng(17)
    for nx, ny in ((17, 34), (1009, 64), (64, 2 * 1031)):
        x = rng.uniform(-1, 1, (nx, ny))
        got, _ = forward(gpu_lib, cuda, x, "f64-native")
        assert rel_l2(got, oracle_lib.fft_2d_r2c(padded(x), nthreads=16)) <= 1e-12, (nx, ny)


def test_batch_of_three(gpu_lib, cuda, oracle_lib):
    rng = np.random.default_rng(3)
    for nx, ny in ((97, 2 * 89), (1009, 64), (8, 2 * 3 * 16384)):
        xs = rng.uniform(-1, 1, (3, nx, ny))
        got, _ = forward(gpu_lib, cuda, xs, "f64", batch=3)
        for b in range(3):
            assert rel_l2(got[b], oracle_lib.fft_2d_r2c(padded(xs[b]), nthreads=16)) <= 1e-12, (nx, ny, b)


def half_spectrum(rng, nx, ny):
    g = rng.standard_normal((nx, ny // 2 + 1)) + 1j * rng.standard_normal((nx, ny // 2 + 1))
    return np.ascontiguousarray(g).view(np.float64).copy()


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("op", ["c2r", "backward"])
def test_inverse_and_adjoint_match_oracle(gpu_lib, cuda, oracle_lib, prec, op):
    """Random half spectra, non-zero imaginary parts at DC and Nyquist
    included (the c2r ignores them)."""
    rng = np.random.default_rng(811)
    dt = np.float32 if prec == "f32" else np.float64
    for nx, ny, _, _, _ in SHAPES[:9]:
        spec = half_spectrum(rng, nx, ny)
        if prec == "f32":
            spec = spec.astype(np.float32).astype(np.float64)
        with gpu_lib.Plan(nx, spec.shape[1], 1, prec, "estimate") as plan:
            got = run_device(cuda, plan, spec.astype(dt), op).astype(np.float64)
        if op == "c2r":
            ref = oracle_lib.fft_2d_c2r(spec.copy(), nthreads=16)
        else:
            ref = oracle_lib.fft_2d_r2c_adjoint(spec.copy(), nthreads=16)
        err = rel_l2(got[:, :ny], ref[:, :ny])
        assert err <= TOL[prec], (prec, op, nx, ny, err)
        assert not got[:, ny:].any(), "pad reals must be zero"


def test_round_trip_and_large_primes_against_pocketfft(gpu_lib, cuda):
    """4099 x 8198 (4099 prime along both axes, Bluestein on both passes),
    FP64: the forward against numpy's pocketfft, and c2r(r2c(x)) = nx ny x."""
    rng = np.random.default_rng(4099)
    nx, ny = 4099, 8198
    x = rng.uniform(-1, 1, (nx, ny))
    host = padded(x)
    with gpu_lib.Plan(nx, host.shape[1], 1, "f64", "estimate") as plan:
        assert plan.measurement("bluestein_rows") == 16384  # 2 * 4099 - 1 rounded up
        assert plan.measurement("bluestein_columns") == 16384
        X = run_device(cuda, plan, host)
        back = run_device(cuda, plan, X.copy(), "c2r")
    assert rel_l2(X, np.fft.rfft2(x).view(np.float64)) <= 1e-12
    assert rel_l2(back[:, :ny] / (nx * ny), x) <= 1e-12


def test_host_buffers_and_plan_search(gpu_lib, cuda, oracle_lib):
    """The host-buffer entry point (staged copies) and a "measure" plan on a
    Bluestein shape; the plan description names the path."""
    rng = np.random.default_rng(97)
    nx, ny = 97, 2 * 89
    x = rng.uniform(-1, 1, (nx, ny))
    ref = oracle_lib.fft_2d_r2c(padded(x), nthreads=16)
    with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, "f64", "measure") as plan:
        got = plan.execute_host(padded(x))
        assert plan.measurement("bluestein_columns") == 256
    assert rel_l2(got, ref) <= 1e-12


def test_plan_description_names_the_path(gpu_lib, cuda, tmp_path):
    path = tmp_path / "plans.txt"
    with gpu_lib.Plan(97, 2 * 90, 1, "f64", "estimate") as plan:
        plan.write_plan(str(path))
    text = path.read_text()
    assert "Bluestein, length 89 through 256" in text
    assert "Bluestein, length 97 through 256" in text


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_random_sizes_against_pocketfft(gpu_lib, cuda, prec):
    """30 seeded random shapes, n_row in [1, 6000] and even ny in [2, 12000]
    (smooth, prime and mixed lengths, so every path and the direct kernels
    alternate), forward and c2r against numpy's pocketfft."""
    rng = np.random.default_rng(40)
    dt = np.float32 if prec == "f32" else np.float64
    tol = TOL[prec]
    for _ in range(30):
        nx = int(rng.integers(1, 6001))
        ny = 2 * int(rng.integers(1, 6001))
        x = rng.uniform(-1, 1, (nx, ny))
        if prec == "f32":
            x = x.astype(np.float32).astype(np.float64)
        with gpu_lib.Plan(nx, 2 * (ny // 2 + 1), 1, prec, "estimate") as plan:
            X = run_device(cuda, plan, padded(x).astype(dt)).astype(np.float64)
            back = run_device(cuda, plan, X.astype(dt), "c2r").astype(np.float64)
        ref = np.fft.rfft2(x)
        assert rel_l2(X.view(np.complex128), ref) <= tol, (prec, nx, ny)
        assert rel_l2(back[:, :ny] / (nx * ny), x) <= 2 * tol, (prec, nx, ny)

