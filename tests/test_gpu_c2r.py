"""Inverse (c2r) path vs the oracle's c2r on arbitrary half spectra (GPU).

The FFTW backward direction is declared by the reference
(core/include/hpxfft/util/adapter_fftw.hpp:11) but never planned; the
oracle's fft_2d_c2r restates the unnormalised 2D inverse: inverse c2c along
x over every complex column, then a c2r along y that ignores the imaginary
parts of the DC and Nyquist bins of each row.  The spectra here are random
everywhere, DC and Nyquist imaginary parts included, so a kernel that used
those parts (or dropped them before the column pass) fails the comparison.

Tolerances (relative L2 over the nx*ny real outputs):
  f64 (float-float arithmetic)  <= 1e-12
  f32                           <= 2e-6   (against the FP64 oracle)
"""
import numpy as np
import pytest

from gpu_helpers import rel_l2, run_device

pytestmark = pytest.mark.gpu
TOL = {"f64": 1e-12, "f32": 2e-6}


def half_spectrum(rng, nx, ny):
    """Random complex half spectrum in the padded layout (float64), with
    non-zero imaginary parts at ky = 0 and ky = ny/2."""
    g = rng.standard_normal((nx, ny // 2 + 1)) + 1j * rng.standard_normal((nx, ny // 2 + 1))
    assert np.all(g[:, 0].imag != 0) and np.all(g[:, -1].imag != 0)
    return np.ascontiguousarray(g).view(np.float64).copy()


def c2r_gpu(gpu_lib, cuda, spec, prec):
    nx, n_col = spec.shape
    dt = np.float32 if prec == "f32" else np.float64
    with gpu_lib.Plan(nx, n_col, 1, prec, "estimate") as plan:
        return run_device(cuda, plan, spec.astype(dt), "c2r")


def c2r_oracle(oracle_lib, spec):
    return oracle_lib.fft_2d_c2r(np.ascontiguousarray(spec, dtype=np.float64).copy(), nthreads=8)


# small and ragged (odd radices, packed rows), the cluster column kernel,
# the two-kernel four-step column pass, long rows
SHAPES = [(1, 2), (2, 4), (3, 6), (5, 10), (7, 14), (12, 40), (77, 130), (143, 182), (256, 256),
          (384, 640), (1024, 36), (4096, 64), (8192, 18), (64, 8192), (16, 16384)]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_c2r_matches_oracle_on_random_half_spectra(gpu_lib, cuda, oracle_lib, prec):
    rng = np.random.default_rng(808)
    for nx, ny in SHAPES:
        spec = half_spectrum(rng, nx, ny)
        if prec == "f32":
            spec = spec.astype(np.float32).astype(np.float64)
        got = c2r_gpu(gpu_lib, cuda, spec, prec)
        ref = c2r_oracle(oracle_lib, spec)
        err = rel_l2(got[:, :ny], ref[:, :ny])
        assert err <= TOL[prec], (prec, nx, ny, err)
        assert not got[:, ny:].any(), "pad reals must be zero"


@pytest.mark.parametrize("strategy", ["cluster", "steps"])
def test_c2r_both_column_strategies(gpu_lib, cuda, oracle_lib, monkeypatch, strategy):
    monkeypatch.setenv("HPXFFT_COLUMNS", strategy)
    rng = np.random.default_rng(809)
    for nx, ny in ((2048, 40), (16384, 18)):
        spec = half_spectrum(rng, nx, ny)
        for prec in ("f64", "f32"):
            s = spec.astype(np.float32).astype(np.float64) if prec == "f32" else spec
            got = c2r_gpu(gpu_lib, cuda, s, prec)
            assert rel_l2(got[:, :ny], c2r_oracle(oracle_lib, s)[:, :ny]) <= TOL[prec], (strategy, prec, nx, ny)


def test_c2r_ignores_dc_and_nyquist_imaginary_parts(gpu_lib, cuda, oracle_lib):
    """Changing only Im X[kx][0] and Im X[kx][ny/2] after the column inverse
    must leave the output unchanged; at the spectrum level that is the
    inverse column transform of those parts, so compare two spectra that
    differ by a purely imaginary column pair whose column inverse is purely
    imaginary (a real, even-symmetric column vector times i)."""
    rng = np.random.default_rng(810)
    nx, ny = 64, 96
    spec = half_spectrum(rng, nx, ny)
    g = spec.view(np.complex128)
    # a column whose inverse DFT along x is real: Hermitian in kx
    h = rng.standard_normal(nx) + 1j * rng.standard_normal(nx)
    h = h + np.conj(np.roll(h[::-1], 1))
    g2 = g.copy()
    g2[:, 0] += 1j * h
    g2[:, -1] += 1j * h
    spec2 = np.ascontiguousarray(g2).view(np.float64).copy()
    a = c2r_gpu(gpu_lib, cuda, spec, "f64")
    b = c2r_gpu(gpu_lib, cuda, spec2, "f64")
    assert rel_l2(b[:, :ny], a[:, :ny]) <= 1e-13
    assert rel_l2(b[:, :ny], c2r_oracle(oracle_lib, spec2)[:, :ny]) <= 1e-12


def test_c2r_4096_squared_fp64(gpu_lib, cuda, oracle_lib):
    """The FP64 inverse at the 4096^2 configuration's size."""
    rng = np.random.default_rng(811)
    spec = half_spectrum(rng, 4096, 4096)
    got = c2r_gpu(gpu_lib, cuda, spec, "f64")
    ref = c2r_oracle(oracle_lib, spec)
    err = rel_l2(got[:, :4096], ref[:, :4096])
    assert err <= 1e-12, err
