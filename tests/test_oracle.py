"""The CPU oracle pinned against the reference's known answers (CPU only)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def ramp_spectrum(nx, ny):
    """Closed form of the examples' ramp input x[i][j] = j
    (examples/hpxfft/shared_loop_2d.cpp:33-40): X[kx != 0] = 0,
    X[0][0] = nx ny (ny-1)/2, X[0][k] = nx ny / (exp(-2 pi i k/ny) - 1)."""
    X = np.zeros((nx, ny // 2 + 1), dtype=np.complex128)
    X[0, 0] = nx * ny * (ny - 1) / 2
    k = np.arange(1, ny // 2 + 1)
    X[0, 1:] = nx * ny / (np.exp(-2j * np.pi * k / ny) - 1)
    return X


def test_kat_4x6_exact(oracle_lib):
    kat = json.load(open(os.path.join(GOLDEN, "kat_4x6.json")))
    v = np.array(kat["input_rows"], dtype=np.float64)
    oracle_lib.fft_2d_r2c(v)
    assert np.array_equal(v, np.array(kat["expected"]))  # REQUIRE(out == expected), test_shared_loop.cpp:53


@pytest.mark.parametrize("threads", [1, 3])
def test_rfft2_fixtures(oracle_lib, threads):
    data = np.load(os.path.join(GOLDEN, "rfft2_small.npz"))
    names = sorted(k[2:] for k in data.files if k.startswith("x_"))
    assert names
    for name in names:
        x, X = data["x_" + name], data["X_" + name]
        p = oracle_lib.padded(x)
        oracle_lib.fft_2d_r2c(p, nthreads=threads)
        assert oracle_lib.rel_l2(oracle_lib.spectrum(p), X) < 1e-14, name


@pytest.mark.parametrize("nx,ny", [(8, 14), (64, 64), (256, 1024), (384, 640)])
def test_ramp_closed_form(oracle_lib, nx, ny):
    x = np.tile(np.arange(ny, dtype=np.float64), (nx, 1))
    p = oracle_lib.padded(x)
    oracle_lib.fft_2d_r2c(p, nthreads=2)
    assert oracle_lib.rel_l2(oracle_lib.spectrum(p), ramp_spectrum(nx, ny)) < 1e-13


def test_one_dimensional_engines(oracle_lib):
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 5, 7, 12, 49, 60, 128, 243, 1000):
        z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        assert oracle_lib.rel_l2(oracle_lib.c2c_1d(z, -1), np.fft.fft(z)) < 1e-14
        assert oracle_lib.rel_l2(oracle_lib.c2c_1d(z, +1), np.fft.ifft(z) * n) < 1e-14
    for n in (2, 4, 6, 10, 30, 256, 1022):
        x = rng.standard_normal(n)
        assert oracle_lib.rel_l2(oracle_lib.r2c_1d(x), np.fft.rfft(x)) < 1e-14


def test_adjoint_against_dense_sum(oracle_lib):
    rng = np.random.default_rng(5)
    for nx, ny in ((4, 4), (6, 10), (16, 12), (5, 2)):
        g = rng.standard_normal((nx, ny // 2 + 1)) + 1j * rng.standard_normal((nx, ny // 2 + 1))
        buf = np.ascontiguousarray(g).view(np.float64).copy()
        oracle_lib.fft_2d_r2c_adjoint(buf)
        e1 = np.exp(2j * np.pi * np.outer(np.arange(nx), np.arange(nx)) / nx)
        e2 = np.exp(2j * np.pi * np.outer(np.arange(ny // 2 + 1), np.arange(ny)) / ny)
        assert oracle_lib.rel_l2(buf[:, :ny], np.real(e1 @ g @ e2)) < 1e-13
        assert not buf[:, ny:].any()


def test_adjoint_is_gradient_of_weighted_power(oracle_lib):
    """L = sum w |X|^2: the adjoint applied to G = 2 w X matches central differences."""
    rng = np.random.default_rng(7)
    nx, ny = 8, 10
    x = rng.uniform(-1, 1, (nx, ny))
    w = rng.uniform(0, 1, (nx, ny // 2 + 1))

    def loss(xx):
        return float(np.sum(w * np.abs(np.fft.rfft2(xx)) ** 2))

    p = oracle_lib.padded(x)
    oracle_lib.fft_2d_r2c(p)
    G = 2 * w * oracle_lib.spectrum(p)
    buf = np.ascontiguousarray(G).view(np.float64).copy()
    oracle_lib.fft_2d_r2c_adjoint(buf)
    h = 1e-6
    for _ in range(20):
        i, j = rng.integers(nx), rng.integers(ny)
        xp, xm = x.copy(), x.copy()
        xp[i, j] += h
        xm[i, j] -= h
        fd = (loss(xp) - loss(xm)) / (2 * h)
        assert abs(buf[i, j] - fd) <= 1e-6 * max(1.0, abs(fd))


def test_c2r_inverts_r2c(oracle_lib):
    rng = np.random.default_rng(9)
    for nx, ny in ((4, 4), (12, 30), (64, 96)):
        x = rng.standard_normal((nx, ny))
        p = oracle_lib.padded(x)
        oracle_lib.fft_2d_r2c(p)
        oracle_lib.fft_2d_c2r(p)
        assert oracle_lib.rel_l2(p[:, :ny] / (nx * ny), x) < 1e-14


def test_rejects_bad_layout(oracle_lib):
    with pytest.raises(RuntimeError):
        oracle_lib.fft_2d_r2c(np.zeros((4, 5)))
    with pytest.raises(ValueError):
        oracle_lib.fft_2d_r2c(np.zeros((4, 6), dtype=np.float32))


PROPERTY_SHAPES = [(77, 130), (96, 160), (256, 512), (2048, 4096)]


def oracle_forward(oracle_lib):
    def fwd(x):
        p = oracle_lib.padded(np.asarray(x, dtype=np.float64))
        oracle_lib.fft_2d_r2c(p, nthreads=8)
        return oracle_lib.spectrum(p)

    return fwd


@pytest.mark.parametrize("nx,ny", PROPERTY_SHAPES)
def test_spectral_properties(oracle_lib, nx, ny):
    """Linearity, Parseval, the shift theorem and exact sinusoid peaks: the
    same checks the GPU parity suite runs on the CUDA path."""
    import spectral_properties as sp

    fwd = oracle_forward(oracle_lib)
    rng = np.random.default_rng(nx * 7 + ny)
    a, b = rng.uniform(-1, 1, (nx, ny)), rng.uniform(-1, 1, (nx, ny))
    assert sp.linearity_error(fwd, a, b) <= 1e-14
    assert sp.parseval_error(fwd, a) <= 1e-13
    assert sp.shift_error(fwd, a, nx // 3 + 1, -(ny // 5) - 1) <= 1e-14
    x, X = sp.pure_sinusoids(nx, ny, 4, nx + ny)
    assert sp.rel_l2(fwd(x), X) <= 1e-14


def test_spectral_properties_catch_planted_mistakes(oracle_lib):
    """Each check fails on a transform with the mistake it is meant to see,
    planted in the oracle's output: the wrong sign (conjugated spectrum), a
    dropped bin and a stray scale."""
    import spectral_properties as sp

    fwd = oracle_forward(oracle_lib)
    nx, ny = 96, 160
    rng = np.random.default_rng(3)
    a, b = rng.uniform(-1, 1, (nx, ny)), rng.uniform(-1, 1, (nx, ny))
    x, X = sp.pure_sinusoids(nx, ny, 4, 11)

    def conj(v):
        return np.conj(fwd(v))

    assert sp.shift_error(conj, a, 5, 7) > 0.1
    assert sp.rel_l2(conj(x), X) > 0.1

    def scaled(v):
        return 1.001 * fwd(v)

    assert sp.parseval_error(scaled, a) > 1e-3

    def drops_bin(v):
        out = fwd(v)
        if np.abs(v).max() > 1.5:  # only the combined input
            out[3, 4] = 0
        return out

    assert sp.linearity_error(drops_bin, a, b) > 1e-4
