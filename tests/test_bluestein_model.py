"""The contracts of the Bluestein / transposed-row kernels compose to the
2D r2c, c2r and adjoint (CPU, numpy).

Each function below restates one kernel's contract as its header comment
gives it (hpx-fft_gb300/csrc/bluestein.cuh) and one plan sequence of
hpx-fft_gb300/csrc/plan.cu (run_alt_columns, run_alt_rows,
run_alt_rows_c2r); the column transforms of the sub-plans are numpy FFTs.
The compositions are checked against numpy.fft on prime, composite and
tiny shapes, and the host-side table rules (convolution length, the chirp's
phase reduced mod 2L) against their definitions.  The kernels themselves
are checked on the GPU by test_gpu_bluestein.py.
"""
import numpy as np
import pytest


def bluestein_length(L):
    M = 1
    while M < 2 * L - 1:
        M <<= 1
    return M


def tables(L, M):
    """chirp[n] = exp(-i pi n^2 / L) with n^2 reduced mod 2L in integers;
    kernel = DFT_M(b) / M, b[m] = b[M - m] = conj chirp[m] (m < L)."""
    n = np.arange(L, dtype=np.uint64)
    r = (n * n) % np.uint64(2 * L)
    chirp = np.exp(-2j * np.pi * r.astype(np.float64) / (2 * L))
    b = np.zeros(M, complex)
    b[:L] = np.conj(chirp)
    b[M - np.arange(1, L)] = np.conj(chirp[1:])
    return chirp, np.fft.fft(b) / M


def scale_rows(inp, tab, conj, rows_in, rows_out):
    f = np.conj(tab) if conj else tab
    out = np.zeros((rows_out, inp.shape[1]), complex)
    out[:rows_in] = inp[:rows_in] * f[:rows_in, None]
    return out


def transpose_scaled(src, src_rows, src_cols, dst_rows, dst_cols, tab, tab_on_col, conj):
    dst = np.zeros((dst_rows, dst_cols), complex)
    nr, nc = min(dst_rows, src_cols), min(dst_cols, src_rows)
    block = src[:nc, :nr].T.copy()  # dst[r][c] = src[c][r]
    if tab is not None:
        f = np.conj(tab) if conj else tab
        block *= f[:nc][None, :] if tab_on_col else f[:nr][:, None]
    dst[:nr, :nc] = block
    return dst


def r2c_split(t, h, chirp, nrows):
    k = np.arange(h + 1)
    ka, kb = k % h, (h - k) % h
    z = t[:h, :nrows] * (chirp[:h, None] if chirp is not None else 1)
    za, zb = z[ka], np.conj(z[kb])
    e, o = (za + zb) / 2, (za - zb) / 2
    wo = np.exp(-1j * np.pi * k / h)[:, None] * o
    return (e - 1j * wo).T  # out[i][k]


def c2r_merge(x, nrows, h, chirp, adjoint, t_rows, t_cols):
    a = x[:nrows, :h].copy()
    c = x[:nrows, h - np.arange(h)].copy()
    a[:, 0] = a[:, 0].real
    c[:, 0] = c[:, 0].real
    if adjoint:
        a[:, 1:] *= 0.5
        c[:, 1:] *= 0.5
    c = np.conj(c)
    s, d = a + c, a - c
    wd = np.conj(np.exp(-1j * np.pi * np.arange(h) / h))[None, :] * d
    z = s + 1j * wd
    if chirp is not None:
        z = z * np.conj(chirp[:h])[None, :]
    t = np.zeros((t_rows, t_cols), complex)
    t[:h, :nrows] = z.T
    return t


def convolve(scr, kernel, direction):
    y = np.fft.fft(scr, axis=0)
    y *= (np.conj(kernel) if direction > 0 else kernel)[:, None]
    return np.fft.ifft(y, axis=0) * scr.shape[0]  # unnormalised inverse


def alt_columns(data, direction):
    nx = data.shape[0]
    M = bluestein_length(nx)
    chirp, kernel = tables(nx, M)
    conj = direction > 0
    scr = scale_rows(data, chirp, conj, nx, M)
    scr = convolve(scr, kernel, direction)
    return scale_rows(scr, chirp, conj, nx, nx)


def alt_rows(data, nx, h, bluestein):
    width = (max(nx, 2) + 3) // 4 * 4
    M = bluestein_length(h) if bluestein else h
    chirp, kernel = tables(h, M) if bluestein else (None, None)
    t = transpose_scaled(data, nx, h, M, width, chirp, 0, 0)
    t = convolve(t, kernel, -1) if bluestein else np.fft.fft(t, axis=0)
    return r2c_split(t, h, chirp, nx)


def alt_rows_c2r(data, nx, h, bluestein, adjoint):
    width = (max(nx, 2) + 3) // 4 * 4
    M = bluestein_length(h) if bluestein else h
    chirp, kernel = tables(h, M) if bluestein else (None, None)
    t = c2r_merge(data, nx, h, chirp, adjoint, M, width)
    t = convolve(t, kernel, +1) if bluestein else np.fft.ifft(t, axis=0) * M
    return transpose_scaled(t, h, nx, nx, h + 1, chirp, 1, 1)


SHAPES = [(17, 34, True), (5, 38, True), (1, 46, True), (19, 22, False), (23, 16, False), (3, 202, True),
          (31, 2 * 97, True), (12, 2 * 60, False)]


@pytest.mark.parametrize("nx,ny,bluestein_rows", SHAPES)
def test_forward_composition(nx, ny, bluestein_rows):
    rng = np.random.default_rng(nx * 1000 + ny)
    h = ny // 2
    x = rng.standard_normal((nx, ny))
    packed = np.zeros((nx, h + 1), complex)
    packed[:, :h] = x[:, 0::2] + 1j * x[:, 1::2]
    rows = alt_rows(packed, nx, h, bluestein_rows)
    assert np.allclose(rows, np.fft.rfft(x, axis=1), rtol=0, atol=1e-12 * np.abs(rows).max())
    full = alt_columns(rows, -1)
    ref = np.fft.rfft2(x)
    assert np.abs(full - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("nx,ny,bluestein_rows", SHAPES)
@pytest.mark.parametrize("adjoint", [False, True])
def test_inverse_and_adjoint_composition(nx, ny, bluestein_rows, adjoint):
    rng = np.random.default_rng(nx * 7 + ny)
    h = ny // 2
    spec = rng.standard_normal((nx, h + 1)) + 1j * rng.standard_normal((nx, h + 1))
    cols = alt_columns(spec, +1)
    assert np.allclose(cols, np.fft.ifft(spec, axis=0) * nx, rtol=0, atol=1e-12 * np.abs(cols).max())
    packed = alt_rows_c2r(cols, nx, h, bluestein_rows, adjoint)
    assert not packed[:, h].any(), "the pad element stays zero"
    got = np.zeros((nx, ny))
    got[:, 0::2], got[:, 1::2] = packed[:, :h].real, packed[:, :h].imag
    half = cols.copy()
    half[:, 0] = half[:, 0].real  # the c2r ignores Im X[0] and Im X[h]
    half[:, -1] = half[:, -1].real
    if adjoint:
        half[:, 1:h] *= 0.5
    ref = np.fft.irfft(half, n=ny, axis=1) * ny
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_table_rules():
    for L in (1, 2, 3, 17, 1009, 4099, 16381):
        M = bluestein_length(L)
        assert M >= 2 * L - 1 and M & (M - 1) == 0 and (M == 1 or M // 2 < 2 * L - 1)
    # the reduced phase equals the unreduced one (exactly representable n here)
    L = 1031
    n = np.arange(L)
    chirp, kernel = tables(L, bluestein_length(L))
    assert np.allclose(chirp, np.exp(-1j * np.pi * (n.astype(np.float64) ** 2) / L), atol=1e-9)
    # the kernel is the spectrum of an even sequence: kernel[k] = kernel[M - k]
    assert np.allclose(kernel[1:], kernel[:0:-1], atol=1e-15)
