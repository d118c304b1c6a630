"""Size-independent properties of the 2D r2c, written once and checked with
any forward transform `fwd(x) -> X` (x: nx x ny reals; X: nx x (ny/2+1)
complex, [kx][ky] orientation, unnormalised, sign -1): the oracle on the
CPU and the CUDA path on the GPU.

Phases and sinusoid arguments are reduced exactly in integers
((a*b) mod (nx*ny)) before the one division and the sin/exp call, so the
reference values carry no argument-reduction error at large sizes.
"""
import numpy as np

from gpu_helpers import rel_l2


def half_weights(ny):
    """Parseval weight of each half-spectrum column: 1 for DC and (even ny)
    Nyquist, 2 for the interior columns, which stand for their mirrors."""
    w = np.full(ny // 2 + 1, 2.0)
    w[0] = 1.0
    if ny % 2 == 0:
        w[-1] = 1.0
    return w


def linearity_error(fwd, a, b, alpha=2.0, beta=-3.0):
    """rel-L2 of F(alpha a + beta b) against alpha F(a) + beta F(b)."""
    return rel_l2(fwd(alpha * a + beta * b), alpha * fwd(a) + beta * fwd(b))


def parseval_error(fwd, x):
    """|sum_half w |X|^2 / (nx ny) - sum x^2| relative to sum x^2."""
    nx, ny = x.shape
    X = fwd(x)
    e_spec = float(np.sum(half_weights(ny) * np.abs(X) ** 2)) / (nx * ny)
    e_sig = float(np.sum(np.asarray(x, dtype=np.float64) ** 2))
    return abs(e_spec - e_sig) / e_sig


def shift_phase(nx, ny, sx, sy):
    """exp(-2 pi i (kx sx/nx + ky sy/ny)) over the half spectrum: the factor
    a circular shift of the input by (sx, sy) puts on each bin."""
    kx = np.arange(nx, dtype=np.int64)[:, None]
    ky = np.arange(ny // 2 + 1, dtype=np.int64)[None, :]
    m = (kx * (sx % nx) * ny + ky * (sy % ny) * nx) % (nx * ny)
    return np.exp(-2j * np.pi * (m / (nx * ny)))


def shift_error(fwd, x, sx, sy):
    """rel-L2 of F(roll(x, (sx, sy))) against shift_phase * F(x)."""
    nx, ny = x.shape
    X = fwd(x)
    Xs = fwd(np.roll(x, (sx, sy), axis=(0, 1)))
    return rel_l2(Xs, shift_phase(nx, ny, sx, sy) * X)


def pure_sinusoids(nx, ny, count, seed, amplitude=10.0):
    """x[i][j] = sum_m A sin(2 pi (fx_m i/nx + fy_m j/ny)) with integer
    frequencies 1 <= fx_m < nx/2, 1 <= fy_m < ny/2, and its exact half
    spectrum. sin t = (e^{it} - e^{-it}) / 2i, so each term puts
    -i A nx ny / 2 in bin (fx, fy); its mirror (nx-fx, ny-fy) has
    ky > ny/2 and lies outside the half spectrum. Needs nx, ny >= 4."""
    rng = np.random.default_rng(seed)
    i = np.arange(nx, dtype=np.int64)[:, None]
    j = np.arange(ny, dtype=np.int64)[None, :]
    x = np.zeros((nx, ny))
    X = np.zeros((nx, ny // 2 + 1), dtype=np.complex128)
    for _ in range(count):
        fx = int(rng.integers(1, nx // 2))
        fy = int(rng.integers(1, ny // 2))
        m = (fx * i * ny + fy * j * nx) % (nx * ny)
        x += amplitude * np.sin(2 * np.pi * (m / (nx * ny)))
        X[fx, fy] += -0.5j * amplitude * nx * ny
    return x, X
