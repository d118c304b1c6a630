"""3D r2c (GPU) against numpy.fft.rfftn in FP64: a batched 2D r2c over the
n0 slabs, then the column pass along axis 0.

Tolerances as the 2D paths: f64 <= 1e-12, f32 <= 2e-6 (relative L2)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(4, 6, 8), (8, 16, 30), (6, 10, 14), (32, 64, 128), (64, 32, 96), (128, 128, 128), (256, 64, 40),
          (1024, 8, 16), (8, 1024, 6)]


def run3d(hpxfft, torch, x, prec, batch=1):
    n0, n1, n2 = x.shape[-3:]
    nc = 2 * (n2 // 2 + 1)
    dt = np.float64 if prec == "f64" else np.float32
    host = np.zeros(x.shape[:-1] + (nc,), dtype=dt)
    host[..., :n2] = x
    dev = torch.from_numpy(host).cuda()
    with hpxfft.Plan3D(n0, n1, nc, batch, prec, "estimate") as plan:
        assert plan.buffer_bytes() == host.nbytes
        plan.set_stream(torch.cuda.current_stream().cuda_stream)
        plan.execute_device(dev.data_ptr())
        torch.cuda.synchronize()
        assert plan.measurement("total") > 0.0
        assert plan.measurement("third_fftw") > 0.0
    out = dev.cpu().numpy()
    return out.view(np.complex128 if dt == np.float64 else np.complex64)


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 2e-6)])
def test_3d_vs_numpy(gpu_lib, cuda, prec, tol):
    rng = np.random.default_rng(3)
    for shape in SHAPES:
        x = rng.uniform(-1, 1, shape)
        if prec == "f32":
            x = x.astype(np.float32).astype(np.float64)
        got = run3d(gpu_lib, cuda, x, prec)
        assert rel(got, np.fft.rfftn(x)) <= tol, (prec, shape)


def test_3d_batch_and_large(gpu_lib, cuda):
    rng = np.random.default_rng(4)
    xs = rng.uniform(-1, 1, (3, 16, 48, 64))
    got = run3d(gpu_lib, cuda, xs, "f64", batch=3)
    for i in range(3):
        assert rel(got[i], np.fft.rfftn(xs[i])) <= 1e-12
    x = rng.uniform(-1, 1, (256, 256, 512))  # 256 MB in, the two-step column pass along axis 0 is not used
    assert rel(run3d(gpu_lib, cuda, x, "f64"), np.fft.rfftn(x)) <= 1e-12
    x = rng.uniform(-1, 1, (8192, 4, 8))  # axis 0 long enough for the two-step column pass
    assert rel(run3d(gpu_lib, cuda, x, "f64"), np.fft.rfftn(x)) <= 1e-12


def test_3d_prime_lengths(gpu_lib, cuda):
    """Primes above 13 along each axis: Bluestein's convolution in the slab
    plan's rows and columns and in the column pass along axis 0."""
    rng = np.random.default_rng(5)
    for shape in ((17, 6, 8), (4, 19, 8), (6, 10, 34), (17, 23, 38)):
        x = rng.uniform(-1, 1, shape)
        assert rel(run3d(gpu_lib, cuda, x, "f64"), np.fft.rfftn(x)) <= 1e-12, shape


def test_3d_argument_errors(gpu_lib, cuda):
    with pytest.raises(gpu_lib.HpxFftError):
        gpu_lib.Plan3D(0, 4, 6)
    with pytest.raises(gpu_lib.HpxFftError):
        gpu_lib.Plan3D(70000, 4, 6)  # n0 * batch above 65535
