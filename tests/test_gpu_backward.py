"""Differentiation: the adjoint kernel (fft_2d_r2c_backward) as the gradient of
L = sum w |X|^2 over the half spectrum, for a batch of 64 FP32 2048 x 2048
transforms (GPU).

Checks, as the workload asks:
  - against FP64 central differences (h = 1e-6) at 256 random coordinates,
    the loss evaluated by the FP64 oracle;
  - against the oracle's FP64 adjoint (the host reference gradient) on two
    batch items: relative L2 <= 2e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

B, N = 64, 2048


def test_weighted_power_gradient_batch64_2048(gpu_lib, cuda, oracle_lib):
    torch = cuda
    rng = np.random.default_rng(2048)
    x = rng.uniform(-1.0, 1.0, (B, N, N)).astype(np.float32)
    w = rng.uniform(0.0, 1.0, (N, N // 2 + 1))
    nc = 2 * (N // 2 + 1)

    host = np.zeros((B, N, nc), dtype=np.float32)
    host[:, :, :N] = x
    dev = torch.from_numpy(host).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    with gpu_lib.Plan(N, nc, B, "f32", "estimate") as plan:
        plan.set_stream(stream)
        plan.execute_device(dev.data_ptr())  # X in place
        Xc = torch.view_as_complex(dev.view(B, N, nc // 2, 2))
        Xc.mul_(2.0 * torch.from_numpy(w).to(torch.float32).cuda())  # G = dL/dRe X + i dL/dIm X = 2 w X
        plan.backward_device(dev.data_ptr())
        torch.cuda.synchronize()
    grad = dev.cpu().numpy()[:, :, :N]
    assert np.isfinite(grad).all()

    def loss(b, xx):
        p = oracle_lib.padded(xx)
        oracle_lib.fft_2d_r2c(p, nthreads=16)
        return float(np.sum(w * np.abs(oracle_lib.spectrum(p)) ** 2))

    # central differences in FP64 on the FP32 input values
    h = 1e-6
    coords = [(rng.integers(B), rng.integers(N), rng.integers(N)) for _ in range(256)]
    by_item = {}
    for b, i, j in coords:
        by_item.setdefault(b, []).append((i, j))
    scale = float(np.sqrt(np.mean(grad[: 2].astype(np.float64) ** 2)))
    worst = 0.0
    for b, ij in by_item.items():
        base = x[b].astype(np.float64)
        # a central difference of an FP64 loss L carries rounding noise of
        # about eps * L / h; at h = 1e-6 that is ~1e-4 of the gradient scale
        fd_noise = 4 * np.finfo(np.float64).eps * loss(b, base) / (2 * h)
        for i, j in ij:
            xp = base.copy()
            xp[i, j] += h
            xm = base.copy()
            xm[i, j] -= h
            fd = (loss(b, xp) - loss(b, xm)) / (2 * h)
            worst = max(worst, abs(float(grad[b, i, j]) - fd) / (1e-5 * scale + fd_noise))
    assert worst <= 1.0, worst

    # the host reference gradient: oracle adjoint of G in FP64
    for b in (0, B - 1):
        p = oracle_lib.padded(x[b].astype(np.float64))
        oracle_lib.fft_2d_r2c(p, nthreads=16)
        G = 2.0 * w * oracle_lib.spectrum(p)
        ref = np.ascontiguousarray(G).view(np.float64).copy()
        oracle_lib.fft_2d_r2c_adjoint(ref, nthreads=16)
        g = grad[b].astype(np.float64)
        err = np.linalg.norm(g - ref[:, :N]) / np.linalg.norm(ref[:, :N])
        assert err <= 2e-6, (b, err)
