"""FP64 at 32768 x 32768 (8.6 GB per array) on the GPU.

The ramp x[i][j] = j has a closed form (no oracle needed); the
uniform-plus-sinusoids input of the scale workload is checked against the
oracle when the host has the memory for it.  Both skip when the host has
too little free memory, rather than push it into swapping.
"""
import numpy as np
import pytest

from gpu_helpers import rel_l2

pytestmark = pytest.mark.gpu
N = 32768
NC = 2 * (N // 2 + 1)


def mem_available_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


def transform(hpxfft, torch, host):
    """In place through the device; returns the complex spectrum."""
    dev = torch.from_numpy(host).cuda()
    del host
    with hpxfft.Plan(N, NC, 1, "f64", "estimate") as plan:
        plan.set_stream(torch.cuda.current_stream().cuda_stream)
        plan.execute_device(dev.data_ptr())
        torch.cuda.synchronize()
        plan.set_stream(None)
    out = dev.cpu().numpy()
    del dev
    torch.cuda.empty_cache()
    return out.view(np.complex128)


def test_ramp_closed_form_32768(gpu_lib, cuda):
    if mem_available_gb() < 40:
        pytest.skip("needs about 40 GB of free host memory")
    host = np.zeros((N, NC))
    host[:, :N] = np.arange(N, dtype=np.float64)[None, :]
    X = transform(gpu_lib, cuda, host)
    k = np.arange(1, N // 2 + 1)
    row0 = np.empty(N // 2 + 1, dtype=np.complex128)
    row0[0] = N * N * (N - 1) / 2
    row0[1:] = N * N / (np.exp(-2j * np.pi * k / N) - 1)
    err2 = np.sum(np.abs(X[0] - row0) ** 2)
    for r0 in range(1, N, 4096):  # every other row is zero
        err2 += np.sum(np.abs(X[r0: r0 + 4096]) ** 2)
    assert np.sqrt(err2) / np.linalg.norm(row0) <= 1e-12


def test_sinusoids_vs_oracle_32768(gpu_lib, cuda, oracle_lib):
    if mem_available_gb() < 64:
        pytest.skip("needs about 64 GB of free host memory")
    rng = np.random.default_rng(32768)
    host = np.zeros((N, NC))
    freqs = [rng.integers(1, N // 2, size=2) for _ in range(4)]
    j = np.arange(N)[None, :]
    for r0 in range(0, N, 2048):  # row chunks keep the temporaries small
        i = np.arange(r0, r0 + 2048)[:, None]
        block = rng.uniform(-1, 1, (2048, N))
        for fx, fy in freqs:
            block += 10.0 * np.sin(2 * np.pi * (((fx * i) % N) / N + ((fy * j) % N) / N))
        host[r0: r0 + 2048, :N] = block
    ref = host.copy()
    got = transform(gpu_lib, cuda, host)
    del host
    oracle_lib.fft_2d_r2c(ref, nthreads=16)
    assert rel_l2(got, oracle_lib.spectrum(ref)) <= 1e-12
