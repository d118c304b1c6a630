"""The reference's own tests, rewritten against the drop-in API (GPU).

Each follows test/src/test_*.cpp: the 4 x 6 padded fixture with rows
[1,2,3,4], initialize(std::move(values), "estimate"), the transform, then
REQUIRE(total >= 0) and REQUIRE(out == expected) with exact equality.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fixture(hpxfft, n_row=4, n_col=6):
    values = hpxfft.util.vector_2d(n_row, n_col, 0.0)
    for i in range(n_row):
        values[i, 0:4] = [1.0, 2.0, 3.0, 4.0]
    expected = hpxfft.util.vector_2d(n_row, n_col, 0.0)
    expected[0, 0] = 40.0
    expected[0, 2] = -8.0
    expected[0, 3] = 8.0
    expected[0, 4] = -8.0
    return values, expected


def test_shared_loop_par_and_seq(gpu_lib, cuda):
    # test/src/test_shared_loop.cpp:10-61
    for method in ("fft_2d_r2c_par", "fft_2d_r2c_seq", "fft_2d_r2c"):
        values, expected = fixture(gpu_lib)
        fft = gpu_lib.shared.loop()
        fft.initialize(values, "estimate")
        assert values.size() == 0  # moved in
        out = getattr(fft, method)()
        assert fft.get_measurement("total") >= 0.0
        assert fft.get_measurement("plan_flops") > 0.0
        assert out == expected


@pytest.mark.parametrize("variant", ["naive", "sync", "opt"])
def test_shared_task_variants(gpu_lib, cuda, variant):
    # test/src/test_naive.cpp, test_shared_sync.cpp, test_shared_opt.cpp
    values, expected = fixture(gpu_lib)
    fft = getattr(gpu_lib.shared, variant)()
    fft.initialize(values, "measure" if variant == "opt" else "estimate")
    out = fft.fft_2d_r2c()
    assert fft.get_measurement("total") >= 0.0
    assert out == expected


def test_distributed_loop_one_locality(gpu_lib, cuda):
    # test/src/test_distributed_loop.cpp:11-51 at one locality
    for comm in ("scatter", "all_to_all"):
        values, expected = fixture(gpu_lib)
        fft = gpu_lib.distributed.loop()
        fft.initialize(values, comm, "estimate")
        out = fft.fft_2d_r2c()
        assert fft.get_measurement("total") >= 0.0
        assert fft.get_measurement("first_comm") == 0.0
        assert out == expected


def test_measurement_keys_and_plan_file(gpu_lib, cuda, tmp_path):
    values, _ = fixture(gpu_lib, 64, 130)
    fft = gpu_lib.shared.loop()
    fft.initialize(values, "estimate")
    fft.fft_2d_r2c_par()
    for key in ("total", "first_fftw", "second_fftw", "plan", "plan_flops", "h2d", "d2h"):
        assert fft.get_measurement(key) >= 0.0, key
    assert fft.get_measurement("first_trans") == 0.0  # fused into the kernels
    assert fft.get_measurement("gbps") > 0.0 and fft.get_measurement("gflops") > 0.0
    assert 0.0 < fft.get_measurement("roofline") < 2.0  # of the nominal DRAM bandwidth
    assert fft.get_measurement("no such key") == 0.0  # loop.cpp:192 default-inserts 0
    path = tmp_path / "plans" / "plan.txt"
    with pytest.raises(RuntimeError, match="Failed to open file"):
        fft.write_plans_to_file(str(path))  # parent folder missing: loop.cpp:197-201
    path.parent.mkdir()
    fft.write_plans_to_file(str(path))
    fft.write_plans_to_file(str(path))
    text = path.read_text()
    assert text.count("GPU r2c 1D plan:") == 2 and text.count("GPU c2c 1D plan:") == 2


def test_ramp_driver_input(gpu_lib, cuda):
    """examples/hpxfft/shared_loop_2d.cpp builds x[i][j] = j (default nx=8, ny=14)."""
    nx, ny = 8, 14
    values = gpu_lib.util.vector_2d(nx, 2 * (ny // 2 + 1))
    for i in range(nx):
        values[i, :ny] = np.arange(ny)
    fft = gpu_lib.shared.loop()
    fft.initialize(values, "estimate")
    out = fft.fft_2d_r2c_par().data().view(np.complex128)
    assert np.allclose(out, np.fft.rfft2(np.tile(np.arange(ny, dtype=float), (nx, 1))), rtol=0, atol=1e-11)


def test_bad_plan_flag_throws_invalid_argument(gpu_lib, cuda):
    values, _ = fixture(gpu_lib)
    with pytest.raises(ValueError):
        gpu_lib.shared.loop().initialize(values, "quick")
    assert values.size() == 24  # nothing was moved


def test_cpp_dropin_headers(gpu_lib, cuda, build_mod):
    """The reference's C++ tests compiled against the drop-in headers."""
    import subprocess

    exe = build_mod.build_cpp()["test_dropin"]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all drop-in checks passed" in r.stdout


def test_cpp_shared_loop_driver(gpu_lib, cuda, build_mod, tmp_path):
    """hpxfft_gpu_shared_loop keeps the reference driver's CLI and output files."""
    import subprocess

    exe = build_mod.build_cpp()["hpxfft_gpu_shared_loop"]
    r = subprocess.run([exe, "--nx=64", "--ny", "96", "--plan=estimate", "--header=1"], capture_output=True,
                       text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FFT 2D runtime:" in r.stdout
    rows = (tmp_path / "runtimes" / "runtimes_hpx_shared_loop.txt").read_text().splitlines()
    assert rows[0].startswith("n_threads;n_x;n_y;plan;run_flag;total;")
    assert rows[1].split(";")[1:5] == ["64", "96", "estimate", "par"]
    plan = (tmp_path / "plans" / "plan_hpx_shared_loop.txt").read_text()
    assert "GPU r2c 1D plan:" in plan and "GPU c2c 1D plan:" in plan


def test_loop_backward_and_precisions(gpu_lib, cuda):
    """fft_2d_r2c_backward on the reference-style class (adjoint of an
    impulse at DC is all ones), and the FP32 / split-BF16 variants."""
    nx, ny = 1024, 64
    nc = 2 * (ny // 2 + 1)
    fft = gpu_lib.shared.loop()
    fft.initialize(gpu_lib.util.vector_2d(nx, nc), "estimate")
    g = gpu_lib.util.vector_2d(nx, nc)
    g[0, 0] = 1.0  # G[0][0] = 1: L = Re X[0][0] = sum of the inputs
    grad = fft.fft_2d_r2c_backward(g).data().reshape(nx, nc)
    assert np.allclose(grad[:, :ny], 1.0, rtol=0, atol=1e-13) and not grad[:, ny:].any()
    assert fft.get_measurement("total") > 0.0
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (nx, ny))
    for prec, tol in (("f32", 2e-6), ("bf16x3", 2e-6)):
        v = gpu_lib.util.vector_2d(nx, nc, dtype=np.float32)
        v.data()[:, :ny] = x
        f = gpu_lib.shared.loop()
        f.initialize(v, "estimate", precision=prec)
        out = f.fft_2d_r2c().data().reshape(nx, nc).astype(np.float64).view(np.complex128)
        ref = np.fft.rfft2(x.astype(np.float32).astype(np.float64))
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= tol, prec
