"""Batching: many uneven 2D r2c transforms in one persistent work-queue launch
replayed from a CUDA graph (GPU).  FP32, relative L2 <= 2e-6 against the
FP64 oracle."""
import numpy as np
import pytest

from gpu_helpers import rel_l2

pytestmark = pytest.mark.gpu

SIZES = [256, 384, 512, 640, 768, 1024, 1536, 2048, 2560, 3072, 4096]


def fill_arena(torch, batch, shapes, seed):
    """Per-instance uniform[-1,1) data generated on the device from per-instance seeds."""
    arena = torch.zeros(batch.arena_bytes // 4, dtype=torch.float32, device="cuda")
    for i, ((nx, ny), off) in enumerate(zip(shapes, batch.offsets)):
        g = torch.Generator(device="cuda")
        g.manual_seed(seed * 100003 + i)
        nc = 2 * (ny // 2 + 1)
        view = arena[off // 4: off // 4 + nx * nc].view(nx, nc)
        view[:, :ny] = torch.rand((nx, ny), generator=g, device="cuda") * 2 - 1
    return arena


def oracle_spectrum(oracle, x):
    p = oracle.padded(x.astype(np.float64))
    oracle.fft_2d_r2c(p, nthreads=16)
    return oracle.spectrum(p)


def run_batch(torch, batch, arena):
    batch.set_stream(torch.cuda.current_stream().cuda_stream)
    batch.execute(arena.data_ptr())
    batch.synchronize()
    torch.cuda.synchronize()


def test_mixed_small_batch_vs_oracle(gpu_lib, cuda, oracle_lib):
    rng = np.random.default_rng(5)
    shapes = [(int(rng.choice([16, 24, 40, 64, 96, 256, 384])), int(rng.choice([8, 12, 20, 64, 160, 640])))
              for _ in range(40)] + [(7, 14), (2, 2), (4096, 16), (16, 4096)]
    with gpu_lib.Batch([s[0] for s in shapes], [2 * (s[1] // 2 + 1) for s in shapes], "f32") as b:
        arena = fill_arena(cuda, b, shapes, 1)
        before = [v.copy() for v in b.views(arena.cpu().numpy().view(np.uint8))]
        run_batch(cuda, b, arena)
        after = b.views(arena.cpu().numpy().view(np.uint8))
        for (nx, ny), x0, y in zip(shapes, before, after):
            ref = oracle_spectrum(oracle_lib, x0[:, :ny])
            assert rel_l2(y.view(np.complex64), ref) <= 2e-6, (nx, ny)


def test_1024_uneven_fp32_transforms(gpu_lib, cuda, oracle_lib):
    """The batching workload: 1024 instances, nx and ny drawn independently
    from {2^k, 3*2^k, 5*2^k} between 256 and 4096."""
    rng = np.random.default_rng(1024)
    shapes = [(int(rng.choice(SIZES)), int(rng.choice(SIZES))) for _ in range(1024)]
    with gpu_lib.Batch([s[0] for s in shapes], [2 * (s[1] // 2 + 1) for s in shapes], "f32") as b:
        arena = fill_arena(cuda, b, shapes, 2)
        x_host = arena.cpu().numpy().view(np.uint8).copy()
        run_batch(cuda, b, arena)
        y_first = arena.cpu().numpy().view(np.uint8).copy()
        xs, ys = b.views(x_host), b.views(y_first)
        # every instance: Parseval over the half spectrum
        for (nx, ny), x, y in zip(shapes, xs, ys):
            X = y.view(np.complex64).astype(np.complex128)
            w = np.full(ny // 2 + 1, 2.0)
            w[0] = 1.0
            if ny % 2 == 0:
                w[-1] = 1.0
            e_spec = float(np.sum(w * np.abs(X) ** 2)) / (nx * ny)
            e_sig = float(np.sum(x[:, :ny].astype(np.float64) ** 2))
            assert abs(e_spec - e_sig) <= 1e-5 * e_sig, (nx, ny)
        # a subset against the oracle
        for i in rng.choice(len(shapes), 16, replace=False):
            nx, ny = shapes[i]
            ref = oracle_spectrum(oracle_lib, xs[i][:, :ny])
            assert rel_l2(ys[i].view(np.complex64), ref) <= 2e-6, shapes[i]
        # graph replay on fresh input gives the same result
        arena.copy_(cuda.from_numpy(x_host.view(np.float32)).cuda())
        run_batch(cuda, b, arena)
        assert np.array_equal(arena.cpu().numpy().view(np.uint8), y_first)
        assert b.measurement("total") > 0 and b.measurement("items") > 1024


def test_measure_flag_tunes_and_wisdom_round_trip(gpu_lib, cuda, oracle_lib, tmp_path):
    from hpxfft import batch as hb

    hb.wisdom_forget()
    shapes = [(256, 512), (384, 256), (512, 640), (1024, 768)] * 8
    nr, nc = [s[0] for s in shapes], [2 * (s[1] // 2 + 1) for s in shapes]
    with gpu_lib.Batch(nr, nc, "f32", "measure") as b:
        assert b.measurement("cached_plan") == 0.0
        tuned = (b.measurement("lag"), b.measurement("ctas_per_sm"))
        arena = fill_arena(cuda, b, shapes, 3)
        x = [v.copy() for v in b.views(arena.cpu().numpy().view(np.uint8))]
        run_batch(cuda, b, arena)
        y = b.views(arena.cpu().numpy().view(np.uint8))
        for (nx, ny), x0, y0 in zip(shapes[:4], x, y):
            assert rel_l2(y0.view(np.complex64), oracle_spectrum(oracle_lib, x0[:, :ny])) <= 2e-6
    path = tmp_path / "wisdom.txt"
    hb.wisdom_export(str(path))
    hb.wisdom_forget()
    with gpu_lib.Batch(nr, nc, "f32", "measure") as b:
        assert b.measurement("cached_plan") == 0.0  # forgotten
    hb.wisdom_forget()
    hb.wisdom_import(str(path))
    with gpu_lib.Batch(nr, nc, "f32", "measure") as b:
        assert b.measurement("cached_plan") == 1.0
        assert (b.measurement("lag"), b.measurement("ctas_per_sm")) == tuned
    bad = tmp_path / "bad.txt"
    bad.write_text("not wisdom\n")
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        hb.wisdom_import(str(bad))


def test_bounded_wait_runs_out_then_clean_run(gpu_lib, cuda, oracle_lib, monkeypatch):
    """The column items' wait for their instance's rows is bounded.  With the
    bound lowered to zero polls, a one-instance batch (1024 row items, then
    its column items, 304 persistent CTAs) hands out its first column items
    while row items are still in flight: those items give up at once, the
    kernel skips them and returns, and synchronize reports
    HPXFFT_ERR_TIMEOUT.  A batch planned afterwards with the default bound
    transforms the same input correctly."""
    shapes = [(4096, 4096)]
    nr, nc = [4096], [4098]
    monkeypatch.setenv("HPXFFT_BATCH_SPIN_LIMIT", "0")
    with gpu_lib.Batch(nr, nc, "f32", "estimate") as b:
        arena = fill_arena(cuda, b, shapes, 9)
        x_host = arena.cpu().numpy().view(np.uint8).copy()
        b.set_stream(cuda.cuda.current_stream().cuda_stream)
        b.execute(arena.data_ptr())
        with pytest.raises(gpu_lib.HpxFftError) as e:
            b.synchronize()
        assert e.value.status == gpu_lib._capi.HPXFFT_ERR_TIMEOUT
        cuda.cuda.synchronize()  # the context is still usable
    monkeypatch.delenv("HPXFFT_BATCH_SPIN_LIMIT")
    with gpu_lib.Batch(nr, nc, "f32", "estimate") as b:
        arena = cuda.from_numpy(x_host.view(np.float32).copy()).cuda()
        run_batch(cuda, b, arena)
        y = b.views(arena.cpu().numpy().view(np.uint8))[0]
        x = b.views(x_host)[0]
        assert rel_l2(y.view(np.complex64), oracle_spectrum(oracle_lib, x[:, :4096])) <= 2e-6


def test_batch_argument_errors(gpu_lib, cuda):
    with pytest.raises(gpu_lib.HpxFftInvalidArgument):
        gpu_lib.Batch([8], [10], "f32", "fast")
    with pytest.raises(gpu_lib.HpxFftError) as e:
        gpu_lib.Batch([8, 17], [10, 10], "f32")  # 17 rows: a prime above 13
    assert e.value.status == gpu_lib._capi.HPXFFT_ERR_UNSUPPORTED_SIZE
    with pytest.raises(gpu_lib.HpxFftError):
        gpu_lib.Batch([16384], [10], "f32")  # a column must fit one CTA
