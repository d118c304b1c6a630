"""bench.py's multi-replica logic on CPU: world size 2 over gloo (no GPU).

With --gpus N each rank runs an independent replica; the reported step time
is the maximum over ranks and the value counts all ranks' bytes.  The
reference arm runs on rank 0 only; other ranks exit 0 silently."""
import importlib.util
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = _bench().replica_max_ms(1.0 + rank, world)  # rank 1 is the slow replica
    q.put((rank, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 2.0, 1: 2.0}


def test_single_rank_is_untouched():
    assert _bench().replica_max_ms(3.5, 1) == 3.5


def test_reference_arm_other_ranks_exit_silently():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_headline_kernels_have_profiled_traffic():
    """bench.py's roofline.traffic comes from the committed ncu summary: every
    kernel the FP64 16384^2 line can name as dominant must be found there,
    at a plausible fraction of the algorithmic bytes per launch (2 S)."""
    bench = _bench()
    alg = 2 * 16384 * 8193 * 16  # read + write of S = nx (ny/2+1) complex doubles
    for label in ("row_r2c_kernel", "colstep_warp_kernel (A)", "colstep_warp_kernel (B)"):
        t = bench.profiled_traffic("f64", 16384, 16384, label)
        assert t is not None and 0.8 * alg <= t <= 1.5 * alg, (label, t)
    assert bench.profiled_traffic("f32", 16384, 16384, "row_r2c_kernel") is None
