"""Slab decomposition over P ranks, host side (CPU, gloo).

hpxfft.distributed.loop at P > 1 runs its local phases on the rank's GPU
(hpxfft_slab_*) and moves the tiles with torch.distributed collectives.  On
this CPU-only check the local phases are a numpy stand-in that follows the
tile layout the C ABI documents (include/hpxfft_gb300.h, hpxfft_slab_*);
everything else is the product's code: the rank and size bookkeeping, the
two exchanges in both of the reference's schemes (one all_to_all or P
scatters, core/src/distributed/loop.cpp:39-84) and the move-in / move-out
ownership.  Every rank's result is compared with its rows of the oracle's
full transform.  The input has energy at every kx, which the reference's
own distributed tests lack (their input varies along y only,
test/src/test_distributed_loop.cpp:22-39), and dcy is not a multiple of P.
The GPU kernels of the same layout are checked in test_gpu_slab.py.
"""
import os
import socket

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class NumpySlabCompute:
    """Local phases with numpy on CPU tensors, in the C ABI's tile layout:
    send[d][x][k] = X[x][d w + k] (zero past dcy), the received tiles are the
    column slab [nx][w], the second exchange's tile s holds columns s w ..
    of this rank's rows."""

    def __init__(self, n_row_local, n_col, n_ranks, rank, precision, plan_flag):
        import torch

        self.torch = torch
        self.nxl, self.ncol, self.P = n_row_local, n_col, n_ranks
        self.dcy = n_col // 2
        self.w = -(-self.dcy // n_ranks)
        n = n_ranks * n_row_local * self.w * 16
        self.recv = torch.zeros(n, dtype=torch.uint8)
        self.recv2 = torch.zeros(n, dtype=torch.uint8)

    def _c(self, t):
        return t.numpy().view(np.complex128)

    def rows(self, values):
        X = np.fft.rfft(values[:, : 2 * self.dcy - 2], axis=1)
        tiles = np.zeros((self.P, self.nxl, self.w), dtype=np.complex128)
        for d in range(self.P):
            cols = X[:, d * self.w: (d + 1) * self.w]
            tiles[d, :, : cols.shape[1]] = cols
        return self.torch.from_numpy(tiles.reshape(-1).view(np.uint8).copy())

    def columns(self, recv):
        slab = self._c(recv).reshape(self.P * self.nxl, self.w)
        slab[...] = np.fft.fft(slab, axis=0)
        return recv

    def finish(self, recv2, values):
        tiles = self._c(recv2).reshape(self.P, self.nxl, self.w)
        out = values.view(np.complex128)
        for s in range(self.P):
            n = min(self.w, self.dcy - s * self.w)
            out[:, s * self.w: s * self.w + n] = tiles[s, :, :n]

    def synchronize(self):
        pass

    def measurement(self, name):
        return 0.0

    def close(self):
        pass


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _full_input(nx, ny, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((nx, 2 * (ny // 2 + 1)))
    x[:, :ny] = rng.uniform(-1, 1, (nx, ny))
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    x[:, :ny] += 5.0 * np.cos(2 * np.pi * (3 * i / nx + 2 * j / ny))  # energy at kx = 3
    return x


def _rank_main(rank, world, port, nx, ny, comm, q):
    import sys

    for p in (os.path.join(REPO, "hpx-fft_gb300", "python"), os.path.join(REPO, "tests")):
        sys.path.insert(0, p)
    import torch.distributed as dist

    import hpxfft
    from test_distributed_slab import NumpySlabCompute, _full_input

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        full = _full_input(nx, ny, 7)
        nxl = nx // world
        mine = hpxfft.util.vector_2d.from_array(full[rank * nxl:(rank + 1) * nxl].copy())
        lp = hpxfft.distributed.loop(local_compute=NumpySlabCompute)
        lp.initialize(mine, comm, "estimate")
        out = lp.fft_2d_r2c()
        q.put((rank, out.data().copy(), lp.get_measurement("first_comm") >= 0.0))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,nx,ny,comm", [(2, 8, 12, "all_to_all"), (2, 6, 10, "scatter"),
                                              (3, 12, 20, "all_to_all"), (3, 9, 16, "scatter")])
def test_slab_exchange_over_gloo_ranks_matches_oracle(oracle_lib, gpu_lib, world, nx, ny, comm):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, world, port, nx, ny, comm, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict((r, (a, ok)) for r, a, ok in (q.get(timeout=120) for _ in range(world)))
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    ref = oracle_lib.fft_2d_r2c(_full_input(nx, ny, 7), nthreads=2)
    nxl = nx // world
    for r in range(world):
        a, ok = got[r]
        assert ok
        assert np.allclose(a, ref[r * nxl:(r + 1) * nxl], rtol=0, atol=1e-10 * np.abs(ref).max()), (r, comm)


def test_reference_cyclic_interleave_would_fail_here(oracle_lib):
    """The reference's post-exchange transpose writes trans[k][2 P j + 2 i]
    (core/src/distributed/loop.cpp:87-106): slab i's row j lands at x = P j +
    i instead of x = i n_x_local + j.  For this input (energy at kx = 3) that
    permutation changes the spectrum, so the comparison above can tell the
    two maps apart."""
    nx, ny, P = 8, 12, 2
    x = _full_input(nx, ny, 7)
    nxl = nx // P
    perm = np.array([P * j + i for i in range(P) for j in range(nxl)])  # row i*nxl+j goes to P*j+i
    cyc = np.zeros_like(x)
    cyc[perm] = x
    ref = oracle_lib.fft_2d_r2c(x.copy(), nthreads=1)
    bad = oracle_lib.fft_2d_r2c(cyc, nthreads=1)
    assert not np.allclose(ref, bad, atol=1e-6)
