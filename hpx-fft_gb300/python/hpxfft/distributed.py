"""hpxfft::distributed::loop (core/include/hpxfft/distributed/loop.hpp:17-31).

The reference slab-decomposes the x rows over P localities: row r2c of the
local rows, pack (split_vec), scatter or all_to_all exchange, transpose,
column c2c, pack, exchange back, transpose back
(core/src/distributed/loop.cpp:130-272).  Here:

- P = 1 (no torch.distributed process group, or one rank): the exchange is
  the identity and the transform is the same fused row and column kernels
  as hpxfft.shared.loop;
- P > 1 (an initialised torch.distributed process group, one rank per
  locality): the local phases run on this rank's GPU through the slab
  decomposition of the C ABI (hpxfft_slab_*), whose index maps are right
  for every P (the reference's transposes are right only for P = 1,
  core/src/distributed/loop.cpp:87-127), and the two exchanges are
  torch.distributed collectives: one all_to_all of equal tiles
  (COMM_FLAG "all_to_all") or P scatters, one per root ("scatter"), as the
  reference's two schemes (core/src/distributed/loop.cpp:39-84).  Each rank
  passes its own n_x_local rows and gets back the same rows of the spectrum.
"""
from __future__ import annotations

import time

import numpy as np

from . import _capi
from .plan import Slab, real_dtype
from .shared import _Base
from .util import vector_2d

COMM_FLAGS = ("scatter", "all_to_all")


def _world():
    """(size, rank) of the default torch.distributed process group, (1, 0) without one."""
    try:
        import torch.distributed as dist

        if dist.is_available() and dist.is_initialized():
            return dist.get_world_size(), dist.get_rank()
    except Exception:
        pass
    return 1, 0


def _world_size() -> int:
    return _world()[0]


def exchange(send, recv, comm_flag: str, n_ranks: int, rank: int) -> None:
    """Tile d of `send` goes to rank d; tile s of `recv` comes from rank s
    (equal tiles, contiguous, n_ranks of them in each buffer)."""
    import torch.distributed as dist

    if comm_flag == "all_to_all":
        dist.all_to_all_single(recv, send)
        return
    # "scatter": root i sends tile d of its buffer to rank d
    sends = list(send.view(n_ranks, -1))
    tiles = recv.view(n_ranks, -1)
    for root in range(n_ranks):
        dist.scatter(tiles[root], scatter_list=sends if rank == root else None, src=root)


class GpuSlabCompute:
    """The local phases on this rank's GPU (hpxfft_slab_* through
    hpxfft.plan.Slab); the buffers the exchanges read and write are device
    tensors, so an NCCL process group moves them GPU to GPU."""

    def __init__(self, n_row_local, n_col, n_ranks, rank, precision, plan_flag):
        import torch

        self.torch = torch
        self.slab = Slab(n_row_local, n_col, n_ranks, rank, precision, plan_flag)
        dev = torch.device("cuda", torch.cuda.current_device())
        tdt = torch.float32 if real_dtype(precision) == np.float32 else torch.float64
        n = self.slab.tile_bytes * n_ranks
        self.values = torch.empty((n_row_local, n_col), dtype=tdt, device=dev)
        self.send = torch.empty(n, dtype=torch.uint8, device=dev)
        self.recv = torch.empty(n, dtype=torch.uint8, device=dev)
        self.recv2 = torch.empty(n, dtype=torch.uint8, device=dev)

    def _stream(self):
        self.slab.set_stream(self.torch.cuda.current_stream().cuda_stream)

    def rows(self, host_values: np.ndarray):
        self.values.copy_(self.torch.from_numpy(host_values))
        self._stream()
        self.slab.rows(self.values.data_ptr(), self.send.data_ptr())
        return self.send

    def columns(self, recv):
        self._stream()
        self.slab.columns(recv.data_ptr())
        return recv

    def finish(self, recv2, host_values: np.ndarray) -> None:
        self._stream()
        self.slab.finish(recv2.data_ptr(), self.values.data_ptr())
        host_values[...] = self.values.cpu().numpy()

    def synchronize(self) -> None:
        self.torch.cuda.synchronize()
        self.slab.synchronize()

    def measurement(self, name: str) -> float:
        return self.slab.measurement(name)

    def close(self) -> None:
        self.slab.close()


class loop(_Base):
    def __init__(self, local_compute=GpuSlabCompute):
        super().__init__()
        self._local_factory = local_compute
        self._local = None

    def initialize(self, values_vec: vector_2d, COMM_FLAG: str, PLAN_FLAG: str, precision: str = "f64") -> None:
        # the reference prints and finalizes on an unknown flag
        # (distributed/loop.cpp:342-346); here it is std::invalid_argument
        if COMM_FLAG not in COMM_FLAGS:
            raise _capi.HpxFftInvalidArgument(
                _capi.HPXFFT_ERR_INVALID_ARG, "Specify communication scheme: scatter or all_to_all"
            )
        self.COMM_FLAG = COMM_FLAG
        self.n_ranks, self.rank = _world()
        if self.n_ranks == 1:
            super().initialize(values_vec, PLAN_FLAG, precision)
            return
        if not isinstance(values_vec, vector_2d):
            raise TypeError("initialize expects a vector_2d")
        dtype = real_dtype(precision)
        if values_vec.data().dtype != dtype:
            raise _capi.HpxFftInvalidArgument(_capi.HPXFFT_ERR_INVALID_ARG, f"values must be {dtype}")
        if not _capi.load().hpxfft_plan_flag_valid(PLAN_FLAG.encode()):
            raise _capi.HpxFftInvalidArgument(_capi.HPXFFT_ERR_INVALID_ARG, "Invalid FFTW plan flag string")
        if self._local is not None:
            self._local.close()
        t0 = time.perf_counter()
        self._local = self._local_factory(values_vec.n_row(), values_vec.n_col(), self.n_ranks, self.rank, precision,
                                          PLAN_FLAG)
        self._values = values_vec.take()
        self._meas = {"plan": time.perf_counter() - t0}

    def fft_2d_r2c(self) -> vector_2d:
        if self.n_ranks == 1:
            out = self._run()
            # the reference's eight timers (distributed/loop.cpp:260-268); the
            # split and exchange phases do not exist at one locality
            for key in ("first_split", "first_comm", "second_split", "second_comm"):
                self._meas[key] = 0.0
            return out
        if self._values is None:
            raise _capi.HpxFftError(_capi.HPXFFT_ERR_STATE, "initialize() must come first")
        local, a = self._local, self._values
        t0 = time.perf_counter()
        send = local.rows(a)
        local.synchronize()
        t1 = time.perf_counter()
        exchange(send, local.recv, self.COMM_FLAG, self.n_ranks, self.rank)
        local.synchronize()
        t2 = time.perf_counter()
        cols = local.columns(local.recv)
        local.synchronize()
        t3 = time.perf_counter()
        exchange(cols, local.recv2, self.COMM_FLAG, self.n_ranks, self.rank)
        local.synchronize()
        t4 = time.perf_counter()
        local.finish(local.recv2, a)
        t5 = time.perf_counter()
        for key in ("first_fftw", "first_split", "first_trans", "second_fftw", "second_split", "second_trans"):
            self._meas[key] = local.measurement(key)
        self._meas.update(total=t5 - t0, first_comm=t2 - t1, second_comm=t4 - t3)
        self._values = None  # moved out (distributed/loop.cpp:271)
        return vector_2d.from_array(a)
