"""hpxfft::distributed::loop (core/include/hpxfft/distributed/loop.hpp:17-31).

The reference slab-decomposes the x rows over P localities and exchanges
slabs with scatter or all_to_all (core/src/distributed/loop.cpp:130-272).  On
one GPU (P = 1) the exchange is the identity and the per-locality compute is
the same fused row and column kernels as hpxfft.shared.loop.  More than one
locality is not supported: this build runs on single-GPU machines.
"""
from __future__ import annotations

from . import _capi
from .shared import _Base
from .util import vector_2d

COMM_FLAGS = ("scatter", "all_to_all")


class loop(_Base):
    def initialize(self, values_vec: vector_2d, COMM_FLAG: str, PLAN_FLAG: str, precision: str = "f64") -> None:
        # the reference prints and finalizes on an unknown flag
        # (distributed/loop.cpp:342-346); here it is std::invalid_argument
        if COMM_FLAG not in COMM_FLAGS:
            raise _capi.HpxFftInvalidArgument(
                _capi.HPXFFT_ERR_INVALID_ARG, "Specify communication scheme: scatter or all_to_all"
            )
        world = _world_size()
        if world != 1:
            raise _capi.HpxFftError(
                _capi.HPXFFT_ERR_UNSUPPORTED_SIZE, f"distributed.loop runs at one locality; world size is {world}"
            )
        self.COMM_FLAG = COMM_FLAG
        super().initialize(values_vec, PLAN_FLAG, precision)

    def fft_2d_r2c(self) -> vector_2d:
        out = self._run()
        # the reference's eight timers (distributed/loop.cpp:260-268); the
        # split and exchange phases do not exist at one locality
        for key in ("first_split", "first_comm", "second_split", "second_comm"):
            self._meas[key] = 0.0
        return out


def _world_size() -> int:
    try:
        import torch.distributed as dist

        if dist.is_available() and dist.is_initialized():
            return dist.get_world_size()
    except Exception:
        pass
    return 1
