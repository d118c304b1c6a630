"""Python mirror of the HPX-FFT API over the GB300 C ABI.

Names and semantics follow the reference's C++ interface so that code and
tests written against it read the same:

  hpxfft.util.vector_2d            core/include/hpxfft/util/vector_2d.hpp:9-86
  hpxfft.shared.loop               core/include/hpxfft/shared/loop.hpp:15-31
  hpxfft.shared.naive/sync/opt     core/include/hpxfft/shared/{naive,sync,opt}.hpp
  hpxfft.distributed.loop          core/include/hpxfft/distributed/loop.hpp:17-31

Every transform runs in libhpxfft_gb300.so on the GPU; there is no CPU path.
"""
from . import _capi
from ._capi import HpxFftError, HpxFftInvalidArgument
from .plan import Plan, Plan3D, Slab
from .batch import Batch
from . import util, shared, distributed

__all__ = ["Plan", "Plan3D", "Slab", "Batch", "HpxFftError", "HpxFftInvalidArgument", "util", "shared", "distributed", "_capi",
           "pipe_peaks"]


def pipe_peaks() -> dict:
    """Measured FP32 and FP64 FMA throughput of the current device (TFLOP/s)."""
    import ctypes

    f32, f64 = ctypes.c_double(), ctypes.c_double()
    _capi.check(_capi.load().hpxfft_measure_pipe_peaks(ctypes.byref(f32), ctypes.byref(f64)))
    return {"fp32_fma_tflops": f32.value, "fp64_fma_tflops": f64.value,
            "fp32_over_fp64": f32.value / f64.value if f64.value > 0 else None}
