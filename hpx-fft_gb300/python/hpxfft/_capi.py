"""ctypes binding of the C ABI declared in include/hpxfft_gb300.h.

The shared library is built in tree by hpx-fft_gb300/build.py.  There is no
fallback: if the library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.normpath(os.path.join(_PKG, "..", "..", "_build", "libhpxfft_gb300.so"))

HPXFFT_OK = 0
HPXFFT_ERR_INVALID_ARG = 1
HPXFFT_ERR_UNSUPPORTED_SIZE = 2
HPXFFT_ERR_ALLOC = 3
HPXFFT_ERR_CUDA = 4
HPXFFT_ERR_TIMEOUT = 5
HPXFFT_ERR_STATE = 6
HPXFFT_ERR_IO = 7

PREC_F64 = 0
PREC_F64_NATIVE = 1
PREC_F32 = 2
PREC_BF16X3 = 3

# every symbol the header declares: name -> (restype, argtypes)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_ci = ctypes.c_int
_cs = ctypes.c_char_p
SIGNATURES = {
    "hpxfft_plan_create": (_ci, [ctypes.POINTER(_vp), _sz, _sz, _sz, _ci, _cs]),
    "hpxfft_plan_destroy": (_ci, [_vp]),
    "hpxfft_plan_set_stream": (_ci, [_vp, _vp]),
    "hpxfft_plan_get_stream": (_ci, [_vp, ctypes.POINTER(_vp)]),
    "hpxfft_plan_buffer_bytes": (_ci, [_vp, ctypes.POINTER(_sz)]),
    "hpxfft_execute_r2c": (_ci, [_vp, _vp]),
    "hpxfft_execute_r2c_oop": (_ci, [_vp, _vp, _vp]),
    "hpxfft_execute_r2c_host": (_ci, [_vp, _vp]),
    "hpxfft_execute_c2r": (_ci, [_vp, _vp]),
    "hpxfft_execute_r2c_backward": (_ci, [_vp, _vp]),
    "hpxfft_get_measurement": (_ci, [_vp, _cs, ctypes.POINTER(ctypes.c_double)]),
    "hpxfft_timing_stats": (_ci, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
    "hpxfft_timing_reset": (_ci, [_vp]),
    "hpxfft_write_plan": (_ci, [_vp, _cs]),
    "hpxfft_plan_flag_valid": (_ci, [_cs]),
    "hpxfft_status_string": (_cs, [_ci]),
    "hpxfft_last_error": (_cs, []),
    "hpxfft_execute_r2c_noalloc": (_ci, [_vp, _vp, _sz, _sz, _vp]),
    "hpxfft_batch_create": (_ci, [ctypes.POINTER(_vp), _sz, ctypes.POINTER(_sz), ctypes.POINTER(_sz), _ci, _cs]),
    "hpxfft_batch_destroy": (_ci, [_vp]),
    "hpxfft_batch_arena_bytes": (_ci, [_vp, ctypes.POINTER(_sz)]),
    "hpxfft_batch_offsets": (_ci, [_vp, ctypes.POINTER(_sz)]),
    "hpxfft_batch_set_stream": (_ci, [_vp, _vp]),
    "hpxfft_batch_execute": (_ci, [_vp, _vp]),
    "hpxfft_batch_synchronize": (_ci, [_vp]),
    "hpxfft_plan_synchronize": (_ci, [_vp]),
    "hpxfft_execute_r2c_backward_host": (_ci, [_vp, _vp]),
    "hpxfft_plan3d_create": (_ci, [ctypes.POINTER(_vp), _sz, _sz, _sz, _sz, _ci, _cs]),
    "hpxfft_plan3d_destroy": (_ci, [_vp]),
    "hpxfft_plan3d_set_stream": (_ci, [_vp, _vp]),
    "hpxfft_plan3d_buffer_bytes": (_ci, [_vp, ctypes.POINTER(_sz)]),
    "hpxfft_execute3d_r2c": (_ci, [_vp, _vp]),
    "hpxfft_plan3d_get_measurement": (_ci, [_vp, _cs, ctypes.POINTER(ctypes.c_double)]),
    "hpxfft_batch_get_measurement": (_ci, [_vp, _cs, ctypes.POINTER(ctypes.c_double)]),
    "hpxfft_wisdom_export": (_ci, [_cs]),
    "hpxfft_wisdom_import": (_ci, [_cs]),
    "hpxfft_wisdom_forget": (_ci, []),
    "hpxfft_slab_create": (_ci, [ctypes.POINTER(_vp), _sz, _sz, _sz, _sz, _ci, _cs]),
    "hpxfft_slab_destroy": (_ci, [_vp]),
    "hpxfft_slab_set_stream": (_ci, [_vp, _vp]),
    "hpxfft_slab_tile_bytes": (_ci, [_vp, ctypes.POINTER(_sz)]),
    "hpxfft_slab_rows": (_ci, [_vp, _vp, _vp]),
    "hpxfft_slab_columns": (_ci, [_vp, _vp]),
    "hpxfft_slab_finish": (_ci, [_vp, _vp, _vp]),
    "hpxfft_slab_synchronize": (_ci, [_vp]),
    "hpxfft_slab_get_measurement": (_ci, [_vp, _cs, ctypes.POINTER(ctypes.c_double)]),
    "hpxfft_measure_pipe_peaks": (_ci, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "hpxfft_host_alloc": (_ci, [ctypes.POINTER(_vp), _sz]),
    "hpxfft_host_free": (_ci, [_vp]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load libhpxfft_gb300.so (raises OSError if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} not built: run hpx-fft_gb300/build.py (no CPU fallback exists)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class HpxFftError(RuntimeError):
    """Failure reported by the C ABI; `status` is the hpxfft_status code."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class HpxFftInvalidArgument(HpxFftError, ValueError):
    """Maps the reference's std::invalid_argument (bad plan flag)."""


def check(status: int) -> None:
    if status == HPXFFT_OK:
        return
    lib = load()
    msg = lib.hpxfft_last_error().decode() or lib.hpxfft_status_string(status).decode()
    text = f"{lib.hpxfft_status_string(status).decode()}: {msg}"
    if status == HPXFFT_ERR_INVALID_ARG:
        raise HpxFftInvalidArgument(status, text)
    raise HpxFftError(status, text)
