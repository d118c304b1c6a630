"""Low-level plan object over the C ABI (include/hpxfft_gb300.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi

_PRECISIONS = {
    "f64": _capi.PREC_F64,
    "f64-native": _capi.PREC_F64_NATIVE,
    "f32": _capi.PREC_F32,
    "bf16x3": _capi.PREC_BF16X3,
}


def precision_code(precision) -> int:
    if isinstance(precision, int):
        return precision
    try:
        return _PRECISIONS[precision]
    except KeyError:
        raise _capi.HpxFftInvalidArgument(_capi.HPXFFT_ERR_INVALID_ARG, f"unknown precision {precision!r}") from None


def real_dtype(precision) -> np.dtype:
    f32 = precision_code(precision) in (_capi.PREC_F32, _capi.PREC_BF16X3)
    return np.dtype(np.float32) if f32 else np.dtype(np.float64)


class Plan:
    """A planned 2D r2c of `batch` arrays of n_row x n_col reals (padded layout).

    n_col = 2*(ny/2+1): the first ny reals of a row are data, the last two
    padding; the forward transform leaves X[kx][ky] (n_col/2 complex) in
    each row.
    """

    def __init__(self, n_row: int, n_col: int, batch: int = 1, precision="f64", plan_flag: str = "estimate"):
        lib = _capi.load()
        self._lib = lib
        self._h = ctypes.c_void_p()
        flag = plan_flag.encode() if isinstance(plan_flag, str) else plan_flag
        _capi.check(lib.hpxfft_plan_create(ctypes.byref(self._h), n_row, n_col, batch, precision_code(precision), flag))
        own = ctypes.c_void_p()
        _capi.check(lib.hpxfft_plan_get_stream(self._h, ctypes.byref(own)))
        self._own_stream = own.value
        self.n_row, self.n_col, self.batch = int(n_row), int(n_col), int(batch)
        self.precision = precision_code(precision)
        self.dtype = real_dtype(precision)

    # -- properties
    @property
    def ny(self) -> int:
        return self.n_col - 2

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._h:
            raise _capi.HpxFftError(_capi.HPXFFT_ERR_STATE, "plan destroyed")
        return self._h

    def buffer_bytes(self) -> int:
        n = ctypes.c_size_t()
        _capi.check(self._lib.hpxfft_plan_buffer_bytes(self.handle, ctypes.byref(n)))
        return n.value

    # -- execution
    def set_stream(self, stream_handle: int | None) -> None:
        """Run on a cudaStream_t handle (0 = legacy default stream); None = the plan's own stream."""
        h = self._own_stream if stream_handle is None else stream_handle
        _capi.check(self._lib.hpxfft_plan_set_stream(self.handle, ctypes.c_void_p(h)))

    def execute_device(self, ptr: int) -> None:
        """In-place forward transform of a device buffer (asynchronous)."""
        _capi.check(self._lib.hpxfft_execute_r2c(self.handle, ctypes.c_void_p(ptr)))

    def execute_oop(self, in_ptr: int, out_ptr: int) -> None:
        _capi.check(self._lib.hpxfft_execute_r2c_oop(self.handle, ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr)))

    def c2r_device(self, ptr: int) -> None:
        _capi.check(self._lib.hpxfft_execute_c2r(self.handle, ctypes.c_void_p(ptr)))

    def backward_device(self, ptr: int) -> None:
        _capi.check(self._lib.hpxfft_execute_r2c_backward(self.handle, ctypes.c_void_p(ptr)))

    def synchronize(self) -> None:
        """Wait for the plan's stream; raises on a timed-out tensor-core wait."""
        _capi.check(self._lib.hpxfft_plan_synchronize(self.handle))

    def execute_host(self, values: np.ndarray) -> np.ndarray:
        """In-place forward transform of a host array (copy in, transform, copy out)."""
        self._check_host(values)
        _capi.check(self._lib.hpxfft_execute_r2c_host(self.handle, values.ctypes.data_as(ctypes.c_void_p)))
        return values

    def backward_host(self, values: np.ndarray) -> np.ndarray:
        """In-place adjoint of a host array (copy in, transform, copy out)."""
        self._check_host(values)
        _capi.check(self._lib.hpxfft_execute_r2c_backward_host(self.handle, values.ctypes.data_as(ctypes.c_void_p)))
        return values

    def _check_host(self, values: np.ndarray) -> None:
        if not isinstance(values, np.ndarray) or not values.flags.c_contiguous:
            raise _capi.HpxFftInvalidArgument(_capi.HPXFFT_ERR_INVALID_ARG, "need a C-contiguous numpy array")
        if values.dtype != self.dtype or values.size != self.batch * self.n_row * self.n_col:
            raise _capi.HpxFftInvalidArgument(
                _capi.HPXFFT_ERR_INVALID_ARG,
                f"array must hold {self.batch}x{self.n_row}x{self.n_col} {self.dtype} values",
            )

    # -- bookkeeping
    def measurement(self, name: str) -> float:
        v = ctypes.c_double()
        _capi.check(self._lib.hpxfft_get_measurement(self.handle, name.encode(), ctypes.byref(v)))
        return v.value

    def timing_stats(self) -> dict:
        """Mean kernel durations (s) over the transforms since timing_reset()."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_longlong()
        _capi.check(self._lib.hpxfft_timing_stats(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                  ctypes.byref(n)))
        return {"first": a.value, "second": b.value, "total": c.value, "count": n.value}

    def timing_reset(self) -> None:
        _capi.check(self._lib.hpxfft_timing_reset(self.handle))

    def write_plan(self, path: str) -> None:
        _capi.check(self._lib.hpxfft_write_plan(self.handle, str(path).encode()))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hpxfft_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_flag_valid(flag: str) -> bool:
    return bool(_capi.load().hpxfft_plan_flag_valid(flag.encode()))


class Plan3D:
    """A planned 3D r2c of `batch` arrays of n0 x n1 x n2 reals, the last axis
    padded to n_col = 2*(n2/2+1); in place, output X[k0][k1][k2] (n_col/2
    complex along the last axis), numpy.fft.rfftn orientation."""

    def __init__(self, n0: int, n1: int, n_col: int, batch: int = 1, precision="f64", plan_flag: str = "estimate"):
        lib = _capi.load()
        self._lib = lib
        self._h = ctypes.c_void_p()
        _capi.check(lib.hpxfft_plan3d_create(ctypes.byref(self._h), n0, n1, n_col, batch, precision_code(precision),
                                             plan_flag.encode()))
        self.shape = (int(n0), int(n1), int(n_col))
        self.batch = int(batch)
        self.dtype = real_dtype(precision)

    def set_stream(self, stream_handle: int | None) -> None:
        """Run both passes on a cudaStream_t handle; None or 0 = the legacy
        default stream (a 3D plan starts on a stream of its own)."""
        _capi.check(self._lib.hpxfft_plan3d_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def execute_device(self, ptr: int) -> None:
        _capi.check(self._lib.hpxfft_execute3d_r2c(self._h, ctypes.c_void_p(ptr)))

    def buffer_bytes(self) -> int:
        n = ctypes.c_size_t()
        _capi.check(self._lib.hpxfft_plan3d_buffer_bytes(self._h, ctypes.byref(n)))
        return n.value

    def measurement(self, name: str) -> float:
        v = ctypes.c_double()
        _capi.check(self._lib.hpxfft_plan3d_get_measurement(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hpxfft_plan3d_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Slab:
    """Local phases of the slab-decomposed 2D r2c on one rank of P
    (hpxfft_slab_* in the C ABI): rank `rank` holds global rows
    rank*n_row_local .. of the padded input; send and receive buffers are
    n_ranks tiles of tile_bytes, tile d for rank d; the caller exchanges
    them (see hpxfft.distributed.loop)."""

    def __init__(self, n_row_local: int, n_col: int, n_ranks: int, rank: int, precision="f64",
                 plan_flag: str = "estimate"):
        lib = _capi.load()
        self._lib = lib
        self._h = ctypes.c_void_p()
        _capi.check(lib.hpxfft_slab_create(ctypes.byref(self._h), n_row_local, n_col, n_ranks, rank,
                                           precision_code(precision), plan_flag.encode()))
        n = ctypes.c_size_t()
        _capi.check(lib.hpxfft_slab_tile_bytes(self._h, ctypes.byref(n)))
        self.tile_bytes = n.value
        self.n_row_local, self.n_col, self.n_ranks, self.rank = int(n_row_local), int(n_col), int(n_ranks), int(rank)
        self.dtype = real_dtype(precision)
        self.tile_columns = -(-(self.n_col // 2) // self.n_ranks)

    def set_stream(self, handle: int) -> None:
        _capi.check(self._lib.hpxfft_slab_set_stream(self._h, ctypes.c_void_p(handle)))

    def rows(self, values_ptr: int, send_ptr: int) -> None:
        _capi.check(self._lib.hpxfft_slab_rows(self._h, ctypes.c_void_p(values_ptr), ctypes.c_void_p(send_ptr)))

    def columns(self, recv_ptr: int) -> None:
        _capi.check(self._lib.hpxfft_slab_columns(self._h, ctypes.c_void_p(recv_ptr)))

    def finish(self, recv_ptr: int, values_ptr: int) -> None:
        _capi.check(self._lib.hpxfft_slab_finish(self._h, ctypes.c_void_p(recv_ptr), ctypes.c_void_p(values_ptr)))

    def synchronize(self) -> None:
        _capi.check(self._lib.hpxfft_slab_synchronize(self._h))

    def measurement(self, name: str) -> float:
        v = ctypes.c_double()
        _capi.check(self._lib.hpxfft_slab_get_measurement(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hpxfft_slab_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
