"""Batches of uneven 2D r2c transforms (hpxfft_batch_* in the C ABI)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .plan import precision_code, real_dtype


class Batch:
    """count independent forward transforms of shapes (n_rows[i], n_cols[i]),
    padded layout, packed in one device arena at `offsets` (bytes)."""

    def __init__(self, n_rows, n_cols, precision="f32", plan_flag="estimate"):
        lib = _capi.load()
        self._lib = lib
        n = len(n_rows)
        if n != len(n_cols):
            raise _capi.HpxFftInvalidArgument(_capi.HPXFFT_ERR_INVALID_ARG, "n_rows and n_cols differ in length")
        nr = (ctypes.c_size_t * n)(*[int(v) for v in n_rows])
        nc = (ctypes.c_size_t * n)(*[int(v) for v in n_cols])
        self._h = ctypes.c_void_p()
        _capi.check(lib.hpxfft_batch_create(ctypes.byref(self._h), n, nr, nc, precision_code(precision),
                                            plan_flag.encode()))
        self.n_rows = [int(v) for v in n_rows]
        self.n_cols = [int(v) for v in n_cols]
        self.dtype = real_dtype(precision)
        size = ctypes.c_size_t()
        _capi.check(lib.hpxfft_batch_arena_bytes(self._h, ctypes.byref(size)))
        self.arena_bytes = size.value
        offs = (ctypes.c_size_t * n)()
        _capi.check(lib.hpxfft_batch_offsets(self._h, offs))
        self.offsets = [int(v) for v in offs]

    def set_stream(self, handle: int) -> None:
        _capi.check(self._lib.hpxfft_batch_set_stream(self._h, ctypes.c_void_p(handle)))

    def execute(self, arena_ptr: int) -> None:
        _capi.check(self._lib.hpxfft_batch_execute(self._h, ctypes.c_void_p(arena_ptr)))

    def synchronize(self) -> None:
        _capi.check(self._lib.hpxfft_batch_synchronize(self._h))

    def measurement(self, name: str) -> float:
        v = ctypes.c_double()
        _capi.check(self._lib.hpxfft_batch_get_measurement(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def views(self, arena: np.ndarray):
        """Per-instance (n_row, n_col) views into a host copy of the arena (bytes)."""
        out = []
        for off, r, c in zip(self.offsets, self.n_rows, self.n_cols):
            out.append(arena[off:off + r * c * self.dtype.itemsize].view(self.dtype).reshape(r, c))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hpxfft_batch_destroy(self._h)
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


def wisdom_export(path: str) -> None:
    _capi.check(_capi.load().hpxfft_wisdom_export(str(path).encode()))


def wisdom_import(path: str) -> None:
    _capi.check(_capi.load().hpxfft_wisdom_import(str(path).encode()))


def wisdom_forget() -> None:
    _capi.check(_capi.load().hpxfft_wisdom_forget())
