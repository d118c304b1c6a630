"""hpxfft::shared::{loop, naive, sync, opt} over the GB300 library.

The reference's shared variants compute the same transform with different
HPX synchronisation (core/src/shared/loop.cpp:56-113, naive.cpp:50-94,
sync.cpp:51-97, opt.cpp:51-96).  On the GPU the whole transform is one
stream-ordered pair of kernels, so every variant maps to the same plan; the
class names and methods are kept so callers switch without edits.
"""
from __future__ import annotations

import numpy as np

from . import _capi
from .plan import Plan, real_dtype
from .util import vector_2d


class _Base:
    """initialize(values, PLAN_FLAG) moves the data in; the transform moves it out."""

    def __init__(self):
        self._values = None
        self._plan = None
        self._meas = {}

    def initialize(self, values_vec: vector_2d, PLAN_FLAG: str, precision: str = "f64") -> None:
        if not isinstance(values_vec, vector_2d):
            raise TypeError("initialize expects a vector_2d")
        dtype = real_dtype(precision)
        if values_vec.data().dtype != dtype:
            raise _capi.HpxFftInvalidArgument(_capi.HPXFFT_ERR_INVALID_ARG, f"values must be {dtype}")
        n_row, n_col = values_vec.n_row(), values_vec.n_col()
        if self._plan is not None:
            self._plan.close()
        self._plan = Plan(n_row, n_col, 1, precision, PLAN_FLAG)  # raises on a bad flag, like loop.cpp:171-180
        self._values = values_vec.take()  # loop.cpp:161, std::move
        self._meas = {"plan": self._plan.measurement("plan"), "plan_flops": self._plan.measurement("plan_flops")}

    def _run(self) -> vector_2d:
        if self._values is None:
            raise _capi.HpxFftError(_capi.HPXFFT_ERR_STATE, "initialize() must come first")
        a = self._values
        self._plan.execute_host(a)
        self._read_measurements()
        self._values = None  # moved out (loop.cpp:112)
        return vector_2d.from_array(a)

    def _read_measurements(self) -> None:
        for key in ("total", "first_fftw", "first_trans", "second_fftw", "second_trans", "h2d", "d2h", "e2e",
                    "gbps", "gflops", "roofline"):
            self._meas[key] = self._plan.measurement(key)

    def fft_2d_r2c_backward(self, grad: vector_2d) -> vector_2d:
        """Adjoint of the transform: grad holds dL/dRe X + i dL/dIm X in the
        output layout; returns dL/dx in the input layout.  No reference
        counterpart."""
        if self._plan is None:
            raise _capi.HpxFftError(_capi.HPXFFT_ERR_STATE, "initialize() must come first")
        a = np.ascontiguousarray(grad.data(), dtype=self._plan.dtype).reshape(self._plan.n_row, self._plan.n_col).copy()
        self._plan.backward_host(a)
        self._read_measurements()
        return vector_2d.from_array(a)

    def get_measurement(self, name: str) -> float:
        return float(self._meas.get(name, 0.0))

    def write_plans_to_file(self, file_path: str) -> None:
        if self._plan is None:
            raise _capi.HpxFftError(_capi.HPXFFT_ERR_STATE, "initialize() must come first")
        try:
            self._plan.write_plan(file_path)
        except _capi.HpxFftError as e:
            if e.status == _capi.HPXFFT_ERR_IO:
                raise RuntimeError(f"Failed to open file: {file_path}") from None
            raise


class loop(_Base):
    """core/include/hpxfft/shared/loop.hpp:15-31."""

    def fft_2d_r2c_par(self) -> vector_2d:
        return self._run()

    def fft_2d_r2c_seq(self) -> vector_2d:
        # the reference's seq loop overruns its transpose bounds when
        # nx > ny/2+1 (loop.cpp:126-130); here it is the same transform as par
        return self._run()

    fft_2d_r2c = fft_2d_r2c_par


class naive(_Base):
    """core/include/hpxfft/shared/naive.hpp."""

    def fft_2d_r2c(self) -> vector_2d:
        return self._run()


class sync(_Base):
    """core/include/hpxfft/shared/sync.hpp."""

    def fft_2d_r2c(self) -> vector_2d:
        return self._run()


class opt(_Base):
    """core/include/hpxfft/shared/opt.hpp."""

    def fft_2d_r2c(self) -> vector_2d:
        return self._run()
