"""hpxfft::util::vector_2d (core/include/hpxfft/util/vector_2d.hpp:9-86).

A row-major owning 2D buffer.  Construction, element access, row(i),
bounds-checked at() raising RuntimeError (the reference's std::runtime_error,
vector_2d.hpp:215-245) and exact ==.  Moving is explicit: `take()` hands the
storage to the caller and leaves this object empty, which is what the
reference's std::move into initialize() does.
"""
from __future__ import annotations

import numpy as np


class vector_2d:
    def __init__(self, n_row: int = 0, n_col: int = 0, value=None, dtype=np.float64):
        self._a = np.zeros((n_row, n_col), dtype=dtype)
        if value is not None:
            self._a.fill(value)

    @classmethod
    def from_array(cls, array: np.ndarray) -> "vector_2d":
        v = cls.__new__(cls)
        a = np.ascontiguousarray(array)
        if a.ndim != 2:
            raise ValueError("vector_2d needs a 2D array")
        v._a = a
        return v

    # element access
    def __call__(self, i: int, j: int):
        return self._a[i, j]

    def __getitem__(self, ij):
        return self._a[ij]

    def __setitem__(self, ij, v):
        self._a[ij] = v

    def at(self, i: int, j: int):
        if i * self.n_col() + j >= self.size() or i < 0 or j < 0:
            raise RuntimeError("out of range exception")
        return self._a.reshape(-1)[i * self.n_col() + j]

    def row(self, i: int) -> np.ndarray:
        return self._a[i]

    def data(self) -> np.ndarray:
        return self._a

    def n_row(self) -> int:
        return self._a.shape[0]

    def n_col(self) -> int:
        return self._a.shape[1]

    def size(self) -> int:
        return self._a.size

    def take(self) -> np.ndarray:
        a = self._a
        self._a = np.zeros((0, 0), dtype=a.dtype)
        return a

    def __eq__(self, other) -> bool:
        if not isinstance(other, vector_2d):
            return NotImplemented
        return self._a.shape == other._a.shape and bool(np.array_equal(self._a, other._a))

    def __repr__(self) -> str:
        return f"vector_2d({self.n_row()}x{self.n_col()}, {self._a.dtype})"
