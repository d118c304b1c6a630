"""ctypes wrapper of the CPU oracle (oracle/hpxfft_oracle.c) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this module.  It restates the reference's FP64 shared::loop algorithm
(core/src/shared/loop.cpp:56-113) in plain C; it is the checker, never the
product.  The library is built by hpx-fft_gb300/build.py (build_oracle).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_DIR, "_build", "libhpxfft_oracle.so")
_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} not built (hpx-fft_gb300/build.py builds it)")
        lib = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_c2c_1d.argtypes = [dp, ctypes.c_size_t, ctypes.c_int]
        lib.oracle_r2c_1d.argtypes = [dp, dp, ctypes.c_size_t]
        lib.oracle_fft_2d_r2c.argtypes = [dp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, dp]
        lib.oracle_fft_2d_r2c_adjoint.argtypes = [dp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int]
        lib.oracle_fft_2d_c2r.argtypes = [dp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int]
        for f in (lib.oracle_c2c_1d, lib.oracle_r2c_1d, lib.oracle_fft_2d_r2c, lib.oracle_fft_2d_r2c_adjoint,
                  lib.oracle_fft_2d_c2r):
            f.restype = ctypes.c_int
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check_2d(values: np.ndarray) -> None:
    if values.dtype != np.float64 or values.ndim != 2 or not values.flags.c_contiguous:
        raise ValueError("oracle works on C-contiguous float64 n_row x n_col arrays")


def fft_2d_r2c(values: np.ndarray, nthreads: int = 1, times: bool = False):
    """In place on the padded layout (n_row x 2*(ny/2+1)); returns values (and phase times)."""
    _check_2d(values)
    t = np.zeros(5)
    rc = load().oracle_fft_2d_r2c(_ptr(values), values.shape[0], values.shape[1], int(nthreads), _ptr(t))
    if rc:
        raise RuntimeError(f"oracle_fft_2d_r2c failed ({rc})")
    if times:
        return values, dict(zip(("total", "first_fftw", "first_trans", "second_fftw", "second_trans"), t))
    return values


def fft_2d_r2c_adjoint(values: np.ndarray, nthreads: int = 1) -> np.ndarray:
    _check_2d(values)
    rc = load().oracle_fft_2d_r2c_adjoint(_ptr(values), values.shape[0], values.shape[1], int(nthreads))
    if rc:
        raise RuntimeError(f"oracle_fft_2d_r2c_adjoint failed ({rc})")
    return values


def fft_2d_c2r(values: np.ndarray, nthreads: int = 1) -> np.ndarray:
    _check_2d(values)
    rc = load().oracle_fft_2d_c2r(_ptr(values), values.shape[0], values.shape[1], int(nthreads))
    if rc:
        raise RuntimeError(f"oracle_fft_2d_c2r failed ({rc})")
    return values


def c2c_1d(x: np.ndarray, sign: int = -1) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    rc = load().oracle_c2c_1d(a.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size, sign)
    if rc:
        raise RuntimeError("oracle_c2c_1d failed")
    return a


def r2c_1d(x: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(a.size // 2 + 1, dtype=np.complex128)
    rc = load().oracle_r2c_1d(_ptr(a), out.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size)
    if rc:
        raise RuntimeError("oracle_r2c_1d failed")
    return out


# ---------------------------------------------------------------- helpers
def padded(x: np.ndarray) -> np.ndarray:
    """Real nx x ny data -> padded nx x 2*(ny/2+1) float64 layout."""
    nx, ny = x.shape
    out = np.zeros((nx, 2 * (ny // 2 + 1)), dtype=np.float64)
    out[:, :ny] = x
    return out


def spectrum(values: np.ndarray) -> np.ndarray:
    """View a transformed padded array as its nx x (ny/2+1) complex spectrum."""
    return np.ascontiguousarray(values).view(np.complex128 if values.dtype == np.float64 else np.complex64)


def rel_l2(got: np.ndarray, ref: np.ndarray) -> float:
    got = np.asarray(got, dtype=np.complex128 if np.iscomplexobj(got) else np.float64)
    ref = np.asarray(ref, dtype=np.complex128 if np.iscomplexobj(ref) else np.float64)
    den = np.linalg.norm(ref.ravel())
    return float(np.linalg.norm((got - ref).ravel()) / (den if den else 1.0))
