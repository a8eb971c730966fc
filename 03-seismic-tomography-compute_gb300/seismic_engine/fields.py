"""Field-health helpers of the reference binding (bindings.cpp:275-301) and
SparseOps.smooth_gradient, computed on the GPU in FP64 (numpy in, numpy out)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import call

_d = C.POINTER(C.c_double)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1)


def check_field_health(data) -> int:
    """Count of NaN/Inf values (FaultTolerance::count_nan_inf)."""
    a = _f64(data)
    out = C.c_int64()
    call("st_field_count_nonfinite", a.ctypes.data_as(_d), a.size, 0, C.byref(out))
    return out.value


def clamp_field_safe(data, lo: float = -1e10, hi: float = 1e10):
    """NaN/Inf -> 0, others clamped to [lo, hi]; returns the array like the
    binding (in place for a contiguous FP64 input)."""
    a = data if (isinstance(data, np.ndarray) and data.dtype == np.float64 and data.flags.c_contiguous) \
        else _f64(data).copy()
    flat = a.reshape(-1)
    call("st_field_clamp", flat.ctypes.data_as(_d), flat.size, float(lo), float(hi), 0)
    return a


def repair_field_nan(data, nx: int, ny: int, nz: int, halo_width: int = 1, replace_value: float = 0.0):
    """Repair NaN/Inf cells by averaging valid neighbours (reference cell order)."""
    a = data if (isinstance(data, np.ndarray) and data.dtype == np.float64 and data.flags.c_contiguous) \
        else _f64(data).copy()
    flat = a.reshape(-1)
    call("st_field_repair_nan", flat.ctypes.data_as(_d), flat.size, nx, ny, nz, halo_width, float(replace_value), 0)
    return a


def smooth_gradient(gradient, nx: int, ny: int, nz: int, sigma: float) -> np.ndarray:
    """SparseOps.smooth_gradient: normalised truncated Gaussian (radius floor(3 sigma))."""
    g = _f64(gradient)
    out = np.zeros(nx * ny * nz)
    call("st_smooth_gradient", g.ctypes.data_as(_d), g.size, nx, ny, nz, float(sigma), 0, out.ctypes.data_as(_d))
    return out
