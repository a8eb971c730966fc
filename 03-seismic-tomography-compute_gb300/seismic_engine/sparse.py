"""Sparse face of seismic_engine: CSRMatrix, SparseOps and compute_fd_stencil
with the names, arguments and defaults of the reference binding
(src/cpp/pybind/bindings.cpp:52-193,243-253), backed by device CSR storage
(int64 row pointers, int32 columns, FP32 values) in libseismic_gb300.so.

numpy FP64 in, numpy FP64 out for the reference names (copy semantics, as
the binding); the *_device / torch entry points are zero-copy.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import call

_d = C.POINTER(C.c_double)
_i64 = C.POINTER(C.c_int64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1)


def _i64a(a):
    return np.ascontiguousarray(a, dtype=np.int64).reshape(-1)


class CSRMatrix:
    """seismic::CSRMatrix (sparse/csr_matrix.h:17-71) on the GPU.

    build_from_triplets produces the canonical CSR (sorted, merged,
    unpadded); pad=True applies the reference's pad_to_alignment rule."""

    def __init__(self, rows: int = 0, cols: int = 0, nnz: int = 0, device: int = 0):
        h = C.c_void_p()
        call("st_csr_create", int(rows), int(cols), int(nnz), device, C.byref(h))
        self._h = h
        self._device = device

    @classmethod
    def _wrap(cls, handle, device):
        m = cls.__new__(cls)
        m._h = handle
        m._device = device
        return m

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().st_csr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ---- construction (csr_matrix.cpp:25-116)
    def build_from_triplets(self, rows, cols, row_idx, col_idx, values, pad: bool = False):
        r, c, v = _i64a(row_idx), _i64a(col_idx), _f64(values)
        n = min(r.size, c.size, v.size)
        call("st_csr_build_from_triplets", self._h, int(rows), int(cols), n, r.ctypes.data_as(_i64),
             c.ctypes.data_as(_i64), v.ctypes.data_as(_d), int(pad))
        return self

    def build_from_triplets_device(self, rows, cols, row_idx, col_idx, values, pad: bool = False):
        """torch CUDA int32 / int32 / float32 triplets (zero-copy)."""
        n = int(row_idx.numel())
        call("st_csr_build_from_triplets_device", self._h, int(rows), int(cols), n, row_idx.data_ptr(),
             col_idx.data_ptr(), values.data_ptr(), int(pad))
        return self

    def build_fd_stencil_7point(self, nx, ny, nz, velocity, dx, dy, dz, dt, pad: bool = False):
        v = _f64(velocity)
        if v.size < nx * ny * nz:
            raise ValueError("velocity has fewer than nx*ny*nz values")
        call("st_csr_build_fd_stencil_7point", self._h, nx, ny, nz, v.ctypes.data_as(_d), dx, dy, dz, dt, int(pad))
        return self

    # ---- accessors (csr_matrix.h:32-38)
    def build_ray_matrix(self, endpoints, nx: int, ny: int, nz: int, cell_size: float = 1.0) -> int:
        """Straight-ray path-length matrix: row i = ray endpoints[i] =
        (x0, y0, z0, x1, y1, z1) in cell units (numpy FP64 or a CUDA FP64
        tensor); returns nnz."""
        nnz = C.c_int64()
        if hasattr(endpoints, "data_ptr"):
            e = endpoints.contiguous()
            assert e.dtype.is_floating_point and e.element_size() == 8 and e.is_cuda
            call("st_csr_build_ray_matrix", self.handle, e.numel() // 6, e.data_ptr(), 1, nx, ny, nz,
                 float(cell_size), C.byref(nnz))
        else:
            e = np.ascontiguousarray(endpoints, np.float64).reshape(-1)
            call("st_csr_build_ray_matrix", self.handle, e.size // 6, e.ctypes.data, 0, nx, ny, nz,
                 float(cell_size), C.byref(nnz))
        return nnz.value

    def _shape(self):
        out = (C.c_int64 * 3)()
        call("st_csr_shape", self._h, out)
        return out[0], out[1], out[2]

    def rows(self):
        return self._shape()[0]

    def cols(self):
        return self._shape()[1]

    def nnz(self):
        return self._shape()[2]

    def row_ptr(self):
        r = np.empty(self.rows() + 1, np.int64)
        call("st_csr_get", self._h, r.ctypes.data_as(_i64), None, None)
        return r

    def col_ind(self):
        c = np.empty(max(self.nnz(), 1), np.int64)
        call("st_csr_get", self._h, None, c.ctypes.data_as(_i64), None)
        return c[:self.nnz()]

    def values(self):
        v = np.empty(max(self.nnz(), 1), np.float64)
        call("st_csr_get", self._h, None, None, v.ctypes.data_as(_d))
        return v[:self.nnz()]

    def device_arrays(self):
        rp, ci, va = C.c_void_p(), C.c_void_p(), C.c_void_p()
        call("st_csr_device_arrays", self._h, C.byref(rp), C.byref(ci), C.byref(va))
        return rp.value, ci.value, va.value

    # ---- operators (csr_matrix.cpp:118-193)
    def spmv(self, x):
        x = _f64(x)
        y = np.empty(self.rows())
        call("st_csr_spmv", self._h, x.ctypes.data_as(_d), x.size, y.ctypes.data_as(_d))
        return y

    def spmv_transpose(self, x):
        x = _f64(x)
        y = np.empty(self.cols())
        call("st_csr_spmv_transpose", self._h, x.ctypes.data_as(_d), x.size, y.ctypes.data_as(_d))
        return y

    def spmv_device(self, x, y, transpose: bool = False):
        """y = A x or A^T x on torch CUDA float32 tensors (on the matrix's stream)."""
        call("st_csr_spmv_device", self._h, int(transpose), x.data_ptr(), y.data_ptr())

    def stream_ptr(self):
        p = C.c_void_p()
        call("st_csr_stream", self._h, C.byref(p))
        return p.value or 0

    def frobenius_norm(self):
        out = C.c_double()
        call("st_csr_frobenius_norm", self._h, C.byref(out))
        return out.value

    def scale(self, alpha):
        call("st_csr_scale", self._h, float(alpha))

    def add_diagonal(self, alpha):
        call("st_csr_add_diagonal", self._h, float(alpha))

    def optimize_cache_blocking(self, block_size: int = 8):
        """Row-block metadata of the CPU SpMV (csr_matrix.cpp:195-210); the GPU
        SpMV assigns rows to thread groups itself, so this only validates."""
        if block_size <= 0:
            raise ValueError("block_size must be positive")

    def clone(self):
        h = C.c_void_p()
        call("st_csr_clone", self._h, C.byref(h))
        return CSRMatrix._wrap(h, self._device)


class SparseOps:
    """seismic::SparseOps (sparse/sparse_ops.h:9-48) on the GPU."""

    @staticmethod
    def _cg(A: CSRMatrix, b, max_iter, tolerance, jacobi):
        b = _f64(b)
        x = np.zeros(A.rows())
        it = C.c_int()
        rel = C.c_double()
        call("st_cg", A.handle, b.ctypes.data_as(_d), b.size, int(max_iter), float(tolerance), int(jacobi),
             x.ctypes.data_as(_d), C.byref(it), C.byref(rel))
        SparseOps.last_iterations = it.value
        SparseOps.last_relative_residual = rel.value
        return x

    @staticmethod
    def conjugate_gradient(A: CSRMatrix, b, max_iter: int = 1000, tolerance: float = 1e-8):
        return SparseOps._cg(A, b, max_iter, tolerance, 0)

    @staticmethod
    def jacobi_preconditioned_cg(A: CSRMatrix, b, max_iter: int = 1000, tolerance: float = 1e-8):
        return SparseOps._cg(A, b, max_iter, tolerance, 1)

    @staticmethod
    def dot_product(a, b):
        a, b = _f64(a), _f64(b)
        n = min(a.size, b.size)
        out = C.c_double()
        call("st_dot", a.ctypes.data_as(_d), b.ctypes.data_as(_d), n, 0, C.byref(out))
        return out.value

    @staticmethod
    def l2_norm(a):
        return float(np.sqrt(SparseOps.dot_product(a, a)))

    @staticmethod
    def build_hessian_approx(forward_operator: CSRMatrix, regularization: float):
        H = forward_operator.clone()
        H.add_diagonal(regularization)
        return H

    @staticmethod
    def smooth_gradient(gradient, nx: int, ny: int, nz: int, sigma: float):
        from .fields import smooth_gradient
        return smooth_gradient(gradient, nx, ny, nz, sigma)


def compute_fd_stencil(nx, ny, nz, velocity, dx, dy, dz, dt) -> CSRMatrix:
    """bindings.cpp:243-253: the 7-point FD stencil as a CSR matrix."""
    return CSRMatrix().build_fd_stencil_7point(nx, ny, nz, velocity, dx, dy, dz, dt)


def normal_pcg_stencil_device(A: CSRMatrix, d, lam: float, w, grid, x, max_iter: int = 1000, tol: float = 1e-6,
                              rhs=None, confirm_true: bool = False):
    """(A^T A + lam I) x = A^T d preconditioned by M r = D r + S K (S r)
    (st_normal_pcg_stencil_device: D Jacobi, S = sqrt(D), K the three-axis
    weighted Dirichlet Laplacian of the (nx, ny, nz) cell grid with weights
    w >= 0); returns (iterations, recurrence relative residual, true relative
    residual)."""
    it = C.c_int()
    rel = C.c_double()
    true_rel = C.c_double()
    wa = (C.c_float * 3)(*[float(v) for v in w])
    nx, ny, nz = (int(v) for v in grid)
    call("st_normal_pcg_stencil_device", A.handle, d.data_ptr() if d is not None else None, float(lam), wa, nx, ny, nz,
         int(max_iter), float(tol), _lib.ST_CG_CONFIRM_TRUE if confirm_true else 0, x.data_ptr(),
         rhs.data_ptr() if rhs is not None else None, C.byref(it), C.byref(rel), C.byref(true_rel))
    return it.value, rel.value, true_rel.value


def normal_cg_device(A: CSRMatrix, d, lam: float, x, max_iter: int = 1000, tol: float = 1e-6,
                     jacobi: bool = True, rhs=None, confirm_true: bool = False):
    """(A^T A + lam I) x = A^T d on torch CUDA float32 tensors; returns
    (iterations, recurrence relative residual, true relative residual).
    With d = None the right-hand side is rhs itself. confirm_true: the stop
    is confirmed on the true residual (the solve continues while it is above
    tol)."""
    it = C.c_int()
    rel = C.c_double()
    true_rel = C.c_double()
    flags = (_lib.ST_CG_JACOBI if jacobi else 0) | (_lib.ST_CG_CONFIRM_TRUE if confirm_true else 0)
    call("st_normal_cg_device", A.handle, d.data_ptr() if d is not None else None, float(lam), int(max_iter),
         float(tol), flags,
         x.data_ptr(), rhs.data_ptr() if rhs is not None else None, C.byref(it), C.byref(rel), C.byref(true_rel))
    return it.value, rel.value, true_rel.value
