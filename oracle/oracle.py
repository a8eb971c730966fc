"""ctypes front end of the CPU oracle (oracle/seismic_oracle.c) and of the
reference build (oracle/_ref/libseismic_ref.so, present only where the
reference sources were available at build time).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, as the checker or the timed CPU baseline. The product
package never imports this module.

Field layout everywhere: the reference's halo-padded array of
(nx+2)*(ny+2)*(nz+2) values, x slowest, z fastest (core/grid.cpp:45-49).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libseismic_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libseismic_ref.so")

_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)
_i64 = C.POINTER(C.c_int64)
_i32 = C.POINTER(C.c_int)


class OrcGrid(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("sponge_width", C.c_int), ("sponge_damping", C.c_double),
                ("amp_limit", C.c_double), ("cfl_safety", C.c_double), ("sponge_mode", C.c_int)]


def build_oracle(force: bool = False) -> str:
    """Compile the C oracle (plain gcc, OpenMP, no fast-math, no FMA
    contraction so x86 and Arm give the same FP64 bits)."""
    src = os.path.join(HERE, "seismic_oracle.c")
    hdr = os.path.join(HERE, "oracle_prop.h")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                           src, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref() -> str | None:
    """Build oracle/_ref from the reference sources when they are present."""
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])
    return REF_SO if os.path.exists(REF_SO) else None


def _p(a, t):
    return a.ctypes.data_as(t)


class Oracle:
    def __init__(self):
        self.lib = C.CDLL(build_oracle())
        L = self.lib
        for pre, ptr in (("orc64", _d), ("orc32", _f)):
            fn = getattr(L, pre + "_run")
            fn.argtypes = [C.POINTER(OrcGrid), ptr, C.c_int, C.c_int, _i64, ptr, C.c_int, _i64, ptr,
                           _i32, ptr, ptr, ptr, ptr, ptr]
            fn.restype = C.c_int
        L.orc64_adjoint.argtypes = [C.POINTER(OrcGrid), _d, C.c_int, C.c_int, _i64, _d, C.c_int, _i64, _d,
                                    _d, _d, _d, _d]
        L.orc64_adjoint.restype = C.c_int
        L.orc64_rtm_image.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_int, _d, _d, _d, _d, _d]
        L.orc_csr_build.argtypes = [C.c_int64, C.c_int64, C.c_int64, _i64, _i64, _d, C.c_int]
        L.orc_csr_build.restype = C.c_void_p
        L.orc_csr_free.argtypes = [C.c_void_p]
        L.orc_csr_nnz.argtypes = [C.c_void_p]
        L.orc_csr_nnz.restype = C.c_int64
        L.orc_csr_copy.argtypes = [C.c_void_p, _i64, _i64, _d]
        L.orc_csr_wrap.argtypes = [C.c_int64, C.c_int64, _i64, _i64, _d]
        L.orc_csr_wrap.restype = C.c_void_p
        L.orc_csr_unwrap.argtypes = [C.c_void_p]
        L.orc_spmv.argtypes = [C.c_void_p, _d, _d]
        L.orc_spmv_t.argtypes = [C.c_void_p, _d, _d]
        L.orc_dot.argtypes = [_d, _d, C.c_int64]
        L.orc_dot.restype = C.c_double
        L.orc_cg.argtypes = [C.c_void_p, _d, C.c_int, C.c_double, C.c_int, _d, _d]
        L.orc_cg.restype = C.c_int
        L.orc_normal_cg.argtypes = [C.c_void_p, _d, C.c_double, C.c_int, C.c_double, C.c_int, _d, _d, _d]
        L.orc_normal_cg.restype = C.c_int
        L.orc_normal_apply.argtypes = [C.c_void_p, C.c_double, _d, _d]
        L.orc_smooth_gradient.argtypes = [_d, C.c_int64, C.c_int64, C.c_int64, C.c_double, _d]
        L.orc_num_threads.restype = C.c_int
        L.orc_ray_triplets.argtypes = [C.c_int64, _d, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int64, _i64, _i64,
                                       _d]
        L.orc_ray_triplets.restype = C.c_int64
        _u8 = C.POINTER(C.c_uint8)
        L.orc_slice_checksum.argtypes = [_u8, C.c_size_t]
        L.orc_slice_checksum.restype = C.c_uint32
        L.orc_slice_frame.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int, _d, _d, _d,
                                      C.c_int64, C.c_double, _u8, C.c_int64]
        L.orc_slice_frame.restype = C.c_int64
        L.orc_sampled_traveltimes.argtypes = [_i64, _d, _d, C.c_int64, _d, _d, _d, _u8, _d, _d]
        L.orc_sampled_gradient.argtypes = [_i64, _d, _d, C.c_int64, _d, _d, _d, _u8, _d, _d, _d, _d]
        L.orc64_repair_field_nan.argtypes = [_d, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_double]
        L.orc64_repair_field_nan.restype = C.c_int64
        L.orc64_clamp_field.argtypes = [_d, C.c_int64, C.c_double, C.c_double]
        L.orc64_count_nan_inf.argtypes = [_d, C.c_int64]
        L.orc64_count_nan_inf.restype = C.c_int64

    # ------------------------------------------------------------ propagator
    @staticmethod
    def grid(nx, ny, nz, dx, dy, dz, dt, sponge_width=20, sponge_damping=0.015, amp_limit=1e10,
             sponge_mode="reference"):
        """sponge_mode: "reference" (the reference's rule) or "stable" (Cerjan
        form: the new field and the current are damped)."""
        return OrcGrid(nx, ny, nz, dx, dy, dz, dt, sponge_width, sponge_damping, amp_limit, 0.49,
                       1 if sponge_mode == "stable" else 0)

    def run(self, g: OrcGrid, vel, nsteps, src_xyz, src_w, rec_xyz, fp32=False, keep_states=False,
            init_cur=None, init_prev=None):
        """Reference stepping (inject, step, sample) in FP64 or FP32, from zero
        fields or from init_cur / init_prev (reference layout).
        Returns dict(seis [nsteps,nrec], status [nsteps], cur, prev, states)."""
        dt = np.float32 if fp32 else np.float64
        ptr = _f if fp32 else _d
        npad = (g.nx + 2) * (g.ny + 2) * (g.nz + 2)
        vel = np.ascontiguousarray(vel, dtype=dt).reshape(-1)
        assert vel.size == npad
        src_xyz = np.ascontiguousarray(src_xyz, dtype=np.int64).reshape(-1, 3)
        rec_xyz = np.ascontiguousarray(rec_xyz, dtype=np.int64).reshape(-1, 3)
        ns, nr = src_xyz.shape[0], rec_xyz.shape[0]
        src_w = np.ascontiguousarray(src_w, dtype=dt).reshape(nsteps, ns)
        seis = np.zeros((nsteps, max(nr, 1)), dt)
        st = np.zeros(nsteps, np.int32)
        cur = np.zeros(npad, dt)
        prev = np.zeros(npad, dt)
        states = np.zeros((nsteps, npad), dt) if keep_states else None
        fn = self.lib.orc32_run if fp32 else self.lib.orc64_run
        nul = C.cast(None, ptr)
        ic = None if init_cur is None else np.ascontiguousarray(init_cur, dtype=dt).reshape(-1)
        ip = None if init_prev is None else np.ascontiguousarray(init_prev, dtype=dt).reshape(-1)
        rc = fn(C.byref(g), _p(vel, ptr), nsteps, ns, _p(src_xyz, _i64), _p(src_w, ptr), nr, _p(rec_xyz, _i64),
                _p(seis, ptr), _p(st, _i32), _p(cur, ptr), _p(prev, ptr),
                _p(states, ptr) if states is not None else nul,
                _p(ic, ptr) if ic is not None else nul, _p(ip, ptr) if ip is not None else nul)
        assert rc == 0, rc
        return dict(seis=seis[:, :nr], status=st, cur=cur, prev=prev, states=states)

    def adjoint(self, g: OrcGrid, vel, nt, rec_xyz, resid, src_xyz=None, states=None,
                want_image=False, want_grad=False):
        npad = (g.nx + 2) * (g.ny + 2) * (g.nz + 2)
        n = g.nx * g.ny * g.nz
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        rec_xyz = np.ascontiguousarray(rec_xyz, dtype=np.int64).reshape(-1, 3)
        resid = np.ascontiguousarray(resid, dtype=np.float64).reshape(nt, rec_xyz.shape[0])
        src_xyz = np.zeros((0, 3), np.int64) if src_xyz is None else np.ascontiguousarray(src_xyz, np.int64).reshape(-1, 3)
        ns = src_xyz.shape[0]
        src_adj = np.zeros((nt, max(ns, 1)))
        image = np.zeros(n) if want_image else None
        illum = np.zeros(n) if want_image else None
        grad = np.zeros(n) if want_grad else None
        if states is not None:
            states = np.ascontiguousarray(states, dtype=np.float64).reshape(nt, npad)
        nul = C.cast(None, _d)
        rc = self.lib.orc64_adjoint(C.byref(g), _p(vel, _d), nt, rec_xyz.shape[0], _p(rec_xyz, _i64),
                                    _p(resid, _d), ns, _p(src_xyz, _i64), _p(src_adj, _d),
                                    _p(states, _d) if states is not None else nul,
                                    _p(image, _d) if image is not None else nul,
                                    _p(illum, _d) if illum is not None else nul,
                                    _p(grad, _d) if grad is not None else nul)
        assert rc == 0, rc
        return dict(src_adj=src_adj[:, :ns], image=image, illum=illum, grad_c=grad)

    def rtm_image(self, nx, ny, nz, fwd, adj):
        nsteps = fwd.shape[0]
        n = nx * ny * nz
        fwd = np.ascontiguousarray(fwd, np.float64)
        adj = np.ascontiguousarray(adj, np.float64)
        image, illum, refl = np.zeros(n), np.zeros(n), np.zeros(n)
        self.lib.orc64_rtm_image(nx, ny, nz, nsteps, _p(fwd, _d), _p(adj, _d), _p(image, _d), _p(illum, _d),
                                 _p(refl, _d))
        return image, illum, refl

    # ---------------------------------------------------------------- sparse
    def csr_build(self, rows, cols, r, c, v, pad=False):
        r = np.ascontiguousarray(r, np.int64)
        c = np.ascontiguousarray(c, np.int64)
        v = np.ascontiguousarray(v, np.float64)
        h = self.lib.orc_csr_build(rows, cols, r.size, _p(r, _i64), _p(c, _i64), _p(v, _d), int(pad))
        assert h
        nnz = self.lib.orc_csr_nnz(h)
        rp = np.zeros(rows + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int64)
        val = np.zeros(max(nnz, 1), np.float64)
        self.lib.orc_csr_copy(h, _p(rp, _i64), _p(col, _i64), _p(val, _d))
        self.lib.orc_csr_free(h)
        return rp, col[:nnz], val[:nnz]

    class _Wrapped:
        def __init__(self, lib, rows, cols, rp, col, val):
            self.lib = lib
            self.rows, self.cols = rows, cols
            self.rp = np.ascontiguousarray(rp, np.int64)
            self.col = np.ascontiguousarray(col, np.int64)
            self.val = np.ascontiguousarray(val, np.float64)
            if self.col.size == 0:
                self.col = np.zeros(1, np.int64)
                self.val = np.zeros(1, np.float64)
            self.h = lib.orc_csr_wrap(rows, cols, _p(self.rp, _i64), _p(self.col, _i64), _p(self.val, _d))

        def __del__(self):
            if getattr(self, "h", None):
                self.lib.orc_csr_unwrap(self.h)
                self.h = None

    def csr(self, rows, cols, rp, col, val):
        return Oracle._Wrapped(self.lib, rows, cols, rp, col, val)

    def spmv(self, m, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(m.rows)
        self.lib.orc_spmv(m.h, _p(x, _d), _p(y, _d))
        return y

    def spmv_t(self, m, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(m.cols)
        self.lib.orc_spmv_t(m.h, _p(x, _d), _p(y, _d))
        return y

    def dot(self, a, b):
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        return self.lib.orc_dot(_p(a, _d), _p(b, _d), min(a.size, b.size))

    def cg(self, m, b, max_iter=1000, tol=1e-8, jacobi=False):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(m.rows)
        rel = C.c_double(0)
        it = self.lib.orc_cg(m.h, _p(b, _d), max_iter, tol, int(jacobi), _p(x, _d), C.byref(rel))
        return x, it, rel.value

    def normal_cg(self, m, d, lam, max_iter=1000, tol=1e-6, jacobi=True):
        d = np.ascontiguousarray(d, np.float64)
        x = np.zeros(m.cols)
        rhs = np.zeros(m.cols)
        rel = C.c_double(0)
        it = self.lib.orc_normal_cg(m.h, _p(d, _d), lam, max_iter, tol, int(jacobi), _p(x, _d), _p(rhs, _d),
                                    C.byref(rel))
        return x, it, rel.value, rhs

    def normal_apply(self, m, lam, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(m.cols)
        self.lib.orc_normal_apply(m.h, lam, _p(x, _d), _p(y, _d))
        return y

    def ray_matrix(self, ends, nx, ny, nz, h=1.0):
        """Straight-ray path-length CSR (row_ptr, col, FP64 val) of rays
        ends[i] = (x0, y0, z0, x1, y1, z1) in cell units."""
        e = np.ascontiguousarray(ends, np.float64).reshape(-1, 6)
        cap = max(1, e.shape[0] * (nx + ny + nz + 3))
        r = np.zeros(cap, np.int64)
        c = np.zeros(cap, np.int64)
        v = np.zeros(cap, np.float64)
        k = self.lib.orc_ray_triplets(e.shape[0], _p(e, _d), nx, ny, nz, h, cap, _p(r, _i64), _p(c, _i64), _p(v, _d))
        assert k >= 0
        return self.csr_build(e.shape[0], nx * ny * nz, r[:k], c[:k], v[:k])

    @staticmethod
    def _picks(n, d, origin, src_xyz, sta_xyz, valid, dist=None):
        n = np.ascontiguousarray(n, np.int64)
        d = np.ascontiguousarray(d, np.float64)
        o = np.ascontiguousarray(origin, np.float64)
        s = np.ascontiguousarray(src_xyz, np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(sta_xyz, np.float64).reshape(-1, 3)
        v = np.ones(s.shape[0], np.uint8) if valid is None else np.ascontiguousarray(valid, np.uint8)
        dp = None if dist is None else _p(np.ascontiguousarray(dist, np.float64), _d)
        return n, d, o, s, r, v, dp

    def sampled_traveltimes(self, n, d, origin, src_xyz, sta_xyz, valid, vp, dist=None):
        """Midpoint-sampled straight-ray traveltimes of the reference's Python
        inversion (inversion.py:329-381); vp (nx, ny, nz) FP64; dist = the
        per-pick source-station distances to use (None: computed)."""
        dist = None if dist is None else np.ascontiguousarray(dist, np.float64)
        n, d, o, s, r, v, dp = self._picks(n, d, origin, src_xyz, sta_xyz, valid, dist)
        vp = np.ascontiguousarray(vp, np.float64).reshape(-1)
        t = np.zeros(s.shape[0])
        u8 = C.POINTER(C.c_uint8)
        self.lib.orc_sampled_traveltimes(_p(n, _i64), _p(d, _d), _p(o, _d), s.shape[0], _p(s, _d), _p(r, _d),
                                         dp, _p(v, u8), _p(vp, _d), _p(t, _d))
        return t

    def sampled_gradient(self, n, d, origin, src_xyz, sta_xyz, valid, weight, vp, residuals, dist=None):
        """Its gradient (inversion.py:383-433), FP64 over the nx*ny*nz cells."""
        dist = None if dist is None else np.ascontiguousarray(dist, np.float64)
        n, d, o, s, r, v, dp = self._picks(n, d, origin, src_xyz, sta_xyz, valid, dist)
        vp = np.ascontiguousarray(vp, np.float64).reshape(-1)
        w = np.ascontiguousarray(weight, np.float64)
        res = np.ascontiguousarray(residuals, np.float64)
        g = np.zeros(int(np.prod(n)))
        u8 = C.POINTER(C.c_uint8)
        self.lib.orc_sampled_gradient(_p(n, _i64), _p(d, _d), _p(o, _d), s.shape[0], _p(s, _d), _p(r, _d),
                                      dp, _p(v, u8), _p(w, _d), _p(vp, _d), _p(res, _d), _p(g, _d))
        return g

    def slice_checksum(self, payload: bytes) -> int:
        """LockFreeSnapshotBuffer::compute_checksum (snapshot_buffer.cpp:207-229)."""
        buf = np.frombuffer(bytes(payload), np.uint8).copy()
        return int(self.lib.orc_slice_checksum(buf.ctypes.data_as(C.POINTER(C.c_uint8)), buf.size))

    def slice_frame(self, axis, index, nx, ny, nz, fwd, adj, ic, timestep, timestamp=0.0) -> bytes:
        """One serialized slice frame (capture_single_slice + serialize_slice)
        from reference-layout FP64 fields fwd / adj and the interior ic."""
        f = np.ascontiguousarray(fwd, np.float64).reshape(-1)
        a = np.ascontiguousarray(adj, np.float64).reshape(-1)
        c = np.ascontiguousarray(ic, np.float64).reshape(-1)
        cap = 128 + 3 * 8 * max(nx, ny) * max(ny, nz)
        out = np.zeros(cap, np.uint8)
        n = self.lib.orc_slice_frame(axis, index, nx, ny, nz, 1, _p(f, _d), _p(a, _d), _p(c, _d), timestep,
                                     float(timestamp), out.ctypes.data_as(C.POINTER(C.c_uint8)), cap)
        assert n > 0
        return out[:n].tobytes()

    def smooth_gradient(self, g, nx, ny, nz, sigma):
        g = np.ascontiguousarray(g, np.float64).reshape(-1)
        out = np.zeros(nx * ny * nz)
        if g.size < nx * ny * nz:
            return out
        self.lib.orc_smooth_gradient(_p(g, _d), nx, ny, nz, sigma, _p(out, _d))
        return out

    def repair_field_nan(self, data, nx, ny, nz, hw=1, repl=0.0):
        d = np.array(data, np.float64, copy=True)
        self.lib.orc64_repair_field_nan(_p(d, _d), d.size, nx, ny, nz, hw, repl)
        return d

    def clamp_field(self, data, lo, hi):
        d = np.array(data, np.float64, copy=True)
        self.lib.orc64_clamp_field(_p(d, _d), d.size, lo, hi)
        return d

    def count_nan_inf(self, data):
        d = np.ascontiguousarray(data, np.float64)
        return self.lib.orc64_count_nan_inf(_p(d, _d), d.size)

    def num_threads(self):
        return self.lib.orc_num_threads()


class Reference:
    """The reference's own C++ through oracle/ref_harness.cpp (x86 only)."""

    def __init__(self):
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        L = self.lib = C.CDLL(REF_SO)
        L.ref_run_steps.argtypes = [C.c_int64] * 3 + [C.c_double] * 4 + [C.c_int, C.c_double, _d, C.c_int, _i64,
                                                                          _d, C.c_int, _i64, _d, C.c_int, C.c_int,
                                                                          _i32, _d, _d]
        L.ref_forward_propagate.argtypes = [C.c_int64] * 3 + [C.c_double] * 4 + [C.c_int, C.c_int, C.c_double,
                                                                                  C.c_int, _d, _d, C.c_int64, _d,
                                                                                  _d, _d, C.c_int64, _i64]
        L.ref_rtm_image.argtypes = [C.c_int64] * 3 + [C.c_int, _d, _d, _d, _d, _d]
        L.ref_csr_build.argtypes = [C.c_int64, C.c_int64, C.c_int64, _i64, _i64, _d]
        L.ref_csr_build.restype = C.c_int64
        L.ref_csr_get.argtypes = [_i64, _i64, _d]
        L.ref_csr_spmv.argtypes = [_d, C.c_int64, _d]
        L.ref_repair_field_nan.argtypes = [_d, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_double]
        L.ref_count_nan_inf.argtypes = [_d, C.c_int64]
        L.ref_count_nan_inf.restype = C.c_int64
        L.ref_clamp_field.argtypes = [_d, C.c_int64, C.c_double, C.c_double]
        L.ref_load_config.argtypes = [C.c_char_p, _d]
        _u8 = C.POINTER(C.c_uint8)
        L.ref_extract_slices.argtypes = [C.c_int64] * 3 + [C.c_int, _i32, _i64, _d, _d, _d, C.c_int64, C.c_int64,
                                                           _d, _i64]
        L.ref_mmap_write.argtypes = [C.c_char_p, C.c_int64, C.c_int, _u8, _i64, _i64]
        L.ref_mmap_read_frame.argtypes = [C.c_char_p, C.c_int64, _u8, C.c_int64]
        L.ref_mmap_read_frame.restype = C.c_int64
        L.ref_terrain.argtypes = ([C.c_int64] * 3 + [C.c_double] * 6 + [C.c_int, C.c_double, C.c_int, C.c_double,
                                                                        C.c_double, C.c_int, _d, _d, _i64,
                                                                        C.c_double, C.c_double, _d,
                                                                        C.POINTER(C.c_uint8), _d, _d, _d, C.c_int,
                                                                        C.c_double])
        L.ref_mmap_count_frames.argtypes = [C.c_char_p]
        L.ref_mmap_count_frames.restype = C.c_int64
        L.ref_csr_fd_stencil.argtypes = [C.c_int64] * 3 + [_d] + [C.c_double] * 4
        L.ref_csr_fd_stencil.restype = C.c_int64
        L.ref_csr_spmv_t.argtypes = [_d, C.c_int64, _d]
        L.ref_hessian_approx.argtypes = [C.c_double]
        L.ref_hessian_approx.restype = C.c_int64
        L.ref_cg.argtypes = [C.c_int, _d, C.c_int64, C.c_int, C.c_double, _d]
        L.ref_dot.argtypes = [_d, _d, C.c_int64]
        L.ref_dot.restype = C.c_double
        L.ref_smooth_gradient.argtypes = [_d, C.c_int64, C.c_int64, C.c_int64, C.c_double, _d]
        L.ref_adjoint_propagate.argtypes = ([C.c_int64] * 3 + [C.c_double] * 4 + [C.c_int, C.c_int, C.c_double, _d, _d,
                                                                                   C.c_int64, _d, C.c_int64, _d, _d,
                                                                                   _i64])
        L.ref_rtm_building_blocks.argtypes = ([C.c_int64] * 3 + [C.c_double] * 4 + [C.c_int, C.c_double, _d, _d,
                                                                                     C.c_int, _i32, C.c_int64, _d, _d,
                                                                                     _d, _d, _d, _i64])

    def extract_slices(self, nx, ny, nz, specs, fwd, adj, ic, timestep=0):
        """RTMEngine::extract_slices with a collecting callback: a list of
        (axis, index, forward, adjoint, ic) with (dim0, dim1) arrays."""
        axes = np.array([a for a, _ in specs], np.int32)
        idx = np.array([i for _, i in specs], np.int64)
        f = np.ascontiguousarray(fwd, np.float64).reshape(-1)
        a = np.ascontiguousarray(adj, np.float64).reshape(-1)
        c = np.ascontiguousarray(ic, np.float64).reshape(-1)
        cap = 3 * len(specs) * max(nx, ny) * max(ny, nz)
        vals = np.zeros(cap)
        meta = np.zeros(4 * len(specs), np.int64)
        k = self.lib.ref_extract_slices(nx, ny, nz, len(specs), _p(axes, _i32), _p(idx, _i64), _p(f, _d), _p(a, _d),
                                        _p(c, _d), timestep, cap, _p(vals, _d), _p(meta, _i64))
        assert k >= 0
        out, o = [], 0
        for j in range(k):
            ax, ix, d0, d1 = (int(v) for v in meta[4 * j:4 * j + 4])
            n = d0 * d1
            out.append((ax, ix, vals[o:o + n].reshape(d0, d1), vals[o + n:o + 2 * n].reshape(d0, d1),
                        vals[o + 2 * n:o + 3 * n].reshape(d0, d1)))
            o += 3 * n
        return out

    def terrain(self, n, d, origin, water_depth, synthetic=False, gradient=0.0, roughness=0.0, points=None,
                water_vp=1500.0, sediment_vp=3000.0, velocity=None, fields=None, sponge_width=3, damping=0.5):
        """TerrainBoundary on a single-rank grid (halo 1): returns dict(bathy,
        sf_index, velocity, mask, free, seafloor, absorbing)."""
        nx, ny, nz = (int(v) for v in n)
        npad = (nx + 2) * (ny + 2) * (nz + 2)
        pts = np.ascontiguousarray(points if points is not None else np.zeros((0, 3)), np.float64).reshape(-1)
        bathy = np.zeros(nx * ny)
        sfi = np.zeros(nx * ny, np.int64)
        vel = np.array(velocity if velocity is not None else np.zeros(npad), np.float64, copy=True).reshape(-1)
        mask = np.zeros(npad, np.uint8)
        f = [np.array(fields[k], np.float64, copy=True).reshape(-1) for k in range(3)]
        self.lib.ref_terrain(nx, ny, nz, *(float(v) for v in d), *(float(v) for v in origin), 1, float(water_depth),
                             int(synthetic), float(gradient), float(roughness), pts.size // 3, _p(pts, _d),
                             _p(bathy, _d), _p(sfi, _i64), float(water_vp), float(sediment_vp), _p(vel, _d),
                             mask.ctypes.data_as(C.POINTER(C.c_uint8)), _p(f[0], _d), _p(f[1], _d), _p(f[2], _d),
                             int(sponge_width), float(damping))
        return dict(bathy=bathy, sf_index=sfi, velocity=vel, mask=mask, free=f[0], seafloor=f[1], absorbing=f[2])

    def mmap_write(self, path, max_bytes, frames):
        """MmapSnapshotWriter open / write_frame per frame / close; returns
        (accepted, [frames_written, frames_dropped, total_bytes, mmap_cycles])."""
        data = np.frombuffer(b"".join(frames), np.uint8).copy() if frames else np.zeros(1, np.uint8)
        sizes = np.array([len(f) for f in frames] or [0], np.int64)
        stats = np.zeros(4, np.int64)
        ok = self.lib.ref_mmap_write(os.fsencode(path), max_bytes, len(frames),
                                     data.ctypes.data_as(C.POINTER(C.c_uint8)), _p(sizes, _i64), _p(stats, _i64))
        return ok, [int(v) for v in stats]

    def mmap_read_frame(self, path, index, cap=1 << 26):
        buf = np.zeros(cap, np.uint8)
        n = self.lib.ref_mmap_read_frame(os.fsencode(path), index, buf.ctypes.data_as(C.POINTER(C.c_uint8)), cap)
        return None if n < 0 else buf[:n].tobytes()

    def mmap_count_frames(self, path):
        return int(self.lib.ref_mmap_count_frames(os.fsencode(path)))

    def run_steps(self, nx, ny, nz, dx, dy, dz, dt, sw, damp, vel, nsteps, src_xyz, src_w, rec_xyz, adjoint=False):
        npad = (nx + 2) * (ny + 2) * (nz + 2)
        vel = np.ascontiguousarray(vel, np.float64).reshape(-1)
        src_xyz = np.ascontiguousarray(src_xyz, np.int64).reshape(-1, 3)
        rec_xyz = np.ascontiguousarray(rec_xyz, np.int64).reshape(-1, 3)
        ns, nr = src_xyz.shape[0], rec_xyz.shape[0]
        src_w = np.ascontiguousarray(src_w, np.float64).reshape(nsteps, ns)
        seis = np.zeros((nsteps, max(nr, 1)))
        st = np.zeros(nsteps, np.int32)
        cur = np.zeros(npad)
        prev = np.zeros(npad)
        self.lib.ref_run_steps(nx, ny, nz, dx, dy, dz, dt, sw, damp, _p(vel, _d), ns, _p(src_xyz, _i64),
                               _p(src_w, _d), nr, _p(rec_xyz, _i64), _p(seis, _d), nsteps, int(adjoint),
                               _p(st, _i32), _p(cur, _d), _p(prev, _d))
        return dict(seis=seis[:, :nr], status=st, cur=cur, prev=prev)

    def forward_propagate(self, nx, ny, nz, dx, dy, dz, dt, nt, sw, damp, snap_int, vel, wavelet):
        npad = (nx + 2) * (ny + 2) * (nz + 2)
        vel = np.ascontiguousarray(vel, np.float64).reshape(-1)
        wavelet = np.ascontiguousarray(wavelet, np.float64)
        cur, prev = np.zeros(npad), np.zeros(npad)
        cap = (nt // max(snap_int, 1) + 2) * nx * ny * nz
        snaps = np.zeros(cap)
        res = np.zeros(6, np.int64)
        self.lib.ref_forward_propagate(nx, ny, nz, dx, dy, dz, dt, nt, sw, damp, snap_int, _p(vel, _d),
                                       _p(wavelet, _d), wavelet.size, _p(cur, _d), _p(prev, _d), _p(snaps, _d),
                                       cap, _p(res, _i64))
        return dict(status=int(res[0]), total_nan=int(res[1]), repaired=int(res[2]), steps=int(res[3]),
                    ok=bool(res[4]), cur=cur, prev=prev, snapshots=snaps[:res[5]])

    def rtm_image(self, nx, ny, nz, fwd, adj):
        n = nx * ny * nz
        fwd = np.ascontiguousarray(fwd, np.float64)
        adj = np.ascontiguousarray(adj, np.float64)
        image, illum, refl = np.zeros(n), np.zeros(n), np.zeros(n)
        self.lib.ref_rtm_image(nx, ny, nz, fwd.shape[0], _p(fwd, _d), _p(adj, _d), _p(image, _d),
                               _p(illum, _d), _p(refl, _d))
        return image, illum, refl

    def csr_build(self, rows, cols, r, c, v):
        r = np.ascontiguousarray(r, np.int64)
        c = np.ascontiguousarray(c, np.int64)
        v = np.ascontiguousarray(v, np.float64)
        nnz = self.lib.ref_csr_build(rows, cols, r.size, _p(r, _i64), _p(c, _i64), _p(v, _d))
        rp = np.zeros(rows + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int64)
        val = np.zeros(max(nnz, 1))
        self.lib.ref_csr_get(_p(rp, _i64), _p(col, _i64), _p(val, _d))
        return rp, col[:nnz], val[:nnz]

    def csr_spmv(self, x, rows):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(rows)
        self.lib.ref_csr_spmv(_p(x, _d), x.size, _p(y, _d))
        return y

    def _csr_get(self, rows, nnz):
        rp = np.zeros(rows + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int64)
        val = np.zeros(max(nnz, 1))
        self.lib.ref_csr_get(_p(rp, _i64), _p(col, _i64), _p(val, _d))
        return rp, col[:nnz], val[:nnz]

    def csr_fd_stencil(self, nx, ny, nz, vel, dx, dy, dz, dt):
        """CSRMatrix::build_fd_stencil_7point; becomes the current matrix."""
        v = np.ascontiguousarray(vel, np.float64)
        nnz = self.lib.ref_csr_fd_stencil(nx, ny, nz, _p(v, _d), dx, dy, dz, dt)
        return self._csr_get(nx * ny * nz, nnz)

    def csr_spmv_t(self, x, cols):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(cols)
        self.lib.ref_csr_spmv_t(_p(x, _d), x.size, _p(y, _d))
        return y

    def hessian_approx(self, reg, rows):
        """SparseOps::build_hessian_approx of the current matrix (replaces it)."""
        nnz = self.lib.ref_hessian_approx(reg)
        return self._csr_get(rows, nnz)

    def cg(self, b, max_iter, tol, jacobi=False):
        """SparseOps::conjugate_gradient / jacobi_preconditioned_cg on the
        current matrix (square)."""
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(b.size)
        self.lib.ref_cg(int(jacobi), _p(b, _d), b.size, int(max_iter), float(tol), _p(x, _d))
        return x

    def dot(self, a, b):
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        return self.lib.ref_dot(_p(a, _d), _p(b, _d), min(a.size, b.size))

    def smooth_gradient(self, g, nx, ny, nz, sigma):
        g = np.ascontiguousarray(g, np.float64)
        out = np.zeros(nx * ny * nz)
        self.lib.ref_smooth_gradient(_p(g, _d), nx, ny, nz, float(sigma), _p(out, _d))
        return out

    def adjoint_propagate(self, nx, ny, nz, dx, dy, dz, dt, nt, sw, damp, vel, residual, fwd_wavelet=None):
        """WaveEquationSolver::adjoint_propagate on a fresh solver, after
        forward_propagate(fwd_wavelet) on it when given."""
        v = np.ascontiguousarray(vel, np.float64)
        r = np.ascontiguousarray(residual, np.float64)
        fw = np.ascontiguousarray(fwd_wavelet if fwd_wavelet is not None else np.zeros(1), np.float64)
        nfw = 0 if fwd_wavelet is None else fw.size
        n = (nx + 2) * (ny + 2) * (nz + 2)
        cur, prev, res = np.zeros(n), np.zeros(n), np.zeros(5, np.int64)
        self.lib.ref_adjoint_propagate(nx, ny, nz, dx, dy, dz, dt, nt, sw, damp, _p(v, _d), _p(fw, _d), nfw,
                                       _p(r, _d), r.size, _p(cur, _d), _p(prev, _d), _p(res, _i64))
        return dict(cur=cur, prev=prev, status=int(res[0]), nan=int(res[1]), repaired=int(res[2]),
                    steps=int(res[3]), ok=bool(res[4]))

    def rtm_building_blocks(self, nx, ny, nz, dx, dy, dz, dt, sw, damp, vel, wavelet, ops, ring_capacity):
        """configure_rtm + inject / step_forward / store_forward_wavefield_for_rtm /
        apply_rtm_step / apply_sponge_layer as ops[t] says (bits 1, 2, 4, 8)."""
        v = np.ascontiguousarray(vel, np.float64)
        w = np.ascontiguousarray(wavelet, np.float64)
        o = np.ascontiguousarray(ops, np.int32)
        n = (nx + 2) * (ny + 2) * (nz + 2)
        m = nx * ny * nz
        img, ill, refl, cur, prev = np.zeros(m), np.zeros(m), np.zeros(m), np.zeros(n), np.zeros(n)
        counts = np.zeros(2, np.int64)
        self.lib.ref_rtm_building_blocks(nx, ny, nz, dx, dy, dz, dt, sw, damp, _p(v, _d), _p(w, _d), o.size,
                                         _p(o, _i32), int(ring_capacity), _p(img, _d), _p(ill, _d), _p(refl, _d),
                                         _p(cur, _d), _p(prev, _d), _p(counts, _i64))
        return dict(image=img, illum=ill, refl=refl, cur=cur, prev=prev, captured=int(counts[0]),
                    dropped=int(counts[1]))

    def repair_field_nan(self, data, nx, ny, nz, hw=1, repl=0.0):
        d = np.array(data, np.float64, copy=True)
        self.lib.ref_repair_field_nan(_p(d, _d), d.size, nx, ny, nz, hw, repl)
        return d

    def count_nan_inf(self, data):
        d = np.ascontiguousarray(data, np.float64)
        return self.lib.ref_count_nan_inf(_p(d, _d), d.size)

    def clamp_field(self, data, lo, hi):
        d = np.array(data, np.float64, copy=True)
        self.lib.ref_clamp_field(_p(d, _d), d.size, lo, hi)
        return d

    def load_config(self, path):
        out = np.zeros(17)
        self.lib.ref_load_config(path.encode(), _p(out, _d))
        return out
