"""Midpoint-sampled straight-ray traveltime tomography on the GPU: the
forward model and gradient of the reference's Python inversion driver,
AdjointStateInversion._forward_model and _compute_gradient
(seismic_tomography/inversion.py:329-433), through st_ray_picks_* of the C
ABI.

`SampledRays` builds a pick set's sample list on the device once (the picks'
geometry does not change during an inversion) and then evaluates traveltimes
and gradients for any velocity model: numpy FP64 in and out (copies), or
torch CUDA FP64 tensors (zero-copy, ordered after the caller's current
stream). `forward_model(model, obs_data)` and
`compute_gradient(model, obs_data, residuals)` take the reference's own
VelocityModel / OBSDataCoordinator objects (read by attribute: nx, ny, nz,
dx, dy, dz, origin_*, vp; picks, sources, stations) and return what the
reference's methods return, bit for bit.

Distances: the reference forms each source-station distance from Python
floats with x ** 2, which libm's pow can round one unit in the last place
away from x * x. `from_reference_objects` recomputes them the reference's
way on the host (one Python expression per pick, as the reference's own
loop does) so the device results are the reference's exactly; arrays given
to the constructor without `dist` use the correctly rounded x * x on the
device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import RayModelC, call
from .sparse import CSRMatrix


def _host_f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


class SampledRays:
    """A pick set's midpoint samples on the GPU.

    model: (nx, ny, nz, dx, dy, dz, origin_x, origin_y, origin_z) or an object
    with those attributes (the reference's VelocityModel). src_xyz / sta_xyz:
    [n_picks, 3] world coordinates; weight: [n_picks]; valid: [n_picks] bool
    (False = the pick's source or station id is unknown); dist: optional
    per-pick distances (see the module docstring)."""

    def __init__(self, model, src_xyz, sta_xyz, weight, valid=None, dist=None, device: int = 0):
        if not isinstance(model, (tuple, list)):
            model = (model.nx, model.ny, model.nz, model.dx, model.dy, model.dz,
                     model.origin_x, model.origin_y, model.origin_z)
        nx, ny, nz = (int(v) for v in model[:3])
        self.shape = (nx, ny, nz)
        self.n_cells = nx * ny * nz
        s = _host_f64(src_xyz)
        r = _host_f64(sta_xyz, s.size)
        if s.size % 3:
            raise ValueError("src_xyz must be [n_picks, 3]")
        n = s.size // 3
        w = _host_f64(weight, n)
        v = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8).reshape(-1)
        if v is not None and v.size != n:
            raise ValueError("valid must have one entry per pick")
        d = None if dist is None else _host_f64(dist, n)
        self._model = RayModelC(nx, ny, nz, *(float(x) for x in model[3:9]))
        h = C.c_void_p()
        call("st_ray_picks_create", device, C.byref(self._model), n, s.ctypes.data, r.ctypes.data,
             None if d is None else d.ctypes.data, w.ctypes.data, None if v is None else v.ctypes.data, C.byref(h))
        self._h = h
        self.device = device
        self.n_picks = n
        info = (C.c_int64 * 3)()
        call("st_ray_picks_info", self._h, info)
        self.n_samples = int(info[1])

    @classmethod
    def from_reference_objects(cls, model, obs_data, device: int = 0):
        """The pick set of a VelocityModel / OBSDataCoordinator pair, with the
        reference's own distance expression (inversion.py:339-341)."""
        picks = obs_data.picks
        n = len(picks)
        src = np.zeros((n, 3))
        sta = np.zeros((n, 3))
        weight = np.zeros(n)
        valid = np.zeros(n, np.uint8)
        dist = np.zeros(n)
        for i, p in enumerate(picks):
            weight[i] = p.weight
            s = obs_data.sources.get(p.source_id)
            r = obs_data.stations.get(p.station_id)
            if s is None or r is None:
                continue
            valid[i] = 1
            src[i] = (s.x, s.y, s.z)
            sta[i] = (r.x, r.y, r.z)
            dist[i] = np.sqrt((s.x - r.x)**2 + (s.y - r.y)**2 + (s.z - r.z)**2)
        return cls(model, src, sta, weight, valid, dist, device)

    # ---- lifetime
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            call("st_ray_picks_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def stream_ptr(self) -> int:
        p = C.c_void_p()
        call("st_ray_picks_stream", self._h, C.byref(p))
        return p.value or 0

    # ---- device ordering for torch tensors
    def _enter(self):
        import torch
        ext = torch.cuda.ExternalStream(self.stream_ptr(), device=torch.device("cuda", self.device))
        ext.wait_stream(torch.cuda.current_stream(self.device))
        return ext

    @staticmethod
    def _leave(ext):
        import torch
        torch.cuda.current_stream(ext.device).wait_stream(ext)

    @staticmethod
    def _is_tensor(a):
        return hasattr(a, "data_ptr") and hasattr(a, "is_cuda")

    def _check_tensor(self, a, n, name):
        import torch
        if not (a.is_cuda and a.dtype == torch.float64 and a.is_contiguous() and a.numel() == n):
            raise ValueError(f"{name}: expected a contiguous CUDA float64 tensor of {n} values")

    # ---- the reference's two methods
    def forward_model(self, vp, out=None):
        """Traveltimes of every pick (inversion.py:329-381) for velocities vp
        of shape (nx, ny, nz) (or flat)."""
        if self._is_tensor(vp):
            import torch
            self._check_tensor(vp, self.n_cells, "vp")
            times = torch.empty(self.n_picks, dtype=torch.float64, device=vp.device) if out is None else out
            self._check_tensor(times, self.n_picks, "out")
            ext = self._enter()
            call("st_ray_picks_forward_model", self._h, vp.data_ptr(), 1, times.data_ptr())
            self._leave(ext)
            return times
        v = _host_f64(vp, self.n_cells)
        times = np.zeros(self.n_picks)
        call("st_ray_picks_forward_model", self._h, v.ctypes.data, 0, times.ctypes.data)
        return times

    def compute_gradient(self, vp, residuals, out=None):
        """Gradient over the cells (inversion.py:383-433), flat, FP64."""
        if self._is_tensor(vp):
            import torch
            self._check_tensor(vp, self.n_cells, "vp")
            self._check_tensor(residuals, self.n_picks, "residuals")
            g = torch.empty(self.n_cells, dtype=torch.float64, device=vp.device) if out is None else out
            self._check_tensor(g, self.n_cells, "out")
            ext = self._enter()
            call("st_ray_picks_compute_gradient", self._h, vp.data_ptr(), residuals.data_ptr(), 1, g.data_ptr())
            self._leave(ext)
            return g
        v = _host_f64(vp, self.n_cells)
        r = _host_f64(residuals, self.n_picks)
        g = np.zeros(self.n_cells)
        call("st_ray_picks_compute_gradient", self._h, v.ctypes.data, r.ctypes.data, 0, g.ctypes.data)
        return g

    def matrix(self) -> CSRMatrix:
        """The sampled-ray matrix (rows = picks, columns = cells, FP32 values
        ds * samples in the cell): A (1 / vp) = traveltimes where every
        velocity is valid."""
        m = CSRMatrix(0, 0, 0, self.device)
        nnz = C.c_int64()
        call("st_csr_build_sampled_ray_matrix", m.handle, self._h, C.byref(nnz))
        return m


def forward_model(model, obs_data, rays: SampledRays | None = None) -> np.ndarray:
    """AdjointStateInversion._forward_model (inversion.py:329-381) on the GPU."""
    rays = rays or SampledRays.from_reference_objects(model, obs_data)
    return rays.forward_model(model.vp)


def compute_gradient(model, obs_data, residuals, rays: SampledRays | None = None) -> np.ndarray:
    """AdjointStateInversion._compute_gradient (inversion.py:383-433) on the GPU."""
    rays = rays or SampledRays.from_reference_objects(model, obs_data)
    return rays.compute_gradient(model.vp, residuals)
