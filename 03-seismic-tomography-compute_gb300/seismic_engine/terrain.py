"""Irregular seafloor terrain: seismic::TerrainBoundary (solver/boundary.h,
solver/boundary.cpp), the binding's BathymetryPoint and generate_bathymetry
(pybind/bindings.cpp:195-200,255-270), over the GPU library.

Field operations take the reference's halo-padded FP64 arrays: numpy arrays
(copied to the GPU and back) or CUDA float64 tensors (in place). Terrain-aware
propagation is `WaveEquationSolver.set_terrain`.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import BathymetryPointC, call

_d = C.POINTER(C.c_double)


@dataclass
class BathymetryPoint:
    """seismic::BathymetryPoint (boundary.h:9-13)."""
    x: float = 0.0
    y: float = 0.0
    depth: float = 0.0


def generate_bathymetry(nx: int, ny: int, dx: float, dy: float, origin_x: float, origin_y: float,
                        water_depth: float, gradient: float, roughness: float) -> np.ndarray:
    """The binding's generate_bathymetry: (nx, ny) synthetic depths."""
    out = np.empty(nx * ny)
    call("st_generate_bathymetry", nx, ny, dx, dy, origin_x, origin_y, water_depth, gradient, roughness,
         out.ctypes.data_as(_d))
    return out.reshape(nx, ny)


class TerrainBoundary:
    """seismic::TerrainBoundary(grid, water_depth) on the GPU library; `grid`
    is a GridParams (single domain, its halo_width)."""

    def __init__(self, grid, water_depth: float, device: int = 0):
        h = C.c_void_p()
        call("st_terrain_create", C.byref(grid.c()), float(water_depth), device, C.byref(h))
        self._h = h
        self._grid = grid
        hw = grid.halo_width
        self.shape = (grid.nx_global, grid.ny_global, grid.nz_global)
        self.padded_size = ((grid.nx_global + 2 * hw) * (grid.ny_global + 2 * hw) * (grid.nz_global + 2 * hw))

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.load().st_terrain_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bathymetry_data(self, data):
        pts = list(data)
        arr = (BathymetryPointC * max(len(pts), 1))()
        for k, p in enumerate(pts):
            x, y, dep = (p.x, p.y, p.depth) if hasattr(p, "depth") else p
            arr[k] = BathymetryPointC(float(x), float(y), float(dep))
        call("st_terrain_set_bathymetry_data", self._h, arr, len(pts))

    def generate_synthetic_bathymetry(self, gradient: float, roughness: float):
        call("st_terrain_generate_synthetic_bathymetry", self._h, float(gradient), float(roughness))

    def bathymetry(self) -> np.ndarray:
        out = np.empty(self.shape[0] * self.shape[1])
        call("st_terrain_bathymetry", self._h, out.ctypes.data_as(_d))
        return out

    def seafloor_depth(self, gx: int, gy: int) -> float:
        d = C.c_double()
        call("st_terrain_seafloor", self._h, gx, gy, C.byref(d), None)
        return d.value

    def seafloor_index(self, gx: int, gy: int) -> int:
        i = C.c_int64()
        call("st_terrain_seafloor", self._h, gx, gy, None, C.byref(i))
        return i.value

    def is_subsurface(self, gx: int, gy: int, gz: int) -> bool:
        """boundary.cpp:59-64."""
        g = self._grid
        return g.origin_z + gz * g.dz >= self.seafloor_depth(gx, gy)

    def is_water(self, gx: int, gy: int, gz: int) -> bool:
        return not self.is_subsurface(gx, gy, gz)

    def _field(self, name, field, *extra, dtype=np.float64):
        if hasattr(field, "data_ptr"):
            if field.numel() != self.padded_size:
                raise ValueError(f"expected {self.padded_size} values")
            call(name, self._h, field.data_ptr(), 1, *extra)
            return field
        if not (isinstance(field, np.ndarray) and field.dtype == dtype and field.flags.c_contiguous):
            raise TypeError(f"expected a C-contiguous numpy {np.dtype(dtype).name} array (modified in place)")
        if field.size != self.padded_size:
            raise ValueError(f"expected {self.padded_size} values")
        call(name, self._h, field.ctypes.data, 0, *extra)
        return field

    def update_velocity_mask(self, velocity, water_vp: float, sediment_vp: float):
        return self._field("st_terrain_update_velocity_mask", velocity, float(water_vp), float(sediment_vp))

    def build_boundary_mask(self) -> np.ndarray:
        m = np.zeros(self.padded_size, np.uint8)
        call("st_terrain_build_boundary_mask", self._h, m.ctypes.data, 0)
        self._mask = m
        return m

    def mask(self) -> np.ndarray:
        return getattr(self, "_mask", np.zeros(0, np.uint8))

    def apply_free_surface_bc(self, field):
        return self._field("st_terrain_apply_free_surface_bc", field)

    def apply_seafloor_bc(self, field):
        return self._field("st_terrain_apply_seafloor_bc", field)

    def apply_absorbing_bc(self, field, sponge_width: int, damping: float):
        return self._field("st_terrain_apply_absorbing_bc", field, int(sponge_width), float(damping))
