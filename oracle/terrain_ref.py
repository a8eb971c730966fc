"""CPU restatement of the reference's TerrainBoundary (solver/boundary.cpp)
in numpy FP64 (TEST INFRASTRUCTURE ONLY: the product never imports this
file). Arrays use the reference's halo-padded layout, x slowest.

Pinned against the reference built in place (tests/golden/terrain_small.npz,
made by tests/golden/make_golden_terrain.py). The reference is compiled with
-ffast-math, so its FP64 formulas (synthetic bathymetry, velocity gradient,
sponge factor) may differ from these IEEE evaluations in the last bits."""
from __future__ import annotations

import math

import numpy as np


class Terrain:
    def __init__(self, n, d, origin, water_depth, hw=1):
        self.nx, self.ny, self.nz = (int(v) for v in n)
        self.dx, self.dy, self.dz = (float(v) for v in d)
        self.ox, self.oy, self.oz = (float(v) for v in origin)
        self.hw = hw
        self.water_depth = float(water_depth)
        self.bathy = np.full(self.nx * self.ny, self.water_depth)  # boundary.cpp:8-14

    def set_bathymetry_data(self, points):  # :16-32
        for x, y, dep in points:
            ix = int((x - self.ox) / self.dx)
            iy = int((y - self.oy) / self.dy)
            if 0 <= ix < self.nx and 0 <= iy < self.ny:
                self.bathy[ix * self.ny + iy] = dep

    def generate_synthetic_bathymetry(self, gradient, roughness):  # :34-57
        for ix in range(self.nx):
            for iy in range(self.ny):
                x, y = ix * self.dx, iy * self.dy
                d = (self.water_depth + gradient * x
                     + roughness * math.sin(2.0 * math.pi * x / 5000.0) * math.cos(2.0 * math.pi * y / 7000.0)
                     + roughness * 0.5 * math.sin(4.0 * math.pi * x / 3000.0))
                self.bathy[ix * self.ny + iy] = min(max(d, 500.0), 8000.0)

    def seafloor_index(self):  # :71-86, per column
        return np.array([int(v / self.dz) for v in self.bathy], np.int64)

    def _pad(self):
        h = self.hw
        return self.nx + 2 * h, self.ny + 2 * h, self.nz + 2 * h

    def update_velocity_mask(self, vel, water_vp, sediment_vp):  # :158-186
        v = np.array(vel, np.float64, copy=True).reshape(self._pad())
        sfi = self.seafloor_index().reshape(self.nx, self.ny)
        h = self.hw
        iz = np.arange(self.nz)
        for ix in range(self.nx):
            for iy in range(self.ny):
                s = sfi[ix, iy]
                col = np.where(iz < s, water_vp,
                               np.minimum(sediment_vp * (1.0 + 0.3 * ((iz - s) * self.dz / 5000.0)), 8500.0))
                v[ix + h, iy + h, h:h + self.nz] = col
        return v.reshape(-1)

    def build_boundary_mask(self):  # :188-214
        m = np.zeros(self._pad(), np.uint8)
        h = self.hw
        z = self.oz + np.arange(self.nz) * self.dz
        b = self.bathy.reshape(self.nx, self.ny)
        m[h:h + self.nx, h:h + self.ny, h:h + self.nz] = np.where(z[None, None, :] >= b[:, :, None], 1, 2)
        return m.reshape(-1)

    def apply_free_surface_bc(self, f):  # :88-100
        g = np.array(f, np.float64, copy=True).reshape(self._pad())
        h = self.hw
        g[h:h + self.nx, h:h + self.ny, h] = 0.0
        return g.reshape(-1)

    def apply_seafloor_bc(self, f):  # :102-124 (flat index ranges, as the reference writes them)
        g = np.array(f, np.float64, copy=True).reshape(-1)
        NX, NY, NZ = self._pad()
        h = self.hw
        sfi = self.seafloor_index().reshape(self.nx, self.ny)
        for ix in range(self.nx):
            for iy in range(self.ny):
                base = ((ix + h) * NY + (iy + h)) * NZ + h
                g[base:min(base + max(sfi[ix, iy], 0), g.size)] = 0.0
        return g

    def apply_absorbing_bc(self, f, sw, damping):  # :126-156
        g = np.array(f, np.float64, copy=True).reshape(self._pad())
        h = self.hw
        ix, iy, iz = np.meshgrid(np.arange(self.nx), np.arange(self.ny), np.arange(self.nz), indexing="ij")
        d = np.minimum.reduce([iz, self.nz - 1 - iz, ix, self.nx - 1 - ix, iy, self.ny - 1 - iy]).astype(np.float64)
        fac = np.where((d < sw) & (d >= 0), 1.0 - damping * (sw - d) * (sw - d) / float(sw * sw), 1.0)
        inner = g[h:h + self.nx, h:h + self.ny, h:h + self.nz]
        g[h:h + self.nx, h:h + self.ny, h:h + self.nz] = np.where(fac != 1.0, inner * fac, inner)
        return g.reshape(-1)
