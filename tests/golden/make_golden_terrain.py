"""Generates tests/golden/terrain_small.npz with the reference's own
TerrainBoundary (solver/boundary.cpp, compiled in place into
oracle/_ref/libseismic_ref.so by oracle/build_ref.sh) on a single-rank grid
with a one-cell halo:

  case "points": bathymetry from set_bathymetry_data (seeded depths, some
    deeper than the grid so apply_seafloor_bc runs past its column), then
    seafloor_index, update_velocity_mask, build_boundary_mask and the three
    boundary conditions on seeded fields;
  case "synthetic": generate_synthetic_bathymetry(gradient, roughness) and
    the same chain (the reference is built with -ffast-math, so its sines
    may differ from a plain build in the last bits: compare with tolerance).

    python tests/golden/make_golden_terrain.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from oracle import Reference, build_ref  # noqa: E402


def main():
    if build_ref() is None:
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    ref = Reference()
    rng = np.random.default_rng(88)
    n = np.array([10, 8, 12])
    d = np.array([100.0, 120.0, 50.0])
    origin = np.array([0.0, 0.0, 0.0])
    nx, ny, nz = (int(v) for v in n)
    npad = (nx + 2) * (ny + 2) * (nz + 2)
    fields = [rng.standard_normal(npad) for _ in range(3)]
    vel0 = rng.uniform(1500, 4000, npad)
    out = {"n": n, "d": d, "origin": origin, "fields": np.stack(fields), "vel0": vel0}
    # points: depths on cell-centred columns, a few below the grid bottom (nz * dz = 600 m)
    pts = []
    for ix in range(nx):
        for iy in range(ny):
            if rng.uniform() < 0.8:
                pts.append((ix * d[0] + 30.0, iy * d[1] + 40.0, float(rng.choice([rng.uniform(0, 550),
                                                                                   rng.uniform(600, 900)]))))
    pts = np.array(pts)
    r = ref.terrain(n, d, origin, 300.0, points=pts, velocity=vel0, fields=fields, sponge_width=3, damping=0.4)
    out.update({"points": pts, **{f"points_{k}": v for k, v in r.items()}})
    r = ref.terrain(n, d, origin, 320.0, synthetic=True, gradient=0.05, roughness=100.0, velocity=vel0,
                    fields=fields, sponge_width=3, damping=0.4)
    out.update({f"synthetic_{k}": v for k, v in r.items()})
    np.savez_compressed(os.path.join(HERE, "terrain_small.npz"), **out)
    print(f"terrain_small.npz: {len(pts)} bathymetry points; seafloor indices "
          f"{out['points_sf_index'].min()}..{out['points_sf_index'].max()} (nz = {nz})")


if __name__ == "__main__":
    main()
