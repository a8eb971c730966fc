"""Generates tests/golden/rays_small.npz by running the reference's own Python
inversion driver (src/python/seismic_tomography of
13262233692/03-seismic-tomography-compute): AdjointStateInversion's
straight-ray traveltime forward model and its gradient
(seismic_tomography/inversion.py:329-433) on a small seeded model.

    python tests/golden/make_golden_rays.py

Fixtures: rays_small.npz (the guard case below) and rays_medium.npz (300
picks between 12 sources and 25 stations over a 40 x 32 x 24 model).

The reference package is loaded module by module from its source directory
(its __init__ pulls in the HTTP server and the visualisation client, and
hdf5_writer needs h5py, none of which these two functions use): hdf5_writer
is replaced by a stub module and `seismic_engine` is made unimportable, so
the pure-numpy paths the reference takes without its compiled engine run.

The case exercises every guard of the two functions: invalid velocities
(NaN, +inf, zero, negative) that the forward model replaces by 1500 and the
gradient skips, a residual that is NaN and one that is infinite (skipped),
picks whose source or station id is unknown (time 0, no gradient), a source
outside the grid (cell indices clamped), a source-station pair at one point
(distance 0: two samples of length 0), anisotropic spacing and a non-zero
origin.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("SEISMIC_REFERENCE_DIR", "/root/reference")
PKG = os.path.join(REFERENCE, "src", "python", "seismic_tomography")


def load_reference():
    if not os.path.isdir(PKG):
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    sys.modules["seismic_engine"] = None  # the reference's optional compiled engine: absent
    pkg = types.ModuleType("stref")
    pkg.__path__ = [PKG]
    sys.modules["stref"] = pkg
    stub = types.ModuleType("stref.hdf5_writer")
    stub.InversionHDF5Writer = object
    sys.modules["stref.hdf5_writer"] = stub
    return (importlib.import_module("stref.inversion"), importlib.import_module("stref.model"),
            importlib.import_module("stref.obs_data"))


def make_case(model_mod, obs_mod):
    rng = np.random.default_rng(2024)
    nx, ny, nz = 12, 10, 14
    dx, dy, dz = 250.0, 200.0, 150.0
    ox, oy, oz = -500.0, 300.0, 0.0
    m = model_mod.VelocityModel(nx, ny, nz, dx, dy, dz, ox, oy, oz)
    vp = rng.uniform(1500.0, 6000.0, (nx, ny, nz))
    vp[1, 2, 3] = np.nan
    vp[5, 5, 7] = np.inf
    vp[6, 4, 6] = 0.0
    vp[7, 5, 8] = -2000.0
    vp[3, 3, 3] = np.nan
    m.vp = vp
    obs = obs_mod.OBSDataCoordinator()
    ext = np.array([nx * dx, ny * dy, nz * dz])
    org = np.array([ox, oy, oz])
    srcs = [org + rng.uniform(0.05, 0.95, 3) * ext for _ in range(4)]
    srcs.append(org + np.array([-0.3, 0.5, 1.2]) * ext)       # outside the grid: clamped cells
    stas = [org + rng.uniform(0.0, 1.0, 3) * ext for _ in range(6)]
    stas.append(srcs[1].copy())                                # coincident with source 1
    for i, p in enumerate(srcs):
        obs.add_source(f"S{i}", *p)
    for i, p in enumerate(stas):
        obs.add_station(f"R{i}", *p)
    for si in range(len(srcs)):
        for ri in range(len(stas)):
            obs.add_pick(f"R{ri}", f"S{si}", "P", float(rng.uniform(0.5, 3.0)),
                         weight=float(rng.uniform(0.5, 1.5)))
    obs.add_pick("R_missing", "S0", "P", 1.0, weight=1.0)      # unknown station
    obs.add_pick("R2", "S_missing", "P", 1.0, weight=1.0)      # unknown source
    # a pick whose ray runs through the invalid cells
    obs.add_source("S_bad", ox + 1.5 * dx, oy + 2.5 * dy, oz + 3.5 * dz)
    obs.add_station("R_bad", ox + 7.5 * dx, oy + 5.5 * dy, oz + 8.5 * dz)
    obs.add_pick("R_bad", "S_bad", "P", 2.0, weight=0.75)
    return m, obs, srcs, stas


def make_medium(model_mod, obs_mod):
    rng = np.random.default_rng(31)
    nx, ny, nz = 40, 32, 24
    m = model_mod.VelocityModel(nx, ny, nz, 100.0, 100.0, 100.0)
    m.vp = rng.integers(1500, 6000, (nx, ny, nz)).astype(np.float64)  # whole m/s: compresses well
    obs = obs_mod.OBSDataCoordinator()
    ext = np.array([nx * 100.0, ny * 100.0, nz * 100.0])
    for i in range(12):
        obs.add_source(f"S{i}", *(rng.uniform(0.0, 1.0, 3) * ext))
    for i in range(25):
        obs.add_station(f"R{i}", *(rng.uniform(0.0, 1.0, 2) * ext[:2]), 50.0)
    for si in range(12):
        for ri in range(25):
            obs.add_pick(f"R{ri}", f"S{si}", "P", float(rng.uniform(0.5, 3.0)),
                         weight=float(rng.uniform(0.5, 1.5)))
    return m, obs


def run_case(inv_mod, m, obs, name, bad_residuals):
    inv = inv_mod.AdjointStateInversion(m, obs, hdf5_writer=None)
    times = inv._forward_model()
    rng = np.random.default_rng(77)
    resid = rng.standard_normal(len(obs.picks))
    if bad_residuals:
        resid[3] = np.nan
        resid[10] = np.inf
    grad = inv._compute_gradient(resid)

    src_xyz = np.zeros((len(obs.picks), 3))
    sta_xyz = np.zeros((len(obs.picks), 3))
    valid = np.zeros(len(obs.picks), np.uint8)
    weight = np.zeros(len(obs.picks))
    dist = np.zeros(len(obs.picks))
    for i, p in enumerate(obs.picks):
        s = obs.sources.get(p.source_id)
        r = obs.stations.get(p.station_id)
        weight[i] = p.weight
        if s is None or r is None:
            continue
        valid[i] = 1
        src_xyz[i] = (s.x, s.y, s.z)
        sta_xyz[i] = (r.x, r.y, r.z)
        # the distance exactly as inversion.py:339-341 forms it (x ** 2 on scalars)
        dist[i] = np.sqrt((s.x - r.x)**2 + (s.y - r.y)**2 + (s.z - r.z)**2)
    np.savez_compressed(os.path.join(HERE, name),
                        n=np.array([m.nx, m.ny, m.nz]), d=np.array([m.dx, m.dy, m.dz]),
                        origin=np.array([m.origin_x, m.origin_y, m.origin_z]), vp=m.vp,
                        src_xyz=src_xyz, sta_xyz=sta_xyz, dist=dist, valid=valid, weight=weight,
                        residuals=resid, times=times, gradient=grad)
    print(f"{name}: {len(obs.picks)} picks, {int(valid.sum())} valid, "
          f"{int(np.count_nonzero(grad))} cells with gradient")


def main():
    inv_mod, model_mod, obs_mod = load_reference()
    m, obs, _, _ = make_case(model_mod, obs_mod)
    run_case(inv_mod, m, obs, "rays_small.npz", True)
    m, obs = make_medium(model_mod, obs_mod)
    run_case(inv_mod, m, obs, "rays_medium.npz", False)


if __name__ == "__main__":
    main()
