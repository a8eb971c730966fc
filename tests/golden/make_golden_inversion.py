"""Generates tests/golden/inversion_small.npz by running the reference's own
Python inversion driver, AdjointStateInversion.run
(seismic_tomography/inversion.py:118-274), for a few iterations on a small
model, with the reference's own synthetic OBS data
(OBSDataCoordinator.generate_synthetic_data, obs_data.py:155-182) and the
gradient model's velocities (VelocityModel.initialize_gradient_model,
model.py:46-64).

    python tests/golden/make_golden_inversion.py

The driver's compiled-engine calls (check_field_health, repair_field_nan,
SparseOps.smooth_gradient; inversion.py:10-18, gradient.py:5-9) are served
by the oracle's C restatements (pinned to the reference's C++ where it
compiles), so the driver takes its with-engine path, the path the GPU
driver replaces; HDF5 output goes to a stub writer. Recorded per iteration:
misfit, step length and the velocity model; then the final model and the
driver's result dict.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE = os.environ.get("SEISMIC_REFERENCE_DIR", "/root/reference")
PKG = os.path.join(REFERENCE, "src", "python", "seismic_tomography")
sys.path.insert(0, os.path.join(REPO, "oracle"))

from oracle import Oracle  # noqa: E402


def oracle_engine():
    """A stand-in `seismic_engine` module backed by the oracle."""
    orc = Oracle()
    eng = types.ModuleType("seismic_engine")

    def check_field_health(data):
        return orc.count_nan_inf(np.ascontiguousarray(data, np.float64))

    def repair_field_nan(data, nx, ny, nz, halo_width=1, replace_value=0.0):
        data[:] = orc.repair_field_nan(data, nx, ny, nz, halo_width, replace_value)

    def clamp_field_safe(data, lo, hi):
        data[:] = orc.clamp_field(data, lo, hi)

    class SparseOps:
        @staticmethod
        def smooth_gradient(g, nx, ny, nz, sigma):
            return orc.smooth_gradient(g, nx, ny, nz, sigma)

    class CSRMatrix:  # not used by the driver's loop
        pass

    def compute_fd_stencil(*args, **kw):
        raise NotImplementedError

    eng.check_field_health = check_field_health
    eng.repair_field_nan = repair_field_nan
    eng.clamp_field_safe = clamp_field_safe
    eng.SparseOps = SparseOps
    eng.CSRMatrix = CSRMatrix
    eng.compute_fd_stencil = compute_fd_stencil
    eng.StepResult = object
    eng.HealthStatus = object
    return eng


class NullWriter:
    """InversionHDF5Writer's interface (hdf5_writer.py:13-140), writing nothing."""

    def __getattr__(self, name):
        return lambda *a, **k: None


def load_reference():
    if not os.path.isdir(PKG):
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    sys.modules["seismic_engine"] = oracle_engine()
    pkg = types.ModuleType("stref")
    pkg.__path__ = [PKG]
    sys.modules["stref"] = pkg
    stub = types.ModuleType("stref.hdf5_writer")
    stub.InversionHDF5Writer = NullWriter
    sys.modules["stref.hdf5_writer"] = stub
    return (importlib.import_module("stref.inversion"), importlib.import_module("stref.model"),
            importlib.import_module("stref.obs_data"))


def main():
    inv_mod, model_mod, obs_mod = load_reference()
    nx, ny, nz, d = 24, 20, 16, 2000.0
    m = model_mod.VelocityModel(nx, ny, nz, d, d, d)
    # initialize_gradient_model's vp (model.py:46-64; the method itself fails on
    # its vs line, min() of an array): water above 4000 m, then 3000 (1 + 0.3 depth / 5000)
    z = np.arange(nz) * d
    col = np.where(z < 4000.0, 1500.0, np.minimum(3000.0 * (1.0 + 0.3 * (z - 4000.0) / 5000.0), m.vp_max))
    m.vp[:] = col[None, None, :]
    obs = obs_mod.OBSDataCoordinator()
    obs.generate_synthetic_data(n_sources=6, n_stations=10, domain_size=(nx * d, ny * d, nz * d))
    vp0 = m.vp.copy()
    src = np.array([[obs.sources[p.source_id].x, obs.sources[p.source_id].y, obs.sources[p.source_id].z]
                    for p in obs.picks])
    sta = np.array([[obs.stations[p.station_id].x, obs.stations[p.station_id].y, obs.stations[p.station_id].z]
                    for p in obs.picks])
    tt = np.array([p.travel_time for p in obs.picks])
    w = np.array([p.weight for p in obs.picks])
    steps, models = [], []

    def cb(it, misfit, gradient, step):
        steps.append(step)
        models.append(m.vp.copy())

    inv = inv_mod.AdjointStateInversion(m, obs, NullWriter(), max_iterations=4, step_length=200.0,
                                        smoothing_sigma=1.5, regularization_lambda=1e-4, misfit_type="l2")
    res = inv.run(callback=cb)
    np.savez_compressed(os.path.join(HERE, "inversion_small.npz"),
                        n=np.array([nx, ny, nz]), d=d, vp0=vp0, src_xyz=src, sta_xyz=sta, travel_time=tt,
                        weight=w, misfit=np.array(res["misfit_history"]), steps=np.array(steps),
                        models=np.array(models), final_vp=m.vp, iterations=res["iterations"],
                        converged=res["converged"], max_iterations=4, step_length=200.0, smoothing_sigma=1.5,
                        regularization_lambda=1e-4)
    print(f"inversion_small.npz: {len(obs.picks)} picks, misfit {res['misfit_history']}, steps {steps}")


if __name__ == "__main__":
    main()
