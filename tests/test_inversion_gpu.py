"""The GPU-resident traveltime inversion driver against the reference's own
AdjointStateInversion.run (tests/golden/inversion_small.npz, made by
tests/golden/make_golden_inversion.py): misfit history, line-search steps
and the model after every iteration. The misfit sums and the smoothing add
in another order than numpy and the reference's loops, so the comparison
is to 1e-12 relative; the step lengths (the line search's decisions) must
be identical."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def se():
    import importlib.util
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(repo, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import seismic_engine
    return seismic_engine


class _Obj:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def reference_objects(z):
    nx, ny, nz = (int(v) for v in z["n"])
    d = float(z["d"])
    model = _Obj(nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, origin_x=0.0, origin_y=0.0, origin_z=0.0,
                 vp=z["vp0"].copy(), vp_min=1450.0, vp_max=8500.0)
    sources, stations, picks = {}, {}, []
    for i in range(z["travel_time"].size):
        sources[f"S{i}"] = _Obj(x=z["src_xyz"][i, 0], y=z["src_xyz"][i, 1], z=z["src_xyz"][i, 2])
        stations[f"R{i}"] = _Obj(x=z["sta_xyz"][i, 0], y=z["sta_xyz"][i, 1], z=z["sta_xyz"][i, 2])
        picks.append(_Obj(source_id=f"S{i}", station_id=f"R{i}", travel_time=float(z["travel_time"][i]),
                          weight=float(z["weight"][i])))
    return model, _Obj(picks=picks, sources=sources, stations=stations)


def test_driver_matches_reference_run(se, golden_dir):
    from seismic_engine.inversion import AdjointStateInversion
    z = dict(np.load(os.path.join(golden_dir, "inversion_small.npz")))
    model, obs = reference_objects(z)
    steps, models = [], []

    def cb(it, misfit, gradient, step):
        steps.append(step)
        models.append(model.vp.copy())

    inv = AdjointStateInversion(model, obs, None, max_iterations=int(z["max_iterations"]),
                                step_length=float(z["step_length"]), smoothing_sigma=float(z["smoothing_sigma"]),
                                regularization_lambda=float(z["regularization_lambda"]), misfit_type="l2")
    res = inv.run(callback=cb)
    assert res["iterations"] == int(z["iterations"]) and res["converged"] == bool(z["converged"])
    np.testing.assert_allclose(res["misfit_history"], z["misfit"], rtol=1e-12, atol=0)
    assert steps == list(z["steps"])
    for got, exp in zip(models, z["models"]):
        np.testing.assert_allclose(got, exp, rtol=1e-12, atol=0)
    np.testing.assert_allclose(model.vp, z["final_vp"], rtol=1e-12, atol=0)
