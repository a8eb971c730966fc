"""TerrainBoundary on the host: the oracle's numpy restatement
(oracle/terrain_ref.py) against the reference's own outputs
(tests/golden/terrain_small.npz, made by tests/golden/make_golden_terrain.py
from the reference built in place), and the library's host-only
generate_bathymetry against the reference's synthetic bathymetry.

Exact except the sponge factor of apply_absorbing_bc: the reference is built
with -ffast-math, which re-rounds that expression (observed 1 unit in the
last place); it is compared at rtol 1e-15."""
import os
import sys

import numpy as np
import pytest

CASES = [("points", 300.0, False), ("synthetic", 320.0, True)]


@pytest.fixture(scope="module")
def gold(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "terrain_small.npz")))


def restated(gold, case, wd, synth):
    from terrain_ref import Terrain
    t = Terrain(gold["n"], gold["d"], gold["origin"], wd)
    if synth:
        t.generate_synthetic_bathymetry(0.05, 100.0)
    else:
        t.set_bathymetry_data(gold["points"])
    return t


@pytest.mark.parametrize("case,wd,synth", CASES)
def test_restatement_matches_reference(gold, case, wd, synth):
    t = restated(gold, case, wd, synth)
    f = gold["fields"]
    assert np.array_equal(t.bathy, gold[f"{case}_bathy"])
    assert np.array_equal(t.seafloor_index(), gold[f"{case}_sf_index"])
    assert np.array_equal(t.update_velocity_mask(gold["vel0"], 1500.0, 3000.0), gold[f"{case}_velocity"])
    assert np.array_equal(t.build_boundary_mask(), gold[f"{case}_mask"])
    assert np.array_equal(t.apply_free_surface_bc(f[0]), gold[f"{case}_free"])
    assert np.array_equal(t.apply_seafloor_bc(f[1]), gold[f"{case}_seafloor"])
    np.testing.assert_allclose(t.apply_absorbing_bc(f[2], 3, 0.4), gold[f"{case}_absorbing"], rtol=1e-15, atol=0)


def test_fixture_exercises_the_seafloor_overrun(gold):
    """Columns whose seafloor lies below the grid: the reference's
    apply_seafloor_bc zeroes on into the next cells of the array."""
    nz = int(gold["n"][2])
    assert gold["points_sf_index"].max() > nz + 2


def test_generate_bathymetry_host(gold):
    import importlib.util
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(repo, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import seismic_engine as se
    nx, ny, _ = (int(v) for v in gold["n"])
    dx, dy, _ = gold["d"]
    b = se.generate_bathymetry(nx, ny, dx, dy, 0.0, 0.0, 320.0, 0.05, 100.0)
    assert b.shape == (nx, ny)
    np.testing.assert_allclose(b.reshape(-1), gold["synthetic_bathy"], rtol=1e-14, atol=0)
