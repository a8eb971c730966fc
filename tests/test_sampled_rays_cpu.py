"""The oracle's restatement of the reference's midpoint-sampled straight-ray
forward model and gradient (seismic_tomography/inversion.py:329-433) against
the reference's own outputs (tests/golden/rays_*.npz, made by
tests/golden/make_golden_rays.py from the reference's Python driver).

Bit-exact given the reference's per-pick distances; with distances formed as
x * x the traveltimes may move by a few units in the last place (the
reference squares with libm pow), which is the whole difference."""
import os

import numpy as np
import pytest


def load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name)))


def args(z):
    return z["n"], z["d"], z["origin"], z["src_xyz"], z["sta_xyz"], z["valid"]


@pytest.mark.parametrize("name", ["rays_small.npz", "rays_medium.npz"])
def test_oracle_bit_exact_with_reference_distances(oracle, golden_dir, name):
    z = load(golden_dir, name)
    t = oracle.sampled_traveltimes(*args(z), z["vp"], dist=z["dist"])
    g = oracle.sampled_gradient(*args(z), z["weight"], z["vp"], z["residuals"], dist=z["dist"])
    assert np.array_equal(t, z["times"])
    assert np.array_equal(g, z["gradient"])


@pytest.mark.parametrize("name", ["rays_small.npz", "rays_medium.npz"])
def test_oracle_with_own_distances_within_ulps(oracle, golden_dir, name):
    z = load(golden_dir, name)
    t = oracle.sampled_traveltimes(*args(z), z["vp"])
    g = oracle.sampled_gradient(*args(z), z["weight"], z["vp"], z["residuals"])
    np.testing.assert_allclose(t, z["times"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(g, z["gradient"], rtol=1e-15, atol=1e-30)


def test_fixture_guards_present(golden_dir):
    """The small fixture holds the cases the reference guards against."""
    z = load(golden_dir, "rays_small.npz")
    vp = z["vp"]
    assert np.isnan(vp).any() and np.isinf(vp).any() and (vp == 0).any() and (vp < 0).any()
    assert (z["valid"] == 0).sum() == 2 and np.all(z["times"][z["valid"] == 0] == 0.0)
    assert np.isnan(z["residuals"]).any() and np.isinf(z["residuals"]).any()
    assert (z["dist"][z["valid"] == 1] == 0.0).any()  # a coincident source and station


def test_sample_cells_follow_the_reference_rule(oracle):
    """Straight-line cell sequence: a ray along x from cell 0 to cell 9 with
    n = max(int(dist / (5 dx)), 2) samples visits int((k + 0.5) / n * 9)."""
    n = np.array([10, 4, 4])
    d = np.array([10.0, 10.0, 10.0])
    o = np.zeros(3)
    src = np.array([[5.0, 15.0, 15.0]])
    sta = np.array([[95.0, 15.0, 15.0]])
    vp = np.arange(1, 161, dtype=np.float64).reshape(10, 4, 4) * 100.0
    t = oracle.sampled_traveltimes(n, d, o, src, sta, None, vp)
    steps = max(int(90.0 / 50.0), 2)
    cells = [int(0 + (k + 0.5) / steps * 9) for k in range(steps)]
    expect = sum((90.0 / steps) / vp[c, 1, 1] for c in cells)
    assert t[0] == expect
