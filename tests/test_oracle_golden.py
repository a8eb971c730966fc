"""The CPU oracle against the reference's own outputs (tests/golden/*.npz,
generated by tests/golden/make_golden.py from the reference C++). FP64
comparisons allow a few ulps: the reference is built with -ffast-math."""
import os

import numpy as np
import pytest


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def test_propagator_stepping_matches_reference(oracle, golden_dir):
    g = load(golden_dir, "prop_small.npz")
    nx, ny, nz = (int(v) for v in g["n"])
    grid = oracle.grid(nx, ny, nz, float(g["d"]), float(g["d"]), float(g["d"]), float(g["dt"]),
                       int(g["sw"]), float(g["damp"]))
    nt = g["seis"].shape[0]
    r = oracle.run(grid, g["vel"], nt, g["src"], g["wavelet"][:, None], g["rec"])
    scale = np.abs(g["seis"]).max()
    assert np.abs(r["seis"] - g["seis"]).max() <= 1e-12 * scale
    assert np.abs(r["cur"] - g["cur"]).max() <= 1e-12 * np.abs(g["cur"]).max()
    assert np.abs(r["prev"] - g["prev"]).max() <= 1e-12 * np.abs(g["prev"]).max()
    assert np.array_equal(r["status"], g["status"])


def test_reference_adjoint_stepping_matches_reference(oracle, golden_dir):
    # the reference's step_adjoint is the forward operator; sources at receivers
    g = load(golden_dir, "prop_small.npz")
    nx, ny, nz = (int(v) for v in g["n"])
    grid = oracle.grid(nx, ny, nz, float(g["d"]), float(g["d"]), float(g["d"]), float(g["dt"]),
                       int(g["sw"]), float(g["damp"]))
    nt = g["adj_seis"].shape[0]
    r = oracle.run(grid, g["vel"], nt, g["rec"], g["adj_resid"], g["src"])
    assert np.abs(r["seis"] - g["adj_seis"]).max() <= 1e-12 * np.abs(g["adj_seis"]).max()
    assert np.abs(r["cur"] - g["adj_cur"]).max() <= 1e-12 * np.abs(g["adj_cur"]).max()
    assert np.array_equal(r["status"], g["adj_status"])


def test_forward_propagate_snapshots_match_reference(oracle, golden_dir):
    g = load(golden_dir, "fwdprop_small.npz")
    p = load(golden_dir, "prop_small.npz")
    nx, ny, nz = (int(v) for v in p["n"])
    nt, si = int(g["nt"]), int(g["snap_interval"])
    assert int(g["status"]) == 0 and int(g["steps"]) == nt and bool(g["ok"])
    assert int(g["cfl_bad_status"]) == 2 and int(g["cfl_bad_steps"]) == 0
    grid = oracle.grid(nx, ny, nz, float(p["d"]), float(p["d"]), float(p["d"]), float(g["dt"]),
                       int(p["sw"]), float(p["damp"]))
    centre = np.array([[nx // 2, ny // 2, nz // 2]])
    w = p["wavelet"][:nt, None]
    snaps = []
    for t in range(0, nt, si):
        r = oracle.run(grid, p["vel"], t + 1, centre, w[:t + 1], np.zeros((0, 3)))
        snaps.append(r["cur"].reshape(nx + 2, ny + 2, nz + 2)[1:-1, 1:-1, 1:-1].ravel())
    snaps = np.concatenate(snaps)
    assert snaps.shape == g["snapshots"].shape
    assert np.abs(snaps - g["snapshots"]).max() <= 1e-12 * np.abs(g["snapshots"]).max()
    r = oracle.run(grid, p["vel"], nt, centre, w, np.zeros((0, 3)))
    assert np.abs(r["cur"] - g["cur"]).max() <= 1e-12 * np.abs(g["cur"]).max()


def test_rtm_imaging_matches_reference(oracle, golden_dir):
    g = load(golden_dir, "rtm_small.npz")
    nx, ny, nz = (int(v) for v in g["n"])
    img, ill, refl = oracle.rtm_image(nx, ny, nz, g["fwd"], g["adj"])
    np.testing.assert_allclose(img, g["image"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(ill, g["illum"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(refl, g["refl"], rtol=1e-12, atol=1e-12)


def test_csr_build_bit_exact_against_reference(oracle, golden_dir):
    g = load(golden_dir, "csr_small.npz")
    rp, col, val = oracle.csr_build(int(g["rows"]), int(g["cols"]), g["r"], g["c"], g["v"])
    assert np.array_equal(rp, g["row_ptr"])
    assert np.array_equal(col, g["col"])
    assert np.array_equal(val, g["val"])  # dyadic duplicates: sums are exact
    m = oracle.csr(int(g["rows"]), int(g["cols"]), rp, col, val)
    y = oracle.spmv(m, g["x"])
    np.testing.assert_allclose(y, g["y"], rtol=1e-14, atol=1e-13)


def test_fault_helpers_match_reference(oracle, golden_dir):
    g = load(golden_dir, "fault_small.npz")
    nx, ny, nz = (int(v) for v in g["n"])
    rep = oracle.repair_field_nan(g["field"], nx + 2, ny + 2, nz + 2, 1, 0.0)
    np.testing.assert_allclose(rep, g["repaired"], rtol=1e-15, atol=0)
    np.testing.assert_array_equal(oracle.clamp_field(g["field"], -500.0, 500.0), g["clamped"])
    assert oracle.count_nan_inf(g["field"]) == int(g["nan_count"])


def test_config_reader_matches_reference(golden_dir, tmp_path):
    from seismic_engine.config import load_config, config_vector
    g = load(golden_dir, "config_small.npz")
    p1 = tmp_path / "default.yaml"
    p1.write_text(str(g["default_yaml"]))
    p2 = tmp_path / "edited.yaml"
    p2.write_text(str(g["edited_yaml"]))
    np.testing.assert_array_equal(config_vector(load_config(str(p1))), g["default"])
    np.testing.assert_array_equal(config_vector(load_config(str(p2))), g["edited"])
    np.testing.assert_array_equal(config_vector(load_config(str(tmp_path / "missing.yaml"))), g["missing"])
