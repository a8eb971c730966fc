"""The header-only C++ face (include/seismic_gb300.hpp): compiles and links
against the library on CPU; on the GPU its figures equal those of the same
calls through the Python face (same library), and its CG solves."""
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "03-seismic-tomography-compute_gb300")
OUT = os.path.join(REPO, "tests", "_build")


def build_demo():
    import importlib.util
    spec = importlib.util.spec_from_file_location("st_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    lib = mod.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "face_demo")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(REPO, "include"),
           os.path.join(REPO, "tests", "cpp", "face_demo.cpp"), "-L", libdir, "-lseismic_gb300",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_face_compiles_and_links():
    assert os.path.exists(build_demo())


@pytest.mark.gpu
def test_cpp_face_matches_python_face(tmp_path):
    import seismic_engine as se
    exe = build_demo()
    ring = str(tmp_path / "ring.dat")
    r = subprocess.run([exe, "", ring], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = {}
    for line in r.stdout.splitlines():
        k, *v = line.split()
        vals[k] = [float(t) for t in v]
    s = se.WaveEquationSolver(se.GridParams(20, 18, 22, 10.0, 10.0, 10.0),
                              se.SolverConfig(dt=0.001, sponge_width=4, sponge_damping=0.015))
    s.initialize_velocity(2500.0)
    for t in range(30):
        s.inject_source(10, 9, 5, [np.sin(0.3 * t)])
        s.step_forward(t)
    e = s.compute_energy()
    assert vals["energy"][0] == pytest.approx(e, rel=1e-12)
    assert vals["energy"][1] == pytest.approx(e, rel=1e-6)
    assert vals["cfl"][0] == 1 and vals["mpi"][0] == 2.0
    f = s.field()
    eng = se.RTMEngine(20, 18, 22, 10.0, 10.0, 10.0, 1)
    eng.apply_image_condition(f.current, f.previous, 20, 24, 0)
    eng.finalize_image()
    assert vals["image"][0] == pytest.approx(float(eng.result().image.sum()), rel=1e-12)
    assert vals["cg_rel"][0] < 1e-5
    assert vals["nnz"][0] > 0 and vals["nnz"][1] == 512
    # terrain through the C++ class vs the Python class
    g = se.GridParams(20, 18, 22, 10.0, 10.0, 10.0)
    t = se.TerrainBoundary(g, 50.0)
    t.set_bathymetry_data([(15.0, 15.0, 120.0), (105.0, 95.0, 30.0)])
    tv = t.update_velocity_mask(np.zeros(t.padded_size), 1500.0, 3000.0)
    tf = t.apply_seafloor_bc(np.ones(t.padded_size))
    assert vals["terrain"][:2] == [t.seafloor_index(1, 1), t.seafloor_index(10, 9)] == [12.0, 3.0]
    # (sums over the padded arrays: C++ adds in index order, numpy pairwise)
    assert vals["terrain"][2] == pytest.approx(float(tv.sum()), rel=1e-12)
    assert vals["terrain"][3] == pytest.approx(float(tf.sum()), rel=1e-12)
    # the ring file: two frames written, frame 1 read back (500 bytes)
    assert vals["ring"] == [1.0, 2.0, 1.0, 500.0]
    assert se.MmapSnapshotWriter.read_frame(ring, 0) == bytes([7]) * 300
    # the RTM driver, sponge, fault-tolerance and adjoint_propagate methods of the C++ class
    s2 = se.WaveEquationSolver(se.GridParams(20, 18, 22, 10.0, 10.0, 10.0),
                               se.SolverConfig(dt=0.001, nt=24, sponge_width=4, sponge_damping=0.015))
    s2.initialize_velocity(2500.0)
    off = s2.run_rtm([1.0], [])
    rec = se.workloads.ReceiverGrid(0, 2, 10, 0, 2, 9, 0)
    s2.configure_rtm(se.RTMConfig(enable_rtm=True, receivers=rec, snap_kind=se._lib.ST_SNAP_FP32))
    wav = np.sin(0.4 * np.arange(24))
    res = 1e-3 * np.cos(0.1 * np.arange(24 * 90))
    pr = s2.run_rtm(wav, res)
    rimg = float(np.sum(s2.rtm_engine().result().image))
    assert vals["run_rtm"][:3] == [1.0, 0.0, 24.0] and off.completed_successfully and pr.timesteps_completed == 24
    assert vals["run_rtm"][3] == pytest.approx(rimg, rel=1e-12)
    s2.reset_field()
    s2.rtm_engine().reset_image()
    for t in range(10):
        s2.inject_source(10, 9, 11, [wav[t]])
        s2.step_forward(t)
        if t == 4:
            s2.store_forward_wavefield_for_rtm(t)
        s2.apply_rtm_step(t, t % 3 == 0)
    s2.apply_sponge_layer()
    s2.rtm_engine().finalize_image()
    bimg = float(np.sum(s2.rtm_engine().result().image))
    assert vals["blocks"][0] == pytest.approx(bimg, rel=1e-12)
    assert vals["blocks"][1] == pytest.approx(s2.compute_energy(), rel=1e-12)
    assert vals["blocks"][2:] == [12.0, 0.0] == [s2.snapshots_captured(), s2.snapshots_dropped()]
    assert vals["fault"] == [0.99, 3.0, 0.0]
    ap = s2.adjoint_propagate([0.5, -0.25, 0.125])
    assert vals["adjoint"][:2] == [0.0, 24.0] and ap.timesteps_completed == 24
    assert vals["adjoint"][2] == pytest.approx(s2.compute_energy(), rel=1e-12)
