"""TerrainBoundary on the GPU: every operation against the reference's own
outputs (tests/golden/terrain_small.npz) and against the oracle's
restatement (oracle/terrain_ref.py) on a larger seeded case, on host and
device arrays; terrain-aware propagation (per-column z limits fused into the
stencil) against the FP64 oracle stepped one step at a time with the same
masks; the exact-adjoint paths refusing while a terrain is attached.

Tolerances: exact (bit-identical FP64) except the reference's sponge factor
(built with -ffast-math: rtol 1e-15); propagation FP32 vs FP64 relative L2
<= 1e-4."""
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


@pytest.fixture(scope="module")
def gold(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "terrain_small.npz")))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def terrain(se, n, d, origin, wd, points=None, synthetic=None):
    g = se.GridParams(int(n[0]), int(n[1]), int(n[2]), *(float(v) for v in d), *(float(v) for v in origin))
    t = se.TerrainBoundary(g, wd)
    if synthetic:
        t.generate_synthetic_bathymetry(*synthetic)
    if points is not None:
        t.set_bathymetry_data([tuple(p) for p in points])
    return t


@pytest.mark.parametrize("case,wd,synth", [("points", 300.0, None), ("synthetic", 320.0, (0.05, 100.0))])
@pytest.mark.parametrize("on_device", [False, True])
def test_matches_reference(se, gold, case, wd, synth, on_device):
    import torch
    t = terrain(se, gold["n"], gold["d"], gold["origin"], wd, gold["points"] if case == "points" else None, synth)
    assert np.array_equal(t.bathymetry(), gold[f"{case}_bathy"])
    nx, ny, _ = (int(v) for v in gold["n"])
    assert [t.seafloor_index(ix, iy) for ix in range(nx) for iy in range(ny)] == list(gold[f"{case}_sf_index"])
    assert np.array_equal(t.build_boundary_mask(), gold[f"{case}_mask"])

    def run(fn, arr, *extra):
        if on_device:
            d = torch.from_numpy(np.array(arr, np.float64)).cuda()
            fn(d, *extra)
            return d.cpu().numpy()
        h = np.array(arr, np.float64)
        fn(h, *extra)
        return h
    f = gold["fields"]
    assert np.array_equal(run(t.update_velocity_mask, gold["vel0"], 1500.0, 3000.0), gold[f"{case}_velocity"])
    assert np.array_equal(run(t.apply_free_surface_bc, f[0]), gold[f"{case}_free"])
    assert np.array_equal(run(t.apply_seafloor_bc, f[1]), gold[f"{case}_seafloor"])
    np.testing.assert_allclose(run(t.apply_absorbing_bc, f[2], 3, 0.4), gold[f"{case}_absorbing"], rtol=1e-15, atol=0)
    t.close()


def test_matches_restatement_larger(se):
    from terrain_ref import Terrain
    rng = np.random.default_rng(12)
    n, d, o = (40, 30, 50), (25.0, 30.0, 20.0), (-100.0, 50.0, 0.0)
    pts = np.stack([rng.uniform(-150, 1000, 900), rng.uniform(0, 1000, 900), rng.uniform(0, 1300, 900)], axis=1)
    t = terrain(se, n, d, o, 400.0, pts)
    r = Terrain(n, d, o, 400.0)
    r.set_bathymetry_data(pts)
    assert np.array_equal(t.bathymetry(), r.bathy)
    npad = (n[0] + 2) * (n[1] + 2) * (n[2] + 2)
    f = rng.standard_normal(npad)
    v = rng.uniform(1500, 5000, npad)
    assert np.array_equal(t.update_velocity_mask(v.copy(), 1480.0, 2900.0), r.update_velocity_mask(v, 1480.0, 2900.0))
    assert np.array_equal(t.build_boundary_mask(), r.build_boundary_mask())
    assert np.array_equal(t.apply_free_surface_bc(f.copy()), r.apply_free_surface_bc(f))
    assert np.array_equal(t.apply_seafloor_bc(f.copy()), r.apply_seafloor_bc(f))
    assert np.array_equal(t.apply_absorbing_bc(f.copy(), 5, 0.3), r.apply_absorbing_bc(f, 5, 0.3))


def test_terrain_aware_propagation_matches_masked_oracle(se, oracle):
    import torch
    from terrain_ref import Terrain
    w = se.workloads.small_case(n=(24, 20, 28), nt=60, seed=9, sponge_width=4)
    rng = np.random.default_rng(3)
    pts = [(ix * w.d + 1.0, iy * w.d + 1.0, float(rng.uniform(40.0, 140.0)))
           for ix in range(w.nx) for iy in range(w.ny)]
    grid = se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d)
    t = se.TerrainBoundary(grid, 100.0)
    t.set_bathymetry_data(pts)
    s = se.WaveEquationSolver(grid, se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                                    sponge_damping=w.sponge_damping))
    vel = se.workloads.to_reference_layout(w.vel)
    s.set_velocity_field(vel)
    s.set_terrain(t)
    src = (w.nx // 2, w.ny // 2, 20)
    rec = se.workloads.ReceiverGrid(2, 4, 5, 2, 4, 4, 22)
    seis = torch.zeros((w.nt, rec.count), device="cuda")
    wav = w.shots[0].wavelet
    assert se.shot_forward(s, src, wav, w.nt, rec, seis=seis) == 0
    torch.cuda.synchronize()
    cur = s.get_field(se._lib.ST_FIELD_CURRENT)
    # oracle: one reference step at a time, the same per-column limits after each
    r = Terrain((w.nx, w.ny, w.nz), (w.d,) * 3, (0.0,) * 3, 100.0)
    r.set_bathymetry_data(pts)
    zl = np.minimum(np.maximum(r.seafloor_index(), 1), w.nz).reshape(w.nx, w.ny)
    keep = np.ones((w.nx + 2, w.ny + 2, w.nz + 2), bool)
    for ix in range(w.nx):
        for iy in range(w.ny):
            keep[ix + 1, iy + 1, 1:1 + zl[ix, iy]] = False
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    oc = op = None
    oseis = []
    for step in range(w.nt):
        o = oracle.run(g, vel, 1, np.array([src]), wav[step:step + 1, None], rec.coords(), init_cur=oc, init_prev=op)
        oc = np.where(keep.reshape(-1), o["cur"], 0.0)
        op = o["prev"]
        oseis.append(o["seis"][0])
    assert np.all(cur.reshape(keep.shape)[~keep] == 0.0)
    e_f = rel(cur, oc)
    e_s = rel(seis.cpu().numpy(), np.array(oseis))
    print(f"terrain propagation: field rel L2 {e_f:.2e}, seismograms {e_s:.2e}")
    assert e_f < 1e-4 and e_s < 1e-4
    # the exact adjoint is unavailable while the terrain is attached
    image = torch.zeros(w.points, device="cuda")
    illum = torch.zeros(w.points, device="cuda")
    with pytest.raises(se.SeismicError):
        se.rtm_shot(s, src, wav, w.nt, rec, seis, image, illum)
    s.set_terrain(None)
    assert se.rtm_shot(s, src, wav, w.nt, rec, seis, image, illum) == 0
    s.close()
