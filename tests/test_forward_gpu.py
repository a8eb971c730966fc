"""GPU parity of the propagator (forward and the reference's stepping API)
against the reference fixtures and the FP64 oracle, through the C ABI.

Tolerances (FP32 on the GPU vs FP64): relative L2 <= 2e-5 on the small
fixtures (measured FP32 floor of the same arithmetic on CPU: ~1e-6) and
<= 1e-4 on the 128^3 x 1000-step workload."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_SMALL = 2e-5
REL_FULL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


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
    import torch
    assert torch.cuda.is_available()
    return seismic_engine


def golden(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def make_solver(se, nx, ny, nz, d, dt, sw, damp, nt=100, snap=100):
    return se.WaveEquationSolver(se.GridParams(nx, ny, nz, d, d, d),
                                 se.SolverConfig(dt=dt, nt=nt, sponge_width=sw, sponge_damping=damp,
                                                 snapshot_interval=snap))


def sample(field, rec, n):
    nx, ny, nz = n
    f = field.reshape(nx + 2, ny + 2, nz + 2)
    return f[rec[:, 0] + 1, rec[:, 1] + 1, rec[:, 2] + 1]


def test_step_api_matches_reference_fixture(se, golden_dir):
    g = golden(golden_dir, "prop_small.npz")
    n = tuple(int(v) for v in g["n"])
    s = make_solver(se, *n, float(g["d"]), float(g["dt"]), int(g["sw"]), float(g["damp"]))
    s.set_velocity_field(g["vel"])
    src, rec, w = g["src"][0], g["rec"], g["wavelet"]
    seis = []
    for t in range(g["seis"].shape[0]):
        s.inject_source(*src, [w[t]])
        assert s.step_forward(t) == se.StepResult.OK
        seis.append(sample(s.get_field(0), rec, n))
    seis = np.array(seis)
    assert rel(seis, g["seis"]) < REL_SMALL
    f = s.field()
    assert rel(f.current, g["cur"]) < REL_SMALL
    assert rel(f.previous, g["prev"]) < REL_SMALL
    np.testing.assert_array_equal(f.velocity, g["vel"])


def test_step_adjoint_api_matches_reference_fixture(se, golden_dir):
    g = golden(golden_dir, "prop_small.npz")
    n = tuple(int(v) for v in g["n"])
    s = make_solver(se, *n, float(g["d"]), float(g["dt"]), int(g["sw"]), float(g["damp"]))
    s.set_velocity_field(g["vel"])
    rec, resid, src = g["rec"], g["adj_resid"], g["src"]
    out = []
    for t in range(resid.shape[0]):
        for q in range(rec.shape[0]):
            s.inject_source(*rec[q], [resid[t, q]])
        assert s.step_adjoint(t) == se.StepResult.OK
        out.append(sample(s.get_field(0), src, n))
    assert rel(np.array(out), g["adj_seis"]) < REL_SMALL
    assert rel(s.get_field(0), g["adj_cur"]) < REL_SMALL


def test_forward_propagate_matches_reference_fixture(se, golden_dir):
    p = golden(golden_dir, "prop_small.npz")
    g = golden(golden_dir, "fwdprop_small.npz")
    n = tuple(int(v) for v in p["n"])
    nt, si = int(g["nt"]), int(g["snap_interval"])
    s = make_solver(se, *n, float(p["d"]), float(g["dt"]), int(p["sw"]), float(p["damp"]), nt=nt, snap=si)
    s.set_velocity_field(p["vel"])
    r = s.forward_propagate(p["wavelet"][:nt])
    assert r.status == se.StepResult.OK and r.completed_successfully and r.timesteps_completed == nt
    f = s.field()
    assert f.snapshots.shape == g["snapshots"].shape
    assert rel(f.snapshots, g["snapshots"]) < REL_SMALL
    assert rel(f.current, g["cur"]) < REL_SMALL
    assert rel(f.previous, g["prev"]) < REL_SMALL
    # CFL violation: dt ten times larger, nothing propagated
    s2 = make_solver(se, *n, float(p["d"]), 10 * float(g["dt"]), int(p["sw"]), float(p["damp"]), nt=nt, snap=si)
    s2.set_velocity_field(p["vel"])
    r2 = s2.forward_propagate(p["wavelet"][:nt])
    assert r2.status == se.StepResult.CFL_VIOLATION and r2.timesteps_completed == 0
    assert not s2.verify_cfl() and s.verify_cfl()


@pytest.mark.parametrize("n", [(24, 20, 28), (17, 21, 13), (9, 40, 70), (70, 5, 130)])
def test_fused_shot_matches_oracle(se, oracle, n):
    import torch
    w = se.workloads.small_case(n=n, nt=60, seed=3, sponge_width=4)
    shot = w.shots[0]
    s = make_solver(se, w.nx, w.ny, w.nz, w.d, w.dt, w.sponge_width, w.sponge_damping)
    vel = se.workloads.to_reference_layout(w.vel)
    s.set_velocity_field(vel)
    seis = torch.zeros((w.nt, shot.rec.count), device="cuda")
    rc = se.shot_forward(s, shot.src, shot.wavelet, w.nt, shot.rec, seis=seis)
    torch.cuda.synchronize()
    assert rc == 0
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    ref = oracle.run(g, vel, w.nt, np.array([shot.src]), shot.wavelet[:, None], shot.rec.coords())
    assert rel(seis.cpu().numpy(), ref["seis"]) < REL_SMALL
    # final state: current = U_nt; previous = D * V_{nt-1}
    assert rel(s.get_field(0), ref["cur"]) < REL_SMALL
    assert rel(s.get_field(1), ref["prev"]) < REL_SMALL
    # host-buffer entry point gives the same seismograms
    host = se.shot_forward_host(s, None, shot.src, shot.wavelet, w.nt, shot.rec)
    np.testing.assert_allclose(host, seis.cpu().numpy().astype(np.float64), rtol=0, atol=0)


def test_snapshot_store_quantisation(se, oracle):
    import torch
    w = se.workloads.small_case(n=(20, 16, 24), nt=40, seed=9, sponge_width=4)
    shot = w.shots[0]
    vel = se.workloads.to_reference_layout(w.vel)
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    ref = oracle.run(g, vel, w.nt, np.array([shot.src]), shot.wavelet[:, None], shot.rec.coords(),
                     keep_states=True)
    V = ref["states"].reshape(w.nt, w.nx + 2, w.ny + 2, w.nz + 2)[:, 1:-1, 1:-1, 1:-1]
    s = make_solver(se, w.nx, w.ny, w.nz, w.d, w.dt, w.sponge_width, w.sponge_damping)
    s.set_velocity_field(vel)
    npts = w.nx * w.ny * w.nz
    for kind, dtype, tol in ((1, torch.bfloat16, 2.0 ** -8), (2, torch.float16, 2.0 ** -10),
                             (3, torch.float32, 1e-5)):
        snaps = torch.zeros((w.nt, npts), dtype=dtype, device="cuda")
        amax = torch.zeros(w.nt + 1, dtype=torch.int32, device="cuda")
        assert se.shot_forward(s, shot.src, shot.wavelet, w.nt, shot.rec,
                               seis=torch.zeros((w.nt, shot.rec.count), device="cuda"),
                               snap_kind=kind, snaps=snaps, snap_amax=amax) == 0
        torch.cuda.synchronize()
        m = amax.cpu().numpy().view(np.float32).astype(np.float64)
        Vt = V.reshape(w.nt, -1)
        np.testing.assert_allclose(m[:w.nt], np.abs(Vt).max(1), rtol=1e-4)
        deq = snaps.float().cpu().numpy().astype(np.float64) * (m[:w.nt, None] / 16384.0)
        err = np.abs(deq - Vt).max(1) / np.maximum(np.abs(Vt).max(1), 1e-30)
        assert err.max() < tol * 1.01 + 1e-6, (kind, err.max())


def test_nan_guards_match_oracle(se, oracle):
    w = se.workloads.small_case(n=(12, 10, 14), nt=6, seed=4, sponge_width=3)
    vel = se.workloads.to_reference_layout(w.vel)
    s = make_solver(se, w.nx, w.ny, w.nz, w.d, w.dt, w.sponge_width, w.sponge_damping)
    s.set_velocity_field(vel)
    rng = np.random.default_rng(1)
    cur = rng.standard_normal(vel.size).astype(np.float32).astype(np.float64)
    prev = rng.standard_normal(vel.size).astype(np.float32).astype(np.float64)
    shape = (w.nx + 2, w.ny + 2, w.nz + 2)
    i1 = np.ravel_multi_index((5, 5, 7), shape)
    i2 = np.ravel_multi_index((3, 8, 4), shape)
    cur[i1] = np.nan
    prev[i2] = np.inf
    s.set_field(0, cur)
    s.set_field(1, prev)
    r = s.step_forward(0)
    assert r == se.StepResult.NAN_DETECTED_AND_REPAIRED
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    ref = oracle.run(g, vel, 1, np.zeros((0, 3)), np.zeros((1, 0)), np.zeros((0, 3)), fp32=True,
                     init_cur=cur, init_prev=prev)
    assert ref["status"][0] == 1
    out = s.get_field(0)
    assert np.isfinite(out).all()
    np.testing.assert_allclose(out, ref["cur"].astype(np.float64), rtol=2e-6, atol=2e-6)
    assert s.nan_count_current() == 0
    assert abs(s.compute_energy() - float(np.sum(out ** 2))) <= 1e-5 * float(np.sum(out ** 2))


@pytest.mark.parametrize("mode", ["reference", "stable"])
def test_forward_128_config_matches_oracle(se, oracle, mode):
    """128^3, 1000 steps, 64x64 receivers: seismograms and the final field
    against the FP64 oracle (relative L2), in both sponge modes."""
    import torch
    w = se.workloads.forward_128(nt=1000)
    shot = w.shots[0]
    vel = se.workloads.to_reference_layout(w.vel)
    s = make_solver(se, w.nx, w.ny, w.nz, w.d, w.dt, w.sponge_width, w.sponge_damping)
    s.set_sponge_mode(mode)
    s.set_velocity_field(vel)
    seis = torch.zeros((w.nt, shot.rec.count), device="cuda")
    assert se.shot_forward(s, shot.src, shot.wavelet, w.nt, shot.rec, seis=seis) == 0
    torch.cuda.synchronize()
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping, sponge_mode=mode)
    ref = oracle.run(g, vel, w.nt, np.array([shot.src]), shot.wavelet[:, None], shot.rec.coords())
    e_seis = rel(seis.cpu().numpy(), ref["seis"])
    e_cur = rel(s.get_field(0), ref["cur"])
    peak = float(np.abs(ref["seis"]).max())
    print(f"128^3 x 1000 ({mode} sponge): rel L2 seismograms {e_seis:.3e}, final field {e_cur:.3e}, "
          f"peak |seismogram| {peak:.3e}")
    assert e_seis < REL_FULL and e_cur < REL_FULL
