"""GPU parity of the exact adjoint and of RTM imaging against the FP64
oracle, through the C ABI.

Tolerances: FP32 GPU vs FP64 oracle relative L2 <= 1e-4 for adjoint traces
and images; BF16 / FP16 snapshot storage vs FP32 storage relative image
error <= 1e-3 (the stated storage-error bound); the GPU dot-product test
<F s, r> = <s, F^T r> to 1e-5 relative."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
    return seismic_engine


def solver_for(se, w, vel_ref):
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping))
    s.set_velocity_field(vel_ref)
    return s


@pytest.mark.parametrize("coincident", [False, True])
def test_adjoint_dot_product_and_trace(se, oracle, coincident):
    import torch
    w = se.workloads.small_case(n=(22, 18, 26), nt=70, seed=2, sponge_width=4)
    shot = w.shots[0]
    rec = shot.rec
    src = (rec.x0 + 2 * rec.sx, rec.y0 + rec.sy, rec.z) if coincident else shot.src
    vel = se.workloads.to_reference_layout(w.vel)
    s = solver_for(se, w, vel)
    rng = np.random.default_rng(7)
    sw = rng.standard_normal(w.nt)
    r = rng.standard_normal((w.nt, rec.count)).astype(np.float32)
    seis = torch.zeros((w.nt, rec.count), device="cuda")
    assert se.shot_forward(s, src, sw, w.nt, rec, seis=seis) == 0
    trace = torch.zeros(w.nt, device="cuda")
    assert se.shot_adjoint(s, src, w.nt, rec, torch.from_numpy(r).cuda(), trace) == 0
    torch.cuda.synchronize()
    lhs = float(np.sum(seis.cpu().numpy().astype(np.float64) * r))
    tr = trace.cpu().numpy().astype(np.float64)
    rhs = float(np.sum(sw * tr))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    ref = oracle.adjoint(g, vel, w.nt, rec.coords(), r.astype(np.float64), src_xyz=np.array([src]))
    assert rel(tr, ref["src_adj"][:, 0]) < 1e-4


def test_rtm_engine_matches_reference_fixture(se, golden_dir):
    """RTMEngine face: the reference's own imaging-condition outputs (FP64)."""
    g = np.load(os.path.join(golden_dir, "rtm_small.npz"))
    nx, ny, nz = (int(v) for v in g["n"])
    e = se.RTMEngine(nx, ny, nz, 10.0, 10.0, 10.0, 1)
    for t in range(g["fwd"].shape[0]):
        e.apply_image_condition(g["fwd"][t], g["adj"][t], ny + 2, nz + 2, t)
    e.finalize_image()
    r = e.result()
    np.testing.assert_allclose(r.image, g["image"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(r.illumination, g["illum"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(r.reflectivity, g["refl"], rtol=1e-12, atol=1e-12)
    e.reset_image()
    assert not e.result().image.any()


def rtm_case(se, oracle, n=(28, 24, 32), nt=90):
    w = se.workloads.small_case(n=n, nt=nt, seed=12, sponge_width=5)
    shot = w.shots[0]
    true_ref = se.workloads.to_reference_layout(w.vel)
    mig = se.workloads.smooth(w.vel, 2.0)
    mig_ref = se.workloads.to_reference_layout(mig)
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    d_obs = oracle.run(g, true_ref, w.nt, np.array([shot.src]), shot.wavelet[:, None], shot.rec.coords())["seis"]
    return w, shot, g, mig_ref, d_obs.astype(np.float32)


@pytest.mark.parametrize("n", [(28, 24, 32), (27, 23, 30)])
def test_rtm_image_matches_oracle(se, oracle, n):
    """nz = 32: imaging operands staged through the TMA ring; nz = 30 (rows
    not a multiple of 16 bytes for 16-bit snapshots): loaded at use."""
    import torch
    w, shot, g, mig_ref, d_obs = rtm_case(se, oracle, n=n)
    fwd = oracle.run(g, mig_ref, w.nt, np.array([shot.src]), shot.wavelet[:, None], shot.rec.coords(),
                     keep_states=True)
    ref = oracle.adjoint(g, mig_ref, w.nt, shot.rec.coords(), d_obs.astype(np.float64), states=fwd["states"],
                         want_image=True)
    refl_ref = np.where(ref["illum"] > 1e-10, ref["image"] / np.where(ref["illum"] > 1e-10, ref["illum"], 1), 0)
    s = solver_for(se, w, mig_ref)
    n = w.points
    data = torch.from_numpy(d_obs).cuda()
    images = {}
    for kind in (3, 1, 2):
        image = torch.zeros(n, device="cuda")
        illum = torch.zeros(n, device="cuda")
        refl = torch.zeros(n, device="cuda")
        assert se.rtm_shot(s, shot.src, shot.wavelet, w.nt, shot.rec, data, image, illum, refl, snap_kind=kind) == 0
        torch.cuda.synchronize()
        images[kind] = (image.cpu().numpy(), illum.cpu().numpy(), refl.cpu().numpy())
    img32, ill32, refl32 = images[3]
    assert rel(img32, ref["image"]) < 1e-4
    assert rel(ill32, ref["illum"]) < 1e-4
    assert rel(refl32, refl_ref) < 1e-3
    for kind in (1, 2):
        e = rel(images[kind][0], img32)
        print(f"snapshot kind {kind}: image error vs FP32 storage {e:.2e}")
        assert e < 1e-3
    # host-buffer entry point, every copy included
    out = se.rtm_shot_host(s, mig_ref, shot.src, shot.wavelet, w.nt, shot.rec, d_obs, snap_kind=3)
    np.testing.assert_allclose(out["image"], img32.astype(np.float64), rtol=1e-6, atol=1e-12 * np.abs(img32).max())
    np.testing.assert_allclose(out["illumination"], ill32.astype(np.float64), rtol=1e-6, atol=0)


def test_rtm_bf16_storage_error_at_128(se):
    """128^3 x 600 steps: BF16 and FP16 snapshot storage against FP32 storage."""
    import torch
    w = se.workloads.forward_128(nt=600)
    shot = w.shots[0]
    s = solver_for(se, w, se.workloads.to_reference_layout(se.workloads.smooth(w.vel, 6.0)))
    # observed data from the true model
    t = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping))
    t.set_velocity_field(se.workloads.to_reference_layout(w.vel))
    data = torch.zeros((w.nt, shot.rec.count), device="cuda")
    assert se.shot_forward(t, shot.src, shot.wavelet, w.nt, shot.rec, seis=data) == 0
    n = w.points
    imgs = {}
    for kind in (3, 1, 2):
        image = torch.zeros(n, device="cuda")
        illum = torch.zeros(n, device="cuda")
        assert se.rtm_shot(s, shot.src, shot.wavelet, w.nt, shot.rec, data, image, illum, snap_kind=kind) == 0
        torch.cuda.synchronize()
        imgs[kind] = image.cpu().numpy()
    for kind in (1, 2):
        e = rel(imgs[kind], imgs[3])
        print(f"128^3 x 600, snapshot kind {kind}: image error vs FP32 storage {e:.2e}")
        assert e < 1e-3
