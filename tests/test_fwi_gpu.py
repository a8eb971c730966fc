"""GPU adjoint-state gradients (FWI) through the C ABI and torch.autograd:
parity with the FP64 oracle's exact discrete gradient, the error of BF16 /
FP16 snapshot storage against FP32 storage, a Taylor test with second-order
remainder decay, and the autograd Function against the direct entry point.

Tolerances: FP32-snapshot gradient vs FP64 oracle relative L2 <= 1e-4;
FP16 storage <= 1e-2 and BF16 storage <= 5e-2 relative to FP32 storage (the
stated storage error; the imaging path's bound is 1e-3)."""
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
    import seismic_engine.fwi  # noqa: F401
    return seismic_engine


def case(se, n=(20, 18, 24), nt=70, seed=21):
    w = se.workloads.small_case(n=n, nt=nt, seed=seed, sponge_width=4)
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping))
    s.set_velocity_field(se.workloads.to_reference_layout(w.vel))
    return w, s


def test_gradient_matches_oracle(se, oracle):
    import torch
    w, s = case(se)
    sh = w.shots[0]
    rng = np.random.default_rng(3)
    adj = rng.standard_normal((w.nt, sh.rec.count)).astype(np.float32)
    vel = se.workloads.to_reference_layout(w.vel)
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    fwd = oracle.run(g, vel, w.nt, np.array([sh.src]), sh.wavelet[:, None], sh.rec.coords(), keep_states=True)
    ref = oracle.adjoint(g, vel, w.nt, sh.rec.coords(), adj.astype(np.float64), states=fwd["states"], want_grad=True)
    ref_v = ref["grad_c"] * 2.0 * w.vel.reshape(-1) * w.dt * w.dt
    grads = {}
    for kind in (3, 1, 2):
        gv = torch.zeros(w.points, device="cuda")
        assert se.fwi.shot_gradient(s, sh.src, sh.wavelet, w.nt, sh.rec, torch.from_numpy(adj).cuda(), gv, kind) == 0
        torch.cuda.synchronize()
        grads[kind] = gv.cpu().numpy()
    e32 = rel(grads[3], ref_v)
    e16 = rel(grads[2], grads[3])
    ebf = rel(grads[1], grads[3])
    print(f"gradient: FP32 storage vs FP64 oracle {e32:.2e}; FP16 vs FP32 storage {e16:.2e}; "
          f"BF16 vs FP32 storage {ebf:.2e}")
    assert e32 < 1e-4
    assert e16 < 1e-2
    assert ebf < 5e-2


def test_taylor_second_order(se):
    """J(v) = 1/2 ||F(v) - d_obs||^2: |J(v+h dv) - J(v) - h <g, dv>| = O(h^2)."""
    import torch
    w, s = case(se, n=(24, 20, 28), nt=90, seed=22)
    sh = w.shots[0]
    v0 = torch.from_numpy(w.vel.astype(np.float32)).cuda()
    # observed data on a perturbed model
    se.fwi.set_velocity_device(s, v0 * 1.02)
    d_obs = torch.zeros((w.nt, sh.rec.count), device="cuda")
    se.shot_forward(s, sh.src, sh.wavelet, w.nt, sh.rec, seis=d_obs)
    se.fwi.set_velocity_device(s, v0)
    g = torch.zeros(w.points, device="cuda")
    j0 = se.fwi.fwi_gradient(s, sh.src, sh.wavelet, w.nt, sh.rec, d_obs, g, snap_kind=3)
    rng = np.random.default_rng(5)
    dv = se.workloads.smooth(rng.standard_normal(w.vel.shape), 2.0)
    dv = torch.from_numpy((0.01 * np.abs(w.vel).max() * dv / np.abs(dv).max()).astype(np.float32)).cuda()
    gd = float(torch.dot(g.double(), dv.reshape(-1).double()))
    rems = []
    for k in range(4):
        h = 2.0 ** -k
        se.fwi.set_velocity_device(s, v0 + h * dv)
        jh = se.fwi.fwi_gradient(s, sh.src, sh.wavelet, w.nt, sh.rec, d_obs, None)
        rems.append(abs(jh - j0 - h * gd))
    ratios = [rems[i] / rems[i + 1] for i in range(3)]
    print("Taylor remainders", rems, "ratios", ratios)
    assert all(3.0 < q < 5.0 for q in ratios), (rems, ratios)


def test_autograd_function_matches_entry_point(se):
    import torch
    w, s = case(se, n=(18, 16, 20), nt=60, seed=23)
    shots = [w.shots[0], se.workloads.ShotSpec((5, 6, 4), w.shots[0].wavelet, w.shots[0].rec)]
    v = torch.from_numpy(w.vel.astype(np.float32)).cuda()
    d_obs = torch.zeros((2, w.nt, shots[0].rec.count), device="cuda")
    se.fwi.set_velocity_device(s, v * 0.98)
    for i, sh in enumerate(shots):
        se.shot_forward(s, sh.src, sh.wavelet, w.nt, sh.rec, seis=d_obs[i])
    vv = v.clone().requires_grad_(True)
    d = se.fwi.modeling(vv, s, shots, w.nt)
    loss = 0.5 * ((d.double() - d_obs.double()) ** 2).sum()
    loss.backward()
    se.fwi.set_velocity_device(s, v)
    g = torch.zeros(w.points, device="cuda")
    m = 0.0
    for i, sh in enumerate(shots):
        m += se.fwi.fwi_gradient(s, sh.src, sh.wavelet, w.nt, sh.rec, d_obs[i].contiguous(), g, snap_kind=3)
    assert abs(float(loss.detach()) - m) <= 1e-6 * m
    assert rel(vv.grad.reshape(-1).cpu().numpy(), g.cpu().numpy()) < 1e-5


def test_autograd_function_on_a_side_stream(se, monkeypatch):
    """The autograd Function runs on torch's current stream: on a side stream,
    with torch.cuda.synchronize made to fail, the seismograms and the
    gradient equal those of the same call on the default stream bit for bit."""
    import torch
    w, s = case(se, n=(18, 16, 20), nt=40, seed=25)
    shots = [w.shots[0]]
    v = torch.from_numpy(w.vel.astype(np.float32)).cuda()
    v0 = v.clone().requires_grad_(True)
    d0 = se.fwi.modeling(v0, s, shots, w.nt)
    (d0.double() ** 2).sum().backward()
    torch.cuda.synchronize()

    def no_device_sync(*a, **k):
        raise AssertionError("device-wide synchronisation inside the autograd Function")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        monkeypatch.setattr(torch.cuda, "synchronize", no_device_sync)
        v1 = v.clone().requires_grad_(True)
        d1 = se.fwi.modeling(v1, s, shots, w.nt)
        (d1.double() ** 2).sum().backward()
        monkeypatch.undo()
    side.synchronize()
    assert s.stream_ptr() != side.cuda_stream  # the solver is back on its own stream
    assert torch.equal(d0, d1)
    assert torch.equal(v0.grad, v1.grad)


def test_exact_gradient_vs_reference_pointwise_formula(se):
    """The reference's adjoint-state gradient (seismic_tomography/gradient.py:
    24-40) is the pointwise g = -u * lambda * 2 v dt^2; summed over time that is
    -2 v dt^2 times the zero-lag image of the forward and adjoint fields. The
    exact discrete gradient correlates lambda with L u instead of u (L u ~ -k^2
    u for band-limited waves), so the two agree in direction but not exactly:
    their cosine similarity is stated and required to be clearly positive."""
    import torch
    w = se.workloads.small_case(n=(32, 28, 40), nt=160, seed=24, sponge_width=6)
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping, sponge_mode="stable"))
    sh = w.shots[0]
    v0 = torch.from_numpy(se.workloads.smooth(w.vel, 2.0).astype(np.float32)).cuda()
    se.fwi.set_velocity_device(s, torch.from_numpy(w.vel.astype(np.float32)).cuda())
    d_obs = torch.zeros((w.nt, sh.rec.count), device="cuda")
    se.shot_forward(s, sh.src, sh.wavelet, w.nt, sh.rec, seis=d_obs)
    se.fwi.set_velocity_device(s, v0)
    g = torch.zeros(w.points, device="cuda")
    res = torch.zeros_like(d_obs)
    se.fwi.fwi_gradient(s, sh.src, sh.wavelet, w.nt, sh.rec, d_obs, g, snap_kind=3, residual=res)
    image = torch.zeros(w.points, device="cuda")
    illum = torch.zeros(w.points, device="cuda")
    assert se.rtm_shot(s, sh.src, sh.wavelet, w.nt, sh.rec, res, image, illum, snap_kind=3) == 0
    torch.cuda.synchronize()
    g_ref = -image * 2.0 * v0.reshape(-1) * w.dt * w.dt
    cos = float(torch.dot(g.double(), g_ref.double()) / (torch.linalg.norm(g.double()) *
                                                          torch.linalg.norm(g_ref.double())))
    print(f"cosine(exact gradient, reference pointwise formula) = {cos:.3f}")
    assert cos > 0.5
