"""The host-buffer entry points upload a whole velocity model straight to the
device (CFL maximum found on the GPU, host mirror refreshed on demand): they
must give the same seismograms and images as the set_velocity_field path,
and field().velocity / the CFL rule must see the uploaded model, including
a model that trips the CFL damping."""
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


@pytest.mark.parametrize("vscale", [1.0, 4.0])  # 4x: CFL > 1, the reference's damping applies
def test_host_upload_matches_set_velocity(se, vscale):
    import torch
    w = se.workloads.small_case(n=(22, 18, 26), nt=60, seed=4, sponge_width=4)
    sh = w.shots[0]
    vel = se.workloads.to_reference_layout(w.vel) * vscale
    vel.reshape(-1)[5] = np.nan  # a non-finite value: the CFL maximum skips it
    grid = se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d)
    cfg = se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width, sponge_damping=w.sponge_damping)
    a = se.WaveEquationSolver(grid, cfg)
    b = se.WaveEquationSolver(grid, cfg)
    a.set_velocity_field(vel)
    seis_a = torch.zeros((w.nt, sh.rec.count), device="cuda")
    assert se.shot_forward(a, sh.src, sh.wavelet, w.nt, sh.rec, seis=seis_a) == 0
    seis_b = se.shot_forward_host(b, vel, sh.src, sh.wavelet, w.nt, sh.rec)
    torch.cuda.synchronize()
    assert np.array_equal(seis_a.cpu().numpy().astype(np.float64), seis_b)
    got = b.get_field(se._lib.ST_FIELD_VELOCITY)
    assert np.array_equal(np.isnan(got), np.isnan(vel.reshape(-1)))
    assert np.array_equal(np.nan_to_num(got), np.nan_to_num(vel.reshape(-1)))
    # RTM through the host entry vs the device entry, same model
    data = torch.randn((w.nt, sh.rec.count), device="cuda") * 1e-3
    img = torch.zeros(w.points, device="cuda")
    ill = torch.zeros(w.points, device="cuda")
    assert se.rtm_shot(a, sh.src, sh.wavelet, w.nt, sh.rec, data, img, ill) == 0
    torch.cuda.synchronize()
    buf = np.empty(w.points)
    out = se.rtm_shot_host(b, vel, sh.src, sh.wavelet, w.nt, sh.rec, data.cpu().numpy(), want=("image",),
                           out={"image": buf})
    assert out["image"] is buf
    assert np.array_equal(buf, img.cpu().numpy().astype(np.float64))
    a.close()
    b.close()
