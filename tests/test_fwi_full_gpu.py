"""The FWI gradient at its full workload size (192^3, 4 shots on a 2x2
surface grid, 1500 steps, start model = the true model smoothed with a
6-cell Gaussian): the torch.autograd.Function against the direct entry
point, checkpointed (segments of 100 steps, 8 slots) against stored
snapshots, and the Taylor test along a smooth seeded perturbation
(remainder ratios of the halved steps near 4: second order)."""
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
    import seismic_engine.fwi  # noqa: F401
    return seismic_engine


def test_fwi_192_full_size(se):
    import torch
    w = se.workloads.fwi_192()
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping, sponge_mode=w.sponge_mode))
    v_true = torch.from_numpy(w.vel.astype(np.float32)).cuda()
    v0 = torch.from_numpy(se.workloads.smooth(w.vel, 6.0).astype(np.float32)).cuda()
    nrec = w.shots[0].rec.count
    d_obs = torch.zeros((len(w.shots), w.nt, nrec), device="cuda")
    se.fwi.set_velocity_device(s, v_true)
    for i, sh in enumerate(w.shots):
        se.shot_forward(s, sh.src, sh.wavelet, w.nt, sh.rec, seis=d_obs[i])

    def J(v, grad=None, checkpoint=None):
        se.fwi.set_velocity_device(s, v)
        m = 0.0
        for i, sh in enumerate(w.shots):
            m += se.fwi.fwi_gradient(s, sh.src, sh.wavelet, w.nt, sh.rec, d_obs[i].contiguous(), grad,
                                     snap_kind=se._lib.ST_SNAP_FP32, checkpoint=checkpoint)
        torch.cuda.synchronize()
        return m

    g = torch.zeros(w.points, device="cuda")
    j0 = J(v0, g)
    gc = torch.zeros(w.points, device="cuda")
    jc = J(v0, gc, checkpoint=(100, 8))
    # checkpointed recomputation: the gradient is bit-identical; the FP64 misfit is summed with
    # atomics, so its last bit may differ
    assert abs(jc - j0) <= 1e-14 * j0 and torch.equal(gc, g)
    # autograd Function
    vv = v0.clone().requires_grad_(True)
    d = se.fwi.modeling(vv, s, w.shots, w.nt)
    loss = 0.5 * ((d.double() - d_obs.double()) ** 2).sum()
    loss.backward()
    ga = vv.grad.reshape(-1)
    assert abs(float(loss.detach()) - j0) <= 1e-6 * j0
    assert float(torch.linalg.norm(ga - g) / torch.linalg.norm(g)) < 1e-5
    # Taylor test
    rng = np.random.default_rng(8)
    dv = se.workloads.smooth(rng.standard_normal(w.vel.shape), 4.0)
    dv = torch.from_numpy((20.0 * dv / np.abs(dv).max()).astype(np.float32)).cuda()
    gd = float(torch.dot(g.double(), dv.reshape(-1).double()))
    rems = []
    for k in range(4):
        h = 2.0 ** -k
        rems.append(abs(J(v0 + h * dv) - j0 - h * gd))
    ratios = [rems[i] / rems[i + 1] for i in range(3)]
    print(f"192^3 FWI: misfit {j0:.6e}, Taylor remainders {rems}, ratios {ratios}")
    assert all(3.0 < q < 5.0 for q in ratios), (rems, ratios)
    s.close()
