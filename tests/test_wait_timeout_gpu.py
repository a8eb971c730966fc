"""The bounded-wait error path of the stencil kernels, exercised without a GPU
fault: the solver's test hook (st_solver_set_wait_test) withholds the copy of
one plane of every CTA's march, so the waits on it run out after a 1 ms limit;
the kernel drains its other copies, records the timeout and exits, and the
call returns ST_ERR_TIMEOUT. The handle stays usable: after reset_field the
same solver steps and shoots exactly as a fresh one, matching the FP64
oracle (relative L2 <= 2e-5)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


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


def test_withheld_copy_times_out_and_handle_recovers(se, oracle):
    import torch
    from seismic_engine._lib import ST_ERR_TIMEOUT, call
    w = se.workloads.small_case(n=(20, 18, 24), nt=16, seed=4, sponge_width=4)
    shot = w.shots[0]
    vel = se.workloads.to_reference_layout(w.vel)
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping))
    s.set_velocity_field(vel)
    # one step per launch (the reference stepping API)
    call("st_solver_set_wait_test", s.handle, 1_000_000, 3)
    with pytest.raises(se.SeismicError) as e:
        s.step_forward(0)
    assert e.value.code == ST_ERR_TIMEOUT
    # two steps per launch (the fused forward shot): the first launch times out
    seis = torch.zeros((w.nt, shot.rec.count), device="cuda")
    call("st_solver_set_wait_test", s.handle, 1_000_000, 2)
    with pytest.raises(se.SeismicError) as e:
        se.shot_forward(s, shot.src, shot.wavelet, w.nt, shot.rec, seis=seis)
    assert e.value.code == ST_ERR_TIMEOUT
    call("st_solver_set_wait_test", s.handle, 0, -1)
    # the same handle afterwards: stepping and a fused shot match the oracle
    s.reset_field()
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping)
    ref = oracle.run(g, vel, w.nt, np.array([shot.src]), shot.wavelet[:, None], shot.rec.coords())
    cur = None
    for t in range(w.nt):
        s.inject_source(*shot.src, [shot.wavelet[t]])
        assert s.step_forward(t) == se.StepResult.OK
    cur = s.get_field(se._lib.ST_FIELD_CURRENT)
    assert rel(cur, ref["cur"]) < 2e-5
    assert se.shot_forward(s, shot.src, shot.wavelet, w.nt, shot.rec, seis=seis) == 0
    torch.cuda.synchronize()
    assert rel(seis.cpu().numpy().astype(np.float64), ref["seis"]) < 2e-5
    s.close()
