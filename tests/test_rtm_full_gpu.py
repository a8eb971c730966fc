"""RTM at its full workload size (256^3, 2000 steps, 128x128 receivers,
stable sponge, migration model = the true model smoothed with a 6-cell
Gaussian): the image error of BF16 and FP16 snapshot storage against FP32
storage (the stated bound is 1e-3 relative L2), and the checkpointed pass
(100-step segments, 20 state slots) against store-all, bit for bit."""
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


def test_rtm_256_storage_error_and_checkpointing(se):
    import torch
    w = se.workloads.rtm_256()
    sh = w.shots[0]
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping, sponge_mode=w.sponge_mode))
    s.set_velocity_field(se.workloads.to_reference_layout(w.vel))
    data = torch.zeros((w.nt, sh.rec.count), device="cuda")
    assert se.shot_forward(s, sh.src, sh.wavelet, w.nt, sh.rec, seis=data) == 0
    s.set_velocity_field(se.workloads.to_reference_layout(se.workloads.smooth(w.vel, 6.0)))
    images = {}
    for kind in (se._lib.ST_SNAP_FP32, se._lib.ST_SNAP_BF16, se._lib.ST_SNAP_FP16):
        img = torch.zeros(w.points, device="cuda")
        ill = torch.zeros(w.points, device="cuda")
        assert se.rtm_shot(s, sh.src, sh.wavelet, w.nt, sh.rec, data, img, ill, snap_kind=kind) == 0
        torch.cuda.synchronize()
        images[kind] = img.double()
        if kind == se._lib.ST_SNAP_BF16:
            ck = torch.zeros(w.points, device="cuda")
            cil = torch.zeros(w.points, device="cuda")
            st = se.rtm_shot_checkpointed(s, sh.src, sh.wavelet, w.nt, sh.rec, data, ck, cil, snap_kind=kind,
                                          segment_steps=100, max_slots=20)
            torch.cuda.synchronize()
            assert torch.equal(ck, img) and torch.equal(cil, ill)
            assert st["segments"] == 20
    ref = images[se._lib.ST_SNAP_FP32]
    e_bf = float(torch.linalg.norm(images[se._lib.ST_SNAP_BF16] - ref) / torch.linalg.norm(ref))
    e_fp = float(torch.linalg.norm(images[se._lib.ST_SNAP_FP16] - ref) / torch.linalg.norm(ref))
    print(f"256^3 x 2000 RTM: image error vs FP32 storage, BF16 {e_bf:.2e}, FP16 {e_fp:.2e}")
    assert e_bf < 1e-3 and e_fp < 1e-3
    s.close()
