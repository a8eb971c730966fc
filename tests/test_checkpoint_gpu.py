"""Checkpointed adjoint passes (forward history recomputed from FP32 state
checkpoints on a binomial schedule) against the store-every-step passes.

The recomputed snapshots are the stored ones bit for bit, so images,
illuminations, gradients and residuals must be identical (tolerance 0) for
every snapshot kind and every slot budget (misfits to 1e-14, their FP64 sum
is order-dependent); the schedule statistics
must match a Python model of the same binomial recursion."""
import math
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


def binom(s, r):
    return math.comb(s + r, s)


def split(l, s):
    r = 1
    while binom(s, r) < l:
        r += 1
    off = max(1, min(l - binom(s - 1, r), binom(s, r - 1)))
    return min(off, l - 1)


def schedule_model(nt, seg, slots):
    """Forward steps and state copies of the recursion in st_checkpoint.cu."""
    nseg = max(1, -(-nt // seg))
    st = {"at": 0, "free": min(slots, nseg) - 1, "fwd": 0, "copies": 1}

    def seg_len(j):
        return min(nt, (j + 1) * seg) - j * seg

    def restore(j):
        if st["at"] != j:
            st["copies"] += 1
            st["at"] = j

    def rev(a, b):
        if b - a == 1:
            restore(a)
            st["fwd"] += seg_len(a)
            st["at"] = a + 1
            return
        if st["free"] == 0:
            for j in range(b - 1, a - 1, -1):
                restore(a)
                st["fwd"] += (j - a) * seg + seg_len(j)
                st["at"] = j + 1
            return
        m = a + split(b - a, st["free"])
        restore(a)
        st["fwd"] += (m - a) * seg
        st["at"] = m
        st["free"] -= 1
        st["copies"] += 1
        rev(m, b)
        st["free"] += 1
        rev(a, m)

    rev(0, nseg)
    return st["fwd"], st["copies"], nseg


def case(se):
    w = se.workloads.small_case(n=(28, 24, 32), nt=93, seed=12, sponge_width=5)
    vel = se.workloads.to_reference_layout(se.workloads.smooth(w.vel, 2.0))
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping))
    s.set_velocity_field(vel)
    return w, s


@pytest.mark.parametrize("kind", [1, 3])
def test_rtm_checkpointed_equals_store_all(se, kind):
    import torch
    w, s = case(se)
    shot = w.shots[0]
    rng = np.random.default_rng(5)
    data = torch.from_numpy(rng.standard_normal((w.nt, shot.rec.count)).astype(np.float32)).cuda()
    n = w.points
    ref = [torch.zeros(n, device="cuda") for _ in range(3)]
    assert se.rtm_shot(s, shot.src, shot.wavelet, w.nt, shot.rec, data, *ref, snap_kind=kind) == 0
    torch.cuda.synchronize()
    for seg, slots in [(10, 100), (10, 3), (10, 1), (7, 2), (93, 1), (1, 4)]:
        out = [torch.full((n,), 7.0, device="cuda") for _ in range(3)]
        st = se.rtm_shot_checkpointed(s, shot.src, shot.wavelet, w.nt, shot.rec, data, *out, snap_kind=kind,
                                      segment_steps=seg, max_slots=slots)
        torch.cuda.synchronize()
        for a, b in zip(out, ref):
            assert torch.equal(a, b), (seg, slots)
        fwd, copies, nseg = schedule_model(w.nt, seg, slots)
        assert st["segments"] == nseg and st["adjoint_steps"] == w.nt
        assert st["forward_steps"] == fwd and st["state_copies"] == copies, (seg, slots, st, fwd, copies)
        assert st["slots_used"] <= min(slots, nseg)
    # with a slot per segment: one plain sweep plus one recompute
    fwd, _, _ = schedule_model(w.nt, 10, 100)
    assert fwd == w.nt + (w.nt - w.nt % 10)


@pytest.mark.parametrize("kind", [1, 3])
def test_gradients_checkpointed_equal_store_all(se, kind):
    import torch
    w, s = case(se)
    shot = w.shots[0]
    rng = np.random.default_rng(9)
    adj = torch.from_numpy(rng.standard_normal((w.nt, shot.rec.count)).astype(np.float32)).cuda()
    g_ref = torch.zeros(w.points, device="cuda")
    se.fwi.shot_gradient(s, shot.src, shot.wavelet, w.nt, shot.rec, adj, g_ref, snap_kind=kind)
    d_obs = adj * 0.01
    gf_ref = torch.zeros(w.points, device="cuda")
    r_ref = torch.zeros_like(adj)
    m_ref = se.fwi.fwi_gradient(s, shot.src, shot.wavelet, w.nt, shot.rec, d_obs, gf_ref, snap_kind=kind,
                                residual=r_ref)
    torch.cuda.synchronize()
    assert float(g_ref.abs().max()) > 0 and m_ref > 0
    for seg, slots in [(12, 100), (12, 2), (31, 1)]:
        g = torch.zeros(w.points, device="cuda")
        st = se.fwi.shot_gradient(s, shot.src, shot.wavelet, w.nt, shot.rec, adj, g, snap_kind=kind,
                                  checkpoint=(seg, slots))
        gf = torch.zeros(w.points, device="cuda")
        r = torch.zeros_like(adj)
        m = se.fwi.fwi_gradient(s, shot.src, shot.wavelet, w.nt, shot.rec, d_obs, gf, snap_kind=kind, residual=r,
                                checkpoint=(seg, slots))
        torch.cuda.synchronize()
        assert torch.equal(g, g_ref), (seg, slots)
        assert torch.equal(gf, gf_ref) and torch.equal(r, r_ref), (seg, slots)
        # the FP64 misfit is summed with atomics, so its last bit depends on block order
        assert abs(m - m_ref) <= 1e-14 * m_ref, (seg, slots)
        assert st["forward_steps"] == schedule_model(w.nt, seg, slots)[0]


def test_checkpointed_autograd_matches_stored(se):
    import torch
    w, s = case(se)
    shots = w.shots[:1]
    v = torch.from_numpy(se.workloads.smooth(w.vel, 2.0).astype(np.float32)).cuda()
    grads = []
    for ck in (None, (16, 2)):
        vv = v.clone().requires_grad_(True)
        d = se.fwi.modeling(vv, s, shots, w.nt, checkpoint=ck)
        (d.double() ** 2).sum().backward()
        grads.append(vv.grad.detach().clone())
    assert torch.equal(grads[0], grads[1])


def test_checkpoint_argument_errors(se):
    import torch
    from seismic_engine import _lib
    w, s = case(se)
    shot = w.shots[0]
    data = torch.zeros((w.nt, shot.rec.count), device="cuda")
    out = [torch.zeros(w.points, device="cuda") for _ in range(3)]
    for seg, slots in [(0, 4), (10, 0)]:
        with pytest.raises(_lib.SeismicError) as e:
            se.rtm_shot_checkpointed(s, shot.src, shot.wavelet, w.nt, shot.rec, data, *out, segment_steps=seg,
                                     max_slots=slots)
        assert e.value.code == _lib.ST_ERR_ARG
