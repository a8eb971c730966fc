"""Two time steps per launch against one step per launch, through the C ABI.
RTM imaging pass: image, illumination and the final adjoint fields; forward
pass: seismograms, snapshot bytes, snapshot scales and the final fields. All
must be bit-identical (each point is updated by the same arithmetic in the
same order), for odd and even step counts, both sponge rules, every snapshot
kind, receivers and sources on the recomputed ring of a tile, grids that end
inside a tile, and different x-chunkings of the grid. The two-step path is
also the default one the oracle parity tests of test_rtm_gpu.py,
test_forward_gpu.py and test_fwi_gpu.py run. Velocity gradients (FWI
gradient epilogue) are compared the same way, stored and checkpointed."""
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


def run_rtm(se, n, nt, sponge, rec_z, kind, steps, seed=3):
    import torch
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    vel = 1500.0 + 1500.0 * rng.random((nx, ny, nz))
    d = 10.0
    dt = se.workloads.cfl_dt(d, 3000.0)
    s = se.WaveEquationSolver(se.GridParams(nx, ny, nz, d, d, d),
                              se.SolverConfig(dt=dt, nt=nt, sponge_width=6, sponge_damping=0.015))
    try:
        s.set_sponge_mode(sponge)
        s.set_velocity_field(se.workloads.to_reference_layout(vel))
        s.set_step_fusion(steps)
        rec = se.workloads.ReceiverGrid(1, 2, (nx - 2) // 2, 0, 1, ny, rec_z)
        data = torch.from_numpy((rng.standard_normal((nt, rec.count)) * 1e-3).astype(np.float32)).cuda()
        wav = se.workloads.ricker(25.0, dt, nt)
        image = torch.zeros(nx * ny * nz, device="cuda")
        illum = torch.zeros(nx * ny * nz, device="cuda")
        # the source sits three cells from the receiver plane, so that the
        # forward and adjoint fields overlap within a few steps
        src_z = rec_z - 3 if rec_z >= 3 else rec_z + 3
        assert se.rtm_shot(s, (nx // 2, ny // 2, src_z), wav, nt, rec, data, image, illum, snap_kind=kind) == 0
        torch.cuda.synchronize()
        return (image.cpu().numpy(), illum.cpu().numpy(), s.get_field(0), s.get_field(1))
    finally:
        s.close()


# nz is a multiple of 8 throughout: 16-bit snapshot rows are then whole
# 16-byte units, the condition for the staged (and two-step) imaging path
CASES = [
    # (nx, ny, nz), nt, sponge rule, receiver plane z
    ((28, 24, 32), 41, "reference", 5),
    ((40, 20, 72), 40, "stable", 63),   # second z tile holds 8 z; forcing on its ring point z0 - 1
    ((70, 33, 64), 23, "stable", 31),   # third y tile holds one row
    ((9, 17, 40), 12, "stable", 39),    # forcing on the last z; ring rows y0 - 1 / y0 + 16 carry receivers
]


@pytest.mark.parametrize("n,nt,sponge,rec_z", CASES)
def test_two_steps_per_launch_bit_identical(se, n, nt, sponge, rec_z):
    one = run_rtm(se, n, nt, sponge, rec_z, 1, steps=1)
    two = run_rtm(se, n, nt, sponge, rec_z, 1, steps=2)
    assert np.abs(one[0]).max() > 0 and np.abs(one[1]).max() > 0
    for a, b, what in zip(one, two, ("image", "illumination", "current field", "previous field")):
        assert np.array_equal(a, b), f"{what}: max |diff| {np.abs(a - b).max():.3e}"


@pytest.mark.parametrize("kind", [2, 3])
def test_two_steps_per_launch_snapshot_kinds(se, kind):
    one = run_rtm(se, (28, 24, 32), 30, "stable", 5, kind, steps=1)
    two = run_rtm(se, (28, 24, 32), 30, "stable", 5, kind, steps=2)
    for a, b in zip(one, two):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("chunks", ["1", "3", "7"])
def test_two_steps_per_launch_any_chunking(se, monkeypatch, chunks):
    base = run_rtm(se, (40, 20, 72), 17, "stable", 63, 1, steps=1)
    monkeypatch.setenv("SEISMIC_GB300_XCHUNKS", chunks)
    two = run_rtm(se, (40, 20, 72), 17, "stable", 63, 1, steps=2)
    for a, b in zip(base, two):
        assert np.array_equal(a, b)


def test_step_fusion_argument_checked(se):
    s = se.WaveEquationSolver(se.GridParams(8, 8, 8, 10.0, 10.0, 10.0), se.SolverConfig(dt=1e-3, nt=4))
    try:
        with pytest.raises(Exception):
            s.set_step_fusion(3)
    finally:
        s.close()


def run_forward(se, n, nt, sponge, src, rec_z, kind, steps, seed=5):
    """One forward shot; returns seismograms, snapshot bytes, the scale array
    and the two final fields."""
    import torch
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    vel = 1500.0 + 1500.0 * rng.random((nx, ny, nz))
    d = 10.0
    dt = se.workloads.cfl_dt(d, 3000.0)
    s = se.WaveEquationSolver(se.GridParams(nx, ny, nz, d, d, d),
                              se.SolverConfig(dt=dt, nt=nt, sponge_width=6, sponge_damping=0.015))
    try:
        s.set_sponge_mode(sponge)
        s.set_velocity_field(se.workloads.to_reference_layout(vel))
        s.set_step_fusion(steps)
        rec = se.workloads.ReceiverGrid(0, 3, (nx + 2) // 3, 0, 1, ny, rec_z)
        seis = torch.zeros((nt, rec.count), device="cuda")
        wav = se.workloads.ricker(30.0, dt, nt)
        es = {0: 0, 1: 2, 2: 2, 3: 4}[kind]
        snaps = torch.zeros(max(nt * nx * ny * nz * es, 1), dtype=torch.uint8, device="cuda")
        amax = torch.zeros(nt + 1, dtype=torch.int32, device="cuda")
        if kind:
            assert se.shot_forward(s, src, wav, nt, rec, seis=seis, snap_kind=kind, snaps=snaps, snap_amax=amax) == 0
        else:
            assert se.shot_forward(s, src, wav, nt, rec, seis=seis) == 0
        torch.cuda.synchronize()
        return (seis.cpu().numpy(), snaps.cpu().numpy(), amax.cpu().numpy(), s.get_field(0), s.get_field(1))
    finally:
        s.close()


FWD_CASES = [
    # (nx, ny, nz), nt, sponge rule, source, receiver plane z, snapshot kind
    ((28, 24, 32), 41, "reference", (14, 16, 5), 5, 1),    # source on row y0 of tile 1: the ring row of tile 0
    ((40, 20, 72), 40, "stable", (20, 15, 64), 63, 1),     # source on z0 of tile 1 / ring point of tile 0
    ((70, 33, 64), 23, "stable", (35, 31, 63), 60, 2),     # source on the last z of tile 0
    ((9, 17, 40), 12, "stable", (4, 16, 39), 39, 3),       # source in the one-row tile, on the last z
    ((30, 20, 36), 17, "stable", (15, 10, 18), 18, 0),     # no snapshots; nz % 8 != 0
]


@pytest.mark.parametrize("n,nt,sponge,src,rec_z,kind", FWD_CASES)
def test_two_forward_steps_per_launch_bit_identical(se, n, nt, sponge, src, rec_z, kind):
    one = run_forward(se, n, nt, sponge, src, rec_z, kind, steps=1)
    two = run_forward(se, n, nt, sponge, src, rec_z, kind, steps=2)
    assert np.abs(one[0]).max() > 0
    for a, b, what in zip(one, two, ("seismograms", "snapshots", "snapshot scales", "current field",
                                     "previous field")):
        assert np.array_equal(a, b), f"{what} differ"


@pytest.mark.parametrize("chunks", ["1", "4"])
def test_two_forward_steps_any_chunking(se, monkeypatch, chunks):
    base = run_forward(se, (40, 20, 72), 19, "stable", (20, 15, 64), 63, 1, steps=1)
    monkeypatch.setenv("SEISMIC_GB300_XCHUNKS", chunks)
    two = run_forward(se, (40, 20, 72), 19, "stable", (20, 15, 64), 63, 1, steps=2)
    for a, b in zip(base, two):
        assert np.array_equal(a, b)


def run_gradient(se, n, nt, sponge, src, rec_z, kind, steps, checkpoint=None, seed=9):
    """Velocity gradient of one shot for a seeded adjoint source; returns the
    gradient and the two final fields."""
    import torch
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    vel = 1500.0 + 1500.0 * rng.random((nx, ny, nz))
    d = 10.0
    dt = se.workloads.cfl_dt(d, 3000.0)
    s = se.WaveEquationSolver(se.GridParams(nx, ny, nz, d, d, d),
                              se.SolverConfig(dt=dt, nt=nt, sponge_width=6, sponge_damping=0.015))
    try:
        s.set_sponge_mode(sponge)
        s.set_velocity_field(se.workloads.to_reference_layout(vel))
        s.set_step_fusion(steps)
        rec = se.workloads.ReceiverGrid(1, 2, (nx - 2) // 2, 0, 1, ny, rec_z)
        adj = torch.from_numpy((rng.standard_normal((nt, rec.count)) * 1e-3).astype(np.float32)).cuda()
        wav = se.workloads.ricker(30.0, dt, nt)
        gv = torch.zeros(nx * ny * nz, device="cuda")
        r = se.fwi.shot_gradient(s, src, wav, nt, rec, adj, gv, kind, checkpoint=checkpoint)
        assert (r == 0) if checkpoint is None else isinstance(r, dict)
        torch.cuda.synchronize()
        return (gv.cpu().numpy(), s.get_field(0), s.get_field(1))
    finally:
        s.close()


GRAD_CASES = [
    # (nx, ny, nz), nt, sponge rule, source, receiver plane z, snapshot kind
    ((28, 24, 32), 41, "reference", (14, 16, 5), 8, 1),
    ((40, 20, 72), 40, "stable", (20, 15, 64), 61, 3),     # second z tile; receivers by the tile seam
    ((9, 17, 40), 13, "stable", (4, 16, 36), 39, 2),
]


@pytest.mark.parametrize("n,nt,sponge,src,rec_z,kind", GRAD_CASES)
def test_two_gradient_steps_per_launch_bit_identical(se, n, nt, sponge, src, rec_z, kind):
    one = run_gradient(se, n, nt, sponge, src, rec_z, kind, steps=1)
    two = run_gradient(se, n, nt, sponge, src, rec_z, kind, steps=2)
    assert np.abs(one[0]).max() > 0
    for a, b, what in zip(one, two, ("gradient", "current field", "previous field")):
        assert np.array_equal(a, b), f"{what} differ"


def test_two_gradient_steps_checkpointed(se):
    """Pairs inside checkpoint segments of odd and even length against one step per launch."""
    base = run_gradient(se, (28, 24, 32), 41, "stable", (14, 16, 5), 8, 1, steps=1)
    for seg, slots in [(10, 2), (7, 3)]:
        two = run_gradient(se, (28, 24, 32), 41, "stable", (14, 16, 5), 8, 1, steps=2, checkpoint=(seg, slots))
        assert np.array_equal(base[0], two[0]), (seg, slots)


@pytest.mark.parametrize("n,nt", [((4, 5, 8), 9), ((5, 17, 16), 6), ((6, 3, 72), 5)])
def test_two_steps_per_launch_small_grids(se, n, nt):
    """Grids thinner than a tile along every axis, with few steps."""
    nx, ny, nz = n
    rz = nz - 2
    src = (nx // 2, ny // 2, rz - 1)
    for run, args in ((run_rtm, (n, nt, "stable", rz, 1)),
                      (run_forward, (n, nt, "stable", src, rz, 1)),
                      (run_gradient, (n, nt, "stable", src, rz, 1))):
        one = run(se, *args, steps=1)
        two = run(se, *args, steps=2)
        for a, b in zip(one, two):
            assert np.array_equal(a, b), run.__name__


def test_two_steps_per_launch_mid_size_partial_tiles(se):
    """301 x 203 x 136: several x-chunks, a last y tile of 11 rows and a last
    z tile of 8 points, in all three modes."""
    n, nt, rz = (301, 203, 136), 14, 100
    src = (150, 101, 97)
    for run, args in ((run_rtm, (n, nt, "stable", rz, 1)),
                      (run_forward, (n, nt, "stable", src, rz, 1)),
                      (run_gradient, (n, nt, "stable", src, rz, 1))):
        one = run(se, *args, steps=1)
        two = run(se, *args, steps=2)
        for a, b in zip(one, two):
            assert np.array_equal(a, b), run.__name__
