"""GPU slice capture and the slice stream: frames serialized on the GPU from
device fields (reference-layout FP64 and device-layout FP32) byte-identical
to the oracle's restatement of capture_single_slice + serialize_slice; the
asynchronous stream's file holding the same frames in capture order; and
the solver's configure_rtm path capturing the shot's fields and image."""
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
    return dict(np.load(os.path.join(golden_dir, "slices_small.npz")))


def to_device_layout(se, ref_field, nx, ny, nz):
    """Reference layout (FP64, pitch nz + 2) -> device layout (FP32)."""
    L = se.field_layout(nx, ny, nz)
    out = np.zeros(L["elems"], np.float32)
    r = ref_field.reshape(nx + 2, ny + 2, nz + 2)
    d = out.reshape(L["NXh"], L["NYh"], L["NZP"])
    d[:, :, L["ZOFF"] - 1:L["ZOFF"] + nz + 1] = r.astype(np.float32)
    return out


SPECS = [(0, 2), (1, -1), (2, 5), (3, 0), (0, -1)]


def resolved(nx, ny, nz):
    return [(a, (i if i >= 0 else (nx, ny, nz)[a] // 2)) for a, i in SPECS if a < 3]


def test_capture_fp64_reference_layout_byte_exact(se, oracle, gold):
    import torch
    nx, ny, nz = (int(v) for v in gold["n"])
    f = torch.from_numpy(gold["fwd"]).cuda()
    a = torch.from_numpy(gold["adj"]).cuda()
    c = torch.from_numpy(gold["ic"]).cuda()
    frames = se.capture_slice_frames(nx, ny, nz, SPECS, f, a, c, timestep=9, timestamp=77.25,
                                     field_kind=se.slices.FIELD_REFERENCE_FP64)
    want = [oracle.slice_frame(ax, ix, nx, ny, nz, gold["fwd"], gold["adj"], gold["ic"], 9, 77.25)
            for ax, ix in resolved(nx, ny, nz)]
    assert len(frames) == len(want)
    for got, exp in zip(frames, want):
        assert got == exp


def test_capture_fp32_device_layout_byte_exact(se, oracle, gold):
    import torch
    nx, ny, nz = (int(v) for v in gold["n"])
    f32 = gold["fwd"].astype(np.float32)
    a32 = gold["adj"].astype(np.float32)
    c32 = gold["ic"].astype(np.float32)
    f = torch.from_numpy(to_device_layout(se, f32, nx, ny, nz)).cuda()
    a = torch.from_numpy(to_device_layout(se, a32, nx, ny, nz)).cuda()
    c = torch.from_numpy(c32).cuda()
    frames = se.capture_slice_frames(nx, ny, nz, SPECS, f, a, c, timestep=3, timestamp=1.5)
    want = [oracle.slice_frame(ax, ix, nx, ny, nz, f32.astype(np.float64), a32.astype(np.float64),
                               c32.astype(np.float64), 3, 1.5) for ax, ix in resolved(nx, ny, nz)]
    for got, exp in zip(frames, want):
        assert got == exp


def _strip_ts(b):
    return b[:100] + b[108:]


def test_slice_stream_file_holds_captures_in_order(se, gold, tmp_path):
    import torch
    from seismic_engine.slices import MmapSnapshotWriter, deserialize_slice
    nx, ny, nz = (int(v) for v in gold["n"])
    f = torch.from_numpy(gold["fwd"]).cuda()
    a = torch.from_numpy(gold["adj"]).cuda()
    c = torch.from_numpy(gold["ic"]).cuda()
    path = str(tmp_path / "stream.dat")
    ss = se.SliceStream(path, nx, ny, nz, specs=SPECS, max_bytes=1 << 20, capacity=8)
    expect = []
    for t in range(6):
        ft = f * (t + 1)
        ss.capture(ft, a, c, timestep=t, field_kind=se.slices.FIELD_REFERENCE_FP64)
        expect += se.capture_slice_frames(nx, ny, nz, SPECS, ft, a, c, timestep=t,
                                          field_kind=se.slices.FIELD_REFERENCE_FP64)
    ss.flush()
    st = ss.stats()
    ss.close()
    assert st["captured"] + st["dropped"] == 6 * 4 and st["written"] == st["captured"]
    assert MmapSnapshotWriter.count_frames(path) == st["written"]
    got = [MmapSnapshotWriter.read_frame(path, k) for k in range(st["written"])]
    if st["dropped"] == 0:
        assert [_strip_ts(g) for g in got] == [_strip_ts(e) for e in expect]
    for g in got:
        assert deserialize_slice(g) is not None  # checksum and magic hold


def test_configure_rtm_streams_shot_fields(se, tmp_path):
    import torch
    from seismic_engine.slices import MmapSnapshotWriter, deserialize_slice
    w = se.workloads.small_case(n=(20, 18, 22), nt=11, seed=5, sponge_width=4)
    s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d),
                              se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width,
                                              sponge_damping=w.sponge_damping))
    s.set_velocity_field(se.workloads.to_reference_layout(w.vel))
    path = str(tmp_path / "rtm.dat")
    s.configure_rtm(se.RTMConfig(enable_rtm=True, enable_mmap_writer=True, mmap_filename=path,
                                 mmap_max_bytes=1 << 22, snapshot_interval=5))
    sh = w.shots[0]
    seis = torch.zeros((w.nt, sh.rec.count), device="cuda")
    assert se.shot_forward(s, sh.src, sh.wavelet, w.nt, sh.rec, seis=seis) == 0
    torch.cuda.synchronize()
    cur = s.get_field(se._lib.ST_FIELD_CURRENT).reshape(w.nx + 2, w.ny + 2, w.nz + 2)
    s.slice_stream().flush()
    frames = [deserialize_slice(MmapSnapshotWriter.read_frame(path, k)) for k in range(9)]
    assert all(fr is not None for fr in frames)
    assert [fr.timestep for fr in frames] == [0] * 3 + [5] * 3 + [10] * 3
    assert [int(fr.axis) for fr in frames[:3]] == [2, 1, 0]  # default specs: Z, Y, X
    last_z = frames[6]
    assert last_z.index == w.nz // 2
    np.testing.assert_array_equal(last_z.forward_slice, cur[1:-1, 1:-1, 1 + w.nz // 2])
    assert not last_z.adjoint_slice.any() and not last_z.ic_slice.any()
    # RTM: the imaging pass captures (forward snapshot, adjoint field, image so far)
    data = torch.randn((w.nt, sh.rec.count), device="cuda") * 1e-3
    image = torch.zeros(w.points, device="cuda")
    illum = torch.zeros(w.points, device="cuda")
    n0 = MmapSnapshotWriter.count_frames(path)
    assert se.rtm_shot(s, sh.src, sh.wavelet, w.nt, sh.rec, data, image, illum,
                       snap_kind=se._lib.ST_SNAP_FP32) == 0
    torch.cuda.synchronize()
    s.slice_stream().flush()
    n1 = MmapSnapshotWriter.count_frames(path)
    # the imaging pass runs backward in time: captures at t = 10, 5, 0, 3 specs each
    assert n1 - n0 == 9
    rtm = [deserialize_slice(MmapSnapshotWriter.read_frame(path, k)) for k in range(n0, n1)]
    assert [fr.timestep for fr in rtm] == [10] * 3 + [5] * 3 + [0] * 3
    final = rtm[-1]  # X slice at t = 0: the image is complete
    n = final.dim0 * final.dim1
    np.testing.assert_array_equal(final.ic_slice.ravel(), image.cpu().numpy()[:n].astype(np.float64))
    assert np.abs(final.adjoint_slice).max() > 0 and np.abs(final.forward_slice).max() > 0
    s.shutdown_rtm_resources()
    s.close()
