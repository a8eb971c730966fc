"""RTM slice frames and the mmap slice ring on the host: the oracle's
restatement of capture_single_slice against the reference's own
RTMEngine::extract_slices output, the checksum's closed form against its
recurrence, and the library's C++ ring writer (host code, no GPU) against
the reference's MmapSnapshotWriter: byte-identical files through two ring
wraps, the same read_frame and count_frames results (golden fixture
tests/golden/slices_small.npz, made by tests/golden/make_golden_slices.py)."""
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def gold(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "slices_small.npz")))


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


def test_oracle_slices_match_reference_extract(oracle, gold):
    nx, ny, nz = (int(v) for v in gold["n"])
    o = 0
    for ax, ix, d0, d1 in gold["meta"]:
        fr = oracle.slice_frame(int(ax), int(ix), nx, ny, nz, gold["fwd"], gold["adj"], gold["ic"], 11)
        n = int(d0 * d1)
        payload = np.frombuffer(fr[128:], np.float64)
        assert np.array_equal(payload, gold["vals"][o:o + 3 * n])
        o += 3 * n
    assert o == gold["vals"].size
    # the VOLUME spec captured nothing; default (-1) indices resolved to n // 2
    assert len(gold["meta"]) == len(gold["specs"]) - 1
    assert [int(m[1]) for m in gold["meta"] if m[0] == 1][0] == ny // 2


def test_checksum_closed_form_matches_recurrence(oracle):
    from seismic_engine.slices import slice_checksum
    rng = np.random.default_rng(1)
    for size in (0, 1, 3, 4, 7, 8, 64, 1001, 4096):
        b = rng.integers(0, 256, size, dtype=np.uint8).tobytes()
        s = 0
        for i in range(size // 4):
            s ^= int.from_bytes(b[4 * i:4 * i + 4], "little")
            s = ((s << 13) | (s >> 19)) & 0xFFFFFFFF
        rest = b[4 * (size // 4):]
        s ^= int.from_bytes(rest, "little") if rest else 0
        assert slice_checksum(b) == s == oracle.slice_checksum(b)


def test_frames_deserialize(oracle, gold):
    from seismic_engine.slices import deserialize_slice
    nx, ny, nz = (int(v) for v in gold["n"])
    fr = oracle.slice_frame(2, 3, nx, ny, nz, gold["fwd"], gold["adj"], gold["ic"], 42, 123.5)
    s = deserialize_slice(fr)
    assert s is not None and s.timestep == 42 and int(s.axis) == 2 and s.index == 3
    assert (s.dim0, s.dim1) == (nx, ny) and s.capture_timestamp == 123.5
    assert np.all(np.isfinite(s.forward_slice)) and np.all(np.isfinite(s.adjoint_slice))
    bad = bytearray(fr)
    bad[200] ^= 1
    assert deserialize_slice(bytes(bad)) is None


def test_ring_writer_byte_identical_to_reference(se, gold, tmp_path):
    from seismic_engine.slices import MmapSnapshotWriter
    sizes = gold["frame_sizes"]
    data = gold["frames"].tobytes()
    path = str(tmp_path / "ring.dat")
    w = MmapSnapshotWriter()
    w.open(path, int(gold["max_bytes"]))
    o = 0
    for sz in sizes:
        assert w.write_frame(data[o:o + int(sz)])
        o += int(sz)
    st = w.stats()
    assert [st.frames_written, st.frames_dropped_buffer_full, st.total_bytes_written, st.mmap_cycles] == \
        [int(v) for v in gold["stats"]]
    assert w.frame_count() == int(gold["count"])
    w.close()
    assert np.array_equal(np.fromfile(path, np.uint8), gold["ring_file"])
    assert MmapSnapshotWriter.count_frames(path) == int(gold["count"])
    reads = gold["reads"].tobytes()
    o = 0
    for k, sz in enumerate(gold["read_sizes"]):
        assert MmapSnapshotWriter.read_frame(path, k) == reads[o:o + int(sz)]
        o += int(sz)
    assert MmapSnapshotWriter.read_frame(path, len(gold["read_sizes"])) is None


def test_ring_writer_refuses_oversize_frames(se, tmp_path):
    from seismic_engine import SeismicError
    from seismic_engine.slices import MmapSnapshotWriter
    w = MmapSnapshotWriter()
    w.open(str(tmp_path / "r.dat"), 1000)
    with pytest.raises(SeismicError):
        w.write_frame(b"x" * 900)  # 120 + 8 + 900 > 1000: the reference would write past its mapping
    assert w.write_frame(b"y" * 800)
    w.close()
    assert MmapSnapshotWriter.count_frames(str(tmp_path / "missing.dat")) == -1
