"""Generates tests/golden/slices_small.npz with the reference's own C++
(oracle/_ref/libseismic_ref.so, built in place from the reference sources by
oracle/build_ref.sh):

  - RTMEngine::extract_slices (rtm/rtm_engine.cpp:59-168) on seeded
    halo-padded fields holding NaN and Inf, for X, Y and Z specs at given
    and default (-1) indices and a VOLUME spec (which captures nothing);
  - MmapSnapshotWriter (rtm/mmap_writer.cpp) writing a sequence of frames
    into a ring small enough to wrap twice: the whole file afterwards, its
    read_frame results and count_frames.

The frames written are serialized by the oracle's restatement of
serialize_slice (the reference's snapshot_buffer.cpp does not compile), so
the file pins the writer, and the extract_slices output pins the gather.

    python tests/golden/make_golden_slices.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from oracle import Oracle, Reference, build_ref  # noqa: E402


def main():
    if build_ref() is None:
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    ref, orc = Reference(), Oracle()
    rng = np.random.default_rng(404)
    nx, ny, nz = 9, 7, 8
    npad = (nx + 2) * (ny + 2) * (nz + 2)
    fwd = rng.standard_normal(npad)
    adj = rng.standard_normal(npad)
    ic = rng.standard_normal(nx * ny * nz)
    fwd[rng.integers(0, npad, 6)] = np.nan
    adj[rng.integers(0, npad, 6)] = np.inf
    ic[rng.integers(0, ic.size, 4)] = -np.inf
    specs = [(0, 2), (1, -1), (2, 5), (2, -1), (0, -1), (3, 0), (1, 6)]
    got = ref.extract_slices(nx, ny, nz, specs, fwd, adj, ic, timestep=11)
    meta = np.array([[a, i, f.shape[0], f.shape[1]] for a, i, f, _, _ in got], np.int64)
    vals = np.concatenate([np.concatenate([f.ravel(), a.ravel(), c.ravel()]) for _, _, f, a, c in got])

    # frames: three captures of the resolved specs at increasing time steps
    frames = []
    for t in (0, 5, 10):
        for a, i, *_ in got:
            frames.append(orc.slice_frame(a, i, nx, ny, nz, fwd * (t + 1), adj, ic, t, 1000.0 + t))
    max_bytes = 120 + 4 * (8 + max(len(f) for f in frames)) + 50
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ring.dat")
        ok, stats = ref.mmap_write(path, max_bytes, frames)
        file_bytes = np.fromfile(path, np.uint8)
        count = ref.mmap_count_frames(path)
        reads = []
        k = 0
        while True:
            f = ref.mmap_read_frame(path, k)
            if f is None:
                break
            reads.append(f)
            k += 1
    sizes = np.array([len(f) for f in frames], np.int64)
    np.savez_compressed(os.path.join(HERE, "slices_small.npz"),
                        n=np.array([nx, ny, nz]), fwd=fwd, adj=adj, ic=ic, specs=np.array(specs, np.int64),
                        timestep=11, meta=meta, vals=vals,
                        frames=np.frombuffer(b"".join(frames), np.uint8), frame_sizes=sizes,
                        max_bytes=max_bytes, accepted=ok, stats=np.array(stats, np.int64), ring_file=file_bytes,
                        count=count, read_sizes=np.array([len(r) for r in reads], np.int64),
                        reads=np.frombuffer(b"".join(reads), np.uint8))
    print(f"slices_small.npz: {len(got)} slices, {len(frames)} frames into a {max_bytes}-byte ring, "
          f"stats {stats}, {len(reads)} readable, count {count}")


if __name__ == "__main__":
    main()
