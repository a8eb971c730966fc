"""RTM slice frames and the mmap slice ring: the reference's visualisation
stream (RTMEngine::extract_slices / capture_single_slice,
rtm/rtm_engine.cpp:59-168; LockFreeSnapshotBuffer::serialize_slice /
deserialize_slice / compute_checksum, rtm/snapshot_buffer.cpp:102-229;
MmapSnapshotWriter, rtm/mmap_writer.h:26-124) with the names of the
reference's binding (pybind/bindings.cpp:303-377).

Frames are captured on the GPU (`capture_slice_frames`, `SliceStream`) and
written by the library's C++ ring writer (`MmapSnapshotWriter`); this module
also reads them back (`deserialize_slice`, `MmapSnapshotWriter.read_frame`).
The file and frame layouts are documented in include/seismic_gb300.h.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
from dataclasses import dataclass, field

import numpy as np

from ._lib import SliceSpecC, call
from .rtm import SliceAxis, SliceSpec

DEFAULT_MMAP_MAX_BYTES = 4 * 1024 * 1024 * 1024   # mmap_writer.h:26
MMAP_FILE_MAGIC = 0x52544D534E4150                 # mmap_writer.h:27
MMAP_HEADER_SIZE = 120                             # sizeof(MmapFileHeader), packed
SLICE_HEADER_SIZE = 128                            # snapshot_buffer.h:16
FRAME_MAGIC = 0x534C494345303031                   # snapshot_buffer.cpp:107

# SliceFrameHeader (snapshot_buffer.h:18-38), packed little-endian: 124 bytes
_FRAME_HEADER = struct.Struct("<QqiqqqqqqqqqqdQII")

FIELD_DEVICE_FP32 = 0
FIELD_REFERENCE_FP64 = 1
IMAGE_FP32 = 0
IMAGE_FP64 = 1


def _specs_c(specs):
    specs = list(specs)
    arr = (SliceSpecC * max(len(specs), 1))()
    for k, sp in enumerate(specs):
        if isinstance(sp, SliceSpec):
            arr[k] = SliceSpecC(int(sp.axis), int(sp.index), int(sp.stride))
        else:
            ax, ix = sp[0], sp[1]
            arr[k] = SliceSpecC(int(ax), int(ix), 1)
    return arr, len(specs)


def default_slice_specs():
    """The specs configure_rtm installs when none are given
    (wave_equation.cpp:529-535): the middle Z, Y and X planes."""
    return [SliceSpec(SliceAxis.Z, -1, 1), SliceSpec(SliceAxis.Y, -1, 1), SliceSpec(SliceAxis.X, -1, 1)]


@dataclass
class CapturedSlice:
    """RTMEngine::CapturedSlice (rtm_engine.h:62-72)."""
    timestep: int
    axis: SliceAxis
    index: int
    dim0: int
    dim1: int
    capture_timestamp: float
    forward_slice: np.ndarray = field(repr=False)
    adjoint_slice: np.ndarray = field(repr=False)
    ic_slice: np.ndarray = field(repr=False)


def slice_checksum(payload) -> int:
    """compute_checksum (snapshot_buffer.cpp:207-229): s = rotl13(s ^ w) over
    the little-endian 32-bit words, the trailing bytes XORed in unrotated.
    Evaluated in closed form: word j of n is rotated by 13 (n - j) mod 32."""
    b = np.frombuffer(bytes(payload), np.uint8)
    n = b.size // 4
    w = b[:4 * n].view("<u4").astype(np.uint64)
    r = (13 * (n - np.arange(n, dtype=np.uint64))) % np.uint64(32)
    rot = ((w << r) | (w >> ((np.uint64(32) - r) % np.uint64(32)))) & np.uint64(0xFFFFFFFF)
    s = int(np.bitwise_xor.reduce(rot)) if n else 0
    rest = b[4 * n:]
    if rest.size:
        s ^= int(sum(int(v) << (8 * i) for i, v in enumerate(rest)))
    return s & 0xFFFFFFFF


def deserialize_slice(buf) -> CapturedSlice | None:
    """LockFreeSnapshotBuffer::deserialize_slice (snapshot_buffer.cpp:155-205):
    None when the magic, the size or the checksum does not match."""
    buf = bytes(buf)
    if len(buf) < SLICE_HEADER_SIZE:
        return None
    (magic, timestep, axis, index, d0, d1, size, fo, ao, io, fb, ab, ib, ts, _seq, csum,
     _res) = _FRAME_HEADER.unpack_from(buf, 0)
    if magic != FRAME_MAGIC or size > len(buf):
        return None
    if slice_checksum(buf[SLICE_HEADER_SIZE:size]) != csum:
        return None

    def arr(off, nbytes):
        return np.frombuffer(buf[off:off + nbytes], np.float64).reshape(d0, d1).copy() if nbytes else np.zeros(0)
    return CapturedSlice(timestep, SliceAxis(axis), index, d0, d1, ts, arr(fo, fb), arr(ao, ab), arr(io, ib))


@dataclass
class MmapStats:
    """MmapSnapshotWriter::Stats (mmap_writer.h:63-70)."""
    frames_written: int
    frames_dropped_buffer_full: int
    total_bytes_written: int
    mmap_cycles: int


class MmapSnapshotWriter:
    """seismic::MmapSnapshotWriter (rtm/mmap_writer.h:41-124): the ring file."""

    def __init__(self):
        self._h = None
        self._filename = ""
        self._max = 0

    def open(self, filename: str, max_bytes: int = DEFAULT_MMAP_MAX_BYTES) -> bool:
        self.close()
        h = C.c_void_p()
        call("st_mmap_writer_open", os.fsencode(filename), int(max_bytes), C.byref(h))
        self._h, self._filename, self._max = h, filename, int(max_bytes)
        return True

    def close(self):
        if self._h is not None:
            call("st_mmap_writer_close", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def is_open(self) -> bool:
        return self._h is not None

    def write_frame(self, frame) -> bool:
        if self._h is None:
            return False
        b = bytes(frame)
        if not b:
            return False
        buf = (C.c_uint8 * len(b)).from_buffer_copy(b)
        call("st_mmap_writer_write_frame", self._h, C.cast(buf, C.c_void_p), len(b))
        return True

    def _info(self):
        out = (C.c_int64 * 7)()
        call("st_mmap_writer_info", self._h, out)
        return list(out)

    def frame_count(self) -> int:
        return self._info()[0]

    def write_offset(self) -> int:
        return self._info()[1]

    def used_bytes(self) -> int:
        return self.write_offset()

    def capacity_bytes(self) -> int:
        return self._max

    def filename(self) -> str:
        return self._filename

    def stats(self) -> MmapStats:
        i = self._info()
        return MmapStats(i[3], i[4], i[5], i[6])

    @staticmethod
    def read_frame(filename: str, frame_index: int) -> bytes | None:
        size = C.c_int64()
        try:
            call("st_mmap_read_frame", os.fsencode(filename), int(frame_index), None, 0, C.byref(size))
        except Exception:
            return None
        buf = (C.c_uint8 * size.value)()
        call("st_mmap_read_frame", os.fsencode(filename), int(frame_index), C.cast(buf, C.c_void_p), size.value,
             C.byref(size))
        return bytes(buf)

    @staticmethod
    def count_frames(filename: str) -> int:
        n = C.c_int64()
        try:
            call("st_mmap_count_frames", os.fsencode(filename), C.byref(n))
        except Exception:
            return -1
        return n.value


def frame_bytes(nx: int, ny: int, nz: int, spec) -> int:
    arr, _ = _specs_c([spec])
    return int(call("st_slice_frame_bytes", nx, ny, nz, arr))


def _ptr(t):
    return None if t is None else t.data_ptr()


def capture_slice_frames(nx, ny, nz, specs, fwd, adj, ic=None, timestep: int = 0, timestamp: float = 0.0,
                         field_kind: int = FIELD_DEVICE_FP32) -> list:
    """Serialized frames (bytes) of every spec from CUDA tensors: fwd / adj in
    the device layout (FP32) or the reference layout (FP64) per field_kind,
    ic an FP32 or FP64 interior array (or None). Runs on torch's current
    stream and copies the frames back."""
    import torch
    arr, n = _specs_c(specs)
    sizes = [frame_bytes(nx, ny, nz, sp) for sp in specs]
    total = sum(sizes)
    dev = (fwd if fwd is not None else adj).device
    out = torch.empty(max(total, 8), dtype=torch.uint8, device=dev)
    ic_kind = IMAGE_FP64 if ic is not None and ic.dtype == torch.float64 else IMAGE_FP32
    got = C.c_int64()
    call("st_capture_slice_frames", nx, ny, nz, arr, n, _ptr(fwd), _ptr(adj), field_kind, _ptr(ic), ic_kind,
         int(timestep), float(timestamp), out.data_ptr(), out.numel(), C.byref(got),
         torch.cuda.current_stream(dev).cuda_stream)
    host = out[:got.value].cpu().numpy().tobytes()
    frames, o = [], 0
    for sz in sizes:
        if sz:
            frames.append(host[o:o + sz])
            o += sz
    return frames


class SliceStream:
    """GPU slice capture into an mmap ring (the roles of the reference's
    LockFreeSnapshotBuffer and the writer's drain thread): `capture` enqueues
    the frames of every spec on a CUDA stream; a writer thread appends them
    to the file in capture order; a capture that finds its slot still busy is
    dropped and counted."""

    def __init__(self, filename: str, nx: int, ny: int, nz: int, specs=None,
                 max_bytes: int = DEFAULT_MMAP_MAX_BYTES, capacity: int = 1024, device: int = 0):
        specs = default_slice_specs() if not specs else list(specs)
        arr, n = _specs_c(specs)
        h = C.c_void_p()
        call("st_slice_stream_create", os.fsencode(filename), int(max_bytes), nx, ny, nz, arr, n, int(capacity),
             device, C.byref(h))
        self._h = h
        self.filename = filename
        self.shape = (nx, ny, nz)
        self.specs = specs

    @classmethod
    def _borrow(cls, handle, filename, shape, specs):
        """A view of a stream another object owns (the solver's configure_rtm);
        close() leaves it open."""
        ss = cls.__new__(cls)
        ss._h = handle
        ss._borrowed = True
        ss.filename = filename
        ss.shape = shape
        ss.specs = specs
        return ss

    @property
    def handle(self):
        return self._h

    def capture(self, fwd, adj=None, ic=None, timestep: int = 0, field_kind: int = FIELD_DEVICE_FP32,
                stream=None):
        import torch
        t = fwd if fwd is not None else adj
        st = stream if stream is not None else torch.cuda.current_stream(t.device).cuda_stream
        ic_kind = IMAGE_FP64 if ic is not None and ic.dtype == torch.float64 else IMAGE_FP32
        call("st_slice_stream_capture", self._h, _ptr(fwd), _ptr(adj), field_kind, _ptr(ic), ic_kind, int(timestep),
             st)

    def flush(self):
        call("st_slice_stream_flush", self._h)

    def stats(self) -> dict:
        out = (C.c_int64 * 4)()
        call("st_slice_stream_stats", self._h, out)
        return {"captured": out[0], "dropped": out[1], "written": out[2], "bytes_written": out[3]}

    def close(self):
        if getattr(self, "_h", None) is not None:
            if not getattr(self, "_borrowed", False):
                call("st_slice_stream_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
