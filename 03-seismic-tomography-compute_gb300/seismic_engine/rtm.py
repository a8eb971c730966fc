"""RTM face of seismic_engine: RTMEngine / RTMImageCondition / RTMConfig with
the reference's names (rtm/rtm_engine.h:25-96, solver/wave_equation.h:39-48,
pybind/bindings.cpp:303-371). apply_image_condition runs on the GPU with FP64
accumulators; the fused shot-level RTM is seismic_engine.rtm_shot.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import call

_d = C.POINTER(C.c_double)


class SliceAxis(enum.IntEnum):
    """seismic::SliceAxis (rtm_engine.h:12-17)."""
    X = 0
    Y = 1
    Z = 2
    VOLUME = 3


@dataclass
class SliceSpec:
    """seismic::SliceSpec (rtm_engine.h:19-23); index < 0 = the middle plane.
    Slice capture and the mmap ring are in seismic_engine.slices."""
    axis: SliceAxis = SliceAxis.Z
    index: int = -1
    stride: int = 1


@dataclass
class RTMConfig:
    """seismic::RTMConfig (wave_equation.h:39-48), plus the inputs of the true
    RTM that WaveEquationSolver.run_rtm performs here (no reference
    counterpart): `receivers` (a workloads.ReceiverGrid or an object with x0,
    sx, nx, y0, sy, ny, z; None = every interior cell of the plane z = 0),
    `snap_kind` (forward snapshot storage, ST_SNAP_*; 0 = BF16 with a
    per-snapshot scale) and `checkpoint_segment` (binomial checkpointing with
    segments of that many steps; 0 = store every step)."""
    enable_rtm: bool = False
    enable_snapshots: bool = False
    snapshot_interval: int = 50
    enable_mmap_writer: bool = False
    mmap_filename: str = "rtm_snapshots.dat"
    mmap_max_bytes: int = 2 * 1024 * 1024 * 1024
    ring_buffer_capacity: int = 1024
    slice_specs: list = field(default_factory=list)
    receivers: object = None
    snap_kind: int = 0
    checkpoint_segment: int = 0


@dataclass
class RTMImageCondition:
    """seismic::RTMImageCondition (rtm_engine.h:25-29)."""
    image: np.ndarray
    illumination: np.ndarray
    reflectivity: np.ndarray


class RTMEngine:
    """seismic::RTMEngine (rtm_engine.h:31-96) on the GPU."""

    def __init__(self, nx, ny, nz, dx, dy, dz, halo_width=1, device=0):
        h = C.c_void_p()
        call("st_rtm_engine_create", nx, ny, nz, dx, dy, dz, halo_width, device, C.byref(h))
        self._h = h
        self._n = (nx, ny, nz)
        self._specs = []
        self._owner = None

    @classmethod
    def _borrow(cls, handle, n, owner):
        """The engine a solver owns (WaveEquationSolver.rtm_engine()); it
        stays valid while `owner` keeps its RTM configuration."""
        e = cls.__new__(cls)
        e._h = handle
        e._n = n
        e._specs = []
        e._owner = owner
        return e

    def close(self):
        if getattr(self, "_h", None):
            if self._owner is None:
                _lib.load().st_rtm_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nx(self):
        return self._n[0]

    def ny(self):
        return self._n[1]

    def nz(self):
        return self._n[2]

    def total_cells(self):
        return self._n[0] * self._n[1] * self._n[2]

    def set_slice_specs(self, specs):
        self._specs = list(specs)

    def apply_image_condition(self, forward_wavefield, adjoint_wavefield, ny, nz, step_idx=0):
        """ny / nz are the padded extents of the fields (as the reference)."""
        f = np.ascontiguousarray(forward_wavefield, np.float64).reshape(-1)
        a = np.ascontiguousarray(adjoint_wavefield, np.float64).reshape(-1)
        call("st_rtm_engine_apply_image_condition", self._h, f.ctypes.data_as(_d), a.ctypes.data_as(_d), ny, nz,
             step_idx)

    def finalize_image(self):
        call("st_rtm_engine_finalize_image", self._h)

    def reset_image(self):
        call("st_rtm_engine_reset_image", self._h)

    def result(self) -> RTMImageCondition:
        n = self.total_cells()
        im, il, rf = np.empty(n), np.empty(n), np.empty(n)
        call("st_rtm_engine_result", self._h, im.ctypes.data_as(_d), il.ctypes.data_as(_d), rf.ctypes.data_as(_d))
        return RTMImageCondition(im, il, rf)
