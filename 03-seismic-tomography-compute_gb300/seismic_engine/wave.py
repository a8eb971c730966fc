"""Propagator face of seismic_engine: the reference's types and the
WaveEquationSolver class (solver/wave_equation.h:16-144), plus the fused shot
entry points that take torch device tensors without copies.

Every call goes through libseismic_gb300.so; fields returned by `field()` are
FP64 numpy arrays in the reference's halo-padded layout.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field as dc_field

import numpy as np

from . import _lib
from ._lib import call


class StepResult(enum.IntEnum):
    """seismic::StepResult (solver/wave_equation.h:24-29)."""
    OK = 0
    NAN_DETECTED_AND_REPAIRED = 1
    CFL_VIOLATION = 2
    FATAL_DIVERGENCE = 3


class HealthStatus(enum.IntEnum):
    """seismic::HealthStatus (core/fault_tolerance.h:13-20)."""
    HEALTHY = 0
    NAN_DETECTED = 1
    INF_DETECTED = 2
    CFL_VIOLATION = 3
    DIVERGENCE = 4
    COMM_FAILURE = 5


@dataclass
class GridParams:
    """seismic::GridParams (core/grid.h:9-20)."""
    nx_global: int
    ny_global: int
    nz_global: int
    dx: float
    dy: float
    dz: float
    origin_x: float = 0.0
    origin_y: float = 0.0
    origin_z: float = 0.0
    halo_width: int = 1

    def c(self) -> _lib.GridParams:
        return _lib.GridParams(self.nx_global, self.ny_global, self.nz_global, self.dx, self.dy, self.dz,
                               self.origin_x, self.origin_y, self.origin_z, self.halo_width)


@dataclass
class SolverConfig:
    """seismic::SolverConfig (core/config.h:9-19), defaults of load_config
    (core/config.cpp:12-20)."""
    frequency: float = 2.0
    dt: float = 0.001
    nt: int = 5000
    water_depth: float = 4000.0
    seafloor_gradient: float = 0.05
    sponge_width: int = 20
    sponge_damping: float = 0.015
    snapshot_interval: int = 100
    output_dir: str = "./output"
    # "reference": the reference's sponge rule (diverges for wide sponges);
    # "stable": the new field is damped (Cerjan form). Not a reference key.
    sponge_mode: str = "reference"

    def c(self) -> _lib.SolverConfigC:
        return _lib.SolverConfigC(self.frequency, self.dt, self.nt, self.water_depth, self.seafloor_gradient,
                                  self.sponge_width, self.sponge_damping, self.snapshot_interval)


@dataclass
class PropagationResult:
    """seismic::PropagationResult (solver/wave_equation.h:31-37)."""
    status: StepResult
    total_nan_encountered: int
    total_cells_repaired: int
    timesteps_completed: int
    completed_successfully: bool


@dataclass
class FaultStats:
    """seismic::FaultTolerance::FaultStats (core/fault_tolerance.h:61-67)."""
    total_nan_count: int = 0
    total_inf_count: int = 0
    cells_repaired: int = 0
    timesteps_recovered: int = 0
    global_abort_count: int = 0


@dataclass
class WaveField:
    """seismic::WaveField (solver/wave_equation.h:16-22), FP64 host copies."""
    current: np.ndarray
    previous: np.ndarray
    next: np.ndarray
    velocity: np.ndarray
    snapshots: np.ndarray = dc_field(default_factory=lambda: np.zeros(0))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def field_layout(nx: int, ny: int, nz: int) -> dict:
    out = (C.c_int64 * 6)()
    call("st_field_layout", nx, ny, nz, out)
    return dict(NXh=out[0], NYh=out[1], NZP=out[2], ZOFF=out[3], plane=out[4], elems=out[5])


class WaveEquationSolver:
    """seismic::WaveEquationSolver over the GPU library. The constructor takes
    (grid, config) like the reference's (mpi, grid, config) minus the MPI
    context: one device-resident domain, no halo exchange."""

    def __init__(self, grid: GridParams, config: SolverConfig, device: int = 0):
        self._grid = grid
        self._cfg = config
        h = C.c_void_p()
        call("st_solver_create", C.byref(grid.c()), C.byref(config.c()), device, C.byref(h), allow_status=False)
        self._h = h
        self.set_sponge_mode(getattr(config, "sponge_mode", "reference"))
        self.nx, self.ny, self.nz = grid.nx_global, grid.ny_global, grid.nz_global
        self.padded_size = (self.nx + 2) * (self.ny + 2) * (self.nz + 2)

    def close(self):
        if getattr(self, "_h", None):
            self.shutdown_rtm_resources()
            _lib.load().st_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_sponge_mode(self, mode):
        """'reference' (default, the reference's rule) or 'stable' (Cerjan form)."""
        m = {"reference": _lib.ST_SPONGE_REFERENCE, "stable": _lib.ST_SPONGE_STABLE}.get(mode, mode)
        call("st_solver_set_sponge_mode", self._h, int(m))

    def sponge_mode(self) -> str:
        m = C.c_int()
        call("st_solver_sponge_mode", self._h, C.byref(m))
        return "stable" if m.value == _lib.ST_SPONGE_STABLE else "reference"

    def grid(self) -> GridParams:
        return self._grid

    def config(self) -> SolverConfig:
        return self._cfg

    # ---- reference API (wave_equation.h:57-110)
    def initialize_velocity(self, vp0: float):
        call("st_solver_initialize_velocity", self._h, float(vp0))

    def set_velocity_field(self, vp, count: int | None = None):
        a = np.ascontiguousarray(vp, dtype=np.float64).reshape(-1)
        n = a.size if count is None else int(count)
        call("st_solver_set_velocity_field", self._h, _dptr(a), min(n, a.size))

    def inject_source(self, ix: int, iy: int, iz: int, wavelet):
        w = np.ascontiguousarray(wavelet, dtype=np.float64).reshape(-1)
        if w.size == 0:
            return
        call("st_solver_inject_source", self._h, ix, iy, iz, _dptr(w), w.size)

    def step_forward(self, timestep: int) -> StepResult:
        return StepResult(call("st_solver_step_forward", self._h, timestep))

    def step_adjoint(self, timestep: int) -> StepResult:
        return StepResult(call("st_solver_step_adjoint", self._h, timestep))

    def _prop(self, name, w):
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(-1)
        if w.size == 0:
            w = np.zeros(1)
            n = 0
        else:
            n = w.size
        r = _lib.PropagationResultC()
        call(name, self._h, _dptr(w), n, C.byref(r))
        return PropagationResult(StepResult(r.status), r.total_nan_encountered, r.total_cells_repaired,
                                 r.timesteps_completed, bool(r.completed_successfully))

    def forward_propagate(self, wavelet) -> PropagationResult:
        return self._prop("st_solver_forward_propagate", wavelet)

    def adjoint_propagate(self, residual_wavelet) -> PropagationResult:
        return self._prop("st_solver_adjoint_propagate", residual_wavelet)

    def reset_field(self):
        call("st_solver_reset_field", self._h)

    def get_field(self, which: int) -> np.ndarray:
        out = np.empty(self.padded_size)
        call("st_solver_get_field", self._h, which, _dptr(out), out.size)
        return out

    def set_field(self, which: int, values):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        call("st_solver_set_field", self._h, which, _dptr(a), a.size)

    def field(self) -> WaveField:
        return WaveField(self.get_field(_lib.ST_FIELD_CURRENT), self.get_field(_lib.ST_FIELD_PREVIOUS),
                         self.get_field(_lib.ST_FIELD_NEXT), self.get_field(_lib.ST_FIELD_VELOCITY),
                         self.snapshots())

    def snapshots(self) -> np.ndarray:
        n = C.c_int64()
        call("st_solver_snapshot_values", self._h, C.byref(n))
        out = np.empty(n.value)
        if n.value:
            call("st_solver_get_snapshots", self._h, _dptr(out), out.size)
        return out

    def save_snapshot(self, timestep: int):
        call("st_solver_save_snapshot", self._h, timestep)

    def clear_snapshots(self):
        call("st_solver_clear_snapshots", self._h)

    def compute_energy(self) -> float:
        e = C.c_double()
        call("st_solver_compute_energy", self._h, C.byref(e))
        return e.value

    def verify_cfl(self) -> bool:
        ok = C.c_int()
        call("st_solver_verify_cfl", self._h, C.byref(ok))
        return bool(ok.value)

    def set_amplitude_limit(self, limit: float):
        call("st_solver_set_amplitude_limit", self._h, float(limit))

    def amplitude_limit(self) -> float:
        v = C.c_double()
        call("st_solver_amplitude_limit", self._h, C.byref(v))
        return v.value

    def nan_count_current(self) -> int:
        v = C.c_int64()
        call("st_solver_nan_count_current", self._h, C.byref(v))
        return v.value

    def fault_stats(self) -> FaultStats:
        s = _lib.FaultStatsC()
        call("st_solver_fault_stats", self._h, C.byref(s))
        return FaultStats(s.total_nan_count, s.total_inf_count, s.cells_repaired, s.timesteps_recovered,
                          s.global_abort_count)

    # ---- terrain-aware propagation (GB300 addition)
    def set_terrain(self, terrain, free_surface: bool = True, seafloor: bool = True):
        """Attach a TerrainBoundary: every step then zeroes, in each (x, y)
        column, the points above the free-surface plane and / or the seafloor
        index, right after the update (fused into the stencil). The limits
        are copied; terrain=None detaches. The exact-adjoint entry points
        refuse while a terrain is attached."""
        flags = (_lib.ST_TERRAIN_FREE_SURFACE if free_surface else 0) | (_lib.ST_TERRAIN_SEAFLOOR if seafloor else 0)
        call("st_solver_set_terrain", self._h, terrain.handle if terrain is not None else None,
             flags if terrain is not None else 0)

    # ---- FaultTolerance of the solver (wave_equation.h:84-85, 94)
    def fault_tolerance(self) -> "FaultTolerance":
        """The solver's FaultTolerance (core/fault_tolerance.h:31-97)."""
        return FaultTolerance(self)

    # ---- RTM driver (wave_equation.h:96-110, wave_equation.cpp:508-688)
    def configure_rtm(self, cfg):
        """WaveEquationSolver::configure_rtm: releases the previous RTM
        resources; with enable_rtm or enable_snapshots, creates the solver's
        RTMEngine and, with enable_mmap_writer, a GPU slice stream on
        cfg.mmap_filename that captures cfg.slice_specs (default: the middle
        Z, Y and X planes) every cfg.snapshot_interval steps of shot_forward,
        rtm_shot and run_rtm, and at apply_rtm_step(t, True)."""
        from .slices import _specs_c
        specs = list(cfg.slice_specs or [])
        arr, n = _specs_c(specs)
        r = cfg.receivers
        rc = _lib.ReceiverGridC(r.x0, r.sx, r.nx, r.y0, r.sy, r.ny, r.z) if r is not None \
            else _lib.ReceiverGridC(0, 1, 0, 0, 1, 0, 0)
        fname = cfg.mmap_filename.encode() if cfg.mmap_filename else None
        c = _lib.RtmConfigC(int(bool(cfg.enable_rtm)), int(bool(cfg.enable_snapshots)), int(cfg.snapshot_interval),
                            int(bool(cfg.enable_mmap_writer)), fname, int(cfg.mmap_max_bytes),
                            int(cfg.ring_buffer_capacity), arr if n else None, n, rc, int(cfg.snap_kind),
                            int(cfg.checkpoint_segment))
        self._rtm_engine = None
        self._slices = None
        call("st_solver_configure_rtm", self._h, C.byref(c))
        self._rtm_cfg = cfg

    def rtm_config(self):
        """The RTMConfig of the last configure_rtm (a default one before)."""
        from .rtm import RTMConfig
        return getattr(self, "_rtm_cfg", None) or RTMConfig()

    def rtm_engine(self):
        """The solver's RTMEngine (image, illumination, reflectivity of
        run_rtm / apply_rtm_step), or None while RTM is disabled."""
        from .rtm import RTMEngine
        h = C.c_void_p()
        call("st_solver_rtm_engine", self._h, C.byref(h))
        if not h.value:
            return None
        eng = getattr(self, "_rtm_engine", None)
        if eng is None or eng._h is None or eng._h.value != h.value:
            eng = RTMEngine._borrow(h, (self.nx, self.ny, self.nz), self)
            eng.set_slice_specs(self.rtm_config().slice_specs)
            self._rtm_engine = eng
        return eng

    def slice_stream(self):
        """The slice stream configure_rtm created (the reference's
        snapshot_buffer() / mmap_writer() pair), or None."""
        from .slices import SliceStream, default_slice_specs
        h = C.c_void_p()
        call("st_solver_rtm_slice_stream", self._h, C.byref(h))
        if not h.value:
            return None
        ss = getattr(self, "_slices", None)
        if ss is None or ss.handle is None or ss.handle.value != h.value:
            cfg = self.rtm_config()
            ss = SliceStream._borrow(h, cfg.mmap_filename, (self.nx, self.ny, self.nz),
                                     list(cfg.slice_specs) or default_slice_specs())
            self._slices = ss
        return ss

    snapshot_buffer = slice_stream
    mmap_writer = slice_stream

    def snapshots_captured(self) -> int:
        c = C.c_int64()
        call("st_solver_rtm_snapshot_counts", self._h, C.byref(c), None)
        return c.value

    def snapshots_dropped(self) -> int:
        d = C.c_int64()
        call("st_solver_rtm_snapshot_counts", self._h, None, C.byref(d))
        return d.value

    def store_forward_wavefield_for_rtm(self, timestep: int):
        call("st_solver_store_forward_wavefield_for_rtm", self._h, int(timestep))

    def apply_rtm_step(self, timestep: int, with_snapshot: bool):
        call("st_solver_apply_rtm_step", self._h, int(timestep), int(bool(with_snapshot)))

    def run_rtm(self, source_wavelet, receiver_residuals) -> PropagationResult:
        """WaveEquationSolver::run_rtm as true reverse-time migration: the
        source wavelet at the domain centre, receiver_residuals FP64
        [nt][nrec] (time-major; the receivers of rtm_config().receivers, by
        default every interior cell of the plane z = 0). Afterwards
        rtm_engine().result() holds the image. Without enable_rtm /
        enable_snapshots it does nothing and reports success, as the
        reference."""
        w = np.ascontiguousarray(source_wavelet, dtype=np.float64).reshape(-1)
        r = np.ascontiguousarray(receiver_residuals, dtype=np.float64).reshape(-1)
        nul = C.cast(None, C.POINTER(C.c_double))
        res = _lib.PropagationResultC()
        call("st_solver_run_rtm", self._h, _dptr(w) if w.size else nul, w.size, _dptr(r) if r.size else nul,
             r.size, C.byref(res))
        return PropagationResult(StepResult(res.status), res.total_nan_encountered, res.total_cells_repaired,
                                 res.timesteps_completed, bool(res.completed_successfully))

    def apply_sponge_layer(self):
        """WaveEquationSolver::apply_sponge_layer: current and previous times
        the sponge factor over the sponge band."""
        call("st_solver_apply_sponge_layer", self._h)

    def shutdown_rtm_resources(self):
        """Releases the RTM resources (wave_equation.cpp:562-575); the slice
        stream's file holds every captured frame afterwards."""
        if getattr(self, "_h", None):
            self._rtm_engine = None
            self._slices = None
            call("st_solver_configure_rtm", self._h, None)

    # ---- GB300 additions
    def set_step_fusion(self, steps: int):
        """Adjoint steps per launch of the RTM imaging pass: 2 (default) or 1;
        the results are bit-identical either way."""
        call("st_solver_set_step_fusion", self._h, int(steps))

    def device_field_ptr(self, which: int) -> int:
        p = C.c_void_p()
        call("st_solver_device_field", self._h, which, C.byref(p))
        return p.value

    def stream_ptr(self) -> int:
        p = C.c_void_p()
        call("st_solver_stream", self._h, C.byref(p))
        return p.value or 0

    def set_stream(self, stream):
        """Runs the solver's work on `stream` (a torch.cuda.Stream, a raw
        cudaStream_t as int, or None for the solver's own stream); queued work
        stays ordered before it."""
        ptr = getattr(stream, "cuda_stream", stream)
        call("st_solver_set_stream", self._h, C.c_void_p(int(ptr)) if ptr else None)

    def on_stream(self, stream):
        """Context manager: the solver's work inside runs on `stream` (default:
        torch's current stream), so it is ordered with the surrounding torch
        work without any device-wide synchronisation."""
        import contextlib

        @contextlib.contextmanager
        def cm():
            import torch
            st = stream if stream is not None else torch.cuda.current_stream()
            self.set_stream(st)
            try:
                yield st
            finally:
                self.set_stream(None)
        return cm()


class FaultTolerance:
    """seismic::FaultTolerance (core/fault_tolerance.h:31-97) of a solver:
    its statistics and settings live in the solver handle; the field helpers
    run on the GPU in FP64. One rank: the global checks are the local ones."""

    def __init__(self, solver: WaveEquationSolver):
        self._s = solver

    def stats(self) -> FaultStats:
        return self._s.fault_stats()

    def reset_stats(self):
        call("st_solver_reset_fault_stats", self._s.handle)

    def _get(self, which):
        v = C.c_double()
        call("st_solver_fault_param", self._s.handle, which, C.byref(v))
        return v.value

    def set_max_repair_attempts(self, n: int):
        call("st_solver_set_fault_param", self._s.handle, _lib.ST_FT_MAX_REPAIR_ATTEMPTS, float(n))

    def max_repair_attempts(self) -> int:
        return int(self._get(_lib.ST_FT_MAX_REPAIR_ATTEMPTS))

    def set_amplitude_limit(self, limit: float):
        call("st_solver_set_fault_param", self._s.handle, _lib.ST_FT_AMPLITUDE_LIMIT, float(limit))

    def amplitude_limit(self) -> float:
        return self._get(_lib.ST_FT_AMPLITUDE_LIMIT)

    def set_cfl_safety_factor(self, factor: float):
        call("st_solver_set_fault_param", self._s.handle, _lib.ST_FT_CFL_SAFETY_FACTOR, float(factor))

    def cfl_safety_factor(self) -> float:
        return self._get(_lib.ST_FT_CFL_SAFETY_FACTOR)

    def verify_cfl_condition(self, velocity, count, dx, dy, dz, dt, cfl_limit=0.5) -> bool:
        """fault_tolerance.cpp:49-70: max finite velocity * dt / d <= cfl_limit on every axis."""
        v = np.asarray(velocity, np.float64).reshape(-1)[:int(count)]
        v = v[np.isfinite(v)]
        vmax = max(0.0, float(v.max())) if v.size else 0.0
        return max(vmax * dt / dx, vmax * dt / dy, vmax * dt / dz) <= cfl_limit

    def global_health_check(self, local_status) -> int:
        return int(local_status)

    def global_health_check_field(self, data, count=None) -> int:
        from .fields import check_field_health
        a = np.asarray(data, np.float64).reshape(-1)
        return 1 if check_field_health(a if count is None else a[:int(count)]) > 0 else 0

    @staticmethod
    def count_nan_inf(data, count=None) -> int:
        from .fields import check_field_health
        a = np.asarray(data, np.float64).reshape(-1)
        return check_field_health(a if count is None else a[:int(count)])

    @staticmethod
    def is_valid_double(v) -> bool:
        return bool(np.isfinite(v))

    @staticmethod
    def safe_clamp(v, lo, hi) -> float:
        return 0.0 if not np.isfinite(v) else float(max(lo, min(v, hi)))

    @staticmethod
    def clamp_field(data, lo, hi):
        from .fields import clamp_field_safe
        return clamp_field_safe(data, lo, hi)

    def repair_field_nan(self, data, nx, ny, nz, halo_width=1, replace_value=0.0):
        from .fields import repair_field_nan
        return repair_field_nan(data, nx, ny, nz, halo_width, replace_value)


def _shot_c(src, wavelet: np.ndarray, nt: int, rec):
    w = np.ascontiguousarray(wavelet, dtype=np.float64).reshape(-1)
    rc = _lib.ReceiverGridC(rec.x0, rec.sx, rec.nx, rec.y0, rec.sy, rec.ny, rec.z) if rec is not None \
        else _lib.ReceiverGridC(0, 1, 0, 0, 1, 0, 0)
    shot = _lib.ShotC(int(src[0]), int(src[1]), int(src[2]), _dptr(w), w.size, int(nt), rc)
    return shot, w


def shot_forward(solver: WaveEquationSolver, src, wavelet, nt: int, rec, seis=None, snap_kind: int = 0,
                 snaps=None, snap_amax=None) -> int:
    """Fused forward shot on the solver's stream. seis / snaps / snap_amax are
    torch CUDA tensors (or None); returns the StepResult code."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    sp = seis.data_ptr() if seis is not None else None
    snp = snaps.data_ptr() if snaps is not None else None
    amp = snap_amax.data_ptr() if snap_amax is not None else None
    return call("st_shot_forward", solver.handle, C.byref(shot), sp, snap_kind, snp, amp)


def shot_adjoint(solver: WaveEquationSolver, src, nt: int, rec, data, src_trace) -> int:
    """Exact adjoint of shot_forward: data (torch CUDA FP32 [nt, nrec]) ->
    src_trace (torch CUDA FP32 [nt]) = d<seismograms, data>/d wavelet."""
    shot, _keep = _shot_c(src, np.zeros(1), nt, rec)
    return call("st_shot_adjoint", solver.handle, C.byref(shot), data.data_ptr(), src_trace.data_ptr())


def rtm_shot(solver: WaveEquationSolver, src, wavelet, nt: int, rec, data, image, illum, refl=None,
             snap_kind: int = _lib.ST_SNAP_BF16, snaps=None, snap_amax=None) -> int:
    """Reverse-time migration of one shot on device tensors: data FP32
    [nt, nrec]; image / illum / refl FP32 interior (nx*ny*nz) outputs. With
    snaps=None the library keeps its own snapshot store."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    return call("st_rtm_shot", solver.handle, C.byref(shot), data.data_ptr(), snap_kind, ptr(snaps),
                ptr(snap_amax), image.data_ptr(), illum.data_ptr(), ptr(refl))


def _stats_dict(st) -> dict:
    return {k: getattr(st, k) for k, _ in _lib.CheckpointStatsC._fields_}


def rtm_shot_checkpointed(solver: WaveEquationSolver, src, wavelet, nt: int, rec, data, image, illum, refl=None,
                          snap_kind: int = _lib.ST_SNAP_BF16, segment_steps: int = 100, max_slots: int = 1 << 30):
    """rtm_shot without the nt-snapshot store: FP32 forward states are kept
    at segment boundaries (at most max_slots of them, binomial schedule) and
    each segment is recomputed into a segment_steps-snapshot buffer. Same
    result as rtm_shot with the same snap_kind. Returns the schedule's
    statistics (forward / adjoint steps run, state copies, device bytes)."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    st = _lib.CheckpointStatsC()
    call("st_rtm_shot_checkpointed", solver.handle, C.byref(shot), data.data_ptr(), snap_kind, int(segment_steps),
         int(max_slots), image.data_ptr(), illum.data_ptr(), refl.data_ptr() if refl is not None else None,
         C.byref(st))
    return _stats_dict(st)


def rtm_shot_host(solver: WaveEquationSolver, vel_ref, src, wavelet, nt: int, rec, data_host,
                  snap_kind: int = _lib.ST_SNAP_BF16, want=("image", "illumination", "reflectivity"), out=None):
    """Host-buffer RTM (every copy included). data_host: FP32 numpy [nt, nrec]
    (pinned memory gives full copy speed). Returns a dict of FP64 interior
    arrays named like RTMImageCondition (rtm/rtm_engine.h:25-29); `out` may
    supply them (C-contiguous float64 arrays of nx*ny*nz values, e.g. pinned
    buffers reused across shots)."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    n = solver.nx * solver.ny * solver.nz
    outs = {}
    for k in want:
        a = None if out is None else out.get(k)
        if a is None:
            a = np.empty(n)
        elif not (a.dtype == np.float64 and a.flags.c_contiguous and a.size == n):
            raise ValueError(f"out[{k!r}] must be a C-contiguous float64 array of {n} values")
        outs[k] = a
    nul = C.cast(None, C.POINTER(C.c_double))
    if vel_ref is None:
        vp, nv = nul, 0
    else:
        v = np.ascontiguousarray(vel_ref, dtype=np.float64).reshape(-1)
        vp, nv = _dptr(v), v.size
    d = data_host if isinstance(data_host, np.ndarray) else data_host.numpy()
    assert d.dtype == np.float32 and d.flags.c_contiguous
    call("st_rtm_shot_host", solver.handle, vp, nv, C.byref(shot), d.ctypes.data_as(C.POINTER(C.c_float)),
         snap_kind, *(_dptr(outs[k]) if k in outs else nul for k in ("image", "illumination", "reflectivity")))
    return outs


def shot_forward_host(solver: WaveEquationSolver, vel_ref, src, wavelet, nt: int, rec) -> np.ndarray:
    """Host-buffer forward shot (all copies included): velocity in the
    reference layout (or None), returns FP64 seismograms [nt, nrec]."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    nrec = rec.nx * rec.ny if rec is not None else 0
    out = np.zeros((nt, max(nrec, 1)))
    if vel_ref is None:
        vp, n = C.cast(None, C.POINTER(C.c_double)), 0
    else:
        v = np.ascontiguousarray(vel_ref, dtype=np.float64).reshape(-1)
        vp, n = _dptr(v), v.size
    call("st_shot_forward_host", solver.handle, vp, n, C.byref(shot), _dptr(out))
    return out[:, :nrec]
