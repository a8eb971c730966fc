"""Loader and ctypes signatures of the C ABI in include/seismic_gb300.h.

The library is the in-tree build lib/libseismic_gb300.so (build.py). There is
no fallback: when it is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libseismic_gb300.so")

ST_OK = 0
ST_NAN_DETECTED_AND_REPAIRED = 1
ST_CFL_VIOLATION = 2
ST_FATAL_DIVERGENCE = 3
ST_ERR_ARG = -1
ST_ERR_CUDA = -2
ST_ERR_ALLOC = -3
ST_ERR_STATE = -4
ST_ERR_TIMEOUT = -5
ST_ERR_UNSUPPORTED = -6

# flags of st_normal_cg_device's jacobi argument
ST_CG_JACOBI = 1
ST_CG_CONFIRM_TRUE = 2

ST_FIELD_CURRENT, ST_FIELD_PREVIOUS, ST_FIELD_NEXT, ST_FIELD_VELOCITY = 0, 1, 2, 3
ST_SNAP_NONE, ST_SNAP_BF16, ST_SNAP_FP16, ST_SNAP_FP32 = 0, 1, 2, 3
ST_SPONGE_REFERENCE, ST_SPONGE_STABLE = 0, 1
ST_TERRAIN_FREE_SURFACE, ST_TERRAIN_SEAFLOOR = 1, 2
ST_FT_MAX_REPAIR_ATTEMPTS, ST_FT_AMPLITUDE_LIMIT, ST_FT_CFL_SAFETY_FACTOR = 0, 1, 2


class SeismicError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"seismic_gb300 error {code}: {msg}")
        self.code = code


class GridParams(C.Structure):
    _fields_ = [("nx_global", C.c_int64), ("ny_global", C.c_int64), ("nz_global", C.c_int64),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("origin_x", C.c_double), ("origin_y", C.c_double), ("origin_z", C.c_double),
                ("halo_width", C.c_int)]


class SolverConfigC(C.Structure):
    _fields_ = [("frequency", C.c_double), ("dt", C.c_double), ("nt", C.c_int), ("water_depth", C.c_double),
                ("seafloor_gradient", C.c_double), ("sponge_width", C.c_int), ("sponge_damping", C.c_double),
                ("snapshot_interval", C.c_int)]


class PropagationResultC(C.Structure):
    _fields_ = [("status", C.c_int), ("total_nan_encountered", C.c_int64), ("total_cells_repaired", C.c_int64),
                ("timesteps_completed", C.c_int), ("completed_successfully", C.c_int)]


class FaultStatsC(C.Structure):
    _fields_ = [("total_nan_count", C.c_int64), ("total_inf_count", C.c_int64), ("cells_repaired", C.c_int64),
                ("timesteps_recovered", C.c_int64), ("global_abort_count", C.c_int)]


class ReceiverGridC(C.Structure):
    _fields_ = [("x0", C.c_int64), ("sx", C.c_int64), ("nx", C.c_int64),
                ("y0", C.c_int64), ("sy", C.c_int64), ("ny", C.c_int64), ("z", C.c_int64)]


class CheckpointStatsC(C.Structure):
    _fields_ = [("forward_steps", C.c_int64), ("adjoint_steps", C.c_int64), ("state_copies", C.c_int64),
                ("segments", C.c_int), ("segment_steps", C.c_int), ("slots_used", C.c_int),
                ("device_bytes", C.c_int64)]


class ShotC(C.Structure):
    _fields_ = [("src_ix", C.c_int64), ("src_iy", C.c_int64), ("src_iz", C.c_int64),
                ("wavelet", C.POINTER(C.c_double)), ("wavelet_len", C.c_int64), ("nt", C.c_int),
                ("rec", ReceiverGridC)]


class SliceSpecC(C.Structure):
    _fields_ = [("axis", C.c_int32), ("index", C.c_int64), ("stride", C.c_int64)]


class RtmConfigC(C.Structure):
    _fields_ = [("enable_rtm", C.c_int), ("enable_snapshots", C.c_int), ("snapshot_interval", C.c_int),
                ("enable_mmap_writer", C.c_int), ("mmap_filename", C.c_char_p), ("mmap_max_bytes", C.c_int64),
                ("ring_buffer_capacity", C.c_int64), ("slice_specs", C.POINTER(SliceSpecC)),
                ("n_slice_specs", C.c_int), ("receivers", ReceiverGridC), ("snap_kind", C.c_int),
                ("checkpoint_segment", C.c_int)]


class BathymetryPointC(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("depth", C.c_double)]


class RayModelC(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("origin_x", C.c_double), ("origin_y", C.c_double), ("origin_z", C.c_double)]


_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)
_i64 = C.POINTER(C.c_int64)
_vp = C.c_void_p

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "st_last_error": [],
    "st_version": [],
    "st_device_count": [C.POINTER(C.c_int)],
    "st_field_layout": [C.c_int64, C.c_int64, C.c_int64, _i64],
    "st_solver_create": [C.POINTER(GridParams), C.POINTER(SolverConfigC), C.c_int, C.POINTER(_vp)],
    "st_solver_destroy": [_vp],
    "st_solver_initialize_velocity": [_vp, C.c_double],
    "st_solver_set_velocity_field": [_vp, _d, C.c_int64],
    "st_solver_inject_source": [_vp, C.c_int64, C.c_int64, C.c_int64, _d, C.c_int64],
    "st_solver_step_forward": [_vp, C.c_int],
    "st_solver_step_adjoint": [_vp, C.c_int],
    "st_solver_forward_propagate": [_vp, _d, C.c_int64, C.POINTER(PropagationResultC)],
    "st_solver_adjoint_propagate": [_vp, _d, C.c_int64, C.POINTER(PropagationResultC)],
    "st_solver_reset_field": [_vp],
    "st_solver_get_field": [_vp, C.c_int, _d, C.c_int64],
    "st_solver_set_field": [_vp, C.c_int, _d, C.c_int64],
    "st_solver_set_sponge_mode": [_vp, C.c_int],
    "st_solver_sponge_mode": [_vp, C.POINTER(C.c_int)],
    "st_solver_compute_energy": [_vp, _d],
    "st_solver_verify_cfl": [_vp, C.POINTER(C.c_int)],
    "st_solver_set_amplitude_limit": [_vp, C.c_double],
    "st_solver_amplitude_limit": [_vp, _d],
    "st_solver_nan_count_current": [_vp, _i64],
    "st_solver_save_snapshot": [_vp, C.c_int],
    "st_solver_clear_snapshots": [_vp],
    "st_solver_snapshot_values": [_vp, _i64],
    "st_solver_get_snapshots": [_vp, _d, C.c_int64],
    "st_solver_fault_stats": [_vp, C.POINTER(FaultStatsC)],
    "st_solver_reset_fault_stats": [_vp],
    "st_solver_set_wait_test": [_vp, C.c_ulonglong, C.c_int],
    "st_solver_set_fault_param": [_vp, C.c_int, C.c_double],
    "st_solver_fault_param": [_vp, C.c_int, _d],
    "st_solver_configure_rtm": [_vp, C.POINTER(RtmConfigC)],
    "st_solver_rtm_engine": [_vp, C.POINTER(_vp)],
    "st_solver_rtm_slice_stream": [_vp, C.POINTER(_vp)],
    "st_solver_rtm_snapshot_counts": [_vp, _i64, _i64],
    "st_solver_store_forward_wavefield_for_rtm": [_vp, C.c_int],
    "st_solver_apply_rtm_step": [_vp, C.c_int, C.c_int],
    "st_solver_run_rtm": [_vp, _d, C.c_int64, _d, C.c_int64, C.POINTER(PropagationResultC)],
    "st_solver_apply_sponge_layer": [_vp],
    "st_solver_device_field": [_vp, C.c_int, C.POINTER(_vp)],
    "st_solver_set_step_fusion": [_vp, C.c_int],
    "st_solver_stream": [_vp, C.POINTER(_vp)],
    "st_solver_set_stream": [_vp, _vp],
    "st_solver_last_phase_ms": [_vp, C.POINTER(C.c_float)],
    "st_launch_count": [C.POINTER(C.c_longlong)],
    "st_shot_forward": [_vp, C.POINTER(ShotC), _vp, C.c_int, _vp, _vp],
    "st_shot_forward_host": [_vp, _d, C.c_int64, C.POINTER(ShotC), _d],
    "st_shot_adjoint": [_vp, C.POINTER(ShotC), _vp, _vp],
    "st_rtm_shot": [_vp, C.POINTER(ShotC), _vp, C.c_int, _vp, _vp, _vp, _vp, _vp],
    "st_rtm_shot_host": [_vp, _d, C.c_int64, C.POINTER(ShotC), _f, C.c_int, _d, _d, _d],
    "st_rtm_engine_create": [C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                             C.POINTER(_vp)],
    "st_rtm_engine_destroy": [_vp],
    "st_rtm_engine_apply_image_condition": [_vp, _d, _d, C.c_int64, C.c_int64, C.c_int64],
    "st_rtm_engine_finalize_image": [_vp],
    "st_rtm_engine_reset_image": [_vp],
    "st_rtm_engine_result": [_vp, _d, _d, _d],
    "st_solver_set_velocity_device": [_vp, _vp],
    "st_shot_gradient": [_vp, C.POINTER(ShotC), _vp, C.c_int, _vp],
    "st_fwi_gradient": [_vp, C.POINTER(ShotC), _vp, C.c_int, _vp, _d, _vp],
    "st_rtm_shot_checkpointed": [_vp, C.POINTER(ShotC), _vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp,
                                 C.POINTER(CheckpointStatsC)],
    "st_shot_gradient_checkpointed": [_vp, C.POINTER(ShotC), _vp, C.c_int, C.c_int, C.c_int, _vp,
                                      C.POINTER(CheckpointStatsC)],
    "st_fwi_gradient_checkpointed": [_vp, C.POINTER(ShotC), _vp, C.c_int, C.c_int, C.c_int, _vp, _d, _vp,
                                     C.POINTER(CheckpointStatsC)],
    "st_conv3d_pack_weights": [_vp, _vp, C.c_int, _vp],
    "st_conv3d_bf16": [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_int, _vp],
    "st_conv3d_check": [_vp],
    "st_pc_in_conv": [_vp, _vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_pc_in_conv_wgrad": [_vp, _vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_pc_out_conv": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_pc_out_conv_bwd": [_vp, _vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_pc_relu_mask": [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_conv3d_wgrad": [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_pc_scales": [_vp, _vp, _vp, _vp, C.c_int64, _vp],
    "st_pc_scale_in": [_vp, _vp, _vp, _vp, C.c_int64, _vp],
    "st_pc_combine": [_vp, _vp, _vp, _vp, _vp, C.c_int64, _vp],
    "st_pc_tconv1": [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    "st_pc_conv1_wgrad": [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, _vp],
    # sparse
    "st_csr_create": [C.c_int64, C.c_int64, C.c_int64, C.c_int, C.POINTER(_vp)],
    "st_csr_destroy": [_vp],
    "st_csr_build_from_triplets": [_vp, C.c_int64, C.c_int64, C.c_int64, _i64, _i64, _d, C.c_int],
    "st_csr_build_from_triplets_device": [_vp, C.c_int64, C.c_int64, C.c_int64, _vp, _vp, _vp, C.c_int],
    "st_csr_build_fd_stencil_7point": [_vp, C.c_int64, C.c_int64, C.c_int64, _d, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_int],
    "st_csr_build_ray_matrix": [_vp, C.c_int64, _vp, C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_double, _i64],
    "st_csr_build_sampled_ray_matrix": [_vp, _vp, _i64],
    "st_ray_picks_create": [C.c_int, C.POINTER(RayModelC), C.c_int64, _vp, _vp, _vp, _vp, _vp, C.POINTER(_vp)],
    "st_ray_picks_destroy": [_vp],
    "st_ray_picks_info": [_vp, _i64],
    "st_ray_picks_stream": [_vp, C.POINTER(_vp)],
    "st_ray_picks_forward_model": [_vp, _vp, C.c_int, _vp],
    "st_ray_picks_compute_gradient": [_vp, _vp, _vp, C.c_int, _vp],
    "st_csr_shape": [_vp, _i64],
    "st_mmap_writer_open": [C.c_char_p, C.c_int64, C.POINTER(_vp)],
    "st_mmap_writer_write_frame": [_vp, _vp, C.c_int64],
    "st_mmap_writer_info": [_vp, _i64],
    "st_mmap_writer_close": [_vp],
    "st_mmap_read_frame": [C.c_char_p, C.c_int64, _vp, C.c_int64, _i64],
    "st_mmap_count_frames": [C.c_char_p, _i64],
    "st_slice_frame_bytes": [C.c_int64, C.c_int64, C.c_int64, C.POINTER(SliceSpecC)],
    "st_capture_slice_frames": [C.c_int64, C.c_int64, C.c_int64, C.POINTER(SliceSpecC), C.c_int, _vp, _vp, C.c_int,
                                _vp, C.c_int, C.c_int64, C.c_double, _vp, C.c_int64, _i64, _vp],
    "st_slice_stream_create": [C.c_char_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.POINTER(SliceSpecC), C.c_int,
                               C.c_int, C.c_int, C.POINTER(_vp)],
    "st_slice_stream_capture": [_vp, _vp, _vp, C.c_int, _vp, C.c_int, C.c_int64, _vp],
    "st_slice_stream_flush": [_vp],
    "st_slice_stream_stats": [_vp, _i64],
    "st_slice_stream_destroy": [_vp],
    "st_solver_set_slice_stream": [_vp, _vp, C.c_int],
    "st_terrain_create": [C.POINTER(GridParams), C.c_double, C.c_int, C.POINTER(_vp)],
    "st_terrain_destroy": [_vp],
    "st_terrain_set_bathymetry_data": [_vp, C.POINTER(BathymetryPointC), C.c_int64],
    "st_terrain_generate_synthetic_bathymetry": [_vp, C.c_double, C.c_double],
    "st_terrain_bathymetry": [_vp, _d],
    "st_terrain_seafloor": [_vp, C.c_int64, C.c_int64, _d, _i64],
    "st_terrain_update_velocity_mask": [_vp, _vp, C.c_int, C.c_double, C.c_double],
    "st_terrain_build_boundary_mask": [_vp, _vp, C.c_int],
    "st_terrain_apply_free_surface_bc": [_vp, _vp, C.c_int],
    "st_terrain_apply_seafloor_bc": [_vp, _vp, C.c_int],
    "st_terrain_apply_absorbing_bc": [_vp, _vp, C.c_int, C.c_int, C.c_double],
    "st_generate_bathymetry": [C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.c_double, C.c_double, _d],
    "st_solver_set_terrain": [_vp, _vp, C.c_int],
    "st_csr_get": [_vp, _i64, _i64, _d],
    "st_csr_device_arrays": [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)],
    "st_csr_stream": [_vp, C.POINTER(_vp)],
    "st_csr_spmv": [_vp, _d, C.c_int64, _d],
    "st_csr_spmv_transpose": [_vp, _d, C.c_int64, _d],
    "st_csr_spmv_device": [_vp, C.c_int, _vp, _vp],
    "st_csr_frobenius_norm": [_vp, _d],
    "st_csr_normal_jacobi": [_vp, C.c_double, _vp],
    "st_pcnet_create": [C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_int, C.POINTER(_vp)],
    "st_pcnet_destroy": [_vp],
    "st_pcnet_set_weights": [_vp, _vp, _vp],
    "st_pcnet_apply": [_vp, _vp, _vp, _vp, _vp],
    "st_normal_fcg_device": [_vp, _vp, C.c_double, C.c_int, C.c_double, _vp, _vp, C.POINTER(C.c_int), _d],
    "st_csr_scale": [_vp, C.c_double],
    "st_csr_add_diagonal": [_vp, C.c_double],
    "st_csr_clone": [_vp, C.POINTER(_vp)],
    "st_cg": [_vp, _d, C.c_int64, C.c_int, C.c_double, C.c_int, _d, C.POINTER(C.c_int), _d],
    "st_cg_device": [_vp, _vp, _vp, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int), _d],
    "st_cg_device_static": [_vp, _vp, _vp, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int), _d],
    "st_normal_cg_device": [_vp, _vp, C.c_double, C.c_int, C.c_double, C.c_int, _vp, _vp, C.POINTER(C.c_int), _d,
                            _d],
    "st_normal_pcg_stencil_device": [_vp, _vp, C.c_double, _f, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_double,
                                     C.c_int, _vp, _vp, C.POINTER(C.c_int), _d, _d],
    "st_dot": [_d, _d, C.c_int64, C.c_int, _d],
    "st_smooth_gradient": [_d, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_int, _d],
    "st_smooth_gradient_device": [_vp, C.c_int64, C.c_int64, C.c_int64, C.c_double, _vp, _vp, _vp],
    "st_field_count_nonfinite": [_d, C.c_int64, C.c_int, _i64],
    "st_field_clamp": [_d, C.c_int64, C.c_double, C.c_double, C.c_int],
    "st_field_repair_nan": [_d, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_double, C.c_int],
}
_RESTYPES = {"st_last_error": C.c_char_p, "st_slice_frame_bytes": C.c_int64}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False):
    """Returns the loaded CDLL. Raises when the library is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if build_if_missing:
                import importlib.util
                spec = importlib.util.spec_from_file_location("_st_build", os.path.join(PKG_ROOT, "build.py"))
                mod = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(mod)
                mod.build()
            else:
                raise ImportError(f"{LIB_PATH} is missing: build it with build.py (there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, C.c_int)
        _lib = L
        return L


def check(rc: int, allow_status: bool = False) -> int:
    """Raises SeismicError for negative codes; returns StepResult codes."""
    if rc < 0:
        msg = load().st_last_error()
        raise SeismicError(rc, msg.decode() if msg else "")
    if rc > 0 and not allow_status:
        return rc
    return rc


def call(name: str, *args, allow_status: bool = True) -> int:
    return check(getattr(load(), name)(*args), allow_status=allow_status)
