/*
 * seismic_gb300 — C ABI of the GB300 (sm_103a) implementation of the seismic
 * hot path of 13262233692/03-seismic-tomography-compute: the 3-D acoustic
 * finite-difference propagator, its exact adjoint and RTM imaging, and the
 * CSR SpMV / CG tomography solve.
 *
 * Conventions
 *  - Every function returns int: 0 = ST_OK; 1..3 mirror seismic::StepResult
 *    (solver/wave_equation.h:24-29); negative values are errors, and
 *    st_last_error() gives the message for the calling thread.
 *  - "Reference layout": the reference's halo-padded FP64 field of
 *    (nx+2)*(ny+2)*(nz+2) doubles, idx = ix*NYh*NZh + iy*NZh + iz
 *    (core/grid.cpp:45-49). Host entry points take and return that layout.
 *  - "Device layout": FP32, x/y halo 1, z interior starting at column 4 of a
 *    row of NZP floats (st_field_layout). Device entry points take device
 *    pointers in that layout and a cudaStream_t passed as void*.
 *  - Handles own their device memory; caller buffers are borrowed for the
 *    duration of a call. One handle per host thread (the reference runs
 *    MPI_THREAD_FUNNELED, core/mpi_context.cpp:10); work is ordered on the
 *    handle's stream and host-visible results synchronise.
 */
#ifndef SEISMIC_GB300_H
#define SEISMIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum st_status {
    ST_OK = 0,
    ST_NAN_DETECTED_AND_REPAIRED = 1, /* StepResult::NAN_DETECTED_AND_REPAIRED */
    ST_CFL_VIOLATION = 2,             /* StepResult::CFL_VIOLATION */
    ST_FATAL_DIVERGENCE = 3,          /* StepResult::FATAL_DIVERGENCE */
    ST_ERR_ARG = -1,
    ST_ERR_CUDA = -2,
    ST_ERR_ALLOC = -3,
    ST_ERR_STATE = -4,
    ST_ERR_TIMEOUT = -5,
    ST_ERR_UNSUPPORTED = -6
};

/* Which field of WaveEquationSolver::field() (wave_equation.h:16-22). */
enum st_field_id { ST_FIELD_CURRENT = 0, ST_FIELD_PREVIOUS = 1, ST_FIELD_NEXT = 2, ST_FIELD_VELOCITY = 3 };

/* Storage of forward snapshots for RTM / gradients (every step, or per
 * segment in the checkpointed entry points). */
enum st_snap_kind { ST_SNAP_NONE = 0, ST_SNAP_BF16 = 1, ST_SNAP_FP16 = 2, ST_SNAP_FP32 = 3 };

/* seismic::GridParams (core/grid.h:9-20). halo_width must be 1 (7-point stencil). */
typedef struct st_grid_params {
    int64_t nx_global, ny_global, nz_global;
    double dx, dy, dz;
    double origin_x, origin_y, origin_z;
    int halo_width;
} st_grid_params;

/* seismic::SolverConfig (core/config.h:9-19) without output_dir. */
typedef struct st_solver_config {
    double frequency;
    double dt;
    int nt;
    double water_depth;
    double seafloor_gradient;
    int sponge_width;
    double sponge_damping;
    int snapshot_interval;
} st_solver_config;

/* seismic::PropagationResult (wave_equation.h:31-37). */
typedef struct st_propagation_result {
    int status;
    int64_t total_nan_encountered;
    int64_t total_cells_repaired;
    int timesteps_completed;
    int completed_successfully;
} st_propagation_result;

/* seismic::FaultTolerance::FaultStats (core/fault_tolerance.h:61-67). */
typedef struct st_fault_stats {
    int64_t total_nan_count;
    int64_t total_inf_count;
    int64_t cells_repaired;
    int64_t timesteps_recovered;
    int global_abort_count;
} st_fault_stats;

/* Receivers on a regular grid of one z-plane (interior coordinates):
 * receiver q = irx*ny + iry sits at (x0 + irx*sx, y0 + iry*sy, z). */
typedef struct st_receiver_grid {
    int64_t x0, sx, nx;
    int64_t y0, sy, ny;
    int64_t z;
} st_receiver_grid;

/* One shot: a point source (interior coordinates) with an nt-sample wavelet
 * on the host, injected raw into the current field before each step as
 * inject_source does (wave_equation.cpp:39-54), and a receiver grid. */
typedef struct st_shot {
    int64_t src_ix, src_iy, src_iz;
    const double* wavelet; /* host, nt values (fewer: missing samples are 0) */
    int64_t wavelet_len;
    int nt;
    st_receiver_grid rec;
} st_shot;

typedef struct st_solver st_solver;

/* ---------------------------------------------------------------- library */
const char* st_last_error(void);
int st_version(void);
int st_device_count(int* count);

/* Device layout of an nx*ny*nz interior: out = {NXh, NYh, NZP, ZOFF, plane, elems}. */
int st_field_layout(int64_t nx, int64_t ny, int64_t nz, int64_t out[6]);

/* ------------------------------------------ seismic::WaveEquationSolver face */
/* Replaces WaveEquationSolver::WaveEquationSolver (wave_equation.cpp:10-23). */
int st_solver_create(const st_grid_params* grid, const st_solver_config* cfg, int device, st_solver** out);
/* Replaces ~WaveEquationSolver (wave_equation.cpp:25-27). */
int st_solver_destroy(st_solver* s);
/* Replaces initialize_velocity (wave_equation.cpp:29-31). */
int st_solver_initialize_velocity(st_solver* s, double vp0);
/* Replaces set_velocity_field (wave_equation.cpp:33-37): linear copy of
 * min(count, padded size) values into the reference-layout velocity. */
int st_solver_set_velocity_field(st_solver* s, const double* vp, int64_t count);
/* Replaces inject_source (wave_equation.cpp:39-54): current[pad(ix,iy,iz)] += wavelet[0]
 * unless non-finite or out of the padded array. */
int st_solver_inject_source(st_solver* s, int64_t ix, int64_t iy, int64_t iz, const double* wavelet, int64_t len);
/* Replace step_forward / step_adjoint (wave_equation.cpp:56-98); return StepResult. */
int st_solver_step_forward(st_solver* s, int timestep);
int st_solver_step_adjoint(st_solver* s, int timestep);
/* Replace forward_propagate / adjoint_propagate (wave_equation.cpp:100-194). */
int st_solver_forward_propagate(st_solver* s, const double* wavelet, int64_t len, st_propagation_result* out);
int st_solver_adjoint_propagate(st_solver* s, const double* residual, int64_t len, st_propagation_result* out);
/* Replaces reset_field (wave_equation.cpp:501-506). */
int st_solver_reset_field(st_solver* s);
/* field() / mutable_field() (wave_equation.h:72-73) in the reference layout. */
int st_solver_get_field(st_solver* s, int which, double* out, int64_t count);
int st_solver_set_field(st_solver* s, int which, const double* in, int64_t count);
/* Sponge rule of every step taken by the handle. ST_SPONGE_REFERENCE (the
 * default) is apply_sponge_layer as the reference calls it
 * (wave_equation.cpp:56-76,262-297): current and previous damped after the
 * update, u_{n+1} = 2u_n - D u_{n-1} + c L u_n, which grows without bound for
 * smooth modes in wide sponges (the 20-cell, 0.015 default diverges within a
 * few hundred steps). ST_SPONGE_STABLE damps the new field instead (Cerjan
 * form), u_{n+1} = D (2u_n - D u_{n-1} + c L u_n), and is stable; the adjoint,
 * imaging, gradient and checkpointed entry points follow the mode. No
 * reference counterpart for the stable mode. */
enum st_sponge_mode { ST_SPONGE_REFERENCE = 0, ST_SPONGE_STABLE = 1 };
int st_solver_set_sponge_mode(st_solver* s, int mode);
int st_solver_sponge_mode(st_solver* s, int* mode);
/* Replaces compute_energy (wave_equation.cpp:482-490): FP64 sum of squares of finite current values. */
int st_solver_compute_energy(st_solver* s, double* out);
/* Replaces verify_cfl (wave_equation.cpp:445-451). */
int st_solver_verify_cfl(st_solver* s, int* ok);
/* Replace set_amplitude_limit / amplitude_limit (wave_equation.cpp:453-456, .h:90). */
int st_solver_set_amplitude_limit(st_solver* s, double limit);
int st_solver_amplitude_limit(st_solver* s, double* out);
/* Replaces nan_count_current (wave_equation.cpp:458-461). */
int st_solver_nan_count_current(st_solver* s, int64_t* out);
/* Replace save_snapshot / clear_snapshots / field().snapshots (wave_equation.cpp:463-480, .h:78). */
int st_solver_save_snapshot(st_solver* s, int timestep);
int st_solver_clear_snapshots(st_solver* s);
int st_solver_snapshot_values(st_solver* s, int64_t* count);
int st_solver_get_snapshots(st_solver* s, double* out, int64_t count);
/* Replaces fault_stats (wave_equation.h:94). */
int st_solver_fault_stats(st_solver* s, st_fault_stats* out);
/* The solver's FaultTolerance (fault_tolerance(), wave_equation.h:84-85):
 * reset_stats (core/fault_tolerance.cpp:183-186) and its settings with the
 * reference's clamps (:188-198): max_repair_attempts >= 1, amplitude_limit
 * >= 1 (the repair clamp only; the solver's set_amplitude_limit sets both,
 * wave_equation.cpp:453-456), cfl_safety_factor in [0.01, 0.99]. */
enum st_fault_param { ST_FT_MAX_REPAIR_ATTEMPTS = 0, ST_FT_AMPLITUDE_LIMIT = 1, ST_FT_CFL_SAFETY_FACTOR = 2 };
/* Test hook of the bounded-wait error path (no reference counterpart): every
 * wait of the solver's stencil kernels gives up after limit_ns of GPU time (0 =
 * the default, 2 s). With withhold_plane >= 0 the next stencil launch never
 * copies that plane of each CTA's march, so the waits on it run out: the
 * launch drains its other copies (always with the full 2 s limit) and exits,
 * and the call returns ST_ERR_TIMEOUT with the handle still usable (its field
 * values are then undefined until reset_field). The withheld plane applies to
 * one launch; the limit stays until changed. */
int st_solver_set_wait_test(st_solver* s, unsigned long long limit_ns, int withhold_plane);
int st_solver_reset_fault_stats(st_solver* s);
int st_solver_set_fault_param(st_solver* s, int which, double value);
int st_solver_fault_param(st_solver* s, int which, double* out);

/* ----------------------------------------------------- GB300 shot entry points */
/* Device pointers to the solver's fields in the device layout (for zero-copy
 * torch views): which = ST_FIELD_*. Valid until the next call that steps the
 * solver (the imaging pass exchanges field buffers). */
int st_solver_device_field(st_solver* s, int which, float** out);
/* Time steps per launch of the shot-level passes (st_shot_forward, st_rtm_shot
 * and its host variant, the forward and adjoint passes of the FWI gradient
 * and of the checkpointed entry points): 2 (default) runs two
 * steps in one launch (with the imaging or gradient terms of both fused), 1
 * one step per launch; seismograms, snapshots, images, gradients and fields
 * are bit-identical either way. The time loops of WaveEquationSolver::
 * forward_propagate (solver/wave_equation.cpp:100-152) and
 * WaveEquationSolver::run_rtm (solver/wave_equation.cpp:621-688), restructured. */
int st_solver_set_step_fusion(st_solver* s, int steps);
/* The CUDA stream the handle orders its work on (a cudaStream_t). */
int st_solver_stream(st_solver* s, void** out);
/* Runs the handle's work on `stream` (a cudaStream_t of the handle's device,
 * e.g. the caller's torch stream; NULL = the handle's own stream again). The
 * work already queued on the previous stream stays ordered before anything
 * issued afterwards; calls that return host-visible results synchronise that
 * stream only, never the whole device. The stream must outlive its use. */
int st_solver_set_stream(st_solver* s, void* stream);
/* Device time of the two phases of the last st_rtm_shot on this handle, from
 * CUDA events recorded on its stream: out[0] = forward pass (fused steps with
 * snapshot store), out[1] = backward pass (fused adjoint steps with imaging). */
int st_solver_last_phase_ms(st_solver* s, float out[2]);
/* Kernels this library has launched in the process so far. */
int st_launch_count(long long* out);

/* Forward modelling of one shot, one fused kernel launch per step: leapfrog
 * update, sponge, source injection, receiver sampling and (snap_kind != NONE)
 * snapshot store of the post-injection field V_t of every step t.
 *   seis:  device FP32 [nt][nrec], nrec = rec.nx*rec.ny
 *   snaps: device buffer of nt * nx*ny*nz values of snap_kind (NULL if NONE)
 *   snap_amax: device uint32 [nt+1] (float bits of per-snapshot |max|), NULL if NONE
 * The solver's fields are reset first and hold the final state on return. */
int st_shot_forward(st_solver* s, const st_shot* shot, float* seis, int snap_kind, void* snaps,
                    unsigned* snap_amax);

/* Host-buffer convenience around st_shot_forward: velocity in the reference
 * layout (FP64, may be NULL to keep the current model), seismograms returned
 * as FP64 [nt][nrec] on the host. Includes all host<->device copies. */
int st_shot_forward_host(st_solver* s, const double* vp, int64_t vp_count, const st_shot* shot, double* seis_host);

/* Exact transpose of the wavelet -> seismogram map of st_shot_forward: runs
 * the discrete adjoint backward from receiver data (device FP32 [nt][nrec])
 * and returns src_trace[t] = dJ/dw_t for J = <seismograms, data> (device
 * FP32 [nt]). The reference's step_adjoint (wave_equation.cpp:78-98) is the
 * forward operator; this entry point is its true adjoint. */
int st_shot_adjoint(st_solver* s, const st_shot* shot, const float* data, float* src_trace);

/* Reverse-time migration of one shot with the exact discrete adjoint: forward
 * pass storing every post-injection field V_t (snap_kind BF16/FP16/FP32 with
 * a per-snapshot scale), backward pass of lambda (the transpose of the
 * forward step) forced by the receiver data, with the zero-lag
 * cross-correlation of RTMEngine::apply_image_condition fused in
 * (image += V_t*lambda_t, illum += V_t^2; rtm/rtm_engine.cpp:24-57) and
 * finalize_image (:170-182) into refl when refl != NULL.
 *   data: device FP32 [nt][nrec] receiver data
 *   snaps/snap_amax: device buffers as in st_shot_forward, or NULL to use
 *     library-owned ones (kept by the handle between calls)
 *   image/illum/refl: device FP32, nx*ny*nz interior values (x slowest).
 * Replaces the imaging of run_rtm (solver/wave_equation.cpp:621-688). */
int st_rtm_shot(st_solver* s, const st_shot* shot, const float* data, int snap_kind, void* snaps,
                unsigned* snap_amax, float* image, float* illum, float* refl);

/* Host-buffer RTM with every copy included: velocity in the reference layout
 * (FP64, NULL keeps the model), receiver data FP32 [nt][nrec] on the host,
 * image / illumination / reflectivity returned as FP64 interior arrays (any
 * may be NULL). The RTMImageCondition of rtm/rtm_engine.h:25-29. */
int st_rtm_shot_host(st_solver* s, const double* vp, int64_t vp_count, const st_shot* shot, const float* data_host,
                     int snap_kind, double* image_host, double* illum_host, double* refl_host);

/* -------------------------------------------------- seismic::RTMEngine face */
/* The imaging condition on caller-provided FP64 halo-padded fields, FP64
 * accumulators on the device. */
typedef struct st_rtm_engine st_rtm_engine;
/* Replaces RTMEngine::RTMEngine (rtm/rtm_engine.cpp:8-16). */
int st_rtm_engine_create(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, int halo_width,
                         int device, st_rtm_engine** out);
int st_rtm_engine_destroy(st_rtm_engine* e);
/* Replaces apply_image_condition (rtm_engine.cpp:24-57): image += f*a,
 * illumination += f*f over the interior, non-finite values taken as 0. */
int st_rtm_engine_apply_image_condition(st_rtm_engine* e, const double* forward_wavefield,
                                        const double* adjoint_wavefield, int64_t ny_padded, int64_t nz_padded,
                                        int64_t step_idx);
/* Replace finalize_image / reset_image / result() (rtm_engine.cpp:170-190, rtm_engine.h:52). */
int st_rtm_engine_finalize_image(st_rtm_engine* e);
int st_rtm_engine_reset_image(st_rtm_engine* e);
int st_rtm_engine_result(st_rtm_engine* e, double* image, double* illumination, double* reflectivity);

/* ------------------------------------------------ seismic::TerrainBoundary */
/* Irregular seafloor terrain (solver/boundary.h:9-52, boundary.cpp). The
 * bathymetry grid (nx*ny depths, column (ix, iy) at ix*ny + iy) is built on
 * the host; the field operations run on the GPU on the reference layout
 * (halo = the grid's halo_width), FP64, host (on_device = 0: copied in and
 * out) or device pointers (1: on the terrain's own stream, synchronous). */
typedef struct st_bathymetry_point { double x, y, depth; } st_bathymetry_point; /* BathymetryPoint */
typedef struct st_terrain st_terrain;
/* TerrainBoundary(grid, water_depth) (boundary.cpp:8-14): flat bathymetry. */
int st_terrain_create(const st_grid_params* grid, double water_depth, int device, st_terrain** out);
int st_terrain_destroy(st_terrain* t);
/* set_bathymetry_data (boundary.cpp:16-32): each point sets its cell's depth. */
int st_terrain_set_bathymetry_data(st_terrain* t, const st_bathymetry_point* points, int64_t n);
/* generate_synthetic_bathymetry (boundary.cpp:34-57). */
int st_terrain_generate_synthetic_bathymetry(st_terrain* t, double gradient, double roughness);
/* bathymetry() (boundary.h:38): nx*ny depths. */
int st_terrain_bathymetry(st_terrain* t, double* out);
/* seafloor_depth / seafloor_index (boundary.cpp:71-86); either output may be NULL. */
int st_terrain_seafloor(st_terrain* t, int64_t gx, int64_t gy, double* depth, int64_t* index);
/* update_velocity_mask (boundary.cpp:158-186) on a padded velocity. */
int st_terrain_update_velocity_mask(st_terrain* t, double* velocity, int on_device, double water_vp,
                                    double sediment_vp);
/* build_boundary_mask (boundary.cpp:188-214): 1 subsurface, 2 water, 0 halo. */
int st_terrain_build_boundary_mask(st_terrain* t, uint8_t* mask, int on_device);
/* apply_free_surface_bc / apply_seafloor_bc / apply_absorbing_bc
 * (boundary.cpp:88-156), in place, with the reference's index ranges (the
 * seafloor range of a column whose seafloor lies below the grid runs on
 * into the following cells, bounded by the array). */
int st_terrain_apply_free_surface_bc(st_terrain* t, double* field, int on_device);
int st_terrain_apply_seafloor_bc(st_terrain* t, double* field, int on_device);
int st_terrain_apply_absorbing_bc(st_terrain* t, double* field, int on_device, int sponge_width, double damping);
/* generate_bathymetry (pybind/bindings.cpp:255-270): nx*ny synthetic depths. */
int st_generate_bathymetry(int64_t nx, int64_t ny, double dx, double dy, double origin_x, double origin_y,
                           double water_depth, double gradient, double roughness, double* out);
/* Terrain-aware propagation (no reference counterpart: the reference never
 * applies its terrain while stepping). With a terrain attached every
 * propagator step sets the points of each (x, y) column above its z limit
 * to 0 right after the update, before receivers sample it: limit 1 for
 * ST_TERRAIN_FREE_SURFACE (the apply_free_surface_bc plane), the seafloor
 * index for ST_TERRAIN_SEAFLOOR (the apply_seafloor_bc range, clamped to the
 * column), the larger of the two for both. The limits are fused into the
 * stencil kernel (one load per row). The exact-adjoint entry points
 * (st_shot_adjoint, st_rtm_shot*, st_shot_gradient*, st_fwi_gradient*)
 * return ST_ERR_UNSUPPORTED while a terrain is attached. t = NULL or
 * flags = 0 detaches. */
enum st_terrain_flags { ST_TERRAIN_FREE_SURFACE = 1, ST_TERRAIN_SEAFLOOR = 2 };
int st_solver_set_terrain(st_solver* s, st_terrain* t, int flags);

/* ---------------------------------------- RTM slice frames and the mmap ring */
/* The on-disk slice stream of the reference's RTM visualisation path:
 * RTMEngine::extract_slices / capture_single_slice (rtm/rtm_engine.cpp:
 * 59-168), LockFreeSnapshotBuffer::serialize_slice + compute_checksum
 * (rtm/snapshot_buffer.cpp:102-153,207-229) and MmapSnapshotWriter
 * (rtm/mmap_writer.h:26-124, mmap_writer.cpp). File: a 120-byte header of 15
 * int64 (magic 0x52544D534E4150, header_size 120, file_size_bytes,
 * frame_count, write_offset, ring_start, ring_capacity, 8 reserved), then
 * records [int64 size][frame]; a frame that does not fit before
 * file_size_bytes restarts the ring at offset 120 (ring_start + 1; the frame
 * count keeps growing). Frame: a 124-byte packed SliceFrameHeader in a
 * 128-byte slot (bytes 124..127 are 0 here; the reference copies them from
 * past its struct), then the forward, adjoint and image-condition slices as
 * FP64, non-finite values written as 0; checksum over the payload:
 * s = rotl13(s ^ w) over little-endian 32-bit words; sequence_id 0. */
enum st_slice_axis { ST_SLICE_X = 0, ST_SLICE_Y = 1, ST_SLICE_Z = 2, ST_SLICE_VOLUME = 3 };
/* SliceSpec (rtm_engine.h:19-23); index < 0 = the middle plane (n / 2). */
typedef struct st_slice_spec {
    int32_t axis;
    int64_t index;
    int64_t stride;
} st_slice_spec;
/* Field kinds of the capture sources. */
enum st_field_kind {
    ST_FIELD_DEVICE_FP32 = 0,   /* the device layout (st_field_layout), FP32 */
    ST_FIELD_REFERENCE_FP64 = 1 /* the reference layout, FP64, on the device */
};
enum st_image_kind { ST_IMAGE_FP32 = 0, ST_IMAGE_FP64 = 1 }; /* nx*ny*nz interior, device */

typedef struct st_mmap_writer st_mmap_writer;
/* MmapSnapshotWriter::open (mmap_writer.cpp:36-127): creates / truncates the
 * file to max_bytes and maps it. max_bytes must exceed the 120-byte header. */
int st_mmap_writer_open(const char* path, int64_t max_bytes, st_mmap_writer** out);
/* write_frame (mmap_writer.cpp:152-176): appends [size][frame]; 0 on
 * success. A frame larger than the ring itself is refused (ST_ERR_ARG; the
 * reference would write past its mapping). */
int st_mmap_writer_write_frame(st_mmap_writer* w, const uint8_t* frame, int64_t size);
/* out = {frame_count, write_offset, capacity_bytes, frames_written,
 *        frames_dropped, total_bytes_written, mmap_cycles} (Stats,
 *        mmap_writer.h:63-70). */
int st_mmap_writer_info(st_mmap_writer* w, int64_t out[7]);
/* close (msync, unmap) and free the handle. */
int st_mmap_writer_close(st_mmap_writer* w);
/* read_frame / count_frames (mmap_writer.cpp:241-331): frame `index` counted
 * from the ring start (out may be NULL to ask the size; cap = out's size);
 * count = the header's frame_count. */
int st_mmap_read_frame(const char* path, int64_t index, uint8_t* out, int64_t cap, int64_t* size);
int st_mmap_count_frames(const char* path, int64_t* count);

/* Bytes of the frame of one spec on an nx*ny*nz interior (0 for VOLUME). */
int64_t st_slice_frame_bytes(int64_t nx, int64_t ny, int64_t nz, const st_slice_spec* spec);
/* Serializes the frames of n_specs specs from device fields fwd / adj (kind
 * field_kind) and the image-condition array ic (kind ic_kind; NULL = zeros)
 * into `frames` (device memory, the frames back to back in spec order,
 * VOLUME specs skipped), on `stream`. timestamp = capture_timestamp.
 * bytes (may be NULL) receives the total. */
int st_capture_slice_frames(int64_t nx, int64_t ny, int64_t nz, const st_slice_spec* specs, int n_specs,
                            const void* fwd, const void* adj, int field_kind, const void* ic, int ic_kind,
                            int64_t timestep, double timestamp, uint8_t* frames, int64_t cap, int64_t* bytes,
                            void* stream);

/* A slice stream: the capture above into `capacity` pinned host slots, each
 * copied back asynchronously and appended to an mmap ring by a writer
 * thread (the roles of LockFreeSnapshotBuffer and the writer's drain
 * thread, mmap_writer.cpp:199-225). A capture that finds its slot busy is
 * dropped and counted, as try_enqueue drops (snapshot_buffer.cpp:28-56). */
typedef struct st_slice_stream st_slice_stream;
int st_slice_stream_create(const char* path, int64_t max_bytes, int64_t nx, int64_t ny, int64_t nz,
                           const st_slice_spec* specs, int n_specs, int capacity, int device, st_slice_stream** out);
/* Captures every spec's frame at this time step (asynchronous on `stream`;
 * the sources may be overwritten once the stream has passed this point). */
int st_slice_stream_capture(st_slice_stream* ss, const void* fwd, const void* adj, int field_kind, const void* ic,
                            int ic_kind, int64_t timestep, void* stream);
/* Waits until every captured frame is in the file. */
int st_slice_stream_flush(st_slice_stream* ss);
/* out = {captured, dropped, written, bytes_written}. */
int st_slice_stream_stats(st_slice_stream* ss, int64_t out[4]);
/* Flushes, stops the writer thread and closes the file. */
int st_slice_stream_destroy(st_slice_stream* ss);
/* Attaches a slice stream to a solver (the streaming half of
 * WaveEquationSolver::configure_rtm, solver/wave_equation.cpp:520-560; the
 * stream is borrowed and must outlive the attachment): every `interval`
 * steps st_shot_forward captures (current field, zeros, zeros) and the
 * imaging pass of st_rtm_shot captures (the stored forward snapshot V_t,
 * the adjoint field, the image so far). ss = NULL or interval <= 0 detaches. */
int st_solver_set_slice_stream(st_solver* s, st_slice_stream* ss, int interval);

/* ------------------------------------------------ RTM driver of the solver */
/* RTMConfig (solver/wave_equation.h:39-48) plus the inputs of the true RTM
 * that run_rtm performs here. A zeroed struct is valid: every GB300 field
 * has its default at 0. */
typedef struct st_rtm_config {
    int enable_rtm;
    int enable_snapshots;
    int snapshot_interval;         /* slice capture every N steps (<= 0: 50) */
    int enable_mmap_writer;
    const char* mmap_filename;     /* NULL or "" disables the writer */
    int64_t mmap_max_bytes;        /* <= 0: 2 GiB */
    int64_t ring_buffer_capacity;  /* <= 0: 1024 */
    const st_slice_spec* slice_specs; /* NULL / 0: the middle Z, Y and X planes */
    int n_slice_specs;
    /* GB300 additions for run_rtm: receivers of the residual traces
     * (nx*ny == 0: every interior cell of the plane z = 0), the forward
     * snapshot storage (ST_SNAP_NONE = BF16 with a per-snapshot scale) and
     * binomial checkpointing (segment length in steps; 0 = store every step). */
    st_receiver_grid receivers;
    int snap_kind;
    int checkpoint_segment;
} st_rtm_config;
/* Replaces configure_rtm / init_rtm_resources / shutdown_rtm_resources
 * (wave_equation.cpp:508-575): drops the previous RTM resources, then, when
 * enable_rtm or enable_snapshots is set, creates the solver's RTMEngine
 * (FP64 image accumulators on the device) and, with enable_mmap_writer and a
 * file name, a slice stream on that file attached to the solver (the ring
 * buffer and mmap writer pair). cfg = NULL disables RTM. */
int st_solver_configure_rtm(st_solver* s, const st_rtm_config* cfg);
/* rtm_engine() (wave_equation.h:99): the solver's engine (borrowed; valid
 * until the next configure_rtm or destroy), NULL while RTM is disabled. */
int st_solver_rtm_engine(st_solver* s, st_rtm_engine** out);
/* snapshot_buffer() / mmap_writer() (wave_equation.h:100-101): the slice
 * stream configure_rtm created (borrowed), NULL when there is none. */
int st_solver_rtm_slice_stream(st_solver* s, st_slice_stream** out);
/* snapshots_captured() / snapshots_dropped() (wave_equation.h:106-107):
 * slices handed to the ring buffer. Without a slice stream the ring is the
 * reference's never-drained one (capacity rounded up to a power of two;
 * once full, every other capture is dropped, snapshot_buffer.cpp:28-56). */
int st_solver_rtm_snapshot_counts(st_solver* s, int64_t* captured, int64_t* dropped);
/* store_forward_wavefield_for_rtm (wave_equation.cpp:577-596): copies the
 * current field into the solver's forward-wavefield buffer (no-op while RTM
 * is disabled). */
int st_solver_store_forward_wavefield_for_rtm(st_solver* s, int timestep);
/* apply_rtm_step (wave_equation.cpp:598-619): the engine's imaging condition
 * on (the stored forward wavefield, or the current field when none was
 * stored; the current field), and with with_snapshot the slices of (that
 * forward field, the current field, the image) to the ring. No-op while RTM
 * is disabled. */
int st_solver_apply_rtm_step(st_solver* s, int timestep, int with_snapshot);
/* run_rtm (wave_equation.cpp:621-688) as true reverse-time migration: while
 * RTM is disabled it returns OK with completed_successfully set and does
 * nothing, as the reference. Otherwise a forward pass of config.nt steps
 * from zero fields with the source wavelet injected at the domain centre
 * (nx/2, ny/2, nz/2) for t < n_src (non-finite samples skipped), the exact
 * adjoint pass forced by receiver_residuals (FP64 [nt][nrec], time-major,
 * receiver q = irx*ny + iry of the configured receiver grid; exactly
 * nt*nrec values), the zero-lag imaging condition fused into it, and
 * finalize_image: the solver's engine then holds image, illumination and
 * reflectivity. Slices are captured every snapshot_interval steps of both
 * passes when a slice stream exists. The reference instead correlates the
 * forward field with itself and reads the residuals as a halo-padded field. */
int st_solver_run_rtm(st_solver* s, const double* source_wavelet, int64_t n_src, const double* receiver_residuals,
                      int64_t n_res, st_propagation_result* out);
/* apply_sponge_layer (wave_equation.cpp:262-297) as a standalone call:
 * field().current and field().previous are multiplied by the sponge factor D
 * over the sponge band, exactly as the reference's call does. */
int st_solver_apply_sponge_layer(st_solver* s);

/* ------------------------------------------------------ FWI gradients */
/* Sets the model from a device FP32 interior velocity (nx*ny*nz, x slowest);
 * the host copy (reference layout, edge-replicated halo) is refreshed too. */
int st_solver_set_velocity_device(st_solver* s, const float* vel);
/* Gradient of <seismograms, adj_src> with respect to the velocity for one
 * shot: forward with snapshot store (snap_kind BF16/FP16/FP32), then the
 * exact discrete adjoint forced by adj_src (device FP32 [nt][nrec]) with the
 * fused epilogue grad_c += lambda_t * L S_t; grad_v (device FP32 interior)
 * receives += dJ/dv = grad_c * 2 v dt^2. No reference counterpart (the
 * reference's adjoint-state gradient, seismic_tomography/gradient.py:24-40,
 * is a pointwise formula). Needs nz * snapshot bytes divisible by 16. */
int st_shot_gradient(st_solver* s, const st_shot* shot, const float* adj_src, int snap_kind, float* grad_v);
/* L2 FWI for one shot: misfit += 1/2 sum (d - d_obs)^2 (FP64) and, when
 * grad_v != NULL, grad_v += its velocity gradient; residual (device FP32
 * [nt][nrec], may be NULL) receives d - d_obs. */
int st_fwi_gradient(st_solver* s, const st_shot* shot, const float* d_obs, int snap_kind, float* grad_v,
                    double* misfit, float* residual);

/* ------------------------------------------- checkpointed adjoint passes */
/* The RTM and gradient passes above store one snapshot per time step
 * (nt * nx*ny*nz values). These variants keep exact FP32 forward states
 * (current + previous field) at segment boundaries of segment_steps steps,
 * in at most max_slots slots (>= 1) chosen by a binomial (revolve) schedule,
 * recompute one segment at a time into a segment_steps-snapshot buffer of
 * snap_kind, and run that segment's adjoint steps from it. Results equal the
 * store-every-step entry points with the same snap_kind. Device memory:
 * (3 + 2 * min(max_slots, segments)) fields + segment_steps snapshots. With
 * max_slots >= segments the cost is one extra forward sweep; fewer slots
 * trade memory for more recomputation. No reference counterpart (the
 * reference keeps its history in host memory, solver/wave_equation.cpp:463-480). */
typedef struct st_checkpoint_stats {
    int64_t forward_steps;  /* forward time steps run (first sweep + recomputes) */
    int64_t adjoint_steps;
    int64_t state_copies;   /* checkpoint stores and restores */
    int segments;
    int segment_steps;
    int slots_used;
    int64_t device_bytes;   /* scratch of the call */
} st_checkpoint_stats;
int st_rtm_shot_checkpointed(st_solver* s, const st_shot* shot, const float* data, int snap_kind,
                             int segment_steps, int max_slots, float* image, float* illum, float* refl,
                             st_checkpoint_stats* stats);
int st_shot_gradient_checkpointed(st_solver* s, const st_shot* shot, const float* adj_src, int snap_kind,
                                  int segment_steps, int max_slots, float* grad_v, st_checkpoint_stats* stats);
int st_fwi_gradient_checkpointed(st_solver* s, const st_shot* shot, const float* d_obs, int snap_kind,
                                 int segment_steps, int max_slots, float* grad_v, double* misfit, float* residual,
                                 st_checkpoint_stats* stats);

/* ------------------------------------- learned-preconditioner conv layer */
/* 3x3x3 convolution of a 32-channel volume on the tensor cores (tcgen05,
 * BF16 operands, FP32 accumulation); no reference counterpart (the learned
 * CG preconditioner is new). Volumes of D x H x W voxels are padded and
 * channels-last: [(D+2)(H+2)(W+2)][32] BF16, zero on the one-voxel border.
 * The kernel writes every row of padded planes 1..D (zero on their border
 * ring) and never planes 0 and D+1, which the caller zeroes once.
 * out = relu?(conv(in) + bias + add), BF16 or,
 * with out_fp32, FP32. packed_w: 55,296 bytes from st_conv3d_pack_weights.
 * Asynchronous on `stream` (a cudaStream_t); W <= 269 (ST_ERR_UNSUPPORTED
 * beyond: the shared-memory plane windows). st_conv3d_check
 * synchronises the stream and reports a bounded-wait timeout of any earlier
 * conv launch (ST_ERR_TIMEOUT), clearing it. */
int st_conv3d_pack_weights(const float* w_oidhw, void* packed_w, int transpose, void* stream);
int st_conv3d_bf16(const void* in, const void* packed_w, const float* bias, const void* add, void* out, int out_fp32,
                   int64_t D, int64_t H, int64_t W, int relu, void* stream);
int st_conv3d_check(void* stream);
/* Other layers of the learned preconditioner z = dinv r + s_out N(r)
 * (no reference counterpart). r, dinv, z, zhat: compact FP32 nx*ny*nz
 * (x slowest); h, dh, g: padded channels-last BF16 32-channel volumes;
 * scale, s_out: one device FP32 each. Weights FP32: w_in [32][2][27],
 * w_out [32][27], conv [32][32][27] (out, in, tap = (kd*3 + kh)*3 + kw).
 *  st_pc_in_conv       h = relu(C_in([scale r, scale dinv r]))
 *  st_pc_in_conv_wgrad dw_in += dL/dw_in for the masked gradient g of h
 *  st_pc_out_conv      zhat = C_out(h); z = dinv r + s_out zhat (z, zhat may be NULL)
 *  st_pc_out_conv_bwd  dh = C_out^T(dzhat); dw_out += dL/dw_out
 *  st_pc_relu_mask     g = dh * [h > 0]
 *  st_conv3d_wgrad     dw += sum_v g[v] (x) x[v + tap] for a 32 -> 32 layer, on the
 *                      tensor cores (tcgen05; g's border rows are ignored; a bounded-wait
 *                      timeout is reported by st_conv3d_check)
 * The others run on CUDA cores. All asynchronous on `stream`; gradients
 * accumulate (zero them first). */
int st_pc_in_conv(const float* r, const float* dinv, const float* scale, const float* w_in, void* h, int64_t nx,
                  int64_t ny, int64_t nz, void* stream);
int st_pc_in_conv_wgrad(const float* r, const float* dinv, const float* scale, const void* g, float* dw_in,
                        int64_t nx, int64_t ny, int64_t nz, void* stream);
int st_pc_out_conv(const void* h, const float* w_out, const float* r, const float* dinv, const float* s_out,
                   float* zhat, float* z, int64_t nx, int64_t ny, int64_t nz, void* stream);
int st_pc_out_conv_bwd(const float* dzhat, const void* h, const float* w_out, void* dh, float* dw_out, int64_t nx,
                       int64_t ny, int64_t nz, void* stream);
int st_pc_relu_mask(const void* dh, const void* h, void* g, int64_t nx, int64_t ny, int64_t nz, void* stream);
int st_conv3d_wgrad(const void* x, const void* g, float* dw, int64_t nx, int64_t ny, int64_t nz, void* stream);
/* Pieces of the symmetric form z = D r + S G^T G S r (st_pcnet below):
 *  st_pc_scales      scales = {1 / rms(r), rms(r) mean(dinv)} (acc: 2 doubles of scratch)
 *  st_pc_scale_in    a = scales[0] * sqrt(dinv) * r
 *  st_pc_combine     z = dinv * r + sqrt(dinv) * y / scales[0]
 *  st_pc_tconv1      h = C^T(a): 1 -> 32 channels, h[v][c] = sum_tap w[c][tap] a[v - tap]
 *  st_pc_conv1_wgrad dw[c][tap] += sum_v dz[v] h[v + tap][c] */
int st_pc_scales(const float* r, const float* dinv, double* acc, float* scales, int64_t n, void* stream);
int st_pc_scale_in(const float* r, const float* dinv, const float* scales, float* a, int64_t n, void* stream);
int st_pc_combine(const float* y, const float* r, const float* dinv, const float* scales, float* z, int64_t n,
                  void* stream);
int st_pc_tconv1(const float* a, const float* w, void* h, int64_t nx, int64_t ny, int64_t nz, void* stream);
int st_pc_conv1_wgrad(const float* dz, const void* h, float* dw, int64_t nx, int64_t ny, int64_t nz, void* stream);

/* ------------------------------------------------ seismic::CSRMatrix face */
/* Device CSR: int64 row pointers, int32 column indices, FP32 values. Host
 * entry points take the reference's int64 indices and FP64 values. */
typedef struct st_csr st_csr;

/* Replaces CSRMatrix(rows, cols, nnz) (sparse/csr_matrix.cpp:19-23); the
 * default CSRMatrix() is st_csr_create(0, 0, 0, ...). Entries are zeroed. */
int st_csr_create(int64_t rows, int64_t cols, int64_t nnz, int device, st_csr** out);
int st_csr_destroy(st_csr* m);
/* Replaces build_from_triplets (csr_matrix.cpp:25-72): entries outside
 * [0,rows)x[0,cols) dropped, rows sorted by column, duplicates summed in
 * input order; row_ptr / col_ind bit-exact with the reference. pad != 0
 * applies pad_to_alignment (:223-264: when it fires, every row is padded to a
 * multiple of 8 with col = row, value 0); it is refused with ST_ERR_ARG when
 * it would fire on a matrix with more rows than columns. */
int st_csr_build_from_triplets(st_csr* m, int64_t rows, int64_t cols, int64_t n, const int64_t* row_idx,
                               const int64_t* col_idx, const double* values, int pad);
/* The same from device triplets (int32 indices, FP32 values), e.g. the ray
 * matrix generator's output. */
int st_csr_build_from_triplets_device(st_csr* m, int64_t rows, int64_t cols, int64_t n, const int32_t* row_idx,
                                      const int32_t* col_idx, const float* values, int pad);
/* Replaces build_fd_stencil_7point (csr_matrix.cpp:74-116); velocity is the
 * nx*ny*nz interior on the host. */
int st_csr_build_fd_stencil_7point(st_csr* m, int64_t nx, int64_t ny, int64_t nz, const double* velocity, double dx,
                                   double dy, double dz, double dt, int pad);
/* Straight-ray path-length matrix for traveltime tomography (no reference
 * counterpart in C++; the reference's Python inversion samples the same
 * straight rays at midpoints, seismic_tomography/inversion.py:329-433): row i
 * = ray i from (x0,y0,z0) to (x1,y1,z1) (endpoints[6*i..6*i+5], in cell units,
 * host or device memory), A[i, (ix*ny + iy)*nz + iz] = length of the ray inside
 * that cell * cell_size, by exact voxel traversal; columns ascending, no
 * padding. nnz (may be NULL) receives the entry count. */
int st_csr_build_ray_matrix(st_csr* m, int64_t n_rays, const double* endpoints, int on_device, int64_t nx,
                            int64_t ny, int64_t nz, double cell_size, int64_t* nnz);
/* ------------------------------------------ sampled straight-ray picks */
/* The traveltime forward model and gradient of the reference's Python
 * inversion driver, AdjointStateInversion._forward_model and
 * _compute_gradient (seismic_tomography/inversion.py:329-433), on the GPU.
 * Each pick's source and station are snapped to cells (int((p - origin) / d)
 * clamped to the grid, :344-350); the ray between the two cells is sampled
 * at n = max(int(dist / (5 dx)), 2) midpoints, cell = int(c_src + frac *
 * (c_sta - c_src)) per axis with frac = (k + 0.5) / n (:352-364), each of
 * length ds = dist / n. The sample list is built once per pick set; the
 * forward model and the gradient then run for any velocity model.
 * Velocities vp are the model's (nx, ny, nz) array in C order (cell (ix, iy,
 * iz) at (ix * ny + iy) * nz + iz, model.py:27,89), FP64. */
typedef struct st_ray_model {
    int64_t nx, ny, nz;                 /* VelocityModel.nx/ny/nz (model.py:13-18) */
    double dx, dy, dz;                  /* cell spacing */
    double origin_x, origin_y, origin_z; /* VelocityModel.origin_* */
} st_ray_model;
typedef struct st_ray_picks st_ray_picks;
/* n_picks picks in the order of OBSDataCoordinator.picks (obs_data.py:38-40):
 * src_xyz / sta_xyz = [n_picks][3] world coordinates of each pick's source
 * and station, weight = pick.weight, valid[i] = 0 for a pick whose source or
 * station id is unknown (time 0, no gradient, :333-335; NULL = all valid).
 * dist (may be NULL) = the source-station distances to use: the reference
 * squares Python floats with x ** 2 (libm pow), which can round one unit in
 * the last place away from the x * x computed here, so passing its
 * distances makes every result the reference's bit for bit. All host
 * arrays, copied. Non-finite coordinates (where the reference's int() would
 * raise) and rays of more than 2^24 samples are refused with ST_ERR_ARG. */
int st_ray_picks_create(int device, const st_ray_model* model, int64_t n_picks, const double* src_xyz,
                        const double* sta_xyz, const double* dist, const double* weight, const uint8_t* valid,
                        st_ray_picks** out);
int st_ray_picks_destroy(st_ray_picks* p);
/* out = {n_picks, n_samples (total midpoint samples), n_cells}. */
int st_ray_picks_info(st_ray_picks* p, int64_t out[3]);
int st_ray_picks_stream(st_ray_picks* p, void** out);
/* _forward_model (inversion.py:329-381): times[i] = sum over the samples in
 * order of ds / v, an invalid velocity (non-finite or <= 0) read as 1500, a
 * non-finite term skipped, a non-finite or negative sum replaced by
 * dist / 6000. FP64, bit-exact against the reference given its distances.
 * on_device = 0: host arrays, returns when done; 1: device arrays, enqueued
 * on the handle's stream. */
int st_ray_picks_forward_model(st_ray_picks* p, const double* vp, int on_device, double* times);
/* _compute_gradient (inversion.py:383-433): gradient (n_cells, overwritten)
 * = sum over picks with a finite residual and their samples at a valid
 * velocity of (residual * (-ds / v^2)) * weight, each cell's terms added in
 * the reference's pick, then sample order (bit-exact as above). */
int st_ray_picks_compute_gradient(st_ray_picks* p, const double* vp, const double* residuals, int on_device,
                                  double* gradient);
/* The sampled-ray matrix of the picks as a CSR (rows = picks, columns =
 * cells, A[i, c] = ds_i * the number of samples of pick i in cell c, FP32),
 * so that A (1 / vp) gives the forward model wherever every velocity is
 * valid, and -(A^T (w r)) / vp^2 the gradient: the system the reference's
 * inversion linearises, for the CG solvers. nnz may be NULL. */
int st_csr_build_sampled_ray_matrix(st_csr* m, st_ray_picks* p, int64_t* nnz);

/* rows(), cols(), nnz() (csr_matrix.h:32-34): out = {rows, cols, nnz}. */
int st_csr_shape(st_csr* m, int64_t out[3]);
/* row_ptr(), col_ind(), values() (csr_matrix.h:36-38) copied to the host (any may be NULL). */
int st_csr_get(st_csr* m, int64_t* row_ptr, int64_t* col_ind, double* values);
/* Device arrays of the matrix (borrowed; valid until the next build). */
int st_csr_device_arrays(st_csr* m, long long** row_ptr, int** col_ind, float** values);
int st_csr_stream(st_csr* m, void** out);
/* Replace spmv / spmv_transpose (csr_matrix.cpp:118-166; the transpose with
 * its accumulator zeroed). Host FP64 vectors in and out. */
int st_csr_spmv(st_csr* m, const double* x, int64_t nx, double* y);
int st_csr_spmv_transpose(st_csr* m, const double* x, int64_t nx, double* y);
/* y = A x (transpose = 0) or A^T x on device FP32 vectors, on the matrix's stream. */
int st_csr_spmv_device(st_csr* m, int transpose, const float* x, float* y);
/* Replace frobenius_norm / scale / add_diagonal (csr_matrix.cpp:168-193). */
int st_csr_frobenius_norm(st_csr* m, double* out);
int st_csr_scale(st_csr* m, double alpha);
int st_csr_add_diagonal(st_csr* m, double alpha);
/* Copy of a matrix (SparseOps::build_hessian_approx copies then adds the
 * diagonal, sparse_ops.cpp:204-210). */
int st_csr_clone(st_csr* m, st_csr** out);

/* ------------------------------------------------ seismic::SparseOps face */
/* Replace conjugate_gradient (jacobi = 0) and jacobi_preconditioned_cg
 * (jacobi = 1) (sparse/sparse_ops.cpp:8-113): x0 = 0, stop when
 * sqrt(<r,r>)/||b|| < tol after an update or when |<p,Ap>| < 1e-30; returns
 * x0 = 0 when ||b|| < 1e-30. FP32 vectors, FP64 inner products and norms. */
int st_cg(st_csr* A, const double* b, int64_t nb, int max_iter, double tol, int jacobi, double* x, int* iters,
          double* final_rel);
int st_cg_device(st_csr* A, const float* b, float* x, int max_iter, double tol, int jacobi, int* iters,
                 double* final_rel);
/* CG without any device allocation (no reference counterpart). Same solver
 * and arguments as st_cg_device, for callers that cannot allocate device
 * memory while they run: services that hand all device memory to their own
 * pool at start-up, plugin hosts that forbid allocation after
 * initialisation, real-time loops that cannot risk an allocator stall or an
 * out-of-memory failure mid-run. Its scratch (5 FP32 vectors of
 * ST_CG_STATIC_MAX_N floats, 20 MiB) is one file-scope device array that
 * every GPU loading this library keeps until the process exits.
 *  - Systems larger than ST_CG_STATIC_MAX_N unknowns are refused (ST_ERR_ARG).
 *  - The call is synchronous (it reads the solver's scalars on the host
 *    every 16 iterations), so it cannot be captured in a CUDA graph. The
 *    first call on a device looks up the array's device address, kept for
 *    the life of the process: a cudaDeviceReset (or any other teardown of the
 *    device's primary context) makes it stale, as it does every handle of
 *    this library.
 *  - All calls on a device share the array, so calls that overlap on the GPU
 *    (other host threads, other streams) race; serialise them. The array keeps
 *    the last call's contents; the solver re-initialises everything it reads. */
#define ST_CG_STATIC_MAX_N 1048576
int st_cg_device_static(st_csr* A, const float* b, float* x, int max_iter, double tol, int jacobi, int* iters,
                        double* final_rel);
/* Learned preconditioner as a native handle (no reference counterpart):
 * the symmetric positive (semi)definite z = D r + S G^T G S r, D = diag(dinv),
 * S = sqrt(D), G = (I + conv_K)...(I + conv_1) C^T with `layers` tensor-core
 * 32 -> 32 layers (G^T by the transposed packing). Weights are device FP32:
 * w_c [32][27], w_k `layers` consecutive [32][32][27] blocks, trained by
 * seismic_engine.precond. */
typedef struct st_pcnet st_pcnet;
int st_pcnet_create(int64_t nx, int64_t ny, int64_t nz, int layers, int device, st_pcnet** out);
int st_pcnet_destroy(st_pcnet* p);
int st_pcnet_set_weights(st_pcnet* p, const float* w_c, const float* w_k);
int st_pcnet_apply(st_pcnet* p, const float* r, const float* dinv, float* z, void* stream);
/* Flexible CG on (A^T A + lam I) x = A^T d (device FP32 d, x) preconditioned
 * by pc, or by Jacobi when pc is NULL; stops when the true relative residual
 * (FP64 norms) is <= tol. No reference counterpart. */
int st_normal_fcg_device(st_csr* A, const float* d, double lam, int max_iter, double tol, st_pcnet* pc, float* x,
                         int* iters, double* true_rel);
/* dinv (device FP32, cols) = 1 / (column sums of A^2 + lam): the Jacobi
 * preconditioner of A^T A + lam I (asynchronous on the matrix's stream). */
int st_csr_normal_jacobi(st_csr* A, double lam, float* dinv);
/* Flags of st_normal_cg_device's `jacobi` argument. */
enum { ST_CG_JACOBI = 1, ST_CG_CONFIRM_TRUE = 2 };
/* Tomography solve: (A^T A + lam I) x = A^T d for a rectangular A (no
 * reference counterpart), Jacobi diagonal = column sums of A^2 + lam when
 * jacobi & ST_CG_JACOBI. rhs (may be NULL) receives A^T d; with d == NULL, rhs
 * is the given right-hand side instead (e.g. a gradient for the regularised
 * update (I + mu L^T L) x = g with A = sqrt(mu) L, lam = 1). true_rel (may be
 * NULL) receives the FP64 relative true residual ||rhs - (A^T A + lam I) x|| /
 * ||rhs||. The solve stops when the recurrence residual falls below tol; with
 * jacobi & ST_CG_CONFIRM_TRUE the stop is confirmed on the true residual:
 * while that is above tol, the iteration continues to a tighter recurrence
 * target (at most ten times, within max_iter). iters and final_rel are those
 * of the last iteration. */
int st_normal_cg_device(st_csr* A, const float* d, double lam, int max_iter, double tol, int jacobi, float* x,
                        float* rhs, int* iters, double* final_rel, double* true_rel);
/* The same solve preconditioned by M r = D r + S K (S r) (no reference
 * counterpart): D the Jacobi diagonal above, S = sqrt(D), K = sum over the
 * three axes of w[a] times the 1-D Dirichlet second difference on the
 * nx x ny x nz cell grid of A's columns (x slowest), w[a] >= 0 (host array):
 * symmetric positive definite, a 7-point stencil per application. The
 * weights are fitted on training systems (seismic_engine.precond.
 * fit_stencil_weights). flags: ST_CG_CONFIRM_TRUE as above (Jacobi implied). */
int st_normal_pcg_stencil_device(st_csr* A, const float* d, double lam, const float* w, int64_t nx, int64_t ny,
                                 int64_t nz, int max_iter, double tol, int flags, float* x, float* rhs, int* iters,
                                 double* final_rel, double* true_rel);
/* Replaces dot_product (sparse_ops.cpp:172-187): FP64 inner product. */
int st_dot(const double* a, const double* b, int64_t n, int device, double* out);
/* Replaces smooth_gradient (sparse_ops.cpp:115-158): truncated Gaussian of
 * radius floor(3 sigma), normalised per point by the in-bounds weight sum,
 * computed as three normalised 1-D passes (the weights and the support
 * factor per axis). FP64. n < nx*ny*nz gives zeros, as the reference. */
int st_smooth_gradient(const double* g, int64_t n, int64_t nx, int64_t ny, int64_t nz, double sigma, int device,
                       double* out);
/* Device version on FP64 arrays (tmp: scratch of nx*ny*nz doubles). */
int st_smooth_gradient_device(const double* g, int64_t nx, int64_t ny, int64_t nz, double sigma, double* out,
                              double* tmp, void* stream);

/* ------------------------------------- FaultTolerance helpers (FP64, host arrays) */
/* check_field_health -> FaultTolerance::count_nan_inf (bindings.cpp:275-280,
 * core/fault_tolerance.cpp:72-80). */
int st_field_count_nonfinite(const double* data, int64_t n, int device, int64_t* out);
/* clamp_field_safe -> FaultTolerance::clamp_field (bindings.cpp:282-289,
 * fault_tolerance.cpp:86-96): non-finite -> 0, else clamped to [lo, hi]. In place. */
int st_field_clamp(double* data, int64_t n, double lo, double hi, int device);
/* repair_field_nan -> FaultTolerance::repair_field_nan (bindings.cpp:290-301,
 * fault_tolerance.cpp:98-157), in the reference's sequential cell order. In
 * place; nx*ny*nz must not exceed n. */
int st_field_repair_nan(double* data, int64_t n, int64_t nx, int64_t ny, int64_t nz, int halo_width,
                        double replace_value, int device);

#ifdef __cplusplus
}
#endif

#endif /* SEISMIC_GB300_H */
