// Internal state of a solver handle, shared by the C-ABI translation units.
#pragma once

#include "st_kernels.cuh"

#include <algorithm>
#include <cstdlib>
#include <functional>
#include <vector>

namespace stg {
// Host array in page-locked memory (plain heap memory if pinning fails), so
// host->device copies from it run at full link speed.
class PinnedVec {
   public:
    PinnedVec() = default;
    PinnedVec(const PinnedVec&) = delete;
    PinnedVec& operator=(const PinnedVec&) = delete;
    ~PinnedVec() { release(); }
    void assign(size_t n, double v) {
        release();
        if (cudaMallocHost(reinterpret_cast<void**>(&p_), n * sizeof(double)) == cudaSuccess) {
            pinned_ = true;
        } else {
            cudaGetLastError();
            p_ = static_cast<double*>(std::malloc(n * sizeof(double)));
            pinned_ = false;
        }
        n_ = p_ ? n : 0;
        std::fill(p_, p_ + n_, v);
    }
    double* data() { return p_; }
    const double* data() const { return p_; }
    size_t size() const { return n_; }
    double* begin() { return p_; }
    double* end() { return p_ + n_; }
    const double* begin() const { return p_; }
    const double* end() const { return p_ + n_; }

   private:
    void release() {
        if (p_) {
            if (pinned_) cudaFreeHost(p_);
            else std::free(p_);
        }
        p_ = nullptr;
        n_ = 0;
    }
    double* p_ = nullptr;
    size_t n_ = 0;
    bool pinned_ = false;
};
}  // namespace stg

struct st_solver {
    int device = 0;
    cudaStream_t stream = nullptr;      // where the handle's work runs (own_stream or a caller's)
    cudaStream_t own_stream = nullptr;  // created with the handle
    stg::Layout L{};
    st_grid_params grid{};
    st_solver_config cfg{};
    double amp_limit = 1e10;     // the stencil's amplitude clamp (the solver's amplitude_limit_)
    double ft_amp_limit = 1e10;  // the repair clamp (its FaultTolerance's amplitude_limit_)
    double cfl_safety = 0.49;
    int max_repair_attempts = 3;
    stg::PinnedVec vel_host;  // reference layout; authoritative unless vel_host_valid is false
    double* vel_dev = nullptr;   // device copy of the last velocity uploaded by upload_velocity
    bool vel_host_valid = true;  // false: vel_dev holds the model, vel_host is refreshed on demand
    float* f[3] = {nullptr, nullptr, nullptr};
    int ic = 0, ip = 1, in = 2;
    float* c = nullptr;
    float* dtab = nullptr;
    int sw = 0;
    double* staging = nullptr;  // FP64 reference-layout buffer on the device
    unsigned* flags = nullptr;
    unsigned long long* counter = nullptr;
    double* dsum = nullptr;
    stg::FieldMaps maps[3];  // TMA maps of f[0..2]
    stg::FieldMaps map_c;    // TMA maps of c
    float* f4 = nullptr;     // spare field of the two-step imaging launches (allocated on first use)
    stg::FieldMaps map4;     // its TMA maps
    int fused_steps = 2;     // time steps per launch of the shot-level passes: 2 (fused pairs) or 1
    bool coeff_dirty = true;
    std::vector<float*> snapshots;  // save_snapshot: interior FP32 copies
    st_fault_stats stats{};
    bool cfl_warned = false;
    // device scratch of the fused shot / RTM / gradient entry points
    void* snap_buf = nullptr;       // forward snapshots (library-owned when the caller passes none)
    size_t snap_cap = 0;
    void* aux_buf = nullptr;        // seismograms / image accumulators / checkpoint states
    size_t aux_cap = 0;
    void* data_buf = nullptr;       // host-API staging of receiver data
    size_t data_cap = 0;
    void* ckpt_buf = nullptr;       // checkpointed adjoint: working set, state slots, segment snapshots
    size_t ckpt_cap = 0;
    int sponge_mode = ST_SPONGE_REFERENCE;  // ST_SPONGE_STABLE: damp the new field (Cerjan form)
    unsigned long long wait_limit_ns = 0;   // bounded-wait limit of the stencil kernels (0: 2 s)
    int withhold = 0;                       // st_solver_set_wait_test: plane + 1 withheld at the next launch
    int* zlim = nullptr;                // terrain: per-column z limits (st_solver_set_terrain), or null
    st_slice_stream* slices = nullptr;  // RTM slice stream (configure_rtm), borrowed
    int slice_interval = 0;             // capture every slice_interval steps
    // RTM driver of the solver face (st_solver_configure_rtm, st_rtm_driver.cu)
    int rtm_enabled = 0;
    st_rtm_engine* rtm_engine = nullptr;    // owned; runs on `stream`
    st_slice_stream* rtm_stream = nullptr;  // owned (configure_rtm with the mmap writer)
    float* rtm_fwd = nullptr;               // store_forward_wavefield_for_rtm's copy of the current field
    bool rtm_fwd_valid = false;
    st_receiver_grid rtm_rec{};
    int rtm_snap_kind = ST_SNAP_BF16;
    int rtm_segment = 0;
    int rtm_interval = 50;
    int rtm_slices_per_capture = 3;          // non-VOLUME slice specs
    int64_t rtm_ring_cap = 1024, rtm_attempts = 0, rtm_captured = 0, rtm_dropped = 0;
    void* rtm_buf = nullptr;                // run_rtm: amax | image | illum | residuals (FP32)
    size_t rtm_cap = 0;
    // phase boundaries of the last shot-level call, recorded on `stream`:
    // [0] start, [1] forward done, [2] backward done
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    int phases_recorded = 0;
    // host entry points: a second stream that uploads the receiver data while
    // the forward pass runs, and the event the adjoint pass waits on
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy = nullptr;
};


namespace stg {
int64_t ref_elems(const st_solver* s);
int ensure_staging(st_solver* s);
int refresh_coeff(st_solver* s);
int ensure_vel_host(st_solver* s);
int upload_velocity(st_solver* s, const double* vp);
int read_flags(st_solver* s, unsigned* out);
StepArgs base_args(st_solver* s, float* out);
// epi: 0 none, 1 imaging, 2 gradient (msnap = the snapshot store's map)
int fused_step(st_solver* s, StepArgs a, int snap_out, int snap_in, int epi, const CUtensorMap* msnap,
               const ImageMaps* imaps = nullptr);
// Two adjoint steps with fused imaging in one launch (launch_fd_step2_image):
// afterwards cur = the field after step t-1 and prev = the field after step t.
int fused_step2(st_solver* s, StepArgs a, int snap_in, const ImageMaps& imaps);
// Two forward steps t, t+1 in one launch (launch_fd_step2_forward):
// afterwards cur = u_{t+2} and prev = u_{t+1}.
int fused_step2_forward(st_solver* s, StepArgs a, int snap_out);
// Two adjoint steps with the gradient epilogue in one launch (launch_fd_step2_grad).
int fused_step2_grad(st_solver* s, StepArgs a, int snap_in, const CUtensorMap& msnap, const CUtensorMap& mgrad);
int zero_fields(st_solver* s);
long long dev_index(const st_solver* s, int64_t ix, int64_t iy, int64_t iz);
bool finite_sample(const double* w, int64_t len, int64_t t, float* out);
inline void set_injection(StepArgs& a, int64_t ix, int64_t iy, int64_t iz, float val) {
    a.inj_x = (int)ix;
    a.inj_y = (int)iy;
    a.inj_z = (int)iz;
    a.inj_val = val;
}
// Device scratch owned by the handle, grown on demand.
int ensure_buffer(st_solver* s, void** buf, size_t* cap, size_t bytes);
// Adjoint forcing of the receiver grid into the current field:
// f += c * row (c * D * row with the stable sponge), st_rtm.cu.
int launch_rec_force(st_solver* s, const st_receiver_grid& R, const float* row);
// Checkpointed adjoint pass (st_checkpoint.cu). epi 1: image / illum get the
// imaging condition; epi 2: grad_c the coefficient gradient. seis (may be
// null) receives the forward seismograms before before_backward runs.
int checkpointed_adjoint(st_solver* s, const st_shot* shot, int snap_kind, int segment_steps, int max_slots, int epi,
                         const float* force, float* image, float* illum, float* grad_c, float* seis,
                         const std::function<int()>& before_backward, st_checkpoint_stats* stats);
// Helpers of the engine a solver's RTM driver owns (st_rtm_engine.cu).
void rtm_engine_set_stream(st_rtm_engine* e, cudaStream_t stream);
int rtm_engine_create_on_stream(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, int device,
                                cudaStream_t stream, st_rtm_engine** out);
// image += fwd * adj, illum += fwd^2 (FP64) over the interior of two device-layout fields.
int rtm_engine_image_fields(st_rtm_engine* e, const float* fwd, const float* adj, const Layout& L);
// Overwrites the engine's FP64 image / illumination with FP32 accumulators.
int rtm_engine_load_fp32(st_rtm_engine* e, const float* image, const float* illum);
const double* rtm_engine_image(const st_rtm_engine* e);
// Releases the RTM driver's resources (st_rtm_driver.cu); used by destroy.
void rtm_release(st_solver* s);
// The exact-adjoint entry points transpose the unmasked step, so they refuse
// while a terrain (st_solver_set_terrain) is attached.
inline int require_no_terrain(const st_solver* s) {
    ST_CHECK(!s->zlim, ST_ERR_UNSUPPORTED, "exact-adjoint paths are unavailable while a terrain is attached");
    return ST_OK;
}

}  // namespace stg
