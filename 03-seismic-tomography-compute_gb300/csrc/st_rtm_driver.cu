// The RTM driver of the WaveEquationSolver face (solver/wave_equation.cpp:
// 262-297, 508-688): configure_rtm / rtm_engine / snapshot counters, the
// per-step building blocks store_forward_wavefield_for_rtm and
// apply_rtm_step with the reference's semantics, run_rtm as true reverse-time
// migration (the fused forward + exact adjoint + imaging of st_rtm_shot), and
// the standalone apply_sponge_layer.
#include "st_solver_impl.cuh"

#include <cstring>
#include <string>
#include <vector>

namespace stg {
namespace {

// apply_sponge_layer (wave_equation.cpp:262-297): current *= D and
// previous *= D over the sponge band. The device keeps previous undamped
// (its reference value is D times it), so scaling the device copy by D scales
// the reference value by D as well.
__global__ void sponge_fields_kernel(float* __restrict__ cur, float* __restrict__ prev, Layout L,
                                     const float* __restrict__ dtab, int sw) {
    const long long n = L.nx * L.ny * L.nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long ix = k / (L.ny * L.nz), r = k % (L.ny * L.nz), iy = r / L.nz, iz = r % L.nz;
        long long d = ix;
        d = min(d, L.nx - 1 - ix);
        d = min(d, iy);
        d = min(d, L.ny - 1 - iy);
        d = min(d, iz);
        d = min(d, L.nz - 1 - iz);
        if (d >= sw) continue;
        const float D = dtab[d];
        const long long i = L.at(ix, iy, iz);
        cur[i] *= D;
        prev[i] *= D;
    }
}

unsigned grid_blocks(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 8));
}

// One capture of every slice spec into the never-drained ring of the
// reference (snapshot_buffer.cpp:28-56 with no reader): the first `cap`
// enqueues succeed; then each enqueue finds its slot full and is dropped
// (freeing the slot), and the next one succeeds.
void count_ring_capture(st_solver* s) {
    for (int k = 0; k < s->rtm_slices_per_capture; ++k) {
        const int64_t a = s->rtm_attempts++;
        if (a < s->rtm_ring_cap || ((a - s->rtm_ring_cap) & 1)) ++s->rtm_captured;
        else ++s->rtm_dropped;
    }
}

}  // namespace

// shutdown_rtm_resources (wave_equation.cpp:563-575). As in the reference,
// the stored forward wavefield and the captured / dropped counters outlive
// it; the ring starts empty at the next configure_rtm.
void rtm_release(st_solver* s) {
    if (s->rtm_stream) {
        if (s->slices == s->rtm_stream) {
            s->slices = nullptr;
            s->slice_interval = 0;
        }
        int64_t st[4] = {0, 0, 0, 0};
        if (st_slice_stream_stats(s->rtm_stream, st) == ST_OK) {
            s->rtm_captured += st[0];
            s->rtm_dropped += st[1];
        }
        st_slice_stream_destroy(s->rtm_stream);
        s->rtm_stream = nullptr;
    }
    if (s->rtm_engine) {
        cudaStreamSynchronize(s->stream);
        st_rtm_engine_destroy(s->rtm_engine);
        s->rtm_engine = nullptr;
    }
    cudaFree(s->rtm_buf);
    s->rtm_buf = nullptr;
    s->rtm_cap = 0;
    s->rtm_enabled = 0;
    s->rtm_attempts = 0;
}

}  // namespace stg

using namespace stg;

extern "C" {

int st_solver_configure_rtm(st_solver* s, const st_rtm_config* cfg) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CUDA(cudaSetDevice(s->device));
    rtm_release(s);
    if (!cfg || !(cfg->enable_rtm || cfg->enable_snapshots)) return ST_OK;
    ST_CHECK(cfg->n_slice_specs >= 0 && (cfg->n_slice_specs == 0 || cfg->slice_specs), ST_ERR_ARG,
             "slice_specs missing");
    ST_CHECK(cfg->snap_kind >= ST_SNAP_NONE && cfg->snap_kind <= ST_SNAP_FP32, ST_ERR_ARG, "bad snapshot kind %d",
             cfg->snap_kind);
    ST_CHECK(cfg->checkpoint_segment >= 0, ST_ERR_ARG, "checkpoint_segment must be >= 0");
    const st_receiver_grid& R = cfg->receivers;
    if (R.nx * R.ny > 0) {
        ST_CHECK(R.nx > 0 && R.ny > 0 && R.x0 >= 0 && R.y0 >= 0 && R.z >= 0 && R.z < s->L.nz &&
                     R.x0 + (R.nx - 1) * R.sx < s->L.nx && R.y0 + (R.ny - 1) * R.sy < s->L.ny &&
                     R.x0 + (R.nx - 1) * R.sx >= 0 && R.y0 + (R.ny - 1) * R.sy >= 0,
                 ST_ERR_ARG, "receiver grid outside the interior");
        s->rtm_rec = R;
    } else {
        s->rtm_rec = st_receiver_grid{0, 1, s->L.nx, 0, 1, s->L.ny, 0};
    }
    s->rtm_snap_kind = cfg->snap_kind == ST_SNAP_NONE ? ST_SNAP_BF16 : cfg->snap_kind;
    s->rtm_segment = cfg->checkpoint_segment;
    s->rtm_interval = cfg->snapshot_interval > 0 ? cfg->snapshot_interval : 50;
    const int64_t want = cfg->ring_buffer_capacity > 0 ? cfg->ring_buffer_capacity : 1024;
    s->rtm_ring_cap = 1;
    while (s->rtm_ring_cap < want) s->rtm_ring_cap <<= 1;
    std::vector<st_slice_spec> specs(cfg->slice_specs, cfg->slice_specs + cfg->n_slice_specs);
    if (specs.empty()) specs = {{ST_SLICE_Z, -1, 1}, {ST_SLICE_Y, -1, 1}, {ST_SLICE_X, -1, 1}};
    s->rtm_slices_per_capture = 0;
    for (const auto& sp : specs) s->rtm_slices_per_capture += sp.axis != ST_SLICE_VOLUME ? 1 : 0;
    ST_TRY(rtm_engine_create_on_stream(s->L.nx, s->L.ny, s->L.nz, s->grid.dx, s->grid.dy, s->grid.dz, s->device,
                                       s->stream, &s->rtm_engine));
    s->rtm_enabled = 1;
    if (cfg->enable_mmap_writer && cfg->mmap_filename && cfg->mmap_filename[0]) {
        const int64_t max_bytes = cfg->mmap_max_bytes > 0 ? cfg->mmap_max_bytes : (int64_t)2 << 30;
        const int cap = (int)std::min<int64_t>(want, 1 << 20);
        const int rc = st_slice_stream_create(cfg->mmap_filename, max_bytes, s->L.nx, s->L.ny, s->L.nz, specs.data(),
                                              (int)specs.size(), cap, s->device, &s->rtm_stream);
        if (rc < 0) {
            // the reference drops the writer when the file cannot be opened (wave_equation.cpp:541-542)
            s->rtm_stream = nullptr;
        } else {
            ST_TRY(st_solver_set_slice_stream(s, s->rtm_stream, s->rtm_interval));
        }
    }
    return ST_OK;
}

int st_solver_rtm_engine(st_solver* s, st_rtm_engine** out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    *out = s->rtm_engine;
    return ST_OK;
}

int st_solver_rtm_slice_stream(st_solver* s, st_slice_stream** out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    *out = s->rtm_stream;
    return ST_OK;
}

int st_solver_rtm_snapshot_counts(st_solver* s, int64_t* captured, int64_t* dropped) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    int64_t c = s->rtm_captured, d = s->rtm_dropped;
    if (s->rtm_stream) {
        int64_t st[4] = {0, 0, 0, 0};
        ST_TRY(st_slice_stream_stats(s->rtm_stream, st));
        c += st[0];
        d += st[1];
    }
    if (captured) *captured = c;
    if (dropped) *dropped = d;
    return ST_OK;
}

int st_solver_store_forward_wavefield_for_rtm(st_solver* s, int timestep) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    (void)timestep;
    if (!s->rtm_enabled) return ST_OK;
    ST_CUDA(cudaSetDevice(s->device));
    const size_t bytes = (size_t)s->L.elems * sizeof(float);
    if (!s->rtm_fwd) ST_CUDA(cudaMalloc(&s->rtm_fwd, bytes));
    ST_CUDA(cudaMemcpyAsync(s->rtm_fwd, s->f[s->ic], bytes, cudaMemcpyDeviceToDevice, s->stream));
    s->rtm_fwd_valid = true;
    return ST_OK;
}

int st_solver_apply_rtm_step(st_solver* s, int timestep, int with_snapshot) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    if (!s->rtm_enabled || !s->rtm_engine) return ST_OK;
    ST_CUDA(cudaSetDevice(s->device));
    const float* fwd = s->rtm_fwd_valid ? s->rtm_fwd : s->f[s->ic];
    ST_TRY(rtm_engine_image_fields(s->rtm_engine, fwd, s->f[s->ic], s->L));
    if (with_snapshot) {
        if (s->rtm_stream) {
            ST_TRY(st_slice_stream_capture(s->rtm_stream, fwd, s->f[s->ic], ST_FIELD_DEVICE_FP32,
                                           rtm_engine_image(s->rtm_engine), ST_IMAGE_FP64, timestep, s->stream));
        } else {
            count_ring_capture(s);
        }
    }
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_solver_run_rtm(st_solver* s, const double* source_wavelet, int64_t n_src, const double* receiver_residuals,
                      int64_t n_res, st_propagation_result* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    std::memset(out, 0, sizeof(*out));
    if (!s->rtm_enabled) {
        // wave_equation.cpp:632-636
        out->status = ST_OK;
        out->completed_successfully = 1;
        return ST_OK;
    }
    ST_TRY(require_no_terrain(s));
    ST_CUDA(cudaSetDevice(s->device));
    const int nt = s->cfg.nt;
    ST_CHECK(nt > 0, ST_ERR_ARG, "config nt must be positive");
    const st_receiver_grid R = s->rtm_rec;
    const int64_t nrec = R.nx * R.ny;
    ST_CHECK(n_res == (int64_t)nt * nrec && (receiver_residuals || n_res == 0), ST_ERR_ARG,
             "receiver_residuals must hold nt*nrec = %d*%lld values ([nt][nrec], time-major), got %lld", nt,
             (long long)nrec, (long long)n_res);
    ST_CHECK(source_wavelet || n_src <= 0, ST_ERR_ARG, "source wavelet missing");
    st_shot shot{};
    shot.src_ix = s->L.nx / 2;
    shot.src_iy = s->L.ny / 2;
    shot.src_iz = s->L.nz / 2;
    shot.wavelet = source_wavelet;
    shot.wavelet_len = std::max<int64_t>(n_src, 0);
    shot.nt = nt;
    shot.rec = R;
    const size_t npts = (size_t)(s->L.nx * s->L.ny * s->L.nz);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t amax_b = up(sizeof(unsigned) * (size_t)(nt + 1)), img_b = up(npts * sizeof(float));
    const size_t data_b = up((size_t)n_res * sizeof(float));
    ST_TRY(ensure_buffer(s, &s->rtm_buf, &s->rtm_cap, amax_b + 2 * img_b + data_b));
    char* base = static_cast<char*>(s->rtm_buf);
    unsigned* amax = reinterpret_cast<unsigned*>(base);
    float* image = reinterpret_cast<float*>(base + amax_b);
    float* illum = reinterpret_cast<float*>(base + amax_b + img_b);
    float* data = reinterpret_cast<float*>(base + amax_b + 2 * img_b);
    if (n_res > 0) {
        std::vector<float> d32((size_t)n_res);
        for (int64_t k = 0; k < n_res; ++k) d32[(size_t)k] = (float)receiver_residuals[k];
        ST_CUDA(cudaMemcpyAsync(data, d32.data(), (size_t)n_res * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        ST_CUDA(cudaStreamSynchronize(s->stream));
    }
    int rc;
    if (s->rtm_segment > 0) {
        st_checkpoint_stats stats{};
        rc = st_rtm_shot_checkpointed(s, &shot, data, s->rtm_snap_kind, s->rtm_segment, 1 << 30, image, illum,
                                      nullptr, &stats);
    } else {
        rc = st_rtm_shot(s, &shot, data, s->rtm_snap_kind, nullptr, amax, image, illum, nullptr);
    }
    if (rc < 0) return rc;
    ST_TRY(rtm_engine_load_fp32(s->rtm_engine, image, illum));
    ST_TRY(st_rtm_engine_finalize_image(s->rtm_engine));
    out->status = rc;
    out->timesteps_completed = nt;
    out->total_cells_repaired = s->stats.cells_repaired;
    out->completed_successfully = rc == ST_FATAL_DIVERGENCE ? 0 : 1;
    return ST_OK;
}

int st_solver_apply_sponge_layer(st_solver* s) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    if (s->sw <= 0) return ST_OK;
    ST_CUDA(cudaSetDevice(s->device));
    const long long n = s->L.nx * s->L.ny * s->L.nz;
    sponge_fields_kernel<<<grid_blocks(n), 256, 0, s->stream>>>(s->f[s->ic], s->f[s->ip], s->L, s->dtab, s->sw);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

}  // extern "C"
