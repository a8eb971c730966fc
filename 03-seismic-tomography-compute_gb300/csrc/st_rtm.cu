// Reverse-time migration of one shot with the exact discrete adjoint.
//
// Forward pass: the fused step (st_shot_forward) stores every post-injection
// forward field V_t as a BF16 / FP16 / FP32 snapshot with a per-snapshot
// scale. Backward pass: mu = c * lambda obeys the forward operator, so the
// same fused kernel runs t = nt-1 .. 0 with the receiver data injected as
// c * d_t at the receiver grid (adjoint forcing) and the zero-lag
// cross-correlation imaging condition of RTMEngine::apply_image_condition
// (rtm/rtm_engine.cpp:24-57) applied in its epilogue:
//     image += V_t * lambda_t,   illum += V_t^2,   lambda_t = mu_t / c;
// then RTMEngine::finalize_image (rtm_engine.cpp:170-182).
//
// The reference's own run_rtm (solver/wave_equation.cpp:621-688) correlates
// the forward field with itself and never back-propagates the data; this
// path keeps its imaging math and its RTMImageCondition outputs and supplies
// the missing adjoint.
#include "st_solver_impl.cuh"
#include "st_slices.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace stg {
namespace {

// f[receiver q] += (c at q) * row[q] over a receiver grid (times the sponge
// factor D at q with the stable sponge: mu = c D lambda).
__global__ void rec_force_kernel(float* f, const float* c, Layout L, st_receiver_grid R, const float* row,
                                 const float* dtab, int sw, int stable) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = R.nx * R.ny;
    if (q >= n) return;
    const long long irx = q / R.ny, iry = q - irx * R.ny;
    const long long ix = R.x0 + irx * R.sx, iy = R.y0 + iry * R.sy;
    const long long i = L.at(ix, iy, R.z);
    const float w = stable ? c[i] * sponge_D(L, dtab, sw, ix, iy, R.z) : c[i];
    f[i] += w * row[q];
}

// trace[t] = lambda at the source before the forcing of step t-1:
// (mu - w * d_{t-1}[q_src]) / w with w = c (w = c D with the stable sponge),
// where q_src < 0 when the source is not a receiver.
__global__ void probe_kernel(const float* f, const float* c, Layout L, long long ix, long long iy, long long iz,
                             const float* force_row, long long q, const float* dtab, int sw, int stable,
                             float* out) {
    const long long idx = L.at(ix, iy, iz);
    const float w = stable ? c[idx] * sponge_D(L, dtab, sw, ix, iy, iz) : c[idx];
    float v = f[idx];
    if (force_row && q >= 0) v -= w * force_row[q];
    *out = v / w;
}

__global__ void f32_to_f64_kernel(const float* a, double* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

int check_receivers(const st_solver* s, const st_receiver_grid& R) {
    const Layout& L = s->L;
    ST_CHECK(R.nx >= 0 && R.ny >= 0, ST_ERR_ARG, "bad receiver counts");
    if (R.nx * R.ny == 0) return ST_OK;
    ST_CHECK(R.sx > 0 && R.sy > 0 && R.x0 >= 0 && R.y0 >= 0 && R.x0 + (R.nx - 1) * R.sx < L.nx &&
                 R.y0 + (R.ny - 1) * R.sy < L.ny && R.z >= 0 && R.z < L.nz,
             ST_ERR_ARG, "receiver grid outside the interior");
    return ST_OK;
}

void set_receivers(StepArgs& a, const st_receiver_grid& R) {
    a.rz = (int)R.z;
    a.rx0 = (int)R.x0;
    a.rsx = (int)R.sx;
    a.rnx = (int)R.nx;
    a.ry0 = (int)R.y0;
    a.rsy = (int)R.sy;
    a.rny = (int)R.ny;
}

}  // namespace

int launch_rec_force(st_solver* s, const st_receiver_grid& R, const float* row) {
    const long long nrec = R.nx * R.ny;
    if (nrec <= 0) return ST_OK;
    rec_force_kernel<<<(unsigned)((nrec + 255) / 256), 256, 0, s->stream>>>(s->f[s->ic], s->c, s->L, R, row, s->dtab,
                                                                           s->sw, s->sponge_mode);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

// Forward shot (shared by st_shot_forward and the RTM / gradient drivers).
// seis may be null (no sampling); snap_kind != NONE needs snaps and amax.
int shot_forward_impl(st_solver* s, const st_shot* shot, float* seis, int snap_kind, void* snaps, unsigned* amax,
                      bool slices = false) {
    const Layout& L = s->L;
    ST_CHECK(shot->src_ix >= 0 && shot->src_ix < L.nx && shot->src_iy >= 0 && shot->src_iy < L.ny &&
                 shot->src_iz >= 0 && shot->src_iz < L.nz,
             ST_ERR_ARG, "source outside the interior");
    ST_CHECK(shot->nt >= 0, ST_ERR_ARG, "negative nt");
    ST_TRY(check_receivers(s, shot->rec));
    const st_receiver_grid& R = shot->rec;
    const int64_t nrec = R.nx * R.ny;
    ST_TRY(refresh_coeff(s));
    ST_TRY(zero_fields(s));
    const int nt = shot->nt;
    const size_t per = (size_t)(L.nx * L.ny * L.nz) * (size_t)snap_bytes(snap_kind);
    if (snap_kind != SNAP_NONE) ST_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned) * (size_t)(nt + 1), s->stream));
    const long long src = dev_index(s, shot->src_ix, shot->src_iy, shot->src_iz);
    float w = 0.0f;
    if (nt > 0 && finite_sample(shot->wavelet, shot->wavelet_len, 0, &w))
        ST_TRY(launch_add_point(s->f[s->ic], src, w, snap_kind != SNAP_NONE ? amax : nullptr, s->stream));
    // pairs of steps share one launch unless a step's field is needed on its
    // own (slice capture) or a terrain is attached; a pair leaves the snapshot
    // of its first output pending: the next pair stores it from its previous
    // field, a single step or the end of the pass stores it here
    const bool pairs = s->fused_steps == 2 && !s->zlim && !(slices && s->slices) && L.nz % 4 == 0;
    bool pending = false;
    auto store_pending = [&](int t) -> int {
        if (!pending) return ST_OK;
        pending = false;
        return launch_snapshot_of_field(s->f[s->ip], L, static_cast<char*>(snaps) + (size_t)(t - 1) * per,
                                        snap_kind, amax + t - 1, s->stream);
    };
    for (int t = 0; t < nt; ++t) {
        if (pairs && t + 1 < nt) {
            StepArgs a = base_args(s, nullptr);
            float w1 = 0.0f, w2 = 0.0f;
            const bool i1 = finite_sample(shot->wavelet, shot->wavelet_len, t + 1, &w1);
            const bool i2 = t + 2 < nt && finite_sample(shot->wavelet, shot->wavelet_len, t + 2, &w2);
            if (i1 || i2) {
                set_injection(a, shot->src_ix, shot->src_iy, shot->src_iz, w1);
                a.inj_val2 = w2;
                a.inj_steps = (i1 ? 1 : 0) | (i2 ? 2 : 0);
            }
            if (nrec > 0 && seis) {
                set_receivers(a, R);
                a.seis_row = seis + (size_t)t * (size_t)nrec;
                a.seis_row2 = seis + (size_t)(t + 1) * (size_t)nrec;
            }
            if (snap_kind != SNAP_NONE) {
                a.snap_out = static_cast<char*>(snaps) + (size_t)t * per;
                a.amax_cur = amax + t;
                if (pending) {
                    a.snap_out2 = static_cast<char*>(snaps) + (size_t)(t - 1) * per;
                    a.amax_cur2 = amax + t - 1;
                }
                a.amax_next = amax + t + 1;
                a.amax_next2 = amax + t + 2;
                pending = true;
            }
            ST_TRY(fused_step2_forward(s, a, snap_kind));
            ++t;
            continue;
        }
        if (snap_kind != SNAP_NONE) ST_TRY(store_pending(t));
        StepArgs a = base_args(s, nullptr);
        float wn = 0.0f;
        if (t + 1 < nt && finite_sample(shot->wavelet, shot->wavelet_len, t + 1, &wn))
            set_injection(a, shot->src_ix, shot->src_iy, shot->src_iz, wn);
        if (nrec > 0 && seis) {
            set_receivers(a, R);
            a.seis_row = seis + (size_t)t * (size_t)nrec;
        }
        if (snap_kind != SNAP_NONE) {
            a.snap_out = static_cast<char*>(snaps) + (size_t)t * per;
            a.amax_cur = amax + t;
            a.amax_next = amax + t + 1;
        }
        ST_TRY(fused_step(s, a, snap_kind, SNAP_NONE, 0, nullptr));
        if (slices && s->slices && t % s->slice_interval == 0) {
            const SliceSrc S{s->f[s->ic], nullptr, nullptr, ST_FIELD_DEVICE_FP32, ST_IMAGE_FP32, L};
            ST_TRY(slice_stream_capture(s->slices, S, t, s->stream));
        }
    }
    if (snap_kind != SNAP_NONE) ST_TRY(store_pending(nt));
    return ST_OK;
}

// Receiver number of grid point (ix, iy, iz), or -1.
long long receiver_at(const st_receiver_grid& R, int64_t ix, int64_t iy, int64_t iz) {
    if (R.nx * R.ny == 0 || iz != R.z) return -1;
    const int64_t xx = ix - R.x0, yy = iy - R.y0;
    if (xx < 0 || yy < 0 || xx % R.sx || yy % R.sy || xx / R.sx >= R.nx || yy / R.sy >= R.ny) return -1;
    return (xx / R.sx) * R.ny + yy / R.sy;
}

// Backward pass of the exact adjoint. With snaps != null the imaging
// epilogue runs (image/illum); with src_trace != null lambda at the source
// is sampled after every step (the transpose of the wavelet -> data map).
int rtm_backward_impl(st_solver* s, const st_shot* shot, const float* data, int snap_kind, const void* snaps,
                      const unsigned* amax, float* image, float* illum, float* src_trace = nullptr) {
    const Layout& L = s->L;
    const st_receiver_grid& R = shot->rec;
    const int64_t nrec = R.nx * R.ny;
    const int nt = shot->nt;
    const size_t npts = (size_t)(L.nx * L.ny * L.nz);
    const size_t per = npts * (size_t)snap_bytes(snap_kind);
    const bool imaging = snaps != nullptr;
    // the imaging operands ride the TMA ring when the store's rows allow it
    ImageMaps imaps;
    const bool staged = imaging && image_maps_supported(snap_kind, L);
    if (staged) ST_TRY(build_image_maps(&imaps, snaps, snap_kind, std::max(nt, 1), image, illum, L));
    ST_TRY(zero_fields(s));
    if (imaging) {
        ST_CUDA(cudaMemsetAsync(image, 0, npts * sizeof(float), s->stream));
        ST_CUDA(cudaMemsetAsync(illum, 0, npts * sizeof(float), s->stream));
    }
    if (nt <= 0) return ST_OK;
    if (nrec > 0) {
        ST_TRY(launch_rec_force(s, R, data + (size_t)(nt - 1) * nrec));
    }
    const long long src = dev_index(s, shot->src_ix, shot->src_iy, shot->src_iz);
    const long long q_src = receiver_at(R, shot->src_ix, shot->src_iy, shot->src_iz);
    // pairs of steps share one launch unless a step's field is needed on its
    // own (slice capture, source trace)
    const bool pairs = staged && s->fused_steps == 2 && !s->slices && !src_trace;
    for (int t = nt - 1; t >= 0; --t) {
        if (pairs && t >= 1) {
            StepArgs a = base_args(s, nullptr);
            if (nrec > 0) {
                set_receivers(a, R);
                a.force_row = data + (size_t)(t - 1) * nrec;
                if (t >= 2) a.force_row2 = data + (size_t)(t - 2) * nrec;
            }
            a.snap_t = t;
            a.amax_in = amax + t;
            a.amax_in2 = amax + t - 1;
            a.image = image;
            a.illum = illum;
            ST_TRY(fused_step2(s, a, snap_kind, imaps));
            --t;
            continue;
        }
        StepArgs a = base_args(s, nullptr);
        if (nrec > 0 && t >= 1) {
            set_receivers(a, R);
            a.force_row = data + (size_t)(t - 1) * nrec;
        }
        if (imaging) {
            a.snap_in = static_cast<const char*>(snaps) + (size_t)t * per;
            a.snap_t = t;
            a.amax_in = amax + t;
            a.image = image;
            a.illum = illum;
        }
        ST_TRY(fused_step(s, a, SNAP_NONE, imaging ? snap_kind : SNAP_NONE, imaging ? 1 : 0, nullptr,
                          staged ? &imaps : nullptr));
        if (imaging && s->slices && t % s->slice_interval == 0) {
            SliceSrc S{a.snap_in, s->f[s->ic], image, ST_FIELD_DEVICE_FP32, ST_IMAGE_FP32, L};
            S.fwd_snap = snap_kind;
            S.fwd_amax = amax + t;
            ST_TRY(slice_stream_capture(s->slices, S, t, s->stream));
        }
        if (src_trace) {
            probe_kernel<<<1, 1, 0, s->stream>>>(s->f[s->ic], s->c, L, shot->src_ix, shot->src_iy, shot->src_iz,
                                                 a.force_row, q_src, s->dtab, s->sw, s->sponge_mode, src_trace + t);
    ::stg::count_launch();
            ST_CUDA(cudaGetLastError());
        }
    }
    return ST_OK;
}

}  // namespace stg

using namespace stg;

extern "C" {

int st_shot_forward(st_solver* s, const st_shot* shot, float* seis, int snap_kind, void* snaps, unsigned* snap_amax) {
    ST_CHECK(s && shot, ST_ERR_ARG, "null argument");
    ST_CHECK(snap_kind >= ST_SNAP_NONE && snap_kind <= ST_SNAP_FP32, ST_ERR_ARG, "bad snapshot kind %d", snap_kind);
    ST_CHECK(snap_kind == ST_SNAP_NONE || (snaps && snap_amax), ST_ERR_ARG, "snapshot buffers missing");
    ST_CHECK(shot->rec.nx * shot->rec.ny == 0 || seis, ST_ERR_ARG, "receivers given but no seismogram buffer");
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(shot_forward_impl(s, shot, seis, snap_kind, snaps, snap_amax, true));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

int st_shot_adjoint(st_solver* s, const st_shot* shot, const float* data, float* src_trace) {
    ST_CHECK(s && shot && src_trace, ST_ERR_ARG, "null argument");
    ST_TRY(require_no_terrain(s));
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    ST_CHECK(nrec == 0 || data, ST_ERR_ARG, "receiver data missing");
    ST_CHECK(shot->src_ix >= 0 && shot->src_ix < s->L.nx && shot->src_iy >= 0 && shot->src_iy < s->L.ny &&
                 shot->src_iz >= 0 && shot->src_iz < s->L.nz,
             ST_ERR_ARG, "source outside the interior");
    ST_TRY(check_receivers(s, shot->rec));
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(refresh_coeff(s));
    ST_TRY(rtm_backward_impl(s, shot, data, SNAP_NONE, nullptr, nullptr, nullptr, nullptr, src_trace));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

// RTM shot; data_ready (may be null): an event the adjoint pass waits on
// before it reads `data` (the host entry point's upload runs beside the
// forward pass).
static int rtm_shot_impl(st_solver* s, const st_shot* shot, const float* data, int snap_kind, void* snaps,
                         unsigned* snap_amax, float* image, float* illum, float* refl, cudaEvent_t data_ready) {
    ST_CHECK(s && shot && image && illum, ST_ERR_ARG, "null argument");
    ST_TRY(require_no_terrain(s));
    ST_CHECK(snap_kind >= ST_SNAP_BF16 && snap_kind <= ST_SNAP_FP32, ST_ERR_ARG,
             "RTM snapshot kind must be BF16, FP16 or FP32 (got %d)", snap_kind);
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    ST_CHECK(nrec == 0 || data, ST_ERR_ARG, "receiver data missing");
    ST_CUDA(cudaSetDevice(s->device));
    const size_t npts = (size_t)(s->L.nx * s->L.ny * s->L.nz);
    const size_t snap_total = npts * (size_t)snap_bytes(snap_kind) * (size_t)std::max(shot->nt, 1);
    unsigned* amax = snap_amax;
    if (!snaps) {
        ST_TRY(ensure_buffer(s, &s->snap_buf, &s->snap_cap, snap_total));
        snaps = s->snap_buf;
    }
    if (!amax) {
        ST_TRY(ensure_buffer(s, &s->aux_buf, &s->aux_cap, sizeof(unsigned) * (size_t)(shot->nt + 1)));
        amax = static_cast<unsigned*>(s->aux_buf);
    }
    ST_CUDA(cudaEventRecord(s->ev[0], s->stream));
    ST_TRY(shot_forward_impl(s, shot, nullptr, snap_kind, snaps, amax));
    ST_CUDA(cudaEventRecord(s->ev[1], s->stream));
    if (data_ready) ST_CUDA(cudaStreamWaitEvent(s->stream, data_ready, 0));
    ST_TRY(rtm_backward_impl(s, shot, data, snap_kind, snaps, amax, image, illum));
    ST_CUDA(cudaEventRecord(s->ev[2], s->stream));
    s->phases_recorded = 1;
    if (refl) ST_TRY(launch_finalize_image(image, illum, refl, (long long)npts, s->stream));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

int st_rtm_shot(st_solver* s, const st_shot* shot, const float* data, int snap_kind, void* snaps,
                unsigned* snap_amax, float* image, float* illum, float* refl) {
    return rtm_shot_impl(s, shot, data, snap_kind, snaps, snap_amax, image, illum, refl, nullptr);
}

int st_rtm_shot_host(st_solver* s, const double* vp, int64_t vp_count, const st_shot* shot, const float* data_host,
                     int snap_kind, double* image_host, double* illum_host, double* refl_host) {
    ST_CHECK(s && shot, ST_ERR_ARG, "null argument");
    ST_TRY(require_no_terrain(s));
    ST_CUDA(cudaSetDevice(s->device));
    if (vp) ST_TRY(vp_count >= ref_elems(s) ? upload_velocity(s, vp) : st_solver_set_velocity_field(s, vp, vp_count));
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    const size_t npts = (size_t)(s->L.nx * s->L.ny * s->L.nz);
    const size_t dbytes = (size_t)nrec * (size_t)std::max(shot->nt, 0) * sizeof(float);
    const size_t snap_total = npts * (size_t)snap_bytes(snap_kind) * (size_t)std::max(shot->nt, 1);
    // aux layout: amax[nt+1] | image | illum | refl | fp64 out
    const size_t amax_bytes = ((sizeof(unsigned) * (size_t)(shot->nt + 1) + 255) / 256) * 256;
    const size_t img_bytes = ((npts * sizeof(float) + 255) / 256) * 256;
    ST_TRY(ensure_buffer(s, &s->aux_buf, &s->aux_cap, amax_bytes + 3 * img_bytes + npts * sizeof(double)));
    char* aux = static_cast<char*>(s->aux_buf);
    unsigned* amax = reinterpret_cast<unsigned*>(aux);
    float* image = reinterpret_cast<float*>(aux + amax_bytes);
    float* illum = reinterpret_cast<float*>(aux + amax_bytes + img_bytes);
    float* refl = reinterpret_cast<float*>(aux + amax_bytes + 2 * img_bytes);
    double* out64 = reinterpret_cast<double*>(aux + amax_bytes + 3 * img_bytes);
    ST_TRY(ensure_buffer(s, &s->snap_buf, &s->snap_cap, snap_total));
    float* data = nullptr;
    cudaEvent_t data_ready = nullptr;
    if (dbytes > 0) {
        ST_CHECK(data_host, ST_ERR_ARG, "receiver data missing");
        ST_TRY(ensure_buffer(s, &s->data_buf, &s->data_cap, dbytes));
        data = static_cast<float*>(s->data_buf);
        // the receiver data is read only by the adjoint pass: upload it on a
        // second stream while the forward pass runs (the buffer's last reader,
        // the previous call, has finished: every call ends synchronised)
        if (!s->copy_stream) {
            ST_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
            ST_CUDA(cudaEventCreateWithFlags(&s->ev_copy, cudaEventDisableTiming));
        }
        ST_CUDA(cudaMemcpyAsync(data, data_host, dbytes, cudaMemcpyHostToDevice, s->copy_stream));
        ST_CUDA(cudaEventRecord(s->ev_copy, s->copy_stream));
        data_ready = s->ev_copy;
    }
    int rc = rtm_shot_impl(s, shot, data, snap_kind, s->snap_buf, amax, image, illum, refl, data_ready);
    if (rc < 0 && s->copy_stream) cudaStreamSynchronize(s->copy_stream);
    if (rc < 0) return rc;
    const float* srcs[3] = {image, illum, refl};
    double* dsts[3] = {image_host, illum_host, refl_host};
    for (int k = 0; k < 3; ++k) {
        if (!dsts[k]) continue;
        f32_to_f64_kernel<<<1024, 256, 0, s->stream>>>(srcs[k], out64, (long long)npts);
    ::stg::count_launch();
        ST_CUDA(cudaGetLastError());
        ST_CUDA(cudaMemcpyAsync(dsts[k], out64, npts * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    }
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return rc;
}

}  // extern "C"
