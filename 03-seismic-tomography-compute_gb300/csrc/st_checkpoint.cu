// Checkpointed adjoint passes: RTM imaging and velocity gradients whose
// forward wavefield history does not have to fit in device memory.
//
// The time axis is cut into segments of K steps. A checkpoint is the exact
// FP32 forward state (current and undamped previous field) at a segment
// boundary; the adjoint of one segment is (1) restore the segment's start
// state, (2) recompute its K forward steps storing the snapshots into a
// K-slot buffer (BF16 / FP16 / FP32 with the per-snapshot scale), (3) run the
// K adjoint steps backwards, reading them in the fused imaging or gradient
// epilogue. Which boundaries hold a checkpoint follows the binomial schedule
// of Griewank's revolve (ACM TOMS 26(1), 2000): with s free slots and
// l segments to reverse, the smallest repetition number r with
// C(s+r, s) >= l bounds how often a segment is advanced, and the first
// checkpoint goes at offset  clamp(l - C(s-1+r, s-1), 1, C(s+r-1, s)).
// With at least as many slots as segments this is one plain forward sweep
// plus one recompute, the cheapest schedule that does not store every step.
//
// The recomputed snapshots equal those of the store-everything passes bit
// for bit: the fused step is deterministic and the scale of the first
// snapshot of a segment (the absolute maximum of the restored field) is the
// value the store-everything pass accumulated for it.
#include "st_solver_impl.cuh"

#include <algorithm>
#include <cmath>
#include <functional>
#include <utility>
#include <vector>

namespace stg {
namespace {

__global__ void absmax_kernel(const float* __restrict__ f, long long n, unsigned* out) {
    float m = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(f[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// C(s + r, s), saturated.
double binom_steps(int s, int r) {
    double v = 1.0;
    for (int i = 1; i <= s; ++i) {
        v = v * (double)(r + i) / (double)i;
        if (v > 1e18) return 1e18;
    }
    return v;
}

// First checkpoint offset for reversing l >= 2 segments with s >= 1 free slots.
int split_offset(int l, int s) {
    int r = 1;
    while (binom_steps(s, r) < (double)l) ++r;
    const double right = binom_steps(s - 1, r), left_max = binom_steps(s, r - 1);
    double off = (double)l - right;
    off = std::max(1.0, std::min(off, left_max));
    return (int)std::min<double>(off, (double)(l - 1));
}

}  // namespace

struct CkptRun {
    st_solver* s = nullptr;
    const st_shot* shot = nullptr;
    int kind = SNAP_BF16;
    int seg = 1, nseg = 1, nslots = 1;
    // forward working set (swapped into the handle while forward steps run)
    float* g[3] = {nullptr, nullptr, nullptr};
    FieldMaps gm[3];
    int gc = 0, gp = 1, gn = 2;
    float* g4 = nullptr;  // the set's spare field for two-step launches (swapped with the handle's spare)
    FieldMaps gm4;
    int work_at = -1;  // segment whose start state the working set holds
    float* slots = nullptr;
    std::vector<int> slot_of;  // segment -> slot, -1 when none
    std::vector<int> free_slots;
    char* segbuf = nullptr;
    unsigned* amax_seg = nullptr;
    float* seis = nullptr;  // receiver sampling during forward steps (may be null)
    // backward
    int epi = 1;
    const float* force = nullptr;
    float* image = nullptr;
    float* illum = nullptr;
    float* grad_c = nullptr;
    CUtensorMap msnap;
    CUtensorMap mgrad;     // compact map of grad_c (gradient step pairs)
    bool grad_pairs = false;
    ImageMaps imaps;
    bool staged = false;
    std::function<int()> before_backward;
    bool started = false;
    st_checkpoint_stats stats{};

    size_t per() const { return (size_t)(s->L.nx * s->L.ny * s->L.nz) * (size_t)snap_bytes(kind); }
    int seg_begin(int j) const { return j * seg; }
    int seg_end(int j) const { return std::min(shot->nt, (j + 1) * seg); }
    float* slot_field(int k, int which) const { return slots + ((size_t)k * 2 + which) * (size_t)s->L.elems; }
};

namespace {

void swap_sets(CkptRun& c) {
    st_solver* s = c.s;
    for (int k = 0; k < 3; ++k) {
        std::swap(s->f[k], c.g[k]);
        std::swap(s->maps[k], c.gm[k]);
    }
    std::swap(s->ic, c.gc);
    std::swap(s->ip, c.gp);
    std::swap(s->in, c.gn);
    std::swap(s->f4, c.g4);
    std::swap(s->map4, c.gm4);
}

struct ForwardSet {
    CkptRun& c;
    explicit ForwardSet(CkptRun& r) : c(r) { swap_sets(c); }
    ~ForwardSet() { swap_sets(c); }
};

int copy_field(st_solver* s, float* dst, const float* src) {
    ST_CUDA(cudaMemcpyAsync(dst, src, (size_t)s->L.elems * sizeof(float), cudaMemcpyDeviceToDevice, s->stream));
    return ST_OK;
}

int take_shot(CkptRun& c, int j) {
    ST_CHECK(!c.free_slots.empty(), ST_ERR_STATE, "no free checkpoint slot");
    const int k = c.free_slots.back();
    c.free_slots.pop_back();
    c.slot_of[j] = k;
    ST_TRY(copy_field(c.s, c.slot_field(k, 0), c.g[c.gc]));
    ST_TRY(copy_field(c.s, c.slot_field(k, 1), c.g[c.gp]));
    c.stats.state_copies += 1;
    c.stats.slots_used = std::max(c.stats.slots_used, c.nslots - (int)c.free_slots.size());
    return ST_OK;
}

void release(CkptRun& c, int j) {
    if (c.slot_of[j] >= 0) c.free_slots.push_back(c.slot_of[j]);
    c.slot_of[j] = -1;
}

int restore(CkptRun& c, int j) {
    if (c.work_at == j) return ST_OK;
    const int k = c.slot_of[j];
    ST_CHECK(k >= 0, ST_ERR_STATE, "segment %d has no checkpoint", j);
    c.gc = 0;
    c.gp = 1;
    c.gn = 2;
    ST_TRY(copy_field(c.s, c.g[0], c.slot_field(k, 0)));
    ST_TRY(copy_field(c.s, c.g[1], c.slot_field(k, 1)));
    c.stats.state_copies += 1;
    c.work_at = j;
    return ST_OK;
}

// Forward steps t0..t1-1 on the working set, storing snapshots when `store`.
int forward_steps(CkptRun& c, int t0, int t1, bool store) {
    st_solver* s = c.s;
    const st_shot* shot = c.shot;
    const st_receiver_grid& R = shot->rec;
    const int64_t nrec = R.nx * R.ny;
    const size_t per = c.per();
    ForwardSet fs(c);
    // pairs of steps inside [t0, t1) share one launch; a pair leaves the
    // snapshot of its first output pending, stored by the next pair from its
    // previous field, or here before a single step and at the end
    const bool pairs = s->fused_steps == 2 && s->L.nz % 4 == 0;
    bool pending = false;
    auto store_pending = [&](int t) -> int {
        if (!pending) return ST_OK;
        pending = false;
        return launch_snapshot_of_field(s->f[s->ip], s->L, c.segbuf + (size_t)(t - 1 - t0) * per, c.kind,
                                        c.amax_seg + (t - 1 - t0), s->stream);
    };
    for (int t = t0; t < t1; ++t) {
        if (pairs && t + 1 < t1) {
            StepArgs a = base_args(s, nullptr);
            float w1 = 0.0f, w2 = 0.0f;
            const bool i1 = finite_sample(shot->wavelet, shot->wavelet_len, t + 1, &w1);
            const bool i2 = t + 2 < shot->nt && finite_sample(shot->wavelet, shot->wavelet_len, t + 2, &w2);
            if (i1 || i2) {
                set_injection(a, shot->src_ix, shot->src_iy, shot->src_iz, w1);
                a.inj_val2 = w2;
                a.inj_steps = (i1 ? 1 : 0) | (i2 ? 2 : 0);
            }
            if (nrec > 0 && c.seis) {
                a.rz = (int)R.z;
                a.rx0 = (int)R.x0;
                a.rsx = (int)R.sx;
                a.rnx = (int)R.nx;
                a.ry0 = (int)R.y0;
                a.rsy = (int)R.sy;
                a.rny = (int)R.ny;
                a.seis_row = c.seis + (size_t)t * (size_t)nrec;
                a.seis_row2 = c.seis + (size_t)(t + 1) * (size_t)nrec;
            }
            if (store) {
                a.snap_out = c.segbuf + (size_t)(t - t0) * per;
                a.amax_cur = c.amax_seg + (t - t0);
                if (pending) {
                    a.snap_out2 = c.segbuf + (size_t)(t - 1 - t0) * per;
                    a.amax_cur2 = c.amax_seg + (t - 1 - t0);
                }
                a.amax_next = c.amax_seg + (t - t0) + 1;
                a.amax_next2 = c.amax_seg + (t - t0) + 2;
                pending = true;
            }
            ST_TRY(fused_step2_forward(s, a, store ? c.kind : SNAP_NONE));
            c.stats.forward_steps += 2;
            ++t;
            continue;
        }
        if (store) ST_TRY(store_pending(t));
        StepArgs a = base_args(s, nullptr);
        float wn = 0.0f;
        if (t + 1 < shot->nt && finite_sample(shot->wavelet, shot->wavelet_len, t + 1, &wn))
            set_injection(a, shot->src_ix, shot->src_iy, shot->src_iz, wn);
        if (nrec > 0 && c.seis) {
            a.rz = (int)R.z;
            a.rx0 = (int)R.x0;
            a.rsx = (int)R.sx;
            a.rnx = (int)R.nx;
            a.ry0 = (int)R.y0;
            a.rsy = (int)R.sy;
            a.rny = (int)R.ny;
            a.seis_row = c.seis + (size_t)t * (size_t)nrec;
        }
        if (store) {
            a.snap_out = c.segbuf + (size_t)(t - t0) * per;
            a.amax_cur = c.amax_seg + (t - t0);
            a.amax_next = c.amax_seg + (t - t0) + 1;
        }
        ST_TRY(fused_step(s, a, store ? c.kind : SNAP_NONE, SNAP_NONE, 0, nullptr));
        c.stats.forward_steps += 1;
    }
    if (store) ST_TRY(store_pending(t1));
    return ST_OK;
}

int advance(CkptRun& c, int a, int m) {
    ST_TRY(forward_steps(c, c.seg_begin(a), c.seg_begin(m), false));
    c.work_at = m;
    return ST_OK;
}

int recompute_store(CkptRun& c, int j) {
    st_solver* s = c.s;
    ST_CUDA(cudaMemsetAsync(c.amax_seg, 0, sizeof(unsigned) * (size_t)(c.seg + 1), s->stream));
    absmax_kernel<<<1024, 256, 0, s->stream>>>(c.g[c.gc], s->L.elems, c.amax_seg);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_TRY(forward_steps(c, c.seg_begin(j), c.seg_end(j), true));
    c.work_at = j + 1;
    return ST_OK;
}

int backward(CkptRun& c, int j) {
    st_solver* s = c.s;
    const Layout& L = s->L;
    const st_receiver_grid& R = c.shot->rec;
    const int64_t nrec = R.nx * R.ny;
    const int nt = c.shot->nt;
    const size_t npts = (size_t)(L.nx * L.ny * L.nz);
    const size_t per = c.per();
    if (!c.started) {
        if (c.before_backward) ST_TRY(c.before_backward());
        ST_TRY(zero_fields(s));
        if (c.epi == 1) {
            ST_CUDA(cudaMemsetAsync(c.image, 0, npts * sizeof(float), s->stream));
            ST_CUDA(cudaMemsetAsync(c.illum, 0, npts * sizeof(float), s->stream));
        } else {
            ST_CUDA(cudaMemsetAsync(c.grad_c, 0, npts * sizeof(float), s->stream));
        }
        if (nrec > 0) {
            ST_TRY(launch_rec_force(s, R, c.force + (size_t)(nt - 1) * nrec));
        }
        c.started = true;
    }
    const int t0 = c.seg_begin(j), t1 = c.seg_end(j);
    // imaging and gradient: pairs of steps inside the segment share one
    // launch (the solver's own fields and spare; the checkpoint sets are not
    // involved)
    const bool pairs = (c.epi == 1 && c.staged && s->fused_steps == 2) || (c.epi == 2 && c.grad_pairs);
    for (int t = t1 - 1; t >= t0; --t) {
        if (pairs && t - 1 >= t0) {
            StepArgs a = base_args(s, nullptr);
            if (nrec > 0) {
                a.rz = (int)R.z;
                a.rx0 = (int)R.x0;
                a.rsx = (int)R.sx;
                a.rnx = (int)R.nx;
                a.ry0 = (int)R.y0;
                a.rsy = (int)R.sy;
                a.rny = (int)R.ny;
                a.force_row = c.force + (size_t)(t - 1) * nrec;
                if (t >= 2) a.force_row2 = c.force + (size_t)(t - 2) * nrec;
            }
            a.snap_t = t - t0;
            a.amax_in = c.amax_seg + (t - t0);
            a.amax_in2 = c.amax_seg + (t - 1 - t0);
            if (c.epi == 1) {
                a.image = c.image;
                a.illum = c.illum;
                ST_TRY(fused_step2(s, a, c.kind, c.imaps));
            } else {
                a.grad = c.grad_c;
                ST_TRY(fused_step2_grad(s, a, c.kind, c.msnap, c.mgrad));
            }
            c.stats.adjoint_steps += 2;
            --t;
            continue;
        }
        StepArgs a = base_args(s, nullptr);
        if (nrec > 0 && t >= 1) {
            a.rz = (int)R.z;
            a.rx0 = (int)R.x0;
            a.rsx = (int)R.sx;
            a.rnx = (int)R.nx;
            a.ry0 = (int)R.y0;
            a.rsy = (int)R.sy;
            a.rny = (int)R.ny;
            a.force_row = c.force + (size_t)(t - 1) * nrec;
        }
        a.amax_in = c.amax_seg + (t - t0);
        if (c.epi == 1) {
            a.snap_in = c.segbuf + (size_t)(t - t0) * per;
            a.snap_t = t - t0;
            a.image = c.image;
            a.illum = c.illum;
            ST_TRY(fused_step(s, a, SNAP_NONE, c.kind, 1, nullptr, c.staged ? &c.imaps : nullptr));
        } else {
            a.snap_t = t - t0;
            a.grad = c.grad_c;
            ST_TRY(fused_step(s, a, SNAP_NONE, c.kind, 2, &c.msnap));
        }
        c.stats.adjoint_steps += 1;
    }
    return ST_OK;
}

// Reverses segments [a, b); the start state of segment a is in a slot.
int reverse(CkptRun& c, int a, int b) {
    const int free_n = (int)c.free_slots.size();
    if (b - a == 1) {
        ST_TRY(restore(c, a));
        ST_TRY(recompute_store(c, a));
        return backward(c, a);
    }
    if (free_n == 0) {
        for (int j = b - 1; j >= a; --j) {
            ST_TRY(restore(c, a));
            if (j > a) ST_TRY(advance(c, a, j));
            ST_TRY(recompute_store(c, j));
            ST_TRY(backward(c, j));
        }
        return ST_OK;
    }
    const int m = a + split_offset(b - a, free_n);
    ST_TRY(restore(c, a));
    ST_TRY(advance(c, a, m));
    ST_TRY(take_shot(c, m));
    ST_TRY(reverse(c, m, b));
    release(c, m);
    return reverse(c, a, m);
}

}  // namespace

// Shared driver of the checkpointed RTM and gradient entry points. epi 1:
// image / illum accumulate the imaging condition; epi 2: grad_c accumulates
// the coefficient gradient. seis (may be null) receives the forward
// seismograms before before_backward runs.
int checkpointed_adjoint(st_solver* s, const st_shot* shot, int snap_kind, int segment_steps, int max_slots, int epi,
                         const float* force, float* image, float* illum, float* grad_c, float* seis,
                         const std::function<int()>& before_backward, st_checkpoint_stats* stats) {
    const Layout& L = s->L;
    const int nt = shot->nt;
    ST_CHECK(segment_steps >= 1, ST_ERR_ARG, "segment_steps must be >= 1 (got %d)", segment_steps);
    ST_CHECK(max_slots >= 1, ST_ERR_ARG, "max_slots must be >= 1 (got %d)", max_slots);
    ST_CHECK(shot->src_ix >= 0 && shot->src_ix < L.nx && shot->src_iy >= 0 && shot->src_iy < L.ny &&
                 shot->src_iz >= 0 && shot->src_iz < L.nz,
             ST_ERR_ARG, "source outside the interior");
    const st_receiver_grid& R = shot->rec;
    if (R.nx * R.ny > 0)
        ST_CHECK(R.sx > 0 && R.sy > 0 && R.x0 >= 0 && R.y0 >= 0 && R.x0 + (R.nx - 1) * R.sx < L.nx &&
                     R.y0 + (R.ny - 1) * R.sy < L.ny && R.z >= 0 && R.z < L.nz,
                 ST_ERR_ARG, "receiver grid outside the interior");
    CkptRun c;
    c.s = s;
    c.shot = shot;
    c.kind = snap_kind;
    c.seg = std::max(1, std::min(segment_steps, std::max(nt, 1)));
    c.nseg = std::max(1, (nt + c.seg - 1) / c.seg);
    c.nslots = std::min(max_slots, c.nseg);
    c.epi = epi;
    c.force = force;
    c.image = image;
    c.illum = illum;
    c.grad_c = grad_c;
    c.seis = seis;
    c.before_backward = before_backward;
    c.stats.segments = c.nseg;
    c.stats.segment_steps = c.seg;

    // device memory: 4 working fields | slots x 2 fields | K snapshots | K+1 scales
    auto al = [](size_t b) { return ((b + 255) / 256) * 256; };
    const size_t fbytes = al((size_t)L.elems * sizeof(float));
    const size_t sbytes = al(c.per() * (size_t)c.seg);
    const size_t abytes = al(sizeof(unsigned) * (size_t)(c.seg + 1));
    const size_t total = fbytes * (4 + 2 * (size_t)c.nslots) + sbytes + abytes;
    ST_TRY(ensure_buffer(s, &s->ckpt_buf, &s->ckpt_cap, total));
    c.stats.device_bytes = (int64_t)total;
    char* p = static_cast<char*>(s->ckpt_buf);
    for (int k = 0; k < 3; ++k) c.g[k] = reinterpret_cast<float*>(p + (size_t)k * fbytes);
    c.slots = reinterpret_cast<float*>(p + 3 * fbytes);
    c.g4 = reinterpret_cast<float*>(p + fbytes * (3 + 2 * (size_t)c.nslots));
    c.segbuf = p + fbytes * (4 + 2 * (size_t)c.nslots);
    c.amax_seg = reinterpret_cast<unsigned*>(c.segbuf + sbytes);
    for (int k = 0; k < 3; ++k) ST_TRY(build_field_maps(&c.gm[k], c.g[k], L));
    // the set's spare: zero once, its halo stays zero (two-step launches write interiors only)
    ST_CUDA(cudaMemsetAsync(c.g4, 0, (size_t)L.elems * sizeof(float), s->stream));
    ST_TRY(build_field_maps(&c.gm4, c.g4, L));
    if (epi == 2) ST_TRY(build_snap_map_grad(&c.msnap, c.segbuf, snap_kind, L, c.seg));
    c.grad_pairs = epi == 2 && s->fused_steps == 2 && L.nz % 4 == 0;
    if (c.grad_pairs) ST_TRY(make_compact_map(&c.mgrad, c.grad_c, L, FD_TZ, 16));
    c.staged = epi == 1 && image_maps_supported(snap_kind, L);
    if (c.staged) ST_TRY(build_image_maps(&c.imaps, c.segbuf, snap_kind, c.seg, image, illum, L));
    c.slot_of.assign((size_t)c.nseg, -1);
    for (int k = c.nslots - 1; k >= 0; --k) c.free_slots.push_back(k);

    ST_TRY(refresh_coeff(s));
    // slot fields are full copies of zero-halo fields, so only the working set is cleared
    ST_CUDA(cudaMemsetAsync(p, 0, 3 * fbytes, s->stream));
    if (nt <= 0) {
        ST_TRY(zero_fields(s));
        const size_t npts = (size_t)(L.nx * L.ny * L.nz);
        if (epi == 1) {
            ST_CUDA(cudaMemsetAsync(image, 0, npts * sizeof(float), s->stream));
            ST_CUDA(cudaMemsetAsync(illum, 0, npts * sizeof(float), s->stream));
        } else {
            ST_CUDA(cudaMemsetAsync(grad_c, 0, npts * sizeof(float), s->stream));
        }
        if (stats) *stats = c.stats;
        return ST_OK;
    }
    // state 0: zero fields plus the first wavelet sample at the source
    float w = 0.0f;
    if (finite_sample(shot->wavelet, shot->wavelet_len, 0, &w))
        ST_TRY(launch_add_point(c.g[c.gc], L.at(shot->src_ix, shot->src_iy, shot->src_iz), w, nullptr, s->stream));
    c.work_at = 0;
    ST_TRY(take_shot(c, 0));
    ST_TRY(reverse(c, 0, c.nseg));
    if (stats) *stats = c.stats;
    return ST_OK;
}

}  // namespace stg

using namespace stg;

extern "C" int st_rtm_shot_checkpointed(st_solver* s, const st_shot* shot, const float* data, int snap_kind,
                                        int segment_steps, int max_slots, float* image, float* illum, float* refl,
                                        st_checkpoint_stats* stats) {
    ST_CHECK(s && shot && image && illum, ST_ERR_ARG, "null argument");
    ST_TRY(require_no_terrain(s));
    ST_CHECK(snap_kind >= ST_SNAP_BF16 && snap_kind <= ST_SNAP_FP32, ST_ERR_ARG,
             "RTM snapshot kind must be BF16, FP16 or FP32 (got %d)", snap_kind);
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    ST_CHECK(nrec == 0 || data, ST_ERR_ARG, "receiver data missing");
    ST_CHECK(shot->nt >= 0, ST_ERR_ARG, "negative nt");
    ST_CUDA(cudaSetDevice(s->device));
    ST_CUDA(cudaEventRecord(s->ev[0], s->stream));
    ST_TRY(checkpointed_adjoint(s, shot, snap_kind, segment_steps, max_slots, 1, data, image, illum, nullptr,
                                nullptr, nullptr, stats));
    ST_CUDA(cudaEventRecord(s->ev[1], s->stream));
    ST_CUDA(cudaEventRecord(s->ev[2], s->stream));
    s->phases_recorded = 1;
    if (refl)
        ST_TRY(launch_finalize_image(image, illum, refl, (long long)(s->L.nx * s->L.ny * s->L.nz), s->stream));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}
