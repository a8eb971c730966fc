// Adjoint-state gradients of the forward shot map (FWI).
//
// For J(c) with seismograms d = F(c) (c = v^2 dt^2 per point), the discrete
// adjoint of the forward recursion gives dJ/dc = sum_t lambda_t * L V_t,
// where V_t is the post-injection forward field of step t, lambda_t the
// adjoint state forced by dJ/dd (the transpose of the forward step, run in
// the scaled variable mu = c * lambda by the same fused kernel) and L the
// 7-point Laplacian with the zero halo. The gradient epilogue of the fused
// kernel accumulates lambda_t * L S_t from the stored snapshot S_t (BF16 /
// FP16 / FP32 with a per-snapshot scale), and dJ/dv = dJ/dc * 2 v dt^2
// (times the CFL damping factor^2 when the reference would apply it).
//
// The reference has no such gradient (its Python adjoint-state gradient
// g = -u * lambda * 2 v dt^2, seismic_tomography/gradient.py:24-40, is a
// pointwise formula with no time integration and is never fed a wavefield).
#include "st_solver_impl.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace stg {

int shot_forward_impl(st_solver* s, const st_shot* shot, float* seis, int snap_kind, void* snaps, unsigned* amax,
                      bool slices = false);

namespace {

unsigned nblocks(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, 152 * 16));
}

__global__ void residual_kernel(const float* __restrict__ seis, const float* __restrict__ dobs, long long n,
                                float* __restrict__ res, double* misfit) {
    __shared__ double part[8];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float r = seis[i] - dobs[i];
        res[i] = r;
        s += (double)r * (double)r;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        atomicAdd(misfit, 0.5 * t);
    }
}

// grad_v[i] += grad_c[i] * dc/dv = grad_c * 2 sqrt(c) * (dt * damp).
__global__ void grad_v_kernel(const float* __restrict__ gc, const float* __restrict__ c, Layout L, double dtd,
                              float* __restrict__ gv) {
    const long long n = L.nx * L.ny * L.nz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long ix = e / (L.ny * L.nz), r = e % (L.ny * L.nz), iy = r / L.nz, iz = r % L.nz;
        const float cc = c[L.at(ix, iy, iz)];
        gv[e] += gc[e] * (float)(2.0 * dtd) * sqrtf(cc);
    }
}

// c = v^2 dt2damp from an interior FP32 velocity (fallback 1500 m/s for
// non-finite or non-positive values), zero in the halo.
__global__ void vel_interior_to_coeff_kernel(const float* __restrict__ v, float* __restrict__ c, Layout L,
                                             double dt2damp) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < L.elems;
         e += (long long)gridDim.x * blockDim.x) {
        const long long xd = e / L.plane, r = e % L.plane, yd = r / L.NZP, zd = r % L.NZP;
        const long long ix = xd - 1, iy = yd - 1, iz = zd - Layout::ZOFF;
        float out = 0.0f;
        if (ix >= 0 && ix < L.nx && iy >= 0 && iy < L.ny && iz >= 0 && iz < L.nz) {
            double vv = v[(ix * L.ny + iy) * L.nz + iz];
            if (!isfinite(vv) || vv <= 0.0) vv = 1500.0;
            out = (float)(vv * vv * dt2damp);
        }
        c[e] = out;
    }
}

void set_receivers_args(StepArgs& a, const st_receiver_grid& R) {
    a.rz = (int)R.z;
    a.rx0 = (int)R.x0;
    a.rsx = (int)R.sx;
    a.rnx = (int)R.nx;
    a.ry0 = (int)R.y0;
    a.rsy = (int)R.sy;
    a.rny = (int)R.ny;
}

double cfl_damp(st_solver* s) {
    // the coefficient array already carries damp^2; recover damp from it is
    // not possible per point, so recompute the reference rule on the host copy
    if (ensure_vel_host(s) != ST_OK) return 1.0;  // (a failed download reports through the next CUDA call)
    double vmax = 0.0;
    for (double v : s->vel_host)
        if (std::isfinite(v) && v > vmax) vmax = v;
    const double dt = s->cfg.dt;
    const double cfl = std::max({vmax * dt / s->grid.dx, vmax * dt / s->grid.dy, vmax * dt / s->grid.dz});
    if (cfl <= 1.0) return 1.0;
    const double ratio = vmax * dt / std::min({s->grid.dx, s->grid.dy, s->grid.dz});
    return std::min(1.0, s->cfl_safety / ratio);
}

}  // namespace

// Backward pass of the gradient: adjoint forced by adj (device [nt][nrec]),
// grad_c (compact interior, zeroed here) accumulated from the snapshots.
int gradient_backward_impl(st_solver* s, const st_shot* shot, const float* adj, int snap_kind, const void* snaps,
                           const unsigned* amax, float* grad_c) {
    const Layout& L = s->L;
    const st_receiver_grid& R = shot->rec;
    const int64_t nrec = R.nx * R.ny;
    const int nt = shot->nt;
    const size_t npts = (size_t)(L.nx * L.ny * L.nz);
    CUtensorMap msnap, mgrad;
    ST_TRY(build_snap_map_grad(&msnap, snaps, snap_kind, L, std::max(nt, 1)));
    // pairs of steps share one launch (the gradient of both accumulated once)
    const bool pairs = s->fused_steps == 2 && L.nz % 4 == 0;
    if (pairs) ST_TRY(make_compact_map(&mgrad, grad_c, L, FD_TZ, 16));
    ST_TRY(zero_fields(s));
    ST_CUDA(cudaMemsetAsync(grad_c, 0, npts * sizeof(float), s->stream));
    if (nt <= 0) return ST_OK;
    if (nrec > 0) {
        ST_TRY(launch_rec_force(s, R, adj + (size_t)(nt - 1) * nrec));
    }
    for (int t = nt - 1; t >= 0; --t) {
        if (pairs && t >= 1) {
            StepArgs a = base_args(s, nullptr);
            if (nrec > 0) {
                set_receivers_args(a, R);
                a.force_row = adj + (size_t)(t - 1) * nrec;
                if (t >= 2) a.force_row2 = adj + (size_t)(t - 2) * nrec;
            }
            a.snap_t = t;
            a.amax_in = amax + t;
            a.amax_in2 = amax + t - 1;
            a.grad = grad_c;
            ST_TRY(fused_step2_grad(s, a, snap_kind, msnap, mgrad));
            --t;
            continue;
        }
        StepArgs a = base_args(s, nullptr);
        if (nrec > 0 && t >= 1) {
            set_receivers_args(a, R);
            a.force_row = adj + (size_t)(t - 1) * nrec;
        }
        a.snap_t = t;
        a.amax_in = amax + t;
        a.grad = grad_c;
        ST_TRY(fused_step(s, a, SNAP_NONE, snap_kind, 2, &msnap));
    }
    return ST_OK;
}

}  // namespace stg

using namespace stg;

namespace {

// Device scratch of one gradient call: seismograms / residuals and grad_c.
struct GradScratch {
    float* seis = nullptr;
    float* res = nullptr;
    float* gc = nullptr;
    unsigned* amax = nullptr;
    double* misfit = nullptr;
};

int gradient_scratch(st_solver* s, const st_shot* shot, int snap_kind, GradScratch* g) {
    const size_t npts = (size_t)(s->L.nx * s->L.ny * s->L.nz);
    const size_t nrec = (size_t)(shot->rec.nx * shot->rec.ny);
    const size_t nt = (size_t)std::max(shot->nt, 1);
    auto al = [](size_t b) { return ((b + 255) / 256) * 256; };
    const size_t b_seis = al(nt * nrec * 4), b_gc = al(npts * 4), b_amax = al((nt + 1) * 4);
    ST_TRY(ensure_buffer(s, &s->aux_buf, &s->aux_cap, 2 * b_seis + b_gc + b_amax + 256));
    char* p = static_cast<char*>(s->aux_buf);
    g->seis = reinterpret_cast<float*>(p);
    g->res = reinterpret_cast<float*>(p + b_seis);
    g->gc = reinterpret_cast<float*>(p + 2 * b_seis);
    g->amax = reinterpret_cast<unsigned*>(p + 2 * b_seis + b_gc);
    g->misfit = reinterpret_cast<double*>(p + 2 * b_seis + b_gc + b_amax);
    const size_t snap_total = npts * (size_t)snap_bytes(snap_kind) * nt;
    if (snap_total > 0) ST_TRY(ensure_buffer(s, &s->snap_buf, &s->snap_cap, snap_total));
    return ST_OK;
}

int check_grad_args(st_solver* s, const st_shot* shot, int snap_kind) {
    ST_CHECK(s && shot, ST_ERR_ARG, "null argument");
    ST_TRY(require_no_terrain(s));
    ST_CHECK(snap_kind >= ST_SNAP_BF16 && snap_kind <= ST_SNAP_FP32, ST_ERR_ARG,
             "gradient snapshot kind must be BF16, FP16 or FP32 (got %d)", snap_kind);
    ST_CHECK((s->L.nz * snap_bytes(snap_kind)) % 16 == 0, ST_ERR_UNSUPPORTED,
             "gradients with this snapshot kind need nz*%d bytes divisible by 16 (nz=%lld)", snap_bytes(snap_kind),
             (long long)s->L.nz);
    return ST_OK;
}

int finish_gradient(st_solver* s, const GradScratch& g, float* grad_v) {
    const Layout& L = s->L;
    grad_v_kernel<<<nblocks(L.nx * L.ny * L.nz), 256, 0, s->stream>>>(g.gc, s->c, L, s->cfg.dt * cfl_damp(s), grad_v);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

}  // namespace

extern "C" {

int st_solver_set_velocity_device(st_solver* s, const float* vel) {
    ST_CHECK(s && vel, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(s->device));
    const Layout& L = s->L;
    const long long n = L.nx * L.ny * L.nz;
    // host copy of the model (reference layout, edge-replicated halo) for field().velocity and the CFL rule
    std::vector<float> h((size_t)n);
    ST_CUDA(cudaMemcpyAsync(h.data(), vel, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    const long long NXh = L.NXh, NYh = L.NYh, NZh = L.nz + 2, nx = L.nx, ny = L.ny, nz = L.nz;
    auto clampi = [](long long v, long long hi) { return v < 0 ? 0 : (v > hi ? hi : v); };
    for (long long xd = 0; xd < NXh; ++xd) {
        const long long ix = clampi(xd - 1, nx - 1);
        for (long long yd = 0; yd < NYh; ++yd) {
            const long long iy = clampi(yd - 1, ny - 1);
            double* row = s->vel_host.data() + (xd * NYh + yd) * NZh;
            const float* src = h.data() + (ix * ny + iy) * nz;
            for (long long zr = 0; zr < NZh; ++zr) row[zr] = src[clampi(zr - 1, nz - 1)];
        }
    }
    s->vel_host_valid = true;
    const double damp = cfl_damp(s);
    vel_interior_to_coeff_kernel<<<nblocks(L.elems), 256, 0, s->stream>>>(vel, s->c, L,
                                                                           s->cfg.dt * s->cfg.dt * damp * damp);
    count_launch();
    ST_CUDA(cudaGetLastError());
    s->coeff_dirty = false;
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_shot_gradient(st_solver* s, const st_shot* shot, const float* adj_src, int snap_kind, float* grad_v) {
    ST_TRY(check_grad_args(s, shot, snap_kind));
    ST_CHECK(grad_v && (shot->rec.nx * shot->rec.ny == 0 || adj_src), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(s->device));
    GradScratch g;
    ST_TRY(gradient_scratch(s, shot, snap_kind, &g));
    ST_TRY(shot_forward_impl(s, shot, nullptr, snap_kind, s->snap_buf, g.amax));
    ST_TRY(gradient_backward_impl(s, shot, adj_src, snap_kind, s->snap_buf, g.amax, g.gc));
    ST_TRY(finish_gradient(s, g, grad_v));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

int st_fwi_gradient(st_solver* s, const st_shot* shot, const float* d_obs, int snap_kind, float* grad_v,
                    double* misfit, float* residual) {
    ST_TRY(check_grad_args(s, shot, snap_kind));
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    ST_CHECK(nrec > 0 && d_obs, ST_ERR_ARG, "FWI needs receivers and observed data");
    ST_CUDA(cudaSetDevice(s->device));
    GradScratch g;
    // misfit only (grad_v == NULL): no snapshot store
    const int fk = grad_v ? snap_kind : ST_SNAP_NONE;
    ST_TRY(gradient_scratch(s, shot, fk, &g));
    const long long nd = (long long)shot->nt * nrec;
    ST_TRY(shot_forward_impl(s, shot, g.seis, fk, s->snap_buf, g.amax));
    ST_CUDA(cudaMemsetAsync(g.misfit, 0, sizeof(double), s->stream));
    residual_kernel<<<nblocks(nd), 256, 0, s->stream>>>(g.seis, d_obs, nd, g.res, g.misfit);
    count_launch();
    ST_CUDA(cudaGetLastError());
    if (residual) ST_CUDA(cudaMemcpyAsync(residual, g.res, (size_t)nd * 4, cudaMemcpyDeviceToDevice, s->stream));
    if (grad_v) {
        ST_TRY(gradient_backward_impl(s, shot, g.res, snap_kind, s->snap_buf, g.amax, g.gc));
        ST_TRY(finish_gradient(s, g, grad_v));
    }
    double h = 0.0;
    ST_CUDA(cudaMemcpyAsync(&h, g.misfit, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    if (misfit) *misfit += h;
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

int st_shot_gradient_checkpointed(st_solver* s, const st_shot* shot, const float* adj_src, int snap_kind,
                                  int segment_steps, int max_slots, float* grad_v, st_checkpoint_stats* stats) {
    ST_TRY(check_grad_args(s, shot, snap_kind));
    ST_CHECK(grad_v && (shot->rec.nx * shot->rec.ny == 0 || adj_src), ST_ERR_ARG, "null argument");
    ST_CHECK(shot->nt >= 0, ST_ERR_ARG, "negative nt");
    ST_CUDA(cudaSetDevice(s->device));
    GradScratch g;
    ST_TRY(gradient_scratch(s, shot, ST_SNAP_NONE, &g));
    ST_TRY(checkpointed_adjoint(s, shot, snap_kind, segment_steps, max_slots, 2, adj_src, nullptr, nullptr, g.gc,
                                nullptr, nullptr, stats));
    ST_TRY(finish_gradient(s, g, grad_v));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

int st_fwi_gradient_checkpointed(st_solver* s, const st_shot* shot, const float* d_obs, int snap_kind,
                                 int segment_steps, int max_slots, float* grad_v, double* misfit, float* residual,
                                 st_checkpoint_stats* stats) {
    if (!grad_v) return st_fwi_gradient(s, shot, d_obs, snap_kind, nullptr, misfit, residual);
    ST_TRY(check_grad_args(s, shot, snap_kind));
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    ST_CHECK(nrec > 0 && d_obs, ST_ERR_ARG, "FWI needs receivers and observed data");
    ST_CHECK(shot->nt >= 0, ST_ERR_ARG, "negative nt");
    ST_CUDA(cudaSetDevice(s->device));
    GradScratch g;
    ST_TRY(gradient_scratch(s, shot, ST_SNAP_NONE, &g));
    const long long nd = (long long)shot->nt * nrec;
    ST_CUDA(cudaMemsetAsync(g.misfit, 0, sizeof(double), s->stream));
    // the residual forces the adjoint: it is formed once every seismogram row
    // has been sampled, just before the first adjoint segment
    auto residual_step = [&]() -> int {
        if (nd > 0) {
            residual_kernel<<<nblocks(nd), 256, 0, s->stream>>>(g.seis, d_obs, nd, g.res, g.misfit);
            count_launch();
            ST_CUDA(cudaGetLastError());
            if (residual)
                ST_CUDA(cudaMemcpyAsync(residual, g.res, (size_t)nd * 4, cudaMemcpyDeviceToDevice, s->stream));
        }
        return ST_OK;
    };
    ST_TRY(checkpointed_adjoint(s, shot, snap_kind, segment_steps, max_slots, 2, g.res, nullptr, nullptr, g.gc, g.seis,
                                residual_step, stats));
    ST_TRY(finish_gradient(s, g, grad_v));
    double h = 0.0;
    ST_CUDA(cudaMemcpyAsync(&h, g.misfit, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    if (misfit) *misfit += h;
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

}  // extern "C"
