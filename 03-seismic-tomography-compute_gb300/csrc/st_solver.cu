// C ABI of the propagator: the seismic::WaveEquationSolver face
// (solver/wave_equation.h:50-144) and the fused shot entry points.
//
// State per handle: three device fields in the device layout with roles
// cur (the reference's `current`), prev (the undamped current of the step
// before; the reference's `previous` is D times it) and third (one step
// older; the reference's `next` scratch is D^2 times it), the update
// coefficient c = v^2 dt^2 (times the reference's CFL damping factor^2), the
// sponge table, and an FP64 host copy of the velocity in the reference layout.
#include "st_solver_impl.cuh"
#include "st_slices.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <memory>
#include <vector>

namespace stg {

namespace {
thread_local char g_err[512] = "";
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
const char* last_error() { return g_err; }

// Sequential-order NaN repair of FaultTolerance::repair_field_nan
// (core/fault_tolerance.cpp:98-157): one CTA scans the field in index order,
// compacts the non-finite interior cells of each chunk in order, and one
// thread repairs them in that order, so a repaired cell feeds later averages
// exactly as in the reference loop. Operates on the damped view D^pow * f
// when pow > 0 and stores back undamped. Rare path (only after a user wrote
// non-finite values into a field).
__global__ void repair_nan_kernel(float* f, Layout L, const float* dtab, int sw, int pow, float repl,
                                  unsigned long long* repaired) {
    __shared__ int list[1024];
    __shared__ int cnt;
    const long long NZh = L.nz + 2, total = L.NXh * L.NYh * NZh;
    auto D = [&](long long xd, long long yd, long long zr) -> float {
        if (pow == 0) return 1.0f;
        const long long ix = xd - 1, iy = yd - 1, iz = zr - 1;
        long long d = sw;
        d = min(d, ix); d = min(d, L.nx - 1 - ix); d = min(d, iy); d = min(d, L.ny - 1 - iy);
        d = min(d, iz); d = min(d, L.nz - 1 - iz);
        float v = (d >= 0 && d < sw) ? dtab[d] : 1.0f;
        return pow == 1 ? v : v * v;
    };
    auto dev = [&](long long xd, long long yd, long long zr) { return xd * L.plane + yd * L.NZP + zr + (Layout::ZOFF - 1); };
    unsigned long long nrep = 0;
    for (long long base = 0; base < total; base += blockDim.x) {
        if (threadIdx.x == 0) cnt = 0;
        __syncthreads();
        const long long e = base + threadIdx.x;
        bool bad = false;
        if (e < total) {
            const long long xd = e / (L.NYh * NZh), r = e % (L.NYh * NZh), yd = r / NZh, zr = r % NZh;
            bad = !isfinite(f[dev(xd, yd, zr)]);
        }
        const unsigned m = __ballot_sync(0xffffffffu, bad);
        __shared__ int wbase[32];
        if ((threadIdx.x & 31) == 0) wbase[threadIdx.x >> 5] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { int c = wbase[w]; wbase[w] = acc; acc += c; }
            cnt = acc;
        }
        __syncthreads();
        if (bad) list[wbase[threadIdx.x >> 5] + __popc(m & ((1u << (threadIdx.x & 31)) - 1))] = (int)(e - base);
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int j = 0; j < cnt; ++j) {
                const long long ee = base + list[j];
                const long long xd = ee / (L.NYh * NZh), r = ee % (L.NYh * NZh), yd = r / NZh, zr = r % NZh;
                const bool interior = xd >= 1 && xd <= L.nx && yd >= 1 && yd <= L.ny && zr >= 1 && zr <= L.nz;
                float* p = f + dev(xd, yd, zr);
                if (!interior) continue;  // the reference's second pass handles halo cells
                double sum = 0.0;
                int nv = 0;
                auto take = [&](long long x, long long y, long long z) {
                    const float v = f[dev(x, y, z)] * D(x, y, z);
                    if (isfinite(v)) { sum += v; ++nv; }
                };
                if (xd > 1) take(xd - 1, yd, zr);
                if (xd < L.nx) take(xd + 1, yd, zr);
                if (yd > 1) take(xd, yd - 1, zr);
                if (yd < L.ny) take(xd, yd + 1, zr);
                if (zr > 1) take(xd, yd, zr - 1);
                if (zr < L.nz) take(xd, yd, zr + 1);
                const float val = nv > 0 ? (float)(sum / nv) : repl;
                *p = val / D(xd, yd, zr);
                ++nrep;
            }
        }
        __syncthreads();
    }
    // second pass: anything still non-finite (halo cells) takes repl
    for (long long e = threadIdx.x; e < total; e += blockDim.x) {
        const long long xd = e / (L.NYh * NZh), r = e % (L.NYh * NZh), yd = r / NZh, zr = r % NZh;
        float* p = f + dev(xd, yd, zr);
        if (!isfinite(*p)) { *p = repl; atomicAdd(repaired, 1ull); }
    }
    if (threadIdx.x == 0) atomicAdd(repaired, nrep);
}

// safe_clamp of the damped view (FaultTolerance::clamp_field, fault_tolerance.cpp:91-96).
__global__ void clamp_view_kernel(float* f, Layout L, const float* dtab, int sw, int pow, float lo, float hi) {
    const long long NZh = L.nz + 2, total = L.NXh * L.NYh * NZh;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long xd = e / (L.NYh * NZh), r = e % (L.NYh * NZh), yd = r / NZh, zr = r % NZh;
        float* p = f + xd * L.plane + yd * L.NZP + zr + (Layout::ZOFF - 1);
        float D = 1.0f;
        if (pow > 0) {
            const long long ix = xd - 1, iy = yd - 1, iz = zr - 1;
            long long d = sw;
            d = min(d, ix); d = min(d, L.nx - 1 - ix); d = min(d, iy); d = min(d, L.ny - 1 - iy);
            d = min(d, iz); d = min(d, L.nz - 1 - iz);
            D = (d >= 0 && d < sw) ? dtab[d] : 1.0f;
        }
        const float v = *p * D;
        const float cl = isfinite(v) ? fminf(fmaxf(v, lo), hi) : 0.0f;
        *p = cl / D;
    }
}

}  // namespace stg

using namespace stg;

namespace stg {

int64_t ref_elems(const st_solver* s) { return s->L.NXh * s->L.NYh * (s->L.nz + 2); }

int ensure_staging(st_solver* s) {
    if (!s->staging) ST_CUDA(cudaMalloc(&s->staging, (size_t)ref_elems(s) * sizeof(double)));
    return ST_OK;
}

// Brings the host copy of the model up to date after a device-side upload.
int ensure_vel_host(st_solver* s) {
    if (s->vel_host_valid) return ST_OK;
    ST_CUDA(cudaSetDevice(s->device));
    ST_CUDA(cudaMemcpyAsync(s->vel_host.data(), s->vel_dev, (size_t)ref_elems(s) * sizeof(double),
                            cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    s->vel_host_valid = true;
    return ST_OK;
}

// Largest finite velocity (compute_local_max_velocity, wave_equation.cpp:435-443).
double host_vmax(const st_solver* s) {
    double vmax = 0.0;
    for (double v : s->vel_host)
        if (std::isfinite(v) && v > vmax) vmax = v;
    return vmax;
}

// Square of the reference's CFL damping factor (wave_equation.cpp:316-387):
// 1 unless max(vmax*dt/d) > 1, then min(1, safety/(vmax*dt/min d))^2.
double cfl_damp2_of(st_solver* s, double vmax) {
    const double dt = s->cfg.dt;
    const double cfl = std::max({vmax * dt / s->grid.dx, vmax * dt / s->grid.dy, vmax * dt / s->grid.dz});
    if (cfl <= 1.0) return 1.0;
    const double ratio = vmax * dt / std::min({s->grid.dx, s->grid.dy, s->grid.dz});
    const double f = std::min(1.0, s->cfl_safety / ratio);
    if (!s->cfl_warned) {
        printf("[WARNING] CFL condition violated (max CFL=%.4f). Applying sub-cycling with reduced effective dt.\n",
               cfl);
        fflush(stdout);
        s->cfl_warned = true;
    }
    return f * f;
}

double cfl_damp2(st_solver* s) { return cfl_damp2_of(s, host_vmax(s)); }

// Largest finite velocity of a device FP64 array, as the bits of a
// non-negative double (monotonic as unsigned integers); 0 when none is
// positive, as host_vmax.
__global__ void vmax_finite_kernel(const double* __restrict__ v, long long n, unsigned long long* out) {
    double m = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = v[i];
        if (isfinite(x) && x > m) m = x;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Uploads a whole reference-layout velocity straight to the device (one
// copy from the caller's buffer, the CFL maximum found on the device) and
// rebuilds the coefficients; the host mirror is refreshed only when read.
int upload_velocity(st_solver* s, const double* vp) {
    const size_t bytes = (size_t)ref_elems(s) * sizeof(double);
    if (!s->vel_dev) ST_CUDA(cudaMalloc(&s->vel_dev, bytes));
    ST_CUDA(cudaMemcpyAsync(s->vel_dev, vp, bytes, cudaMemcpyHostToDevice, s->stream));
    ST_CUDA(cudaMemsetAsync(s->counter, 0, sizeof(unsigned long long), s->stream));
    vmax_finite_kernel<<<152 * 8, 256, 0, s->stream>>>(s->vel_dev, ref_elems(s), s->counter);
    count_launch();
    ST_CUDA(cudaGetLastError());
    unsigned long long bits = 0;
    ST_CUDA(cudaMemcpyAsync(&bits, s->counter, sizeof(bits), cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    double vmax;
    std::memcpy(&vmax, &bits, sizeof(vmax));
    ST_TRY(launch_vel_to_coeff(s->vel_dev, s->c, s->L, s->cfg.dt * s->cfg.dt * cfl_damp2_of(s, vmax), s->stream));
    s->vel_host_valid = false;
    s->coeff_dirty = false;
    return ST_OK;
}

int refresh_coeff(st_solver* s) {
    if (!s->coeff_dirty) return ST_OK;
    ST_TRY(ensure_staging(s));
    ST_CUDA(cudaMemcpyAsync(s->staging, s->vel_host.data(), (size_t)ref_elems(s) * sizeof(double),
                            cudaMemcpyHostToDevice, s->stream));
    ST_TRY(launch_vel_to_coeff(s->staging, s->c, s->L, s->cfg.dt * s->cfg.dt * cfl_damp2(s), s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    s->coeff_dirty = false;
    return ST_OK;
}

int read_flags(st_solver* s, unsigned* out) {
    unsigned h = 0;
    ST_CUDA(cudaMemcpyAsync(&h, s->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    ST_CUDA(cudaMemsetAsync(s->flags, 0, sizeof(unsigned), s->stream));
    *out = h;
    if (h & FLAG_TIMEOUT) {
        set_error("propagator pipeline wait timed out (TMA copy did not complete)");
        return ST_ERR_TIMEOUT;
    }
    return ST_OK;
}

StepArgs base_args(st_solver* s, float* out) {
    StepArgs a{};
    a.out = out;
    a.ax = (float)(1.0 / (s->grid.dx * s->grid.dx));
    a.ay = (float)(1.0 / (s->grid.dy * s->grid.dy));
    a.az = (float)(1.0 / (s->grid.dz * s->grid.dz));
    a.amp = (float)s->amp_limit;
    a.sw = s->sw;
    a.dtab = s->dtab;
    a.inj_x = -1;
    a.flags = s->flags;
    a.rsx = a.rsy = 1;
    a.stable_sponge = s->sponge_mode == ST_SPONGE_STABLE;
    a.zlim = s->zlim;
    a.timeout_ns = s->wait_limit_ns;
    a.withhold = s->withhold;  // the test hook applies to one launch
    s->withhold = 0;
    return a;
}

// One fused step out = f[in] from cur = f[ic], prev = f[ip]; then rotates the
// roles so cur = out, prev = old cur, third = old prev.
int fused_step(st_solver* s, StepArgs a, int snap_out, int snap_in, int epi, const CUtensorMap* msnap,
               const ImageMaps* imaps) {
    a.out = s->f[s->in];
    ST_TRY(launch_fd_step(s->L, s->maps[s->ic], s->maps[s->ip], s->map_c, a, snap_out, snap_in, epi, msnap,
                          s->stream, imaps));
    const int old_c = s->ic, old_p = s->ip, old_n = s->in;
    s->ic = old_n;
    s->ip = old_c;
    s->in = old_p;
    return ST_OK;
}

namespace {
int ensure_spare(st_solver* s) {
    if (s->f4) return ST_OK;
    const size_t fb = (size_t)s->L.elems * sizeof(float);
    ST_CUDA(cudaMalloc(&s->f4, fb));
    ST_CUDA(cudaMemsetAsync(s->f4, 0, fb, s->stream));  // its halo stays zero: only interiors are written
    return build_field_maps(&s->map4, s->f4, s->L);
}

// After a two-step launch (first output in f[in], second in the spare): cur
// takes the spare, whose old buffer (the old cur) becomes the spare; prev =
// the first output, and the old prev is free.
void rotate_after_pair(st_solver* s) {
    std::swap(s->f[s->ic], s->f4);
    std::swap(s->maps[s->ic], s->map4);
    std::swap(s->ip, s->in);
}
}  // namespace

int fused_step2(st_solver* s, StepArgs a, int snap_in, const ImageMaps& imaps) {
    ST_TRY(ensure_spare(s));
    a.out = s->f[s->in];
    a.out2 = s->f4;
    ST_TRY(launch_fd_step2_image(s->L, s->maps[s->ic], s->maps[s->ip], s->map_c, a, snap_in, imaps, s->stream));
    rotate_after_pair(s);
    return ST_OK;
}

int fused_step2_grad(st_solver* s, StepArgs a, int snap_in, const CUtensorMap& msnap, const CUtensorMap& mgrad) {
    ST_TRY(ensure_spare(s));
    a.out = s->f[s->in];
    a.out2 = s->f4;
    ST_TRY(launch_fd_step2_grad(s->L, s->maps[s->ic], s->maps[s->ip], s->map_c, a, snap_in, msnap, mgrad,
                                s->stream));
    rotate_after_pair(s);
    return ST_OK;
}

int fused_step2_forward(st_solver* s, StepArgs a, int snap_out) {
    ST_TRY(ensure_spare(s));
    a.out = s->f[s->in];
    a.out2 = s->f4;
    ST_TRY(launch_fd_step2_forward(s->L, s->maps[s->ic], s->maps[s->ip], s->map_c, a, snap_out, s->stream));
    rotate_after_pair(s);
    return ST_OK;
}

long long dev_index(const st_solver* s, int64_t ix, int64_t iy, int64_t iz) { return s->L.at(ix, iy, iz); }

// Reference padded index -> device index, -1 when outside the padded array.
long long ref_to_dev_index(const st_solver* s, int64_t ix, int64_t iy, int64_t iz) {
    const int64_t xd = ix + 1, yd = iy + 1, zr = iz + 1;
    const int64_t NZh = s->L.nz + 2;
    const int64_t r = (xd * s->L.NYh + yd) * NZh + zr;
    if (r < 0 || r >= ref_elems(s)) return -1;
    // the reference adds at a linear index; recover its padded coordinates
    const int64_t X = r / (s->L.NYh * NZh), rem = r % (s->L.NYh * NZh), Y = rem / NZh, Z = rem % NZh;
    return X * s->L.plane + Y * s->L.NZP + Z + (Layout::ZOFF - 1);
}

int health_check(st_solver* s, int timestep, int* result) {
    // perform_health_check (wave_equation.cpp:407-424) -> attempt_recovery
    // (fault_tolerance.cpp:198-257)
    unsigned long long nan = 0;
    ST_TRY(launch_count_nonfinite(s->f[s->ic], s->L.elems, s->counter, s->stream));
    ST_CUDA(cudaMemcpyAsync(&nan, s->counter, sizeof(nan), cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    *result = ST_OK;
    if (nan == 0) return ST_OK;
    (void)timestep;
    s->stats.total_nan_count += (int64_t)nan;
    int64_t global = (int64_t)nan;
    for (int attempt = 0; attempt < s->max_repair_attempts; ++attempt) {
        ST_CUDA(cudaMemsetAsync(s->counter, 0, sizeof(unsigned long long), s->stream));
        repair_nan_kernel<<<1, 1024, 0, s->stream>>>(s->f[s->ic], s->L, s->dtab, s->sw, 0, 0.0f, s->counter);
    ::stg::count_launch();
        repair_nan_kernel<<<1, 1024, 0, s->stream>>>(s->f[s->ip], s->L, s->dtab, s->sw, 1, 0.0f, s->counter);
    ::stg::count_launch();
        clamp_view_kernel<<<256, 256, 0, s->stream>>>(s->f[s->ic], s->L, s->dtab, s->sw, 0,
                                                      (float)-s->ft_amp_limit, (float)s->ft_amp_limit);
    ::stg::count_launch();
        clamp_view_kernel<<<256, 256, 0, s->stream>>>(s->f[s->ip], s->L, s->dtab, s->sw, 1,
                                                      (float)-s->ft_amp_limit, (float)s->ft_amp_limit);
    ::stg::count_launch();
        ST_CUDA(cudaGetLastError());
        unsigned long long post = 0;
        ST_TRY(launch_count_nonfinite(s->f[s->ic], s->L.elems, s->counter, s->stream));
        ST_CUDA(cudaMemcpyAsync(&post, s->counter, sizeof(post), cudaMemcpyDeviceToHost, s->stream));
        ST_CUDA(cudaStreamSynchronize(s->stream));
        s->stats.cells_repaired += global - (int64_t)post;
        if (post == 0) {
            s->stats.timesteps_recovered++;
            *result = ST_NAN_DETECTED_AND_REPAIRED;
            return ST_OK;
        }
        global = (int64_t)post;
    }
    *result = ST_FATAL_DIVERGENCE;
    return ST_OK;
}

int one_reference_step(st_solver* s, int timestep) {
    ST_TRY(refresh_coeff(s));
    StepArgs a = base_args(s, nullptr);
    ST_TRY(fused_step(s, a, SNAP_NONE, SNAP_NONE, 0, nullptr));
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    int health = ST_OK;
    ST_TRY(health_check(s, timestep, &health));
    if (health != ST_OK) return health;
    return (fl & FLAG_GUARD) ? ST_NAN_DETECTED_AND_REPAIRED : ST_OK;
}

int zero_fields(st_solver* s) {
    for (int k = 0; k < 3; ++k) ST_CUDA(cudaMemsetAsync(s->f[k], 0, (size_t)s->L.elems * 4, s->stream));
    s->ic = 0;
    s->ip = 1;
    s->in = 2;
    return ST_OK;
}

int save_snapshot_dev(st_solver* s) {
    const size_t n = (size_t)(s->L.nx * s->L.ny * s->L.nz);
    float* buf = nullptr;
    ST_CUDA(cudaMalloc(&buf, n * sizeof(float)));
    s->snapshots.push_back(buf);
    return launch_interior_copy(s->f[s->ic], s->L, buf, s->stream);
}

void clear_snaps(st_solver* s) {
    for (float* p : s->snapshots) cudaFree(p);
    s->snapshots.clear();
}

bool finite_sample(const double* w, int64_t len, int64_t t, float* out) {
    if (t < 0 || t >= len || !w) return false;
    if (!std::isfinite(w[t])) return false;
    *out = (float)w[t];
    return true;
}

int ensure_buffer(st_solver* s, void** buf, size_t* cap, size_t bytes) {
    if (*cap >= bytes && *buf) return ST_OK;
    if (*buf) {
        ST_CUDA(cudaStreamSynchronize(s->stream));
        cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
    }
    cudaError_t e = cudaMalloc(buf, bytes);
    if (e != cudaSuccess) {
        *buf = nullptr;
        set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return ST_ERR_ALLOC;
    }
    *cap = bytes;
    return ST_OK;
}

}  // namespace stg

extern "C" {

const char* st_last_error(void) { return last_error(); }
int st_version(void) { return 10000; }

int st_device_count(int* count) {
    ST_CHECK(count, ST_ERR_ARG, "null count");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) n = 0;
    *count = n;
    return ST_OK;
}

int st_field_layout(int64_t nx, int64_t ny, int64_t nz, int64_t out[6]) {
    ST_CHECK(nx > 0 && ny > 0 && nz > 0 && out, ST_ERR_ARG, "bad extents");
    Layout L = make_layout(nx, ny, nz);
    out[0] = L.NXh;
    out[1] = L.NYh;
    out[2] = L.NZP;
    out[3] = Layout::ZOFF;
    out[4] = L.plane;
    out[5] = L.elems;
    return ST_OK;
}

int st_solver_create(const st_grid_params* grid, const st_solver_config* cfg, int device, st_solver** out) {
    ST_CHECK(grid && cfg && out, ST_ERR_ARG, "null argument");
    ST_CHECK(grid->halo_width == 1, ST_ERR_UNSUPPORTED, "halo_width must be 1 (7-point stencil), got %d",
             grid->halo_width);
    ST_CHECK(grid->nx_global > 0 && grid->ny_global > 0 && grid->nz_global > 0, ST_ERR_ARG, "bad grid extents");
    ST_CHECK(grid->nx_global < (1 << 30) && grid->ny_global < (1 << 30) && grid->nz_global < (1 << 30), ST_ERR_ARG,
             "grid extents too large");
    ST_CHECK(grid->dx > 0 && grid->dy > 0 && grid->dz > 0, ST_ERR_ARG, "grid spacing must be positive");
    ST_CHECK(cfg->sponge_width >= 0 && cfg->sponge_width <= 4096, ST_ERR_ARG, "bad sponge width");
    int ndev = 0;
    ST_CUDA(cudaGetDeviceCount(&ndev));
    ST_CHECK(device >= 0 && device < ndev, ST_ERR_ARG, "device %d out of range (%d devices)", device, ndev);
    ST_CUDA(cudaSetDevice(device));
    std::unique_ptr<st_solver> s(new st_solver());
    s->device = device;
    s->grid = *grid;
    s->cfg = *cfg;
    s->L = make_layout(grid->nx_global, grid->ny_global, grid->nz_global);
    s->vel_host.assign((size_t)ref_elems(s.get()), 0.0);
    ST_CUDA(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
    s->stream = s->own_stream;
    for (int k = 0; k < 3; ++k) ST_CUDA(cudaEventCreate(&s->ev[k]));
    const size_t fb = (size_t)s->L.elems * sizeof(float);
    for (int k = 0; k < 3; ++k) ST_CUDA(cudaMalloc(&s->f[k], fb));
    ST_CUDA(cudaMalloc(&s->c, fb));
    ST_CUDA(cudaMemsetAsync(s->c, 0, fb, s->stream));
    ST_CUDA(cudaMalloc(&s->flags, sizeof(unsigned)));
    ST_CUDA(cudaMalloc(&s->counter, sizeof(unsigned long long)));
    ST_CUDA(cudaMalloc(&s->dsum, sizeof(double)));
    ST_CUDA(cudaMemsetAsync(s->flags, 0, sizeof(unsigned), s->stream));
    // sponge factors exactly as apply_sponge_layer evaluates them (wave_equation.cpp:288-290)
    s->sw = cfg->sponge_width;
    if (s->sw > 0) {
        std::vector<float> tab((size_t)s->sw);
        for (int d = 0; d < s->sw; ++d) {
            double damp = 1.0 - cfg->sponge_damping * (s->sw - d) * (s->sw - d) / (s->sw * s->sw);
            tab[d] = (float)damp;
        }
        ST_CUDA(cudaMalloc(&s->dtab, tab.size() * sizeof(float)));
        ST_CUDA(cudaMemcpy(s->dtab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    ST_TRY(zero_fields(s.get()));
    for (int k = 0; k < 3; ++k) ST_TRY(build_field_maps(&s->maps[k], s->f[k], s->L));
    ST_TRY(build_field_maps(&s->map_c, s->c, s->L));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    *out = s.release();
    return ST_OK;
}

int st_solver_destroy(st_solver* s) {
    if (!s) return ST_OK;
    cudaSetDevice(s->device);
    rtm_release(s);
    cudaFree(s->rtm_fwd);
    clear_snaps(s);
    for (int k = 0; k < 3; ++k) cudaFree(s->f[k]);
    cudaFree(s->f4);
    cudaFree(s->c);
    cudaFree(s->dtab);
    cudaFree(s->staging);
    cudaFree(s->flags);
    cudaFree(s->counter);
    cudaFree(s->dsum);
    cudaFree(s->snap_buf);
    cudaFree(s->aux_buf);
    cudaFree(s->data_buf);
    cudaFree(s->ckpt_buf);
    cudaFree(s->zlim);
    cudaFree(s->vel_dev);
    for (int k = 0; k < 3; ++k)
        if (s->ev[k]) cudaEventDestroy(s->ev[k]);
    if (s->ev_copy) cudaEventDestroy(s->ev_copy);
    if (s->copy_stream) {
        cudaStreamSynchronize(s->copy_stream);
        cudaStreamDestroy(s->copy_stream);
    }
    if (s->stream != s->own_stream) cudaStreamSynchronize(s->stream);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
    return ST_OK;
}

int st_solver_initialize_velocity(st_solver* s, double vp0) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    std::fill(s->vel_host.begin(), s->vel_host.end(), vp0);
    s->vel_host_valid = true;
    s->coeff_dirty = true;
    return ST_OK;
}

int st_solver_set_velocity_field(st_solver* s, const double* vp, int64_t count) {
    ST_CHECK(s && (vp || count <= 0), ST_ERR_ARG, "null argument");
    const int64_t n = std::min<int64_t>(count, (int64_t)s->vel_host.size());
    ST_TRY(ensure_vel_host(s));
    if (n > 0) std::memcpy(s->vel_host.data(), vp, (size_t)n * sizeof(double));
    s->coeff_dirty = true;
    return ST_OK;
}

int st_solver_inject_source(st_solver* s, int64_t ix, int64_t iy, int64_t iz, const double* wavelet, int64_t len) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    if (!wavelet || len <= 0) return ST_OK;
    const double val = wavelet[0];
    if (!std::isfinite(val)) return ST_OK;
    const long long d = ref_to_dev_index(s, ix, iy, iz);
    if (d < 0) return ST_OK;
    ST_CUDA(cudaSetDevice(s->device));
    return launch_add_point(s->f[s->ic], d, (float)val, nullptr, s->stream);
}

int st_solver_step_forward(st_solver* s, int timestep) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CUDA(cudaSetDevice(s->device));
    return one_reference_step(s, timestep);
}

int st_solver_step_adjoint(st_solver* s, int timestep) {
    // the reference's step_adjoint is the same operator (wave_equation.cpp:78-98)
    return st_solver_step_forward(s, timestep);
}

int st_solver_reset_field(st_solver* s) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(zero_fields(s));
    clear_snaps(s);
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_solver_forward_propagate(st_solver* s, const double* wavelet, int64_t len, st_propagation_result* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(s->device));
    std::memset(out, 0, sizeof(*out));
    ST_TRY(st_solver_reset_field(s));
    s->stats = st_fault_stats{};
    int ok = 0;
    ST_TRY(st_solver_verify_cfl(s, &ok));
    if (!ok) {
        out->status = ST_CFL_VIOLATION;
        return ST_OK;
    }
    ST_TRY(refresh_coeff(s));
    const int nt = s->cfg.nt;
    const int si = s->cfg.snapshot_interval;
    ST_CHECK(si > 0, ST_ERR_ARG, "snapshot_interval must be positive");
    const long long src = dev_index(s, s->L.nx / 2, s->L.ny / 2, s->L.nz / 2);
    float w = 0.0f;
    if (nt > 0 && finite_sample(wavelet, len, 0, &w)) ST_TRY(launch_add_point(s->f[s->ic], src, w, nullptr, s->stream));
    for (int t = 0; t < nt; ++t) {
        StepArgs a = base_args(s, nullptr);
        const bool snap = (t % si == 0);
        float wn = 0.0f;
        const bool inj = t + 1 < nt && finite_sample(wavelet, len, t + 1, &wn);
        if (inj && !snap) set_injection(a, s->L.nx / 2, s->L.ny / 2, s->L.nz / 2, wn);
        ST_TRY(fused_step(s, a, SNAP_NONE, SNAP_NONE, 0, nullptr));
        if (snap) {
            ST_TRY(save_snapshot_dev(s));
            if (inj) ST_TRY(launch_add_point(s->f[s->ic], src, wn, nullptr, s->stream));
        }
    }
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    if (fl & FLAG_GUARD) out->status = ST_NAN_DETECTED_AND_REPAIRED;
    out->timesteps_completed = nt;
    out->total_cells_repaired = s->stats.cells_repaired;
    out->completed_successfully = 1;
    return ST_OK;
}

int st_solver_adjoint_propagate(st_solver* s, const double* residual, int64_t len, st_propagation_result* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(s->device));
    std::memset(out, 0, sizeof(*out));
    ST_TRY(refresh_coeff(s));
    const int nt = s->cfg.nt;
    const long long src = dev_index(s, s->L.nx / 2, s->L.ny / 2, s->L.nz / 2);
    float w = 0.0f;
    if (nt > 0 && finite_sample(residual, len, nt - 1, &w))
        ST_TRY(launch_add_point(s->f[s->ic], src, w, nullptr, s->stream));
    for (int t = nt - 1; t >= 0; --t) {
        StepArgs a = base_args(s, nullptr);
        float wn = 0.0f;
        if (t - 1 >= 0 && finite_sample(residual, len, t - 1, &wn))
            set_injection(a, s->L.nx / 2, s->L.ny / 2, s->L.nz / 2, wn);
        ST_TRY(fused_step(s, a, SNAP_NONE, SNAP_NONE, 0, nullptr));
    }
    unsigned fl = 0;
    ST_TRY(read_flags(s, &fl));
    if (fl & FLAG_GUARD) out->status = ST_NAN_DETECTED_AND_REPAIRED;
    out->timesteps_completed = nt;
    out->total_cells_repaired = s->stats.cells_repaired;
    out->completed_successfully = 1;
    return ST_OK;
}

int st_solver_get_field(st_solver* s, int which, double* out, int64_t count) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    const int64_t n = ref_elems(s);
    ST_CHECK(count >= n, ST_ERR_ARG, "output holds %lld values, field has %lld", (long long)count, (long long)n);
    if (which == ST_FIELD_VELOCITY) {
        ST_TRY(ensure_vel_host(s));
        std::memcpy(out, s->vel_host.data(), (size_t)n * sizeof(double));
        return ST_OK;
    }
    ST_CHECK(which >= 0 && which <= 2, ST_ERR_ARG, "bad field id %d", which);
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(ensure_staging(s));
    const float* src = which == ST_FIELD_CURRENT ? s->f[s->ic] : (which == ST_FIELD_PREVIOUS ? s->f[s->ip] : s->f[s->in]);
    // stored damping of the reference layout: previous D, next D^2 (D with the stable sponge)
    const int pw = (which == ST_FIELD_NEXT && s->sponge_mode == ST_SPONGE_STABLE) ? 1 : which;
    ST_TRY(launch_dev_to_ref(src, s->staging, s->L, s->dtab, s->sw, pw, s->stream));
    ST_CUDA(cudaMemcpyAsync(out, s->staging, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_solver_set_field(st_solver* s, int which, const double* in, int64_t count) {
    ST_CHECK(s && in, ST_ERR_ARG, "null argument");
    const int64_t n = ref_elems(s);
    if (which == ST_FIELD_VELOCITY) return st_solver_set_velocity_field(s, in, count);
    ST_CHECK(which >= 0 && which <= 2, ST_ERR_ARG, "bad field id %d", which);
    ST_CHECK(count >= n, ST_ERR_ARG, "input holds %lld values, field has %lld", (long long)count, (long long)n);
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(ensure_staging(s));
    float* dst = which == ST_FIELD_CURRENT ? s->f[s->ic] : (which == ST_FIELD_PREVIOUS ? s->f[s->ip] : s->f[s->in]);
    ST_CUDA(cudaMemcpyAsync(s->staging, in, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    const int pw = (which == ST_FIELD_NEXT && s->sponge_mode == ST_SPONGE_STABLE) ? 1 : which;
    ST_TRY(launch_ref_to_dev_undamp(s->staging, dst, s->L, s->dtab, s->sw, pw, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_solver_set_sponge_mode(st_solver* s, int mode) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CHECK(mode == ST_SPONGE_REFERENCE || mode == ST_SPONGE_STABLE, ST_ERR_ARG, "bad sponge mode %d", mode);
    s->sponge_mode = mode;
    return ST_OK;
}

int st_solver_set_slice_stream(st_solver* s, st_slice_stream* ss, int interval) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    if (ss && interval > 0) {
        int64_t nx, ny, nz;
        slice_stream_extents(ss, &nx, &ny, &nz);
        ST_CHECK(nx == s->L.nx && ny == s->L.ny && nz == s->L.nz, ST_ERR_ARG,
                 "slice stream grid %lldx%lldx%lld does not match the solver's", (long long)nx, (long long)ny,
                 (long long)nz);
        s->slices = ss;
        s->slice_interval = interval;
    } else {
        s->slices = nullptr;
        s->slice_interval = 0;
    }
    return ST_OK;
}

int st_solver_sponge_mode(st_solver* s, int* mode) {
    ST_CHECK(s && mode, ST_ERR_ARG, "null argument");
    *mode = s->sponge_mode;
    return ST_OK;
}

int st_solver_compute_energy(st_solver* s, double* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(launch_sumsq_finite(s->f[s->ic], s->L.elems, s->dsum, s->stream));
    ST_CUDA(cudaMemcpyAsync(out, s->dsum, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_solver_verify_cfl(st_solver* s, int* ok) {
    // FaultTolerance::verify_cfl_condition (core/fault_tolerance.cpp:49-70)
    ST_CHECK(s && ok, ST_ERR_ARG, "null argument");
    const double vmax = host_vmax(s), dt = s->cfg.dt;
    const double cfl = std::max({vmax * dt / s->grid.dx, vmax * dt / s->grid.dy, vmax * dt / s->grid.dz});
    *ok = cfl <= s->cfl_safety ? 1 : 0;
    return ST_OK;
}

int st_solver_set_amplitude_limit(st_solver* s, double limit) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    s->amp_limit = std::max(1.0, limit);
    s->ft_amp_limit = s->amp_limit;
    return ST_OK;
}

int st_solver_amplitude_limit(st_solver* s, double* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    *out = s->amp_limit;
    return ST_OK;
}

int st_solver_nan_count_current(st_solver* s, int64_t* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(s->device));
    unsigned long long n = 0;
    ST_TRY(launch_count_nonfinite(s->f[s->ic], s->L.elems, s->counter, s->stream));
    ST_CUDA(cudaMemcpyAsync(&n, s->counter, sizeof(n), cudaMemcpyDeviceToHost, s->stream));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    *out = (int64_t)n;
    return ST_OK;
}

int st_solver_save_snapshot(st_solver* s, int timestep) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    (void)timestep;
    ST_CUDA(cudaSetDevice(s->device));
    ST_TRY(save_snapshot_dev(s));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    return ST_OK;
}

int st_solver_clear_snapshots(st_solver* s) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CUDA(cudaSetDevice(s->device));
    ST_CUDA(cudaStreamSynchronize(s->stream));
    clear_snaps(s);
    return ST_OK;
}

int st_solver_snapshot_values(st_solver* s, int64_t* count) {
    ST_CHECK(s && count, ST_ERR_ARG, "null argument");
    *count = (int64_t)s->snapshots.size() * s->L.nx * s->L.ny * s->L.nz;
    return ST_OK;
}

int st_solver_get_snapshots(st_solver* s, double* out, int64_t count) {
    ST_CHECK(s && (out || count == 0), ST_ERR_ARG, "null argument");
    const int64_t per = s->L.nx * s->L.ny * s->L.nz;
    const int64_t total = (int64_t)s->snapshots.size() * per;
    ST_CHECK(count >= total, ST_ERR_ARG, "output holds %lld values, snapshots have %lld", (long long)count,
             (long long)total);
    ST_CUDA(cudaSetDevice(s->device));
    std::vector<float> tmp((size_t)per);
    for (size_t k = 0; k < s->snapshots.size(); ++k) {
        ST_CUDA(cudaMemcpyAsync(tmp.data(), s->snapshots[k], (size_t)per * sizeof(float), cudaMemcpyDeviceToHost,
                                s->stream));
        ST_CUDA(cudaStreamSynchronize(s->stream));
        for (int64_t i = 0; i < per; ++i) out[(int64_t)k * per + i] = tmp[(size_t)i];
    }
    return ST_OK;
}

int st_solver_fault_stats(st_solver* s, st_fault_stats* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    *out = s->stats;
    return ST_OK;
}

int st_solver_set_stream(st_solver* s, void* stream) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CUDA(cudaSetDevice(s->device));
    cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
    if (next == s->stream) return ST_OK;
    // work queued so far stays ordered before everything issued on the new stream
    cudaEvent_t ev = nullptr;
    ST_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    const cudaError_t e1 = cudaEventRecord(ev, s->stream);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(next, ev, 0) : e1;
    cudaEventDestroy(ev);
    ST_CUDA(e2);
    s->stream = next;
    if (s->rtm_engine) rtm_engine_set_stream(s->rtm_engine, next);
    return ST_OK;
}

int st_solver_set_wait_test(st_solver* s, unsigned long long limit_ns, int withhold_plane) {
    ST_CHECK(s && withhold_plane >= -1, ST_ERR_ARG, "bad argument");
    s->wait_limit_ns = limit_ns;
    s->withhold = withhold_plane + 1;
    return ST_OK;
}

int st_solver_reset_fault_stats(st_solver* s) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    s->stats = st_fault_stats{};
    return ST_OK;
}

int st_solver_set_fault_param(st_solver* s, int which, double value) {
    ST_CHECK(s && std::isfinite(value), ST_ERR_ARG, "bad argument");
    switch (which) {
        case ST_FT_MAX_REPAIR_ATTEMPTS: s->max_repair_attempts = (int)std::max(1.0, std::min(value, 1e9)); break;
        case ST_FT_AMPLITUDE_LIMIT: s->ft_amp_limit = std::max(1.0, value); break;
        case ST_FT_CFL_SAFETY_FACTOR: s->cfl_safety = std::max(0.01, std::min(value, 0.99)); break;
        default: ST_CHECK(false, ST_ERR_ARG, "unknown fault-tolerance parameter %d", which);
    }
    return ST_OK;
}

int st_solver_fault_param(st_solver* s, int which, double* out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    switch (which) {
        case ST_FT_MAX_REPAIR_ATTEMPTS: *out = s->max_repair_attempts; break;
        case ST_FT_AMPLITUDE_LIMIT: *out = s->ft_amp_limit; break;
        case ST_FT_CFL_SAFETY_FACTOR: *out = s->cfl_safety; break;
        default: ST_CHECK(false, ST_ERR_ARG, "unknown fault-tolerance parameter %d", which);
    }
    return ST_OK;
}

int st_solver_set_step_fusion(st_solver* s, int steps) {
    ST_CHECK(s, ST_ERR_ARG, "null argument");
    ST_CHECK(steps == 1 || steps == 2, ST_ERR_ARG, "time steps per launch must be 1 or 2 (got %d)", steps);
    s->fused_steps = steps;
    return ST_OK;
}

int st_solver_device_field(st_solver* s, int which, float** out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    switch (which) {
        case ST_FIELD_CURRENT: *out = s->f[s->ic]; break;
        case ST_FIELD_PREVIOUS: *out = s->f[s->ip]; break;
        case ST_FIELD_NEXT: *out = s->f[s->in]; break;
        case ST_FIELD_VELOCITY: {
            int rc = refresh_coeff(s);
            if (rc < 0) return rc;
            *out = s->c;
            break;
        }
        default: ST_CHECK(false, ST_ERR_ARG, "bad field id %d", which);
    }
    return ST_OK;
}

int st_launch_count(long long* out) {
    ST_CHECK(out, ST_ERR_ARG, "null argument");
    *out = launch_count();
    return ST_OK;
}

int st_solver_last_phase_ms(st_solver* s, float out[2]) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    ST_CHECK(s->phases_recorded, ST_ERR_STATE, "no RTM call has recorded its phases yet");
    ST_CUDA(cudaSetDevice(s->device));
    ST_CUDA(cudaEventSynchronize(s->ev[2]));
    ST_CUDA(cudaEventElapsedTime(&out[0], s->ev[0], s->ev[1]));
    ST_CUDA(cudaEventElapsedTime(&out[1], s->ev[1], s->ev[2]));
    return ST_OK;
}

int st_solver_stream(st_solver* s, void** out) {
    ST_CHECK(s && out, ST_ERR_ARG, "null argument");
    *out = (void*)s->stream;
    return ST_OK;
}

int st_shot_forward_host(st_solver* s, const double* vp, int64_t vp_count, const st_shot* shot, double* seis_host) {
    ST_CHECK(s && shot, ST_ERR_ARG, "null argument");
    if (vp) ST_TRY(vp_count >= ref_elems(s) ? upload_velocity(s, vp) : st_solver_set_velocity_field(s, vp, vp_count));
    const int64_t nrec = shot->rec.nx * shot->rec.ny;
    const size_t ns = (size_t)nrec * (size_t)shot->nt;
    ST_CUDA(cudaSetDevice(s->device));
    float* seis = nullptr;
    if (ns > 0) ST_CUDA(cudaMalloc(&seis, ns * sizeof(float)));
    int rc = st_shot_forward(s, shot, seis, ST_SNAP_NONE, nullptr, nullptr);
    if (rc >= 0 && ns > 0 && seis_host) {
        std::vector<float> tmp(ns);
        cudaError_t e = cudaMemcpyAsync(tmp.data(), seis, ns * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            set_error("seismogram download: %s", cudaGetErrorString(e));
            rc = ST_ERR_CUDA;
        } else {
            for (size_t i = 0; i < ns; ++i) seis_host[i] = tmp[i];
        }
    }
    cudaFree(seis);
    return rc;
}

}  // extern "C"
