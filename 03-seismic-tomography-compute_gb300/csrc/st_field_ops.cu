// Field utilities on the GPU: the FaultTolerance helpers exposed by the
// reference binding (check_field_health / clamp_field_safe /
// repair_field_nan, pybind/bindings.cpp:275-301 ->
// core/fault_tolerance.cpp:72-157) and SparseOps::smooth_gradient
// (sparse/sparse_ops.cpp:115-158), all in FP64 like the reference.
//
// smooth_gradient: the reference's weight exp(-(dx^2+dy^2+dz^2)/(2 s^2))
// factors into per-axis weights and its support (the radius-floor(3s) box
// cut to the grid) is a product of per-axis intervals, so the per-point
// normalised 3-D sum equals three 1-D passes, each normalised by its own
// in-bounds weight sum. O(n * 3 * (2r+1)) instead of O(n * (2r+1)^3).
#include "st_common.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace stg {
namespace {

unsigned blocks(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, 152 * 16));
}

__global__ void count_kernel(const double* __restrict__ d, long long n, unsigned long long* out) {
    unsigned long long c = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c += !isfinite(d[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void clamp_kernel(double* __restrict__ d, long long n, double lo, double hi) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = d[i];
        d[i] = isfinite(v) ? fmax(lo, fmin(v, hi)) : 0.0;
    }
}

// In reference loop order: one CTA scans chunks of the array in index order;
// the non-finite interior cells of a chunk are listed in order and repaired
// one after another by one thread, so cells repaired earlier feed later
// averages exactly as in the sequential loop.
__global__ void repair_kernel(double* d, long long count, long long nx, long long ny, long long nz, int hw,
                              double repl) {
    __shared__ int list[1024];
    __shared__ int wsum[32];
    __shared__ int cnt;
    const long long nynz = ny * nz;
    const long long total = nx * ny * nz;
    for (long long base = 0; base < total; base += blockDim.x) {
        const long long e = base + threadIdx.x;
        bool bad = false;
        if (e < total) {
            const long long ix = e / nynz, r = e % nynz, iy = r / nz, iz = r % nz;
            const bool interior = ix >= hw && ix < nx - hw && iy >= hw && iy < ny - hw && iz >= hw && iz < nz - hw;
            bad = interior && !isfinite(d[e]);
        }
        const unsigned m = __ballot_sync(0xffffffffu, bad);
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const int c = wsum[w];
                wsum[w] = acc;
                acc += c;
            }
            cnt = acc;
        }
        __syncthreads();
        if (bad) list[wsum[threadIdx.x >> 5] + __popc(m & ((1u << (threadIdx.x & 31)) - 1))] = threadIdx.x;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int j = 0; j < cnt; ++j) {
                const long long i = base + list[j];
                const long long ix = i / nynz, r = i % nynz, iy = r / nz, iz = r % nz;
                double sum = 0.0;
                int nv = 0;
                if (ix > hw && isfinite(d[i - nynz])) { sum += d[i - nynz]; ++nv; }
                if (ix < nx - hw - 1 && isfinite(d[i + nynz])) { sum += d[i + nynz]; ++nv; }
                if (iy > hw && isfinite(d[i - nz])) { sum += d[i - nz]; ++nv; }
                if (iy < ny - hw - 1 && isfinite(d[i + nz])) { sum += d[i + nz]; ++nv; }
                if (iz > hw && isfinite(d[i - 1])) { sum += d[i - 1]; ++nv; }
                if (iz < nz - hw - 1 && isfinite(d[i + 1])) { sum += d[i + 1]; ++nv; }
                d[i] = nv > 0 ? sum / nv : repl;
            }
        }
        __syncthreads();
    }
    for (long long i = threadIdx.x; i < count; i += blockDim.x)
        if (!isfinite(d[i])) d[i] = repl;
}

// One normalised 1-D pass of the separable Gaussian along `axis` (0 = x, 1 = y, 2 = z).
__global__ void smooth_pass_kernel(const double* __restrict__ in, double* __restrict__ out, long long nx, long long ny,
                                   long long nz, int axis, const double* __restrict__ w, int radius) {
    const long long n = nx * ny * nz;
    const long long stride = axis == 0 ? ny * nz : (axis == 1 ? nz : 1);
    const long long len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long pos = axis == 0 ? e / (ny * nz) : (axis == 1 ? (e / nz) % ny : e % nz);
        const long long lo = -min((long long)radius, pos), hi = min((long long)radius, len - 1 - pos);
        double s = 0.0, ws = 0.0;
        for (long long d = lo; d <= hi; ++d) {
            const double wt = w[d < 0 ? -d : d];
            s += wt * in[e + d * stride];
            ws += wt;
        }
        out[e] = s / ws;
    }
}

}  // namespace
}  // namespace stg

using namespace stg;

namespace {
struct DevMem {
    void* p = nullptr;
    ~DevMem() { cudaFree(p); }
};
}  // namespace

extern "C" {

int st_field_count_nonfinite(const double* data, int64_t n, int device, int64_t* out) {
    ST_CHECK(out && (data || n == 0), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(device));
    *out = 0;
    if (n <= 0) return ST_OK;
    DevMem d, c;
    ST_CUDA(cudaMalloc(&d.p, (size_t)n * 8));
    ST_CUDA(cudaMalloc(&c.p, 8));
    ST_CUDA(cudaMemcpy(d.p, data, (size_t)n * 8, cudaMemcpyHostToDevice));
    ST_CUDA(cudaMemset(c.p, 0, 8));
    count_kernel<<<blocks(n), 256>>>(static_cast<double*>(d.p), n, static_cast<unsigned long long*>(c.p));
    count_launch();
    ST_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    ST_CUDA(cudaMemcpy(&h, c.p, 8, cudaMemcpyDeviceToHost));
    *out = (int64_t)h;
    return ST_OK;
}

int st_field_clamp(double* data, int64_t n, double lo, double hi, int device) {
    ST_CHECK(data || n == 0, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(device));
    if (n <= 0) return ST_OK;
    DevMem d;
    ST_CUDA(cudaMalloc(&d.p, (size_t)n * 8));
    ST_CUDA(cudaMemcpy(d.p, data, (size_t)n * 8, cudaMemcpyHostToDevice));
    clamp_kernel<<<blocks(n), 256>>>(static_cast<double*>(d.p), n, lo, hi);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaMemcpy(data, d.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    return ST_OK;
}

int st_field_repair_nan(double* data, int64_t n, int64_t nx, int64_t ny, int64_t nz, int halo_width,
                        double replace_value, int device) {
    ST_CHECK(data || n == 0, ST_ERR_ARG, "null argument");
    ST_CHECK(nx >= 0 && ny >= 0 && nz >= 0 && halo_width >= 0, ST_ERR_ARG, "bad extents");
    ST_CHECK(nx * ny * nz <= n, ST_ERR_ARG, "nx*ny*nz = %lld exceeds the %lld values given",
             (long long)(nx * ny * nz), (long long)n);
    ST_CUDA(cudaSetDevice(device));
    if (n <= 0) return ST_OK;
    DevMem d;
    ST_CUDA(cudaMalloc(&d.p, (size_t)n * 8));
    ST_CUDA(cudaMemcpy(d.p, data, (size_t)n * 8, cudaMemcpyHostToDevice));
    repair_kernel<<<1, 1024>>>(static_cast<double*>(d.p), n, nx, ny, nz, halo_width, replace_value);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaMemcpy(data, d.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    return ST_OK;
}

int st_smooth_gradient_device(const double* g, int64_t nx, int64_t ny, int64_t nz, double sigma, double* out,
                              double* tmp, void* stream) {
    ST_CHECK(g && out && tmp, ST_ERR_ARG, "null argument");
    ST_CHECK(nx > 0 && ny > 0 && nz > 0, ST_ERR_ARG, "bad extents");
    const long long radius_ll = (long long)(3 * sigma);
    ST_CHECK(radius_ll >= 0 && radius_ll < (1 << 20), ST_ERR_ARG, "bad sigma %g", sigma);
    const int radius = (int)radius_ll;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<double> w((size_t)radius + 1);
    for (int d = 0; d <= radius; ++d) w[d] = std::exp(-(double)(d * d) / (2.0 * sigma * sigma));
    DevMem dw;
    ST_CUDA(cudaMalloc(&dw.p, w.size() * 8));
    ST_CUDA(cudaMemcpyAsync(dw.p, w.data(), w.size() * 8, cudaMemcpyHostToDevice, st));
    const long long n = nx * ny * nz;
    const double* wd = static_cast<const double*>(dw.p);
    smooth_pass_kernel<<<blocks(n), 256, 0, st>>>(g, out, nx, ny, nz, 2, wd, radius);
    count_launch();
    smooth_pass_kernel<<<blocks(n), 256, 0, st>>>(out, tmp, nx, ny, nz, 1, wd, radius);
    count_launch();
    smooth_pass_kernel<<<blocks(n), 256, 0, st>>>(tmp, out, nx, ny, nz, 0, wd, radius);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaStreamSynchronize(st));
    return ST_OK;
}

int st_smooth_gradient(const double* g, int64_t n, int64_t nx, int64_t ny, int64_t nz, double sigma, int device,
                       double* out) {
    ST_CHECK(out && (g || n == 0), ST_ERR_ARG, "null argument");
    ST_CHECK(nx >= 0 && ny >= 0 && nz >= 0, ST_ERR_ARG, "bad extents");
    const long long total = nx * ny * nz;
    if (total == 0) return ST_OK;
    if (n < total) {  // sparse_ops.cpp:123: too few values -> zeros
        std::fill(out, out + total, 0.0);
        return ST_OK;
    }
    ST_CUDA(cudaSetDevice(device));
    DevMem a, b, c;
    ST_CUDA(cudaMalloc(&a.p, (size_t)total * 8));
    ST_CUDA(cudaMalloc(&b.p, (size_t)total * 8));
    ST_CUDA(cudaMalloc(&c.p, (size_t)total * 8));
    ST_CUDA(cudaMemcpy(a.p, g, (size_t)total * 8, cudaMemcpyHostToDevice));
    ST_TRY(st_smooth_gradient_device(static_cast<double*>(a.p), nx, ny, nz, sigma, static_cast<double*>(b.p),
                                     static_cast<double*>(c.p), nullptr));
    ST_CUDA(cudaMemcpy(out, b.p, (size_t)total * 8, cudaMemcpyDeviceToHost));
    return ST_OK;
}

}  // extern "C"
