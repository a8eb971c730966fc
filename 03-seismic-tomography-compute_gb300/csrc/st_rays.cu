// Straight-ray path-length matrix for traveltime tomography.
//
// Row i of A holds, for every cell j that ray i crosses, the length of the
// ray inside that cell (times the cell size), so A s = traveltimes for the
// slowness model s. The traversal is the exact voxel walk of Amanatides and
// Woo ("A fast voxel traversal algorithm for ray tracing", Eurographics
// 1987): the ray p(t) = p0 + t (p1 - p0), t in [0, 1], is cut at every
// cell face it crosses, in order of t; ties go to x, then y, then z. All
// arithmetic is FP64 with explicit rounding (no contractions) so the host
// restatement in the oracle produces the same lengths bit for bit; values
// are rounded to FP32 once, when the CSR is built.
//
// Two passes over the rays (count, then write triplets at scanned offsets)
// feed the general triplet -> CSR builder, which gives the
// CSRMatrix::build_from_triplets semantics (sparse/csr_matrix.cpp:25-72):
// per-row columns ascending, no padding. Columns are j = (ix*ny + iy)*nz + iz.
#include "st_sort.cuh"
#include "st_sparse.cuh"

#include <algorithm>
#include <cmath>

namespace stg {
namespace {

struct RayGrid {
    int nx, ny, nz;
    double h;
};

__host__ __device__ inline double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ inline double dsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ inline double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ inline double ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

__host__ __device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Parameter t at which the ray leaves cell index c along one axis.
__device__ inline double t_exit(int c, int step, double p0, double d) {
    if (step == 0) return 1e300;
    const double face = (double)(step > 0 ? c + 1 : c);
    return ddiv(dsub(face, p0), d);
}

// Walks ray e; emit(col, length) for every crossed cell, in traversal order.
template <class F>
__device__ void walk(const double* e, const RayGrid& G, F emit) {
    const double p0[3] = {e[0], e[1], e[2]};
    const double d[3] = {dsub(e[3], e[0]), dsub(e[4], e[1]), dsub(e[5], e[2])};
    const double len = sqrt(dadd(dadd(dmul(d[0], d[0]), dmul(d[1], d[1])), dmul(d[2], d[2])));
    const int n[3] = {G.nx, G.ny, G.nz};
    int c[3], step[3];
    double tm[3];
    for (int a = 0; a < 3; ++a) {
        c[a] = clampi((int)floor(p0[a]), 0, n[a] - 1);
        step[a] = d[a] > 0.0 ? 1 : (d[a] < 0.0 ? -1 : 0);
        tm[a] = t_exit(c[a], step[a], p0[a], d[a]);
    }
    double t = 0.0;
    const int max_iter = G.nx + G.ny + G.nz + 3;
    for (int it = 0; it < max_iter; ++it) {
        const int ax = (tm[0] <= tm[1] && tm[0] <= tm[2]) ? 0 : (tm[1] <= tm[2] ? 1 : 2);
        const double tn = tm[ax];
        const double te = tn < 1.0 ? tn : 1.0;
        const double seg = dmul(dmul(dsub(te, t), len), G.h);
        if (seg > 0.0) emit(((long long)c[0] * G.ny + c[1]) * G.nz + c[2], seg);
        if (tn >= 1.0) break;
        t = tn;
        c[ax] += step[ax];
        if (c[ax] < 0 || c[ax] >= n[ax]) break;
        tm[ax] = t_exit(c[ax], step[ax], p0[ax], d[ax]);
    }
}

__global__ void ray_count_kernel(const double* __restrict__ ends, long long nrays, RayGrid G, long long* count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nrays;
         i += (long long)gridDim.x * blockDim.x) {
        long long k = 0;
        walk(ends + 6 * i, G, [&](long long, double) { ++k; });
        count[i] = k;
    }
}

__global__ void ray_write_kernel(const double* __restrict__ ends, long long nrays, RayGrid G,
                                 const long long* __restrict__ off, long long* rows, long long* cols, double* vals) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nrays;
         i += (long long)gridDim.x * blockDim.x) {
        long long k = off[i];
        walk(ends + 6 * i, G, [&](long long col, double v) {
            rows[k] = i;
            cols[k] = col;
            vals[k] = v;
            ++k;
        });
    }
}

unsigned grid_for(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 32));
}

}  // namespace

// Builds the ray matrix of nrays rays (device endpoints [nrays][6] =
// x0 y0 z0 x1 y1 z1 in cell units) over an nx*ny*nz grid of cells of size h.
int build_ray_csr(long long nrays, const double* d_ends, int nx, int ny, int nz, double h, DevCsr* out,
                  long long* total_nnz, cudaStream_t st) {
    ST_CHECK(nrays >= 0 && nx > 0 && ny > 0 && nz > 0, ST_ERR_ARG, "bad ray-matrix extents");
    ST_CHECK((long long)nx * ny * nz < (1ll << 31), ST_ERR_ARG, "cell count must fit int32 columns");
    ST_CHECK(h > 0.0 && std::isfinite(h), ST_ERR_ARG, "cell size must be positive");
    const RayGrid G{nx, ny, nz, h};
    DeviceBuffers bufs;
    auto* count = static_cast<long long*>(bufs.get((size_t)(nrays + 1) * 8));
    auto* off = static_cast<long long*>(bufs.get((size_t)(nrays + 1) * 8));
    auto* tot = static_cast<long long*>(bufs.get(64));
    void* stmp = bufs.get(scan_tmp_bytes(std::max<long long>(nrays, 1)));
    if (!count || !off || !tot || !stmp) return bufs.fail();
    long long n = 0;
    if (nrays > 0) {
        ray_count_kernel<<<grid_for(nrays), 256, 0, st>>>(d_ends, nrays, G, count);
        count_launch();
        ST_CUDA(cudaGetLastError());
        ST_TRY(exclusive_scan_i64(count, off, nrays, tot, stmp, st));
        ST_CUDA(cudaMemcpyAsync(&n, tot, sizeof(long long), cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
    }
    if (total_nnz) *total_nnz = n;
    auto* r = static_cast<long long*>(bufs.get((size_t)std::max<long long>(n, 1) * 8));
    auto* c = static_cast<long long*>(bufs.get((size_t)std::max<long long>(n, 1) * 8));
    auto* v = static_cast<double*>(bufs.get((size_t)std::max<long long>(n, 1) * 8));
    if (!r || !c || !v) return bufs.fail();
    if (n > 0) {
        ray_write_kernel<<<grid_for(nrays), 256, 0, st>>>(d_ends, nrays, G, off, r, c, v);
        count_launch();
        ST_CUDA(cudaGetLastError());
    }
    return build_csr<long long, double>(nrays, (long long)nx * ny * nz, n, r, c, v, false, out, st);
}

}  // namespace stg
