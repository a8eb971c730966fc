// C ABI of the sparse path: the seismic::CSRMatrix face
// (sparse/csr_matrix.h:17-71) and the seismic::SparseOps Krylov solvers
// (sparse/sparse_ops.h:9-48), over device CSR storage.
#include "st_sparse.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

using namespace stg;

struct st_csr {
    int device = 0;
    cudaStream_t stream = nullptr;
    DevCsr A;
    DevCsr AT;  // transpose, built on first use, dropped when values change
    bool has_T = false;
    double* dacc = nullptr;
};

namespace {

void drop_transpose(st_csr* m) {
    if (m->has_T) m->AT.release();
    m->has_T = false;
}

int ensure_transpose(st_csr* m) {
    if (m->has_T) return ST_OK;
    ST_TRY(build_transpose(m->A, &m->AT, m->stream));
    m->has_T = true;
    return ST_OK;
}

struct Scratch {
    std::vector<void*> p;
    ~Scratch() {
        for (void* q : p) cudaFree(q);
    }
    template <class T>
    T* get(size_t n) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        p.push_back(q);
        return static_cast<T*>(q);
    }
};

}  // namespace

namespace stg {
// The matrix, device and stream of a handle (for solver variants in other files).
const DevCsr* csr_matrix_of(const st_csr* m, int* device, cudaStream_t* stream) {
    *device = m->device;
    *stream = m->stream;
    return &m->A;
}
}  // namespace stg

namespace {

#define ST_ALLOC(ok) ST_CHECK(static_cast<bool>(ok), ST_ERR_ALLOC, "device allocation failed")

int make_handle(int device, st_csr** out) {
    ST_CHECK(out, ST_ERR_ARG, "null argument");
    int ndev = 0;
    ST_CUDA(cudaGetDeviceCount(&ndev));
    ST_CHECK(device >= 0 && device < ndev, ST_ERR_ARG, "device %d out of range", device);
    ST_CUDA(cudaSetDevice(device));
    std::unique_ptr<st_csr> m(new st_csr());
    m->device = device;
    ST_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    ST_CUDA(cudaMalloc(&m->dacc, 4 * sizeof(double)));
    ST_CUDA(cudaMalloc(&m->A.row_ptr, sizeof(long long)));
    ST_CUDA(cudaMemset(m->A.row_ptr, 0, sizeof(long long)));
    *out = m.release();
    return ST_OK;
}

}  // namespace

extern "C" {

int st_csr_create(int64_t rows, int64_t cols, int64_t nnz, int device, st_csr** out) {
    ST_CHECK(rows >= 0 && cols >= 0 && nnz >= 0, ST_ERR_ARG, "negative CSR extents");
    ST_TRY(make_handle(device, out));
    st_csr* m = *out;
    // CSRMatrix(rows, cols, nnz) (csr_matrix.cpp:19-23): zero row_ptr, nnz zero entries
    cudaFree(m->A.row_ptr);
    m->A.rows = rows;
    m->A.cols = cols;
    m->A.nnz = nnz;
    ST_CUDA(cudaMalloc(&m->A.row_ptr, (size_t)(rows + 1) * sizeof(long long)));
    ST_CUDA(cudaMalloc(&m->A.col, (size_t)std::max<int64_t>(nnz, 1) * sizeof(int)));
    ST_CUDA(cudaMalloc(&m->A.val, (size_t)std::max<int64_t>(nnz, 1) * sizeof(float)));
    ST_CUDA(cudaMemset(m->A.row_ptr, 0, (size_t)(rows + 1) * sizeof(long long)));
    ST_CUDA(cudaMemset(m->A.col, 0, (size_t)std::max<int64_t>(nnz, 1) * sizeof(int)));
    ST_CUDA(cudaMemset(m->A.val, 0, (size_t)std::max<int64_t>(nnz, 1) * sizeof(float)));
    return ST_OK;
}

int st_csr_destroy(st_csr* m) {
    if (!m) return ST_OK;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    m->A.release();
    drop_transpose(m);
    cudaFree(m->dacc);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return ST_OK;
}

int st_csr_build_from_triplets(st_csr* m, int64_t rows, int64_t cols, int64_t n, const int64_t* r, const int64_t* c,
                               const double* v, int pad) {
    ST_CHECK(m && (n == 0 || (r && c && v)), ST_ERR_ARG, "null argument");
    ST_CHECK(n >= 0, ST_ERR_ARG, "negative triplet count");
    ST_CUDA(cudaSetDevice(m->device));
    Scratch sc;
    long long* dr = sc.get<long long>((size_t)n);
    long long* dc = sc.get<long long>((size_t)n);
    double* dv = sc.get<double>((size_t)n);
    ST_ALLOC(dr && dc && dv);
    if (n > 0) {
        ST_CUDA(cudaMemcpyAsync(dr, r, (size_t)n * 8, cudaMemcpyHostToDevice, m->stream));
        ST_CUDA(cudaMemcpyAsync(dc, c, (size_t)n * 8, cudaMemcpyHostToDevice, m->stream));
        ST_CUDA(cudaMemcpyAsync(dv, v, (size_t)n * 8, cudaMemcpyHostToDevice, m->stream));
    }
    DevCsr out;
    int rc = build_csr<long long, double>(rows, cols, n, (const long long*)dr, (const long long*)dc, dv, pad != 0,
                                          &out, m->stream);
    if (rc < 0) {
        out.release();
        return rc;
    }
    ST_CUDA(cudaStreamSynchronize(m->stream));
    m->A.release();
    drop_transpose(m);
    m->A = out;
    return ST_OK;
}

int st_csr_build_from_triplets_device(st_csr* m, int64_t rows, int64_t cols, int64_t n, const int32_t* r,
                                      const int32_t* c, const float* v, int pad) {
    ST_CHECK(m && (n == 0 || (r && c && v)), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    DevCsr out;
    int rc = build_csr<int, float>(rows, cols, n, r, c, v, pad != 0, &out, m->stream);
    if (rc < 0) {
        out.release();
        return rc;
    }
    m->A.release();
    drop_transpose(m);
    m->A = out;
    return ST_OK;
}

int st_csr_build_fd_stencil_7point(st_csr* m, int64_t nx, int64_t ny, int64_t nz, const double* velocity, double dx,
                                   double dy, double dz, double dt, int pad) {
    ST_CHECK(m && velocity, ST_ERR_ARG, "null argument");
    ST_CHECK(nx > 0 && ny > 0 && nz > 0, ST_ERR_ARG, "bad grid extents");
    ST_CUDA(cudaSetDevice(m->device));
    const long long n = nx * ny * nz;
    Scratch sc;
    double* dvel = sc.get<double>((size_t)n);
    long long* tr = sc.get<long long>((size_t)(7 * n));
    long long* tc = sc.get<long long>((size_t)(7 * n));
    double* tv = sc.get<double>((size_t)(7 * n));
    ST_ALLOC(dvel && tr && tc && tv);
    ST_CUDA(cudaMemcpyAsync(dvel, velocity, (size_t)n * 8, cudaMemcpyHostToDevice, m->stream));
    ST_TRY(launch_fd_triplets(dvel, nx, ny, nz, 1.0 / (dx * dx), 1.0 / (dy * dy), 1.0 / (dz * dz), dt * dt, tr, tc,
                              tv, m->stream));
    DevCsr out;
    int rc = build_csr<long long, double>(n, n, 7 * n, tr, tc, tv, pad != 0, &out, m->stream);
    if (rc < 0) {
        out.release();
        return rc;
    }
    m->A.release();
    drop_transpose(m);
    m->A = out;
    return ST_OK;
}

int st_csr_build_ray_matrix(st_csr* m, int64_t n_rays, const double* endpoints, int on_device, int64_t nx,
                            int64_t ny, int64_t nz, double cell_size, int64_t* nnz) {
    ST_CHECK(m && (endpoints || n_rays == 0), ST_ERR_ARG, "null argument");
    ST_CHECK(n_rays >= 0 && n_rays < (1ll << 31), ST_ERR_ARG, "ray count out of range (%lld)", (long long)n_rays);
    ST_CHECK(nx > 0 && ny > 0 && nz > 0 && nx < (1 << 20) && ny < (1 << 20) && nz < (1 << 20), ST_ERR_ARG,
             "bad grid extents");
    ST_CUDA(cudaSetDevice(m->device));
    Scratch sc;
    const double* dends = endpoints;
    if (!on_device && n_rays > 0) {
        double* e = sc.get<double>((size_t)(6 * n_rays));
        ST_ALLOC(e);
        ST_CUDA(cudaMemcpyAsync(e, endpoints, (size_t)n_rays * 6 * 8, cudaMemcpyHostToDevice, m->stream));
        dends = e;
    }
    DevCsr out;
    long long total = 0;
    int rc = build_ray_csr(n_rays, dends, (int)nx, (int)ny, (int)nz, cell_size, &out, &total, m->stream);
    if (rc < 0) {
        out.release();
        return rc;
    }
    m->A.release();
    drop_transpose(m);
    m->A = out;
    if (nnz) *nnz = total;
    return ST_OK;
}

int st_csr_build_sampled_ray_matrix(st_csr* m, st_ray_picks* p, int64_t* nnz) {
    ST_CHECK(m && p, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    DevCsr out;
    long long total = 0;
    int rc = build_sampled_ray_csr(p, &out, &total, m->stream);
    if (rc < 0) {
        out.release();
        return rc;
    }
    m->A.release();
    drop_transpose(m);
    m->A = out;
    if (nnz) *nnz = total;
    return ST_OK;
}

int st_csr_shape(st_csr* m, int64_t out[3]) {
    ST_CHECK(m && out, ST_ERR_ARG, "null argument");
    out[0] = m->A.rows;
    out[1] = m->A.cols;
    out[2] = m->A.nnz;
    return ST_OK;
}

int st_csr_get(st_csr* m, int64_t* row_ptr, int64_t* col, double* val) {
    ST_CHECK(m, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    if (row_ptr)
        ST_CUDA(cudaMemcpyAsync(row_ptr, m->A.row_ptr, (size_t)(m->A.rows + 1) * 8, cudaMemcpyDeviceToHost,
                                m->stream));
    std::vector<int> ci;
    std::vector<float> vf;
    if (col && m->A.nnz) {
        ci.resize((size_t)m->A.nnz);
        ST_CUDA(cudaMemcpyAsync(ci.data(), m->A.col, ci.size() * 4, cudaMemcpyDeviceToHost, m->stream));
    }
    if (val && m->A.nnz) {
        vf.resize((size_t)m->A.nnz);
        ST_CUDA(cudaMemcpyAsync(vf.data(), m->A.val, vf.size() * 4, cudaMemcpyDeviceToHost, m->stream));
    }
    ST_CUDA(cudaStreamSynchronize(m->stream));
    for (size_t i = 0; i < ci.size(); ++i) col[i] = ci[i];
    for (size_t i = 0; i < vf.size(); ++i) val[i] = vf[i];
    return ST_OK;
}

int st_csr_device_arrays(st_csr* m, long long** row_ptr, int** col, float** val) {
    ST_CHECK(m, ST_ERR_ARG, "null argument");
    if (row_ptr) *row_ptr = m->A.row_ptr;
    if (col) *col = m->A.col;
    if (val) *val = m->A.val;
    return ST_OK;
}

int st_csr_stream(st_csr* m, void** out) {
    ST_CHECK(m && out, ST_ERR_ARG, "null argument");
    *out = (void*)m->stream;
    return ST_OK;
}

int st_csr_spmv_device(st_csr* m, int transpose, const float* x, float* y) {
    ST_CHECK(m && x && y, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    if (transpose) {
        ST_TRY(ensure_transpose(m));
        return launch_spmv(m->AT, x, y, nullptr, 0.0f, nullptr, nullptr, nullptr, m->stream);
    }
    return launch_spmv(m->A, x, y, nullptr, 0.0f, nullptr, nullptr, nullptr, m->stream);
}

static int spmv_host(st_csr* m, int transpose, const double* x, int64_t nx, double* y) {
    ST_CHECK(m && (x || nx == 0) && y, ST_ERR_ARG, "null argument");
    const long long in_n = transpose ? m->A.rows : m->A.cols;
    const long long out_n = transpose ? m->A.cols : m->A.rows;
    ST_CHECK(nx >= in_n, ST_ERR_ARG, "x has %lld values, the product needs %lld", (long long)nx, in_n);
    ST_CUDA(cudaSetDevice(m->device));
    Scratch sc;
    double* d64 = sc.get<double>((size_t)std::max(in_n, out_n));
    float* xf = sc.get<float>((size_t)in_n);
    float* yf = sc.get<float>((size_t)out_n);
    ST_ALLOC(d64 && xf && yf);
    ST_CUDA(cudaMemcpyAsync(d64, x, (size_t)in_n * 8, cudaMemcpyHostToDevice, m->stream));
    ST_TRY(launch_f64_to_f32(d64, xf, in_n, m->stream));
    ST_TRY(st_csr_spmv_device(m, transpose, xf, yf));
    ST_TRY(launch_f32_to_f64(yf, d64, out_n, m->stream));
    ST_CUDA(cudaMemcpyAsync(y, d64, (size_t)out_n * 8, cudaMemcpyDeviceToHost, m->stream));
    ST_CUDA(cudaStreamSynchronize(m->stream));
    return ST_OK;
}

int st_csr_spmv(st_csr* m, const double* x, int64_t nx, double* y) { return spmv_host(m, 0, x, nx, y); }
int st_csr_spmv_transpose(st_csr* m, const double* x, int64_t nx, double* y) { return spmv_host(m, 1, x, nx, y); }

int st_csr_normal_jacobi(st_csr* m, double lam, float* dinv) {
    ST_CHECK(m && dinv, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    ST_TRY(ensure_transpose(m));
    return launch_normal_jacobi(m->AT, lam, dinv, m->stream);
}

int st_csr_frobenius_norm(st_csr* m, double* out) {
    ST_CHECK(m && out, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    ST_TRY(launch_sumsq(m->A.val, m->A.nnz, m->dacc, m->stream));
    double s = 0.0;
    ST_CUDA(cudaMemcpyAsync(&s, m->dacc, 8, cudaMemcpyDeviceToHost, m->stream));
    ST_CUDA(cudaStreamSynchronize(m->stream));
    *out = std::sqrt(s);
    return ST_OK;
}

int st_csr_scale(st_csr* m, double alpha) {
    ST_CHECK(m, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    ST_TRY(launch_scale(m->A.val, m->A.nnz, (float)alpha, m->stream));
    drop_transpose(m);
    ST_CUDA(cudaStreamSynchronize(m->stream));
    return ST_OK;
}

int st_csr_add_diagonal(st_csr* m, double alpha) {
    ST_CHECK(m, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    ST_TRY(launch_add_diag(m->A, (float)alpha, m->stream));
    drop_transpose(m);
    ST_CUDA(cudaStreamSynchronize(m->stream));
    return ST_OK;
}

int st_csr_clone(st_csr* m, st_csr** out) {
    ST_CHECK(m && out, ST_ERR_ARG, "null argument");
    ST_TRY(st_csr_create(m->A.rows, m->A.cols, m->A.nnz, m->device, out));
    st_csr* c = *out;
    ST_CUDA(cudaMemcpy(c->A.row_ptr, m->A.row_ptr, (size_t)(m->A.rows + 1) * 8, cudaMemcpyDeviceToDevice));
    if (m->A.nnz) {
        ST_CUDA(cudaMemcpy(c->A.col, m->A.col, (size_t)m->A.nnz * 4, cudaMemcpyDeviceToDevice));
        ST_CUDA(cudaMemcpy(c->A.val, m->A.val, (size_t)m->A.nnz * 4, cudaMemcpyDeviceToDevice));
    }
    return ST_OK;
}

// Device-pointer CG on the square system A x = b (FP32 vectors, FP64 scalars).
int st_cg_device(st_csr* m, const float* b, float* x, int max_iter, double tol, int jacobi, int* iters,
                 double* final_rel) {
    ST_CHECK(m && b && x, ST_ERR_ARG, "null argument");
    ST_CHECK(m->A.rows == m->A.cols, ST_ERR_ARG, "CG needs a square matrix (%lld x %lld)", m->A.rows, m->A.cols);
    ST_CUDA(cudaSetDevice(m->device));
    const long long n = m->A.rows;
    Scratch sc;
    CgWork W;
    W.r = sc.get<float>((size_t)n);
    W.z = sc.get<float>((size_t)n);
    W.p = sc.get<float>((size_t)n);
    W.q = sc.get<float>((size_t)n);
    W.sc = sc.get<CgScalars>(1);
    float* dinv = jacobi ? sc.get<float>((size_t)n) : nullptr;
    ST_ALLOC(W.r && W.z && W.p && W.q && W.sc && (!jacobi || dinv));
    if (jacobi) ST_TRY(launch_jacobi(m->A, dinv, m->stream));
    CgProblem P;
    P.A = &m->A;
    P.n = n;
    P.b = b;
    P.x = x;
    P.dinv = dinv;
    CgResult R;
    ST_TRY(run_cg(P, W, max_iter, tol, 16, &R, m->stream));
    if (n == 0 || R.iters == 0) ST_CUDA(cudaMemsetAsync(x, 0, (size_t)std::max<long long>(n, 1) * 4, m->stream));
    ST_CUDA(cudaStreamSynchronize(m->stream));
    if (iters) *iters = R.iters;
    if (final_rel) *final_rel = R.rel;
    return ST_OK;
}

int st_cg(st_csr* m, const double* b, int64_t nb, int max_iter, double tol, int jacobi, double* x, int* iters,
          double* final_rel) {
    ST_CHECK(m && x && (b || nb == 0), ST_ERR_ARG, "null argument");
    const long long n = m->A.rows;
    ST_CHECK(nb >= n, ST_ERR_ARG, "b has %lld values, the system has %lld rows", (long long)nb, n);
    ST_CUDA(cudaSetDevice(m->device));
    Scratch sc;
    double* d64 = sc.get<double>((size_t)n);
    float* bf = sc.get<float>((size_t)n);
    float* xf = sc.get<float>((size_t)n);
    ST_ALLOC(d64 && bf && xf);
    if (n) ST_CUDA(cudaMemcpyAsync(d64, b, (size_t)n * 8, cudaMemcpyHostToDevice, m->stream));
    ST_TRY(launch_f64_to_f32(d64, bf, n, m->stream));
    ST_TRY(st_cg_device(m, bf, xf, max_iter, tol, jacobi, iters, final_rel));
    ST_TRY(launch_f32_to_f64(xf, d64, n, m->stream));
    if (n) ST_CUDA(cudaMemcpyAsync(x, d64, (size_t)n * 8, cudaMemcpyDeviceToHost, m->stream));
    ST_CUDA(cudaStreamSynchronize(m->stream));
    return ST_OK;
}

// Damped normal equations (A^T A + lam I) x = A^T d of a rectangular A.
// The normal-equation CG of st_normal_cg_device, with the stencil
// preconditioner of st_normal_pcg_stencil_device when stencil is set (three
// axis weights on a gx x gy x gz cell grid).
static int normal_cg_impl(st_csr* m, const float* d, double lam, int max_iter, double tol, int jacobi, float* x,
                          float* rhs, int* iters, double* final_rel, double* true_rel, const float* stencil, int gx,
                          int gy, int gz) {
    ST_CHECK(m && x && (d || rhs), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(m->device));
    ST_TRY(ensure_transpose(m));
    const long long n = m->A.cols, rows = m->A.rows;
    Scratch sc;
    CgWork W;
    W.r = sc.get<float>((size_t)n);
    W.z = sc.get<float>((size_t)n);
    W.p = sc.get<float>((size_t)n);
    W.q = sc.get<float>((size_t)n);
    W.t = sc.get<float>((size_t)rows);
    W.sc = sc.get<CgScalars>(1);
    float* b = rhs ? rhs : sc.get<float>((size_t)n);
    const bool use_jacobi = (jacobi & ST_CG_JACOBI) != 0 || stencil;
    const bool confirm = (jacobi & ST_CG_CONFIRM_TRUE) != 0;
    float* dinv = use_jacobi ? sc.get<float>((size_t)n) : nullptr;
    float* res = sc.get<float>((size_t)n);
    float* sq = stencil ? sc.get<float>((size_t)n) : nullptr;
    ST_ALLOC(W.r && W.z && W.p && W.q && W.t && W.sc && b && (!use_jacobi || dinv) && res && (!stencil || sq));
    if (d) ST_TRY(launch_spmv(m->AT, d, b, nullptr, 0.0f, nullptr, nullptr, nullptr, m->stream));
    if (use_jacobi) ST_TRY(launch_normal_jacobi(m->AT, lam, dinv, m->stream));
    if (stencil) ST_TRY(launch_sqrt(dinv, sq, n, m->stream));
    CgProblem P;
    P.A = &m->A;
    P.AT = &m->AT;
    P.lam = lam;
    P.n = n;
    P.b = b;
    P.x = x;
    P.dinv = dinv;
    if (stencil) {
        P.sq = sq;
        P.gx = gx;
        P.gy = gy;
        P.gz = gz;
        for (int a = 0; a < 3; ++a) P.w[a] = stencil[a];
    }
    CgResult R;
    ST_TRY(run_cg(P, W, max_iter, tol, 16, &R, m->stream));
    if (R.iters == 0) ST_CUDA(cudaMemsetAsync(x, 0, (size_t)std::max<long long>(n, 1) * 4, m->stream));
    // ||A^T d - (A^T A + lam I) x|| / ||A^T d|| in FP64 (t and q are rewritten by every iteration)
    auto residual = [&](double* out) -> int {
        ST_TRY(launch_spmv(m->A, x, W.t, nullptr, 0.0f, nullptr, nullptr, nullptr, m->stream));
        ST_TRY(launch_spmv(m->AT, W.t, W.q, x, (float)lam, nullptr, nullptr, nullptr, m->stream));
        ST_TRY(launch_residual(res, b, W.q, n, m->stream));
        ST_TRY(launch_sumsq(res, n, m->dacc, m->stream));
        ST_TRY(launch_sumsq(b, n, m->dacc + 1, m->stream));
        double h[2];
        ST_CUDA(cudaMemcpyAsync(h, m->dacc, 16, cudaMemcpyDeviceToHost, m->stream));
        ST_CUDA(cudaStreamSynchronize(m->stream));
        *out = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
        return ST_OK;
    };
    // With ST_CG_CONFIRM_TRUE the stop is confirmed on the true residual: the
    // FP32 recurrence residual drifts from it, so while the true one is above
    // tol the solve continues (same Krylov state) to a recurrence target
    // scaled by their ratio, a few times at most.
    double tr = 0.0;
    if (confirm || true_rel) ST_TRY(residual(&tr));
    for (int round = 0; confirm && round < 10 && tr > tol && !R.breakdown && R.iters > 0 && R.iters < max_iter &&
                        R.rel < tol;
         ++round) {
        const double target = R.rel * (tol / tr) * 0.995;
        ST_TRY(resume_cg(P, W, max_iter, target, 16, &R, m->stream));
        ST_TRY(residual(&tr));
    }
    if (true_rel) *true_rel = tr;
    ST_CUDA(cudaStreamSynchronize(m->stream));
    if (iters) *iters = R.iters;
    if (final_rel) *final_rel = R.rel;
    return ST_OK;
}

int st_normal_cg_device(st_csr* m, const float* d, double lam, int max_iter, double tol, int jacobi, float* x,
                        float* rhs, int* iters, double* final_rel, double* true_rel) {
    return normal_cg_impl(m, d, lam, max_iter, tol, jacobi, x, rhs, iters, final_rel, true_rel, nullptr, 0, 0, 0);
}

int st_normal_pcg_stencil_device(st_csr* m, const float* d, double lam, const float* w, int64_t nx, int64_t ny,
                                 int64_t nz, int max_iter, double tol, int flags, float* x, float* rhs, int* iters,
                                 double* final_rel, double* true_rel) {
    ST_CHECK(m && w, ST_ERR_ARG, "null argument");
    ST_CHECK(nx > 0 && ny > 0 && nz > 0 && nx * ny * nz == m->A.cols, ST_ERR_ARG,
             "grid %lld x %lld x %lld does not match the matrix's %lld columns", (long long)nx, (long long)ny,
             (long long)nz, m->A.cols);
    for (int a = 0; a < 3; ++a)
        ST_CHECK(std::isfinite(w[a]) && w[a] >= 0.0f, ST_ERR_ARG, "stencil weights must be finite and >= 0");
    return normal_cg_impl(m, d, lam, max_iter, tol, flags, x, rhs, iters, final_rel, true_rel, w, (int)nx, (int)ny,
                          (int)nz);
}

int st_normal_fcg_device(st_csr* m, const float* d, double lam, int max_iter, double tol, st_pcnet* pc, float* x,
                         int* iters, double* true_rel) {
    ST_CHECK(m && d && x, ST_ERR_ARG, "null argument");
    ST_CHECK(max_iter >= 0, ST_ERR_ARG, "negative iteration limit");
    ST_CUDA(cudaSetDevice(m->device));
    ST_TRY(ensure_transpose(m));
    const long long n = m->A.cols, rows = m->A.rows;
    ST_CHECK(!pc || pcnet_points(pc) == n, ST_ERR_ARG, "network grid has %lld points, the system %lld unknowns",
             pc ? pcnet_points(pc) : 0ll, n);
    Scratch sc;
    float* b = sc.get<float>((size_t)n);
    float* dinv = sc.get<float>((size_t)n);
    float* r = sc.get<float>((size_t)n);
    float* z = sc.get<float>((size_t)n);
    float* p = sc.get<float>((size_t)n);
    float* q = sc.get<float>((size_t)n);
    float* ax = sc.get<float>((size_t)n);
    float* t = sc.get<float>((size_t)rows);
    FcgScalars* s = sc.get<FcgScalars>(1);
    double* acc = sc.get<double>(2);
    ST_ALLOC(b && dinv && r && z && p && q && ax && t && s && acc);
    ST_TRY(launch_spmv(m->AT, d, b, nullptr, 0.0f, nullptr, nullptr, nullptr, m->stream));
    ST_TRY(launch_normal_jacobi(m->AT, lam, dinv, m->stream));
    int it = 0;
    double rel = 0.0;
    ST_TRY(run_fcg(m->A, m->AT, lam, b, x, dinv, pc, max_iter, tol, r, z, p, q, ax, t, s, acc, m->stream, &it, &rel));
    ST_CUDA(cudaStreamSynchronize(m->stream));
    if (iters) *iters = it;
    if (true_rel) *true_rel = rel;
    return ST_OK;
}

// SparseOps::dot_product (sparse_ops.cpp:172-187): FP64 inner product on the GPU.
int st_dot(const double* a, const double* b, int64_t n, int device, double* out) {
    ST_CHECK((a && b) || n == 0, ST_ERR_ARG, "null argument");
    ST_CHECK(out, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(device));
    *out = 0.0;
    if (n <= 0) return ST_OK;
    // FP64 in, FP64 products and sums: one pass on the device
    Scratch sc;
    double* da = sc.get<double>((size_t)n);
    double* db = sc.get<double>((size_t)n);
    double* acc = sc.get<double>(1);
    ST_ALLOC(da && db && acc);
    ST_CUDA(cudaMemcpy(da, a, (size_t)n * 8, cudaMemcpyHostToDevice));
    ST_CUDA(cudaMemcpy(db, b, (size_t)n * 8, cudaMemcpyHostToDevice));
    ST_TRY(launch_dot64(da, db, n, acc, nullptr));
    ST_CUDA(cudaMemcpy(out, acc, 8, cudaMemcpyDeviceToHost));
    return ST_OK;
}

}  // extern "C"
