// Flexible CG on the damped normal equations (A^T A + lam I) x = A^T d with a
// nonlinear preconditioner (the learned network, st_precond.cu) or Jacobi.
//
// Iteration (one-term A-orthogonalisation, FP32 vectors, FP64 scalars kept
// on the device):
//     alpha = p.r / p.q,  x += alpha p,  r -= alpha q
//     z = M(r); if z.r <= 0 (not a descent direction) z = dinv r
//     beta = z.q / p.q,   p = z - beta p,   q = (A^T A + lam I) p
// The recursive residual is read every 16 iterations; a candidate
// convergence is confirmed on the true residual b - (A^T A + lam I) x (FP64
// norms), which otherwise replaces r.
#include "st_sparse.cuh"

#include <cmath>

struct st_pcnet;
extern "C" int st_pcnet_apply(st_pcnet* p, const float* r, const float* dinv, float* z, void* stream);

namespace stg {
namespace {

// Four CTAs per SM: each thread takes a few elements, so that the per-thread
// FP64 sums and block reductions (a slow pipe on this GPU) stay small.
unsigned fcg_blocks(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 4));
}

__device__ __forceinline__ void block_sum3(double a, double b, double c, double* da, double* db, double* dc) {
    __shared__ double s[3][8];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s[0][w] = a;
        s[1][w] = b;
        s[2][w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = b = c = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a += s[0][k];
            b += s[1][k];
            c += s[2][k];
        }
        if (da) atomicAdd(da, a);
        if (db) atomicAdd(db, b);
        if (dc) atomicAdd(dc, c);
    }
}

// pq = p.q, pr = p.r
__global__ void fcg_dots_pq(const float* __restrict__ p, const float* __restrict__ q, const float* __restrict__ r,
                            long long n, FcgScalars* s) {
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        a += (double)p[i] * (double)q[i];
        b += (double)p[i] * (double)r[i];
    }
    block_sum3(a, b, 0.0, &s->pq, &s->pr, nullptr);
}

// x += alpha p, r -= alpha q, rr = r.r
__global__ void fcg_update(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
                           const float* __restrict__ q, long long n, FcgScalars* s) {
    __shared__ float s_alpha;  // formed once per block
    if (threadIdx.x == 0) {
        const double pq = s->pq;
        s_alpha = pq != 0.0 ? (float)(s->pr / pq) : 0.0f;
    }
    __syncthreads();
    const float alpha = s_alpha;
    double a = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        x[i] = fmaf(alpha, p[i], x[i]);
        const float ri = fmaf(-alpha, q[i], r[i]);
        r[i] = ri;
        a += (double)ri * (double)ri;
    }
    block_sum3(a, 0.0, 0.0, &s->rr, nullptr, nullptr);
}

// zr = z.r, zq = z.q, jq = (dinv r).q
__global__ void fcg_dots_z(const float* __restrict__ z, const float* __restrict__ r, const float* __restrict__ q,
                           const float* __restrict__ dinv, long long n, FcgScalars* s) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        a += (double)z[i] * (double)r[i];
        b += (double)z[i] * (double)q[i];
        c += (double)dinv[i] * (double)r[i] * (double)q[i];
    }
    block_sum3(a, b, c, &s->zr, &s->zq, &s->jq);
}

// p = z - beta p (z replaced by dinv r when it is not a descent direction)
__global__ void fcg_pupdate(float* __restrict__ p, const float* __restrict__ z, const float* __restrict__ r,
                            const float* __restrict__ dinv, long long n, const FcgScalars* s, int first) {
    __shared__ float s_beta;  // formed once per block
    __shared__ int s_use_z;
    if (threadIdx.x == 0) {
        const bool uz = s->zr > 0.0;
        const double pq = s->pq;
        s_beta = first || pq == 0.0 ? 0.0f : (float)((uz ? s->zq : s->jq) / pq);
        s_use_z = uz;
    }
    __syncthreads();
    const bool use_z = s_use_z;
    const float beta = s_beta;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float zi = use_z ? z[i] : dinv[i] * r[i];
        p[i] = first ? zi : fmaf(-beta, p[i], zi);
    }
}

__global__ void fcg_mul(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = a[i] * b[i];
}

__global__ void fcg_residual(const float* __restrict__ b, const float* __restrict__ ax, float* __restrict__ r,
                             long long n, double* acc) {
    double a = 0.0, c = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float ri = b[i] - ax[i];
        if (r) r[i] = ri;
        a += (double)ri * (double)ri;
        c += (double)b[i] * (double)b[i];
    }
    block_sum3(a, c, 0.0, acc, acc + 1, nullptr);
}

}  // namespace

// q = A^T (A p) + lam p; t: rows-long scratch.
static int normal_apply(const DevCsr& A, const DevCsr& AT, double lam, const float* p, float* t, float* q,
                        cudaStream_t st) {
    ST_TRY(launch_spmv(A, p, t, nullptr, 0.0f, nullptr, nullptr, nullptr, st));
    return launch_spmv(AT, t, q, p, (float)lam, nullptr, nullptr, nullptr, st);
}

// True relative residual ||b - (A^T A + lam I) x|| / ||b||, optionally stored into r.
static int true_residual(const DevCsr& A, const DevCsr& AT, double lam, const float* b, const float* x, float* t,
                         float* ax, float* r, double* acc, double* out, cudaStream_t st) {
    const long long n = A.cols;
    ST_TRY(normal_apply(A, AT, lam, x, t, ax, st));
    ST_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), st));
    fcg_residual<<<fcg_blocks(n), 256, 0, st>>>(b, ax, r, n, acc);
    count_launch();
    double h[2];
    ST_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaStreamSynchronize(st));
    *out = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
    return ST_OK;
}

// Work vectors: r, z, p, q, ax (n each), t (rows), scalars.
int run_fcg(const DevCsr& A, const DevCsr& AT, double lam, const float* b, float* x, const float* dinv, st_pcnet* pc,
            int max_iter, double tol, float* r, float* z, float* p, float* q, float* ax, float* t, FcgScalars* sc,
            double* acc, cudaStream_t st, int* iters, double* true_rel) {
    const long long n = A.cols;
    const unsigned nb = fcg_blocks(n);
    auto precondition = [&]() -> int {
        if (pc) return st_pcnet_apply(pc, r, dinv, z, st);
        fcg_mul<<<nb, 256, 0, st>>>(dinv, r, z, n);
        count_launch();
        return ST_OK;
    };
    auto direction = [&](int first) -> int {
        ST_CUDA(cudaMemsetAsync(&sc->zr, 0, 3 * sizeof(double), st));
        fcg_dots_z<<<nb, 256, 0, st>>>(z, r, q, dinv, n, sc);
        count_launch();
        fcg_pupdate<<<nb, 256, 0, st>>>(p, z, r, dinv, n, sc, first);
        count_launch();
        return normal_apply(A, AT, lam, p, t, q, st);
    };
    ST_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 4, st));
    ST_CUDA(cudaMemcpyAsync(r, b, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
    ST_CUDA(cudaMemsetAsync(q, 0, (size_t)n * 4, st));
    double bb = 0.0;
    {
        ST_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), st));
        fcg_residual<<<nb, 256, 0, st>>>(b, q, nullptr, n, acc);  // ||b||^2 (q = 0)
        count_launch();
        double h[2];
        ST_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
        bb = h[1];
    }
    *iters = 0;
    *true_rel = 0.0;
    if (bb == 0.0) return ST_OK;
    ST_TRY(precondition());
    ST_TRY(direction(1));
    int it = 0;
    double rel = 1.0;
    while (it < max_iter) {
        ST_CUDA(cudaMemsetAsync(sc, 0, 3 * sizeof(double), st));  // pq, pr, rr
        fcg_dots_pq<<<nb, 256, 0, st>>>(p, q, r, n, sc);
        count_launch();
        fcg_update<<<nb, 256, 0, st>>>(x, r, p, q, n, sc);
        count_launch();
        ++it;
        if (it % 16 == 0 || it == max_iter) {
            FcgScalars h;
            ST_CUDA(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, st));
            ST_CUDA(cudaStreamSynchronize(st));
            rel = std::sqrt(h.rr / bb);
            if (!(h.pq > 0.0) || rel <= tol) {
                ST_TRY(true_residual(A, AT, lam, b, x, t, ax, r, acc, &rel, st));
                if (rel <= tol || !(h.pq > 0.0)) break;
            }
        }
        ST_TRY(precondition());
        ST_TRY(direction(0));
    }
    ST_TRY(true_residual(A, AT, lam, b, x, t, ax, nullptr, acc, &rel, st));
    *iters = it;
    *true_rel = rel;
    return ST_OK;
}

}  // namespace stg
