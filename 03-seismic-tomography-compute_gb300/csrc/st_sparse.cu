// CSR sparse path on the GPU: the triplet -> CSR builder of
// CSRMatrix::build_from_triplets (sparse/csr_matrix.cpp:25-72), the 7-point
// FD stencil matrix (:74-116), SpMV / SpMV^T (:118-166), scale,
// add_diagonal, Frobenius norm (:168-193), and the Krylov solvers of
// SparseOps (sparse/sparse_ops.cpp:8-113) -- plain CG, Jacobi-PCG and the
// damped normal-equation solve of the tomography system -- with FP32
// vectors and matrix values, int32 column indices, int64 row pointers and
// every inner product, residual norm and step scalar in FP64 on the device.
#include "st_sort.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "st_sparse.cuh"

#include <cstdlib>

namespace stg {
namespace {

constexpr unsigned FULL = 0xffffffffu;

int bits_for(long long v) {
    int b = 0;
    while (b < 63 && (1ll << b) <= v) ++b;
    return std::max(b, 1);
}

int grid_cap() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        n = std::max(n, 1);
    }
    return n * 16;
}

unsigned blocks_for(long long work, int threads = 256) {
    long long b = (work + threads - 1) / threads;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, grid_cap()));
}

// The CG vector kernels: four CTAs per SM (each thread a few elements), so
// that their per-thread FP64 partial sums and block reductions stay small.
unsigned cg_blocks(long long work) {
    long long b = (work + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, grid_cap() / 4));
}

// ---------------------------------------------------------------- builder kernels
template <class TI>
__global__ void keys_kernel(const TI* __restrict__ r, const TI* __restrict__ c, long long n, long long R, long long Cc,
                            int cb, unsigned long long* __restrict__ keys, unsigned* __restrict__ pay) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long rr = (long long)r[i], cc = (long long)c[i];
        const bool ok = rr >= 0 && rr < R && cc >= 0 && cc < Cc;
        keys[i] = ok ? (((unsigned long long)rr << cb) | (unsigned long long)cc) : ((unsigned long long)R << cb);
        pay[i] = (unsigned)i;
    }
}

__global__ void heads_kernel(const unsigned long long* __restrict__ keys, long long n, long long R, int cb,
                             long long* __restrict__ flag) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        const bool valid = (long long)(k >> cb) < R;
        flag[i] = (valid && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
    }
}

// One thread per run of equal keys: sums the duplicates in input order (FP64).
template <class TV>
__global__ void merge_kernel(const unsigned long long* __restrict__ keys, const unsigned* __restrict__ pay, long long n,
                             int cb, const long long* __restrict__ flag, const long long* __restrict__ uidx,
                             const TV* __restrict__ v_in, int* __restrict__ col_out, float* __restrict__ val_out,
                             long long* __restrict__ urow) {
    const unsigned long long cmask = (1ull << cb) - 1;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        const unsigned long long k = keys[i];
        long long j = i + 1;
        while (j < n && keys[j] == k) ++j;
        double sum = 0.0;
        if (j - i == 1) {
            sum = (double)v_in[pay[i]];
        } else {
            // visit the run's input positions in increasing order
            unsigned last = 0;
            bool first = true;
            for (long long m = i; m < j; ++m) {
                unsigned best = 0xffffffffu;
                for (long long q = i; q < j; ++q) {
                    const unsigned p = pay[q];
                    if ((first || p > last) && p < best) best = p;
                }
                sum += (double)v_in[best];
                last = best;
                first = false;
            }
        }
        const long long u = uidx[i];
        col_out[u] = (int)(k & cmask);
        val_out[u] = (float)sum;
        urow[u] = (long long)(k >> cb);
    }
}

__global__ void rowptr_kernel(const long long* __restrict__ urow, long long nnz, long long R,
                              long long* __restrict__ rp) {
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nnz; u += (long long)gridDim.x * blockDim.x) {
        const long long r = urow[u];
        const long long prev = u == 0 ? -1 : urow[u - 1];
        for (long long q = prev + 1; q <= r; ++q) rp[q] = u;
        if (u == nnz - 1)
            for (long long q = r + 1; q <= R; ++q) rp[q] = nnz;
    }
}

// pad_to_alignment trigger (csr_matrix.cpp:223-264): a row i with
// roundup8(row_ptr[i]) > row_ptr[i+1].
__global__ void pad_trigger_kernel(const long long* __restrict__ rp, long long R, int* __restrict__ trig) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x)
        if (((rp[i] + 7) / 8) * 8 > rp[i + 1]) atomicOr(trig, 1);
}

__global__ void pad_len_kernel(const long long* __restrict__ rp, long long R, long long* __restrict__ plen) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x)
        plen[i] = ((rp[i + 1] - rp[i] + 7) / 8) * 8;
}

__global__ void pad_scatter_kernel(const long long* __restrict__ rp, const int* __restrict__ col,
                                   const float* __restrict__ val, long long R, const long long* __restrict__ nrp,
                                   int* __restrict__ ncol, float* __restrict__ nval) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x) {
        const long long a = rp[i], len = rp[i + 1] - a, o = nrp[i], plen = nrp[i + 1] - o;
        for (long long k = 0; k < len; ++k) {
            ncol[o + k] = col[a + k];
            nval[o + k] = val[a + k];
        }
        for (long long k = len; k < plen; ++k) {
            ncol[o + k] = (int)i;
            nval[o + k] = 0.0f;
        }
    }
}

__global__ void fill_last_kernel(long long* rp, long long R, const long long* total) { rp[R] = *total; }

// ---------------------------------------------------------------- SpMV
// y[row] = sum val*x[col] with G threads per row (FP32 accumulation, a
// G-way strided partial sum per row reduced by shuffles), optional
// y += add_scale * add and FP64 accumulation of dot(pdot, y).
// Each lane first loads the column and value of up to K of its row's entries
// (coalesced), then issues all K gathers of x before it sums: the gathers,
// which wait on L2, are all in flight at once (the rest of a longer row
// follows in a loop). PF: the group pulls the columns and values of the row
// it takes two rows on into L2. Resident CTAs per SM are pinned (six at 40
// registers, five at 48 for the 10-entry variant): the gathers need the warps.
template <int G, int K, bool PF>
__global__ void __launch_bounds__(256, K >= 10 ? 5 : 6) spmv_kernel(const long long* __restrict__ rp, const int* __restrict__ col,
                                                   const float* __restrict__ val, const float* __restrict__ x,
                                                   float* __restrict__ y, long long rows, const float* __restrict__ add,
                                                   float add_scale, const float* __restrict__ pdot,
                                                   double* __restrict__ dot_acc, const int* __restrict__ done) {
    if (done && *done) return;
    __shared__ double red[8];
    const int lane = threadIdx.x % G;
    const long long gid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
    const long long stride = ((long long)gridDim.x * blockDim.x) / G;
    // the warp's first group: every lane of a warp runs the same number of
    // iterations (groups past the last row idle through them), so the
    // full-warp shuffles below always see all 32 lanes
    const long long gfirst = (blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31u)) / G;
    double local = 0.0;
    constexpr long long PFR = 2;  // rows ahead
    for (long long it = 0; gfirst + it * stride < rows; ++it) {
        const long long row = gid + it * stride;
        const bool active = row < rows;
        const long long a = active ? rp[row] : 0, b = active ? rp[row + 1] : 0;
        if (PF && active && row + PFR * stride < rows) {
            const long long na = rp[row + PFR * stride], nb = rp[row + PFR * stride + 1];
            const long long l0 = na >> 5, l1 = (nb + 31) >> 5;  // 32 four-byte entries per line
            for (long long l = l0 + lane; l < l1; l += G) {
                const long long e = l << 5;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(col + e));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(val + e));
            }
        }
        int cs[K];
        float vs[K], xs[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const long long e = a + lane + (long long)k * G;
            cs[k] = e < b ? __ldg(col + e) : 0;
            vs[k] = e < b ? __ldg(val + e) : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < K; ++k) xs[k] = (a + lane + (long long)k * G < b) ? __ldg(x + cs[k]) : 0.0f;
        float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
        for (int k = 0; k < K; k += 2) {
            s0 = fmaf(vs[k], xs[k], s0);
            if (k + 1 < K) s1 = fmaf(vs[k + 1], xs[k + 1], s1);
        }
        for (long long p = a + lane + (long long)K * G; p < b; p += G) s0 = fmaf(__ldg(val + p), __ldg(x + __ldg(col + p)), s0);
        float sum = s0 + s1;
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o, G);
        if (lane == 0 && active) {
            if (add) sum = fmaf(add_scale, add[row], sum);
            y[row] = sum;
            if (pdot) local += (double)pdot[row] * (double)sum;
        }
    }
    if (dot_acc) {
        // only the groups' first lanes hold row products: fold those of the
        // warp (none to fold for one group per warp), then the block's warps,
        // into one of the accumulator's CG_SLOTS addresses
        for (int o = 16; o >= G; o >>= 1) local += __shfl_xor_sync(FULL, local, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
            atomicAdd(dot_acc + blockIdx.x % CG_SLOTS, t);
        }
    }
}

template <int G, int K, bool PF>
int launch_spmv_g(const DevCsr& A, const float* x, float* y, const float* add, float add_scale, const float* pdot,
                  double* dot_acc, const int* done, cudaStream_t st) {
    // up to 64 CTAs of 256 threads per SM, the rest by the grid-stride loop
    // (measured on the 2M-ray matrix: 16 per SM 0.58 ms, 32 0.56, 64 0.54 for A x)
    const long long b = (A.rows * G + 255) / 256;
    const unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>(b, (long long)grid_cap() * 4));
    spmv_kernel<G, K, PF><<<blocks, 256, 0, st>>>(A.row_ptr, A.col, A.val, x, y, A.rows, add, add_scale, pdot, dot_acc,
                                                  done);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

// ---------------------------------------------------------------- vectors / CG
__global__ void f64_to_f32_kernel(const double* a, float* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void f32_to_f64_kernel(const float* a, double* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// Block sums of a and b added to acc_a / acc_b; slots > 1: into slot
// blockIdx % slots of each (the CG accumulators).
__device__ __forceinline__ void block_add2(double a, double b, double* acc_a, double* acc_b, int slots = 1) {
    __shared__ double ra[8], rb[8];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(FULL, a, o);
        b += __shfl_xor_sync(FULL, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        ra[threadIdx.x >> 5] = a;
        rb[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            ta += ra[w];
            tb += rb[w];
        }
        if (acc_a) atomicAdd(acc_a + blockIdx.x % slots, ta);
        if (acc_b) atomicAdd(acc_b + blockIdx.x % slots, tb);
    }
}

// r = b, z = M r, p = z, x = 0; acc rz = <r,z>, bb = <b,b>.
__global__ void cg_init_kernel(const float* __restrict__ b, const float* __restrict__ dinv, long long n,
                               float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
                               float* __restrict__ p, double* rz, double* bb) {
    double a = 0.0, c = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float bi = b[i];
        const float zi = dinv ? dinv[i] * bi : bi;
        x[i] = 0.0f;
        r[i] = bi;
        if (z) z[i] = zi;
        p[i] = zi;
        a += (double)bi * (double)zi;
        c += (double)bi * (double)bi;
    }
    block_add2(a, c, rz, bb, CG_SLOTS);
}

// x += alpha p, r -= alpha q, z = M r; acc rz_new = <r,z>, rr = <r,r>.
// alpha = rz_old / pq; |pq| < 1e-30 stops the solve (sparse_ops.cpp:37,88).
// The scalars are formed once per block (FP64 is a slow pipe on this GPU).
// skip_rz: <r, z> comes from the stencil preconditioner's kernel instead.
__global__ void cg_update_kernel(long long n, float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
                                 const float* __restrict__ p, const float* __restrict__ q,
                                 const float* __restrict__ dinv, CgScalars* sc, int k, int skip_rz) {
    __shared__ float s_alpha;
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
        int stop = sc->done;
        float alpha = 0.0f;
        if (!stop) {
            const double pq = cg_slot_sum(sc->acc[k % 3].pq);
            if (fabs(pq) < 1e-30) {
                stop = 1;
                if (blockIdx.x == 0) {
                    sc->done = 1;
                    sc->breakdown = 1;
                }
            } else {
                alpha = (float)(cg_slot_sum(sc->acc[(k + 2) % 3].rzn) / pq);
            }
        }
        s_alpha = alpha;
        s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    const float alpha = s_alpha;
    double a = 0.0, c = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        x[i] = fmaf(alpha, p[i], x[i]);
        const float ri = fmaf(-alpha, q[i], r[i]);
        r[i] = ri;
        const float zi = dinv ? dinv[i] * ri : ri;
        if (z) z[i] = zi;
        a += (double)ri * (double)zi;
        c += (double)ri * (double)ri;
    }
    block_add2(a, c, skip_rz ? nullptr : sc->acc[k % 3].rzn, sc->acc[k % 3].rr, CG_SLOTS);
}

// z = dinv r + S sum_a w_a (2 v - v(-e_a) - v(+e_a)), v = S r and 0 outside
// the grid (the weighted Dirichlet Laplacian between the two diagonal
// scalings: symmetric positive definite with dinv); acc += <r, z>; p = z when
// p is set (the first iteration).
__global__ void stencil_prec_kernel(long long n, const float* __restrict__ r, const float* __restrict__ dinv,
                                    const float* __restrict__ sq, int gx, int gy, int gz, float wx, float wy,
                                    float wz, float* __restrict__ z, float* __restrict__ p, double* acc,
                                    const int* done) {
    if (done && *done) return;
    const long long sy = gz, sx = (long long)gy * gz;
    double a = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(i % gz);
        const long long t = i / gz;
        const int iy = (int)(t % gy), ix = (int)(t / gy);
        const float si = sq[i], ri = r[i], vi = si * ri;
        auto v = [&](long long j) { return sq[j] * r[j]; };
        const float lz = 2.0f * vi - (iz > 0 ? v(i - 1) : 0.0f) - (iz < gz - 1 ? v(i + 1) : 0.0f);
        const float ly = 2.0f * vi - (iy > 0 ? v(i - sy) : 0.0f) - (iy < gy - 1 ? v(i + sy) : 0.0f);
        const float lx = 2.0f * vi - (ix > 0 ? v(i - sx) : 0.0f) - (ix < gx - 1 ? v(i + sx) : 0.0f);
        const float zi = fmaf(dinv[i], ri, si * fmaf(wx, lx, fmaf(wy, ly, wz * lz)));
        z[i] = zi;
        if (p) p[i] = zi;
        a += (double)ri * (double)zi;
    }
    block_add2(a, 0.0, acc, nullptr, CG_SLOTS);
}

// Convergence test after the update (sqrt(rr)/||b|| < tol) and
// p = z + beta p with beta = rz_new / rz_old; clears the accumulators of
// iteration k+1.
__global__ void cg_pupdate_kernel(long long n, float* __restrict__ p, const float* __restrict__ z, CgScalars* sc,
                                  int k, double tol) {
    __shared__ float s_beta;
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
        int stop = sc->done;
        float beta = 0.0f;
        if (!stop) {
            const double rel = sqrt(cg_slot_sum(sc->acc[k % 3].rr)) / sqrt(cg_slot_sum(sc->bb));
            if (blockIdx.x == 0) {
                sc->iters = k + 1;
                sc->rel = rel;
                CgAcc& nxt = sc->acc[(k + 1) % 3];
                for (int i = 0; i < CG_SLOTS; ++i) nxt.pq[i] = nxt.rr[i] = nxt.rzn[i] = 0.0;
            }
            if (rel < tol) {
                stop = 1;
                if (blockIdx.x == 0) sc->done = 1;
            } else {
                beta = (float)(cg_slot_sum(sc->acc[k % 3].rzn) / cg_slot_sum(sc->acc[(k + 2) % 3].rzn));
            }
        }
        s_beta = beta;
        s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    const float beta = s_beta;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = fmaf(beta, p[i], z[i]);
}

// Jacobi diagonal of sparse_ops.cpp:60-73: 1/A_ii from the first entry with
// col == row when |A_ii| > 1e-30, otherwise 1.
__global__ void jacobi_kernel(const long long* __restrict__ rp, const int* __restrict__ col,
                              const float* __restrict__ val, long long rows, float* __restrict__ dinv) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
        float d = 1.0f;
        for (long long p = rp[i]; p < rp[i + 1]; ++p)
            if (col[p] == i) {
                if (fabsf(val[p]) > 1e-30f) d = 1.0f / val[p];
                break;
            }
        dinv[i] = d;
    }
}

// diag of A^T A + lam I from the rows of A^T: 1 / (sum_k AT[j,k]^2 + lam).
__global__ void normal_jacobi_kernel(const long long* __restrict__ rp, const float* __restrict__ val, long long rows,
                                     double lam, float* __restrict__ dinv) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (long long p = rp[i]; p < rp[i + 1]; ++p) s += (double)val[p] * (double)val[p];
        dinv[i] = (float)(1.0 / (s + lam));
    }
}

__global__ void scale_kernel(float* v, long long n, float a) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] *= a;
}

__global__ void add_diag_kernel(const long long* __restrict__ rp, const int* __restrict__ col, float* __restrict__ val,
                                long long rows, float a) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x)
        for (long long p = rp[i]; p < rp[i + 1]; ++p)
            if (col[p] == i) {
                val[p] += a;
                break;
            }
}

__global__ void sumsq_kernel(const float* __restrict__ v, long long n, double* acc) {
    double a = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a += (double)v[i] * (double)v[i];
    block_add2(a, 0.0, acc, nullptr);
}

__global__ void dot64_kernel(const double* __restrict__ a, const double* __restrict__ b, long long n, double* acc) {
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    block_add2(s, 0.0, acc, nullptr);
}

__global__ void axpby_kernel(float* __restrict__ out, const float* __restrict__ a, const float* __restrict__ b,
                             float beta, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = a[i] - beta * b[i];
}

// 7-point stencil triplets of build_fd_stencil_7point (csr_matrix.cpp:74-116),
// emitted in the reference's per-row order, 7 slots per row (unused slots get
// an out-of-range row and are dropped by the builder).
__global__ void fd_triplets_kernel(const double* __restrict__ vel, long long nx, long long ny, long long nz, double idx2,
                                   double idy2, double idz2, double dt2, long long* __restrict__ tr,
                                   long long* __restrict__ tc, double* __restrict__ tv) {
    const long long n = nx * ny * nz;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        const long long ix = r / (ny * nz), rem = r % (ny * nz), iy = rem / nz, iz = rem % nz;
        const double v = vel[r];
        const double v2dt2 = v * v * dt2;
        const double diag = -2.0 * v2dt2 * (idx2 + idy2 + idz2) + 2.0;
        long long* rr = tr + 7 * r;
        long long* cc = tc + 7 * r;
        double* vv = tv + 7 * r;
        int k = 0;
        auto put = [&](bool ok, long long c, double val) {
            rr[k] = ok ? r : -1;
            cc[k] = ok ? c : 0;
            vv[k] = ok ? val : 0.0;
            ++k;
        };
        put(true, r, diag);
        put(ix > 0, r - ny * nz, v2dt2 * idx2);
        put(ix < nx - 1, r + ny * nz, v2dt2 * idx2);
        put(iy > 0, r - nz, v2dt2 * idy2);
        put(iy < ny - 1, r + nz, v2dt2 * idy2);
        put(iz > 0, r - 1, v2dt2 * idz2);
        put(iz < nz - 1, r + 1, v2dt2 * idz2);
    }
}

}  // namespace

// ---------------------------------------------------------------- builder (host side)

template <class TI, class TV>
int build_csr(long long rows, long long cols, long long n, const TI* r, const TI* c, const TV* v, bool pad,
              DevCsr* out, cudaStream_t st) {
    ST_CHECK(rows >= 0 && cols >= 0 && n >= 0, ST_ERR_ARG, "negative CSR extents");
    ST_CHECK(cols < (1ll << 31), ST_ERR_ARG, "columns must fit int32 indices");
    ST_CHECK(n < (1ll << 32), ST_ERR_ARG, "at most 2^32-1 triplets per build");
    const int cb = bits_for(cols);
    const int rb = bits_for(rows);  // rows itself (the drop marker) must be representable
    ST_CHECK(cb + rb <= 64, ST_ERR_ARG, "row/column index range too large");
    DeviceBuffers bufs;
    auto alloc = [&](size_t bytes) -> void* { return bufs.get(bytes); };
    ST_CUDA(cudaMalloc(&out->row_ptr, (size_t)(rows + 1) * sizeof(long long)));
    out->rows = rows;
    out->cols = cols;
    if (n == 0) {
        ST_CUDA(cudaMemsetAsync(out->row_ptr, 0, (size_t)(rows + 1) * sizeof(long long), st));
        out->nnz = 0;
        return ST_OK;
    }
    auto* keys = static_cast<unsigned long long*>(alloc((size_t)n * 8));
    auto* pay = static_cast<unsigned*>(alloc((size_t)n * 4));
    auto* keys2 = static_cast<unsigned long long*>(alloc((size_t)n * 8));
    auto* pay2 = static_cast<unsigned*>(alloc((size_t)n * 4));
    void* rtmp = alloc(radix_tmp_bytes(n));
    if (!keys || !pay || !keys2 || !pay2 || !rtmp) return bufs.fail();
    keys_kernel<TI><<<blocks_for(n), 256, 0, st>>>(r, c, n, rows, cols, cb, keys, pay);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_TRY(radix_sort_u64(keys, pay, keys2, pay2, n, cb + rb, rtmp, st));
    // reuse keys2 / pay2 storage for the head flags and unique indices
    auto* flag = reinterpret_cast<long long*>(keys2);
    auto* uidx = static_cast<long long*>(alloc((size_t)n * 8));
    auto* total = static_cast<long long*>(alloc(64));
    void* stmp = alloc(scan_tmp_bytes(n));
    if (!uidx || !total || !stmp) return bufs.fail();
    heads_kernel<<<blocks_for(n), 256, 0, st>>>(keys, n, rows, cb, flag);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_TRY(exclusive_scan_i64(flag, uidx, n, total, stmp, st));
    long long nnz = 0;
    ST_CUDA(cudaMemcpyAsync(&nnz, total, sizeof(long long), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaStreamSynchronize(st));
    out->nnz = nnz;
    ST_CUDA(cudaMalloc(&out->col, (size_t)std::max<long long>(nnz, 1) * sizeof(int)));
    ST_CUDA(cudaMalloc(&out->val, (size_t)std::max<long long>(nnz, 1) * sizeof(float)));
    auto* urow = static_cast<long long*>(alloc((size_t)std::max<long long>(nnz, 1) * 8));
    if (!urow) return bufs.fail();
    merge_kernel<TV><<<blocks_for(n), 256, 0, st>>>(keys, pay, n, cb, flag, uidx, v, out->col, out->val, urow);
    count_launch();
    ST_CUDA(cudaGetLastError());
    if (nnz == 0) {
        ST_CUDA(cudaMemsetAsync(out->row_ptr, 0, (size_t)(rows + 1) * sizeof(long long), st));
    } else {
        rowptr_kernel<<<blocks_for(nnz), 256, 0, st>>>(urow, nnz, rows, out->row_ptr);
        count_launch();
        ST_CUDA(cudaGetLastError());
    }
    if (pad && rows > 0) {
        int* trig = static_cast<int*>(alloc(64));
        if (!trig) return bufs.fail();
        ST_CUDA(cudaMemsetAsync(trig, 0, sizeof(int), st));
        pad_trigger_kernel<<<blocks_for(rows), 256, 0, st>>>(out->row_ptr, rows, trig);
        count_launch();
        int h = 0;
        ST_CUDA(cudaMemcpyAsync(&h, trig, sizeof(int), cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
        if (h) {
            ST_CHECK(rows <= cols, ST_ERR_ARG,
                     "pad-to-8 entries use col = row, out of range for %lld rows x %lld cols", rows, cols);
            auto* plen = static_cast<long long*>(alloc((size_t)(rows + 1) * 8));
            long long* nrp = nullptr;
            ST_CUDA(cudaMalloc(&nrp, (size_t)(rows + 1) * sizeof(long long)));
            if (!plen) return bufs.fail();
            pad_len_kernel<<<blocks_for(rows), 256, 0, st>>>(out->row_ptr, rows, plen);
            count_launch();
            ST_TRY(exclusive_scan_i64(plen, nrp, rows, total, stmp, st));
            fill_last_kernel<<<1, 1, 0, st>>>(nrp, rows, total);
            count_launch();
            long long pn = 0;
            ST_CUDA(cudaMemcpyAsync(&pn, total, sizeof(long long), cudaMemcpyDeviceToHost, st));
            ST_CUDA(cudaStreamSynchronize(st));
            int* ncol = nullptr;
            float* nval = nullptr;
            ST_CUDA(cudaMalloc(&ncol, (size_t)std::max<long long>(pn, 1) * sizeof(int)));
            ST_CUDA(cudaMalloc(&nval, (size_t)std::max<long long>(pn, 1) * sizeof(float)));
            pad_scatter_kernel<<<blocks_for(rows), 256, 0, st>>>(out->row_ptr, out->col, out->val, rows, nrp, ncol,
                                                                 nval);
            count_launch();
            ST_CUDA(cudaGetLastError());
            ST_CUDA(cudaStreamSynchronize(st));
            cudaFree(out->row_ptr);
            cudaFree(out->col);
            cudaFree(out->val);
            out->row_ptr = nrp;
            out->col = ncol;
            out->val = nval;
            out->nnz = pn;
        }
    }
    ST_CUDA(cudaStreamSynchronize(st));
    return ST_OK;
}

template int build_csr<long long, double>(long long, long long, long long, const long long*, const long long*,
                                          const double*, bool, DevCsr*, cudaStream_t);
template int build_csr<int, float>(long long, long long, long long, const int*, const int*, const float*, bool,
                                   DevCsr*, cudaStream_t);

// Transpose: rebuild from (col, row) keys of the existing entries.
__global__ void expand_rows_kernel(const long long* __restrict__ rp, long long rows, int* __restrict__ rowidx) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x)
        for (long long p = rp[i]; p < rp[i + 1]; ++p) rowidx[p] = (int)i;
}

int build_transpose(const DevCsr& A, DevCsr* T, cudaStream_t st) {
    ST_CHECK(A.rows < (1ll << 31), ST_ERR_ARG, "rows must fit int32 to transpose");
    int* rowidx = nullptr;
    ST_CUDA(cudaMalloc(&rowidx, (size_t)std::max<long long>(A.nnz, 1) * sizeof(int)));
    expand_rows_kernel<<<blocks_for(A.rows), 256, 0, st>>>(A.row_ptr, A.rows, rowidx);
    count_launch();
    ST_CUDA(cudaGetLastError());
    int rc = build_csr<int, float>(A.cols, A.rows, A.nnz, A.col, rowidx, A.val, false, T, st);
    cudaFree(rowidx);
    return rc;
}

int launch_spmv(const DevCsr& A, const float* x, float* y, const float* add, float add_scale, const float* pdot,
                double* dot_acc, const int* done, cudaStream_t st) {
    const double avg = A.rows > 0 ? (double)A.nnz / (double)A.rows : 0.0;
    // tuning override: SEISMIC_GB300_SPMV_G=<2|4|8|16|32> threads per row
    static const int forced = [] {
        const char* e = std::getenv("SEISMIC_GB300_SPMV_G");
        return e ? std::atoi(e) : 0;
    }();
    switch (forced) {
        case 32: return launch_spmv_g<32, 6, false>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
        case 16: return launch_spmv_g<16, 10, true>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
        case 8: return launch_spmv_g<8, 4, true>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
        case 4: return launch_spmv_g<4, 4, false>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
        default: break;
    }
    // measured on the 2M-ray matrix (180 entries per row) and its transpose (360): 16 threads per
    // row with 10 entries held per lane and the L2 prefetch 0.545 ms; the transpose with 32
    // threads, 6 entries per lane and no prefetch 0.599 ms (before the held entries: 0.66 / 0.80)
    if (avg >= 256) return launch_spmv_g<32, 6, false>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
    if (avg >= 24) return launch_spmv_g<16, 10, true>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
    if (avg >= 10) return launch_spmv_g<8, 4, true>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
    if (avg >= 5) return launch_spmv_g<4, 4, false>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
    return launch_spmv_g<2, 4, false>(A, x, y, add, add_scale, pdot, dot_acc, done, st);
}

int launch_f64_to_f32(const double* a, float* b, long long n, cudaStream_t st) {
    f64_to_f32_kernel<<<blocks_for(n), 256, 0, st>>>(a, b, n);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_f32_to_f64(const float* a, double* b, long long n, cudaStream_t st) {
    f32_to_f64_kernel<<<blocks_for(n), 256, 0, st>>>(a, b, n);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_jacobi(const DevCsr& A, float* dinv, cudaStream_t st) {
    jacobi_kernel<<<blocks_for(A.rows), 256, 0, st>>>(A.row_ptr, A.col, A.val, A.rows, dinv);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_normal_jacobi(const DevCsr& AT, double lam, float* dinv, cudaStream_t st) {
    normal_jacobi_kernel<<<blocks_for(AT.rows), 256, 0, st>>>(AT.row_ptr, AT.val, AT.rows, lam, dinv);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_scale(float* v, long long n, float a, cudaStream_t st) {
    scale_kernel<<<blocks_for(n), 256, 0, st>>>(v, n, a);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_add_diag(DevCsr& A, float a, cudaStream_t st) {
    add_diag_kernel<<<blocks_for(A.rows), 256, 0, st>>>(A.row_ptr, A.col, A.val, A.rows, a);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_sumsq(const float* v, long long n, double* acc, cudaStream_t st) {
    ST_CUDA(cudaMemsetAsync(acc, 0, sizeof(double), st));
    sumsq_kernel<<<blocks_for(n), 256, 0, st>>>(v, n, acc);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_dot64(const double* a, const double* b, long long n, double* acc, cudaStream_t st) {
    ST_CUDA(cudaMemsetAsync(acc, 0, sizeof(double), st));
    dot64_kernel<<<blocks_for(n), 256, 0, st>>>(a, b, n, acc);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

__global__ void sqrt_kernel(const float* __restrict__ a, float* __restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = sqrtf(a[i]);
}

int launch_sqrt(const float* a, float* out, long long n, cudaStream_t st) {
    sqrt_kernel<<<blocks_for(n), 256, 0, st>>>(a, out, n);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_residual(float* out, const float* b, const float* Ax, long long n, cudaStream_t st) {
    axpby_kernel<<<blocks_for(n), 256, 0, st>>>(out, b, Ax, 1.0f, n);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}
int launch_fd_triplets(const double* vel, long long nx, long long ny, long long nz, double idx2, double idy2,
                       double idz2, double dt2, long long* tr, long long* tc, double* tv, cudaStream_t st) {
    fd_triplets_kernel<<<blocks_for(nx * ny * nz), 256, 0, st>>>(vel, nx, ny, nz, idx2, idy2, idz2, dt2, tr, tc, tv);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

// ---------------------------------------------------------------- CG driver
int cg_loop(const CgProblem& P, CgWork& W, int k0, int max_iter, double tol, int check_every, CgResult* res,
            cudaStream_t st);

int run_cg(const CgProblem& P, CgWork& W, int max_iter, double tol, int check_every, CgResult* res,
           cudaStream_t st) {
    const long long n = P.n;
    ST_CUDA(cudaMemsetAsync(W.sc, 0, sizeof(CgScalars), st));
    // iteration -1 stores rz in acc[2].rzn
    // (stencil: p and <r, z> from the preconditioner kernel below)
    cg_init_kernel<<<cg_blocks(n), 256, 0, st>>>(P.b, P.sq ? nullptr : P.dinv, n, P.x, W.r,
                                                   P.dinv && !P.sq ? W.z : nullptr, W.p,
                                                   P.sq ? nullptr : W.sc->acc[2].rzn, W.sc->bb);
    count_launch();
    ST_CUDA(cudaGetLastError());
    if (P.sq) {
        stencil_prec_kernel<<<cg_blocks(n), 256, 0, st>>>(n, W.r, P.dinv, P.sq, P.gx, P.gy, P.gz, P.w[0], P.w[1],
                                                           P.w[2], W.z, W.p, W.sc->acc[2].rzn, nullptr);
        count_launch();
        ST_CUDA(cudaGetLastError());
    }
    CgScalars h{};
    ST_CUDA(cudaMemcpyAsync(&h, W.sc, sizeof(h), cudaMemcpyDeviceToHost, st));
    ST_CUDA(cudaStreamSynchronize(st));
    res->iters = 0;
    res->rel = 0.0;
    res->breakdown = 0;
    if (std::sqrt(cg_slot_sum(h.bb)) < 1e-30) return ST_OK;  // sparse_ops.cpp:22,83
    return cg_loop(P, W, 0, max_iter, tol, check_every, res, st);
}

int resume_cg(const CgProblem& P, CgWork& W, int max_iter, double tol, int check_every, CgResult* res,
              cudaStream_t st) {
    if (res->breakdown || res->iters == 0 || res->iters >= max_iter) return ST_OK;
    // the last iteration stopped before p = z + beta p: clear the stop and
    // run that update (a zero tolerance never stops it)
    const int k = res->iters;
    ST_CUDA(cudaMemsetAsync(&W.sc->done, 0, sizeof(int), st));
    cg_pupdate_kernel<<<cg_blocks(P.n), 256, 0, st>>>(P.n, W.p, P.dinv || P.sq ? W.z : W.r, W.sc, k - 1, 0.0);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return cg_loop(P, W, k, max_iter, tol, check_every, res, st);
}

// Iterations k0 .. of a solve whose state is in W (check_every iterations
// between host reads of the scalars).
int cg_loop(const CgProblem& P, CgWork& W, int k0, int max_iter, double tol, int check_every, CgResult* res,
            cudaStream_t st) {
    const long long n = P.n;
    CgScalars h{};
    const float* zp = P.dinv ? W.z : W.r;
    int k = k0;
    while (k < max_iter) {
        const int batch = std::min(check_every, max_iter - k);
        for (int j = 0; j < batch; ++j, ++k) {
            if (P.AT) {
                ST_TRY(launch_spmv(*P.A, W.p, W.t, nullptr, 0.0f, nullptr, nullptr, &W.sc->done, st));
                ST_TRY(launch_spmv(*P.AT, W.t, W.q, W.p, (float)P.lam, W.p, W.sc->acc[k % 3].pq, &W.sc->done, st));
            } else {
                ST_TRY(launch_spmv(*P.A, W.p, W.q, nullptr, 0.0f, W.p, W.sc->acc[k % 3].pq, &W.sc->done, st));
            }
            cg_update_kernel<<<cg_blocks(n), 256, 0, st>>>(n, P.x, W.r, P.dinv && !P.sq ? W.z : nullptr, W.p,
                                                             W.q, P.sq ? nullptr : P.dinv, W.sc, k, P.sq != nullptr);
            count_launch();
            if (P.sq) {
                stencil_prec_kernel<<<cg_blocks(n), 256, 0, st>>>(n, W.r, P.dinv, P.sq, P.gx, P.gy, P.gz, P.w[0],
                                                                   P.w[1], P.w[2], W.z, nullptr,
                                                                   W.sc->acc[k % 3].rzn, &W.sc->done);
                count_launch();
            }
            cg_pupdate_kernel<<<cg_blocks(n), 256, 0, st>>>(n, W.p, zp, W.sc, k, tol);
            count_launch();
            ST_CUDA(cudaGetLastError());
        }
        ST_CUDA(cudaMemcpyAsync(&h, W.sc, sizeof(h), cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
        if (h.done) break;
    }
    res->iters = h.iters;
    res->rel = h.rel;
    res->breakdown = h.breakdown;
    return ST_OK;
}

}  // namespace stg
