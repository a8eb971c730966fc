// Internal declarations of the sparse path (CSR build, SpMV, Krylov solves).
#pragma once

#include "st_common.cuh"

#include <vector>

namespace stg {

// Device CSR: int64 row pointers, int32 columns, FP32 values.
struct DevCsr {
    long long rows = 0, cols = 0, nnz = 0;
    long long* row_ptr = nullptr;
    int* col = nullptr;
    float* val = nullptr;
    void release() {
        cudaFree(row_ptr);
        cudaFree(col);
        cudaFree(val);
        row_ptr = nullptr;
        col = nullptr;
        val = nullptr;
    }
};

// Scratch allocations freed together (kernels using them must have finished).
class DeviceBuffers {
   public:
    ~DeviceBuffers() {
        for (void* p : ptrs_) cudaFree(p);
    }
    void* get(size_t bytes) {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
            cudaGetLastError();
            failed_bytes_ = bytes;
            return nullptr;
        }
        ptrs_.push_back(p);
        return p;
    }
    int fail() {
        set_error("device allocation of %zu bytes failed", failed_bytes_);
        return ST_ERR_ALLOC;
    }

   private:
    std::vector<void*> ptrs_;
    size_t failed_bytes_ = 0;
};

// FP64 accumulators of one CG iteration (three rotating sets). Each is
// spread over CG_SLOTS addresses (a block adds into slot blockIdx % CG_SLOTS)
// so that the blocks' atomics do not all queue on one address; readers sum
// the slots.
constexpr int CG_SLOTS = 8;
struct CgAcc {
    double pq[CG_SLOTS];   // <p, A p>
    double rr[CG_SLOTS];   // <r, r> after the update
    double rzn[CG_SLOTS];  // <r, z> after the update
};

struct CgScalars {
    CgAcc acc[3];
    double bb[CG_SLOTS];  // <b, b>
    double rel;           // sqrt(rr)/||b|| of the last iteration
    int iters;
    int done;
    int breakdown;
    int pad_;
};

inline __host__ __device__ double cg_slot_sum(const double* s) {
    double t = 0.0;
    for (int i = 0; i < CG_SLOTS; ++i) t += s[i];
    return t;
}

// Operator and preconditioner of one solve: A (square) or A^T A + lam I
// (A rectangular, AT its explicit transpose); dinv = Jacobi diagonal or null.
struct CgProblem {
    const DevCsr* A = nullptr;
    const DevCsr* AT = nullptr;
    double lam = 0.0;
    long long n = 0;
    const float* b = nullptr;
    float* x = nullptr;
    const float* dinv = nullptr;
    // stencil preconditioner M r = dinv r + S K (S r) (S = sqrt(dinv), K the
    // weighted Dirichlet Laplacian of an nx x ny x nz grid, x slowest) when
    // sq is set; dinv must be set too
    const float* sq = nullptr;
    int gx = 0, gy = 0, gz = 0;
    float w[3] = {0.0f, 0.0f, 0.0f};
};

struct CgWork {
    float *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *t = nullptr;
    CgScalars* sc = nullptr;
};

struct CgResult {
    int iters = 0;
    double rel = 0.0;
    int breakdown = 0;
};

template <class TI, class TV>
int build_csr(long long rows, long long cols, long long n, const TI* r, const TI* c, const TV* v, bool pad,
              DevCsr* out, cudaStream_t st);
int build_transpose(const DevCsr& A, DevCsr* T, cudaStream_t st);
// Straight-ray path-length matrix (st_rays.cu): d_ends = device [nrays][6]
// endpoints in cell units; total_nnz (may be null) receives the entry count.
int build_ray_csr(long long nrays, const double* d_ends, int nx, int ny, int nz, double h, DevCsr* out,
                  long long* total_nnz, cudaStream_t st);
// Sampled-ray matrix of a pick set (st_sampled_rays.cu): rows = picks,
// columns = cells, duplicates (samples of one pick in one cell) summed.
int build_sampled_ray_csr(const st_ray_picks* p, DevCsr* out, long long* nnz, cudaStream_t st);
int launch_spmv(const DevCsr& A, const float* x, float* y, const float* add, float add_scale, const float* pdot,
                double* dot_acc, const int* done, cudaStream_t st);
int launch_f64_to_f32(const double* a, float* b, long long n, cudaStream_t st);
int launch_f32_to_f64(const float* a, double* b, long long n, cudaStream_t st);
int launch_jacobi(const DevCsr& A, float* dinv, cudaStream_t st);
int launch_normal_jacobi(const DevCsr& AT, double lam, float* dinv, cudaStream_t st);
int launch_scale(float* v, long long n, float a, cudaStream_t st);
int launch_add_diag(DevCsr& A, float a, cudaStream_t st);
int launch_sumsq(const float* v, long long n, double* acc, cudaStream_t st);
int launch_residual(float* out, const float* b, const float* Ax, long long n, cudaStream_t st);
int launch_sqrt(const float* a, float* out, long long n, cudaStream_t st);
int launch_dot64(const double* a, const double* b, long long n, double* acc, cudaStream_t st);
int launch_fd_triplets(const double* vel, long long nx, long long ny, long long nz, double idx2, double idy2,
                       double idz2, double dt2, long long* tr, long long* tc, double* tv, cudaStream_t st);
int run_cg(const CgProblem& P, CgWork& W, int max_iter, double tol, int check_every, CgResult* res, cudaStream_t st);
// Continues a solve that run_cg stopped at tolerance (state in W, res from that
// call) down to the tighter recurrence tolerance tol, up to max_iter in all.
int resume_cg(const CgProblem& P, CgWork& W, int max_iter, double tol, int check_every, CgResult* res,
              cudaStream_t st);

// Flexible CG on (A^T A + lam I) x = b (st_fcg.cu); pc = the learned network
// (null: Jacobi with dinv). Work vectors r, z, p, q, ax of A.cols floats, t of
// A.rows floats, acc two doubles.
struct FcgScalars {
    double pq, pr, rr, zr, zq, jq;
};
int run_fcg(const DevCsr& A, const DevCsr& AT, double lam, const float* b, float* x, const float* dinv,
            st_pcnet* pc, int max_iter, double tol, float* r, float* z, float* p, float* q, float* ax, float* t,
            FcgScalars* sc, double* acc, cudaStream_t st, int* iters, double* true_rel);
// Unknowns of a preconditioner network (st_precond.cu).
long long pcnet_points(const st_pcnet* p);

}  // namespace stg
