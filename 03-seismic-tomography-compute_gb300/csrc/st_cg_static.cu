// CG on a square system without any device allocation.
//
// st_cg_device allocates its work vectors (r, z, p, A p, the Jacobi diagonal
// and the FP64 scalars) with cudaMalloc on every call. Some callers cannot
// allow that: services that reserve the whole device memory for their own
// pool at start-up, plugin hosts that forbid allocation once initialised,
// and real-time loops that must not pay an allocator's latency or risk an
// out-of-memory failure mid-run. st_cg_device_static runs the same solver
// with its scratch in one file-scope __device__ array of fixed size, which
// every GPU that loads this library holds until the process exits.
//
// Limit: systems of at most ST_CG_STATIC_MAX_N = 1,048,576 unknowns (5
// FP32 vectors = 20 MiB, plus 256 bytes of FP64 scalars).
#include "st_sparse.cuh"

#include <mutex>

// st_csr is defined in st_csr_capi.cu; this file only needs its matrix.
struct st_csr;

namespace stg {
const DevCsr* csr_matrix_of(const st_csr* m, int* device, cudaStream_t* stream);
}

namespace {

constexpr long long kMaxN = ST_CG_STATIC_MAX_N;

// Five work vectors (r, z, p, q = A p, Jacobi diagonal) of kMaxN floats each,
// followed by the FP64 scalar block. Shared by every call on a device.
constexpr int kTail = 256;
static __device__ __align__(256) float g_cg_scratch[5 * kMaxN + kTail];
static_assert(sizeof(stg::CgScalars) <= kTail * sizeof(float), "CG scalar block does not fit the scratch tail");

std::mutex g_mu;
float* g_scratch_ptr[64] = {nullptr};  // device address of g_cg_scratch, per device

// The symbol's device address, looked up once per device with that device
// current (host code cannot use &g_cg_scratch: on the host it names a
// host-side stand-in, not device memory).
int scratch_for(int device, float** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    ST_CHECK(device >= 0 && device < 64, ST_ERR_ARG, "device %d out of range", device);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_cg_scratch);
        if (e != cudaSuccess || !p) {
            stg::set_error("cudaGetSymbolAddress of the CG scratch failed on device %d: %s", device,
                           cudaGetErrorString(e));
            return ST_ERR_CUDA;
        }
        g_scratch_ptr[device] = static_cast<float*>(p);
    }
    *out = g_scratch_ptr[device];
    return ST_OK;
}

}  // namespace

using namespace stg;

extern "C" int st_cg_device_static(st_csr* m, const float* b, float* x, int max_iter, double tol, int jacobi,
                                   int* iters, double* final_rel) {
    ST_CHECK(m && b && x, ST_ERR_ARG, "null argument");
    int device = 0;
    cudaStream_t st = nullptr;
    const DevCsr* A = csr_matrix_of(m, &device, &st);
    ST_CHECK(A->rows == A->cols, ST_ERR_ARG, "CG needs a square matrix (%lld x %lld)", A->rows, A->cols);
    const long long n = A->rows;
    ST_CHECK(n <= kMaxN, ST_ERR_ARG,
             "st_cg_device_static handles at most %lld unknowns (got %lld); use st_cg_device for larger systems",
             kMaxN, n);
    ST_CUDA(cudaSetDevice(device));
    float* base = nullptr;
    ST_TRY(scratch_for(device, &base));
    CgWork W;
    W.r = base;
    W.z = base + kMaxN;
    W.p = base + 2 * kMaxN;
    W.q = base + 3 * kMaxN;
    float* dinv = jacobi ? base + 4 * kMaxN : nullptr;
    W.sc = reinterpret_cast<CgScalars*>(base + 5 * kMaxN);  // run_cg zeroes it before use
    if (jacobi) ST_TRY(launch_jacobi(*A, dinv, st));
    CgProblem P;
    P.A = A;
    P.n = n;
    P.b = b;
    P.x = x;
    P.dinv = dinv;
    CgResult R;
    ST_TRY(run_cg(P, W, max_iter, tol, 16, &R, st));
    ST_CUDA(cudaStreamSynchronize(st));
    if (iters) *iters = R.iters;
    if (final_rel) *final_rel = R.rel;
    return ST_OK;
}
