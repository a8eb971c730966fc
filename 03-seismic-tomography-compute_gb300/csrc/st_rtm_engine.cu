// C ABI of the seismic::RTMEngine face (rtm/rtm_engine.h:31-96): the
// zero-lag cross-correlation imaging condition on caller-provided
// halo-padded FP64 fields, with FP64 image / illumination / reflectivity
// accumulators on the device (the fused RTM path, st_rtm_shot, applies the
// same condition inside the adjoint kernel instead). Slice capture
// (extract_slices, :59-81) feeds the reference's visualisation stream and is
// not part of this path.
#include "st_common.cuh"

#include <algorithm>
#include <memory>

namespace {

// image += f*a, illum += f*f over the interior, non-finite inputs taken as 0
// (RTMEngine::apply_image_condition, rtm_engine.cpp:24-57). Products and sums
// are rounded separately, as the reference's plain C++ expressions.
__global__ void image_kernel(const double* __restrict__ fwd, const double* __restrict__ adj, long long nx, long long ny,
                             long long nz, long long nyh, long long nzh, int hw, double* __restrict__ image,
                             double* __restrict__ illum) {
    const long long n = nx * ny * nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long ix = k / (ny * nz), r = k % (ny * nz), iy = r / nz, iz = r % nz;
        const long long i = (ix + hw) * nyh * nzh + (iy + hw) * nzh + (iz + hw);
        const double f0 = fwd[i], a0 = adj[i];
        const double f = isfinite(f0) ? f0 : 0.0;
        const double a = isfinite(a0) ? a0 : 0.0;
        image[k] = __dadd_rn(image[k], __dmul_rn(f, a));
        illum[k] = __dadd_rn(illum[k], __dmul_rn(f, f));
    }
}

// The same condition on two FP32 fields of the solver's device layout
// (apply_rtm_step, wave_equation.cpp:598-619): values widened to FP64.
__global__ void image_device_kernel(const float* __restrict__ fwd, const float* __restrict__ adj, stg::Layout L,
                                    double* __restrict__ image, double* __restrict__ illum) {
    const long long n = L.nx * L.ny * L.nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long ix = k / (L.ny * L.nz), r = k % (L.ny * L.nz), iy = r / L.nz, iz = r % L.nz;
        const long long i = L.at(ix, iy, iz);
        const double f0 = fwd[i], a0 = adj[i];
        const double f = isfinite(f0) ? f0 : 0.0;
        const double a = isfinite(a0) ? a0 : 0.0;
        image[k] = __dadd_rn(image[k], __dmul_rn(f, a));
        illum[k] = __dadd_rn(illum[k], __dmul_rn(f, f));
    }
}

// Loads FP32 image / illumination accumulators into the FP64 ones.
__global__ void load_fp32_kernel(const float* __restrict__ image32, const float* __restrict__ illum32,
                                 double* __restrict__ image, double* __restrict__ illum, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        image[k] = image32[k];
        illum[k] = illum32[k];
    }
}

// RTMEngine::finalize_image (rtm_engine.cpp:170-182).
__global__ void finalize_kernel(const double* __restrict__ image, const double* __restrict__ illum,
                                double* __restrict__ refl, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        refl[k] = illum[k] > 1e-10 ? image[k] / illum[k] : 0.0;
}

unsigned blocks(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 16));
}

}  // namespace

struct st_rtm_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    long long nx = 0, ny = 0, nz = 0;
    double dx = 0, dy = 0, dz = 0;
    int hw = 1;
    double* image = nullptr;
    double* illum = nullptr;
    double* refl = nullptr;
    double* fwd = nullptr;  // staging of one padded field each
    double* adj = nullptr;
    size_t stage_cap = 0;
    bool own_stream = true;  // false: the stream of the solver that owns the engine
};

using namespace stg;

extern "C" {

// Replaces RTMEngine::RTMEngine (rtm_engine.cpp:8-16).
int st_rtm_engine_create(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, int halo_width,
                         int device, st_rtm_engine** out) {
    ST_CHECK(out && nx >= 0 && ny >= 0 && nz >= 0 && halo_width >= 0, ST_ERR_ARG, "bad arguments");
    ST_CUDA(cudaSetDevice(device));
    std::unique_ptr<st_rtm_engine> e(new st_rtm_engine());
    e->device = device;
    e->nx = nx;
    e->ny = ny;
    e->nz = nz;
    e->dx = dx;
    e->dy = dy;
    e->dz = dz;
    e->hw = halo_width;
    const size_t n = (size_t)std::max<long long>(nx * ny * nz, 1);
    ST_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    ST_CUDA(cudaMalloc(&e->image, n * 8));
    ST_CUDA(cudaMalloc(&e->illum, n * 8));
    ST_CUDA(cudaMalloc(&e->refl, n * 8));
    ST_CUDA(cudaMemset(e->image, 0, n * 8));
    ST_CUDA(cudaMemset(e->illum, 0, n * 8));
    ST_CUDA(cudaMemset(e->refl, 0, n * 8));
    *out = e.release();
    return ST_OK;
}

int st_rtm_engine_destroy(st_rtm_engine* e) {
    if (!e) return ST_OK;
    cudaSetDevice(e->device);
    cudaFree(e->image);
    cudaFree(e->illum);
    cudaFree(e->refl);
    cudaFree(e->fwd);
    cudaFree(e->adj);
    if (e->stream && e->own_stream) cudaStreamDestroy(e->stream);
    delete e;
    return ST_OK;
}

// Replaces apply_image_condition (rtm_engine.cpp:24-57): fields are host FP64
// halo-padded arrays with padded extents (nx+2hw) x ny_padded x nz_padded.
int st_rtm_engine_apply_image_condition(st_rtm_engine* e, const double* forward_wavefield,
                                        const double* adjoint_wavefield, int64_t ny_padded, int64_t nz_padded,
                                        int64_t step_idx) {
    ST_CHECK(e && forward_wavefield && adjoint_wavefield, ST_ERR_ARG, "null argument");
    ST_CHECK(ny_padded >= e->ny + 2 * e->hw && nz_padded >= e->nz + 2 * e->hw, ST_ERR_ARG,
             "padded extents smaller than the interior plus halo");
    (void)step_idx;
    ST_CUDA(cudaSetDevice(e->device));
    const size_t np = (size_t)((e->nx + 2 * e->hw) * ny_padded * nz_padded);
    if (e->stage_cap < np) {
        cudaFree(e->fwd);
        cudaFree(e->adj);
        e->fwd = e->adj = nullptr;
        e->stage_cap = 0;
        ST_CUDA(cudaMalloc(&e->fwd, np * 8));
        ST_CUDA(cudaMalloc(&e->adj, np * 8));
        e->stage_cap = np;
    }
    ST_CUDA(cudaMemcpyAsync(e->fwd, forward_wavefield, np * 8, cudaMemcpyHostToDevice, e->stream));
    ST_CUDA(cudaMemcpyAsync(e->adj, adjoint_wavefield, np * 8, cudaMemcpyHostToDevice, e->stream));
    image_kernel<<<blocks(e->nx * e->ny * e->nz), 256, 0, e->stream>>>(e->fwd, e->adj, e->nx, e->ny, e->nz,
                                                                        ny_padded, nz_padded, e->hw, e->image,
                                                                        e->illum);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaStreamSynchronize(e->stream));
    return ST_OK;
}

// Replaces finalize_image (rtm_engine.cpp:170-182).
int st_rtm_engine_finalize_image(st_rtm_engine* e) {
    ST_CHECK(e, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(e->device));
    const long long n = e->nx * e->ny * e->nz;
    finalize_kernel<<<blocks(n), 256, 0, e->stream>>>(e->image, e->illum, e->refl, n);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaStreamSynchronize(e->stream));
    return ST_OK;
}

// Replaces reset_image (rtm_engine.cpp:184-190).
int st_rtm_engine_reset_image(st_rtm_engine* e) {
    ST_CHECK(e, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(e->device));
    const size_t n = (size_t)std::max<long long>(e->nx * e->ny * e->nz, 1);
    ST_CUDA(cudaMemsetAsync(e->image, 0, n * 8, e->stream));
    ST_CUDA(cudaMemsetAsync(e->illum, 0, n * 8, e->stream));
    ST_CUDA(cudaMemsetAsync(e->refl, 0, n * 8, e->stream));
    ST_CUDA(cudaStreamSynchronize(e->stream));
    return ST_OK;
}

// result() (rtm_engine.h:52): image / illumination / reflectivity (any may be NULL).
int st_rtm_engine_result(st_rtm_engine* e, double* image, double* illumination, double* reflectivity) {
    ST_CHECK(e, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(e->device));
    const size_t n = (size_t)(e->nx * e->ny * e->nz);
    if (image) ST_CUDA(cudaMemcpyAsync(image, e->image, n * 8, cudaMemcpyDeviceToHost, e->stream));
    if (illumination) ST_CUDA(cudaMemcpyAsync(illumination, e->illum, n * 8, cudaMemcpyDeviceToHost, e->stream));
    if (reflectivity) ST_CUDA(cudaMemcpyAsync(reflectivity, e->refl, n * 8, cudaMemcpyDeviceToHost, e->stream));
    ST_CUDA(cudaStreamSynchronize(e->stream));
    return ST_OK;
}

}  // extern "C"

namespace stg {

// The engine of a solver's RTM driver: it runs on the solver's stream, so
// its work is ordered with the solver's steps.
int rtm_engine_create_on_stream(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, int device,
                                cudaStream_t stream, st_rtm_engine** out) {
    ST_TRY(st_rtm_engine_create(nx, ny, nz, dx, dy, dz, 1, device, out));
    st_rtm_engine* e = *out;
    cudaStreamDestroy(e->stream);
    e->stream = stream;
    e->own_stream = false;
    return ST_OK;
}

int rtm_engine_image_fields(st_rtm_engine* e, const float* fwd, const float* adj, const Layout& L) {
    ST_CHECK(e && fwd && adj && L.nx == e->nx && L.ny == e->ny && L.nz == e->nz, ST_ERR_ARG,
             "engine and field extents differ");
    image_device_kernel<<<blocks(e->nx * e->ny * e->nz), 256, 0, e->stream>>>(fwd, adj, L, e->image, e->illum);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int rtm_engine_load_fp32(st_rtm_engine* e, const float* image, const float* illum) {
    const long long n = e->nx * e->ny * e->nz;
    load_fp32_kernel<<<blocks(n), 256, 0, e->stream>>>(image, illum, e->image, e->illum, n);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

const double* rtm_engine_image(const st_rtm_engine* e) { return e->image; }

void rtm_engine_set_stream(st_rtm_engine* e, cudaStream_t stream) {
    if (!e->own_stream) e->stream = stream;
}

}  // namespace stg
