// CUDA-core layers of the learned CG preconditioner (the 32 -> 32 channel
// layers run on the tensor cores, st_conv.cu).
//
// The network maps a residual r of the damped tomography normal equations
// on an nx x ny x nz cell grid (compact, x slowest) to a correction
//     z = dinv * r + s_out * N(s_in * r, s_in * dinv * r),
//     N = C_out o (relu(conv_K(h) + h))^K o relu(C_in),
// with dinv the Jacobi diagonal, s_in = 1 / rms(r) and s_out = rms(r) *
// mean(dinv); N has no biases, so z scales with r. C_in: 2 -> 32 channels,
// C_out: 32 -> 1, both 3x3x3 with zero padding. Activations h are padded
// channels-last BF16 volumes ([(nx+2)(ny+2)(nz+2)][32], zero border).
//
// Weight layouts (FP32 masters): C_in [32][2][27], C_out [32][27], conv_k
// [32][32][27] (out, in, tap = (kd*3 + kh)*3 + kw).
#include "st_common.cuh"

#include <algorithm>

namespace stg {
namespace {

constexpr int CH = 32;
constexpr int NTAP = 27;

struct Vol {
    int nx, ny, nz;
    __host__ __device__ long long pad_row(int x, int y, int z) const {  // padded row of interior (x, y, z)
        return ((long long)(x + 1) * (ny + 2) + (y + 1)) * (nz + 2) + (z + 1);
    }
    __host__ __device__ long long n() const { return (long long)nx * ny * nz; }
};

__device__ __forceinline__ void decode(long long i, const Vol& v, int& x, int& y, int& z) {
    z = (int)(i % v.nz);
    const long long t = i / v.nz;
    y = (int)(t % v.ny);
    x = (int)(t / v.ny);
}

__device__ __forceinline__ void load_row32(const __nv_bfloat16* p, float f[CH]) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint4 u = q[j];
        const __nv_bfloat162* b = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 t = __bfloat1622float2(b[e]);
            f[8 * j + 2 * e] = t.x;
            f[8 * j + 2 * e + 1] = t.y;
        }
    }
}

__device__ __forceinline__ void store_row32(__nv_bfloat16* p, const float f[CH]) {
    uint4* q = reinterpret_cast<uint4*>(p);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint4 u;
        __nv_bfloat162* b = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
        for (int e = 0; e < 4; ++e) b[e] = __floats2bfloat162_rn(f[8 * j + 2 * e], f[8 * j + 2 * e + 1]);
        q[j] = u;
    }
}

// h0 = relu(C_in([s r, s dinv r])) into the padded layout (interior rows only;
// the border stays as allocated, zero).
__global__ void in_conv_kernel(const float* __restrict__ r, const float* __restrict__ dinv, const float* scale,
                               const float* __restrict__ w, Vol v, __nv_bfloat16* __restrict__ h) {
    __shared__ float ws[CH * 2 * NTAP];
    for (int i = threadIdx.x; i < CH * 2 * NTAP; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    const float s = *scale;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n(); i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        decode(i, v, x, y, z);
        float acc[CH];
#pragma unroll
        for (int c = 0; c < CH; ++c) acc[c] = 0.0f;
        for (int tap = 0; tap < NTAP; ++tap) {
            const int xx = x + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, zz = z + tap % 3 - 1;
            if (xx < 0 || xx >= v.nx || yy < 0 || yy >= v.ny || zz < 0 || zz >= v.nz) continue;
            const long long j = ((long long)xx * v.ny + yy) * v.nz + zz;
            const float a = s * r[j], b = a * dinv[j];
#pragma unroll
            for (int c = 0; c < CH; ++c) acc[c] = fmaf(ws[(c * 2) * NTAP + tap], a, fmaf(ws[(c * 2 + 1) * NTAP + tap], b, acc[c]));
        }
#pragma unroll
        for (int c = 0; c < CH; ++c) acc[c] = fmaxf(acc[c], 0.0f);
        store_row32(h + v.pad_row(x, y, z) * CH, acc);
    }
}

// dW_in[c][k][tap] += sum_v g[v][c] * in_k[v + s_tap]; one block per tap and
// slab of voxels, block-reduced, one atomic per weight per block.
__global__ void in_conv_wgrad_kernel(const float* __restrict__ r, const float* __restrict__ dinv, const float* scale,
                                     const __nv_bfloat16* __restrict__ g, Vol v, float* __restrict__ dw) {
    const int tap = blockIdx.y;
    const int dx = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dz = tap % 3 - 1;
    const float s = *scale;
    float acc[2 * CH];
#pragma unroll
    for (int c = 0; c < 2 * CH; ++c) acc[c] = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n(); i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        decode(i, v, x, y, z);
        const int xx = x + dx, yy = y + dy, zz = z + dz;
        if (xx < 0 || xx >= v.nx || yy < 0 || yy >= v.ny || zz < 0 || zz >= v.nz) continue;
        const long long j = ((long long)xx * v.ny + yy) * v.nz + zz;
        const float a = s * r[j], b = a * dinv[j];
        float gg[CH];
        load_row32(g + v.pad_row(x, y, z) * CH, gg);
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            acc[2 * c] = fmaf(gg[c], a, acc[2 * c]);
            acc[2 * c + 1] = fmaf(gg[c], b, acc[2 * c + 1]);
        }
    }
    __shared__ float red[2 * CH][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 2 * CH; ++c) {
        float t = acc[c];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[c][warp] = t;
    }
    __syncthreads();
    if (threadIdx.x < 2 * CH) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        atomicAdd(&dw[threadIdx.x * NTAP + tap], t);  // [c][k] flattened as c*2+k, times NTAP, plus tap
    }
}

// zhat = C_out(h); z = dinv * r + s_out * zhat (zhat kept for training).
__global__ void out_conv_kernel(const __nv_bfloat16* __restrict__ h, const float* __restrict__ w, Vol v,
                                const float* __restrict__ r, const float* __restrict__ dinv, const float* s_out,
                                float* __restrict__ zhat, float* __restrict__ z) {
    __shared__ float ws[CH * NTAP];
    for (int i = threadIdx.x; i < CH * NTAP; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    const float so = s_out ? *s_out : 0.0f;
    const int W2 = v.nz + 2, P2 = (v.ny + 2) * W2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n(); i += (long long)gridDim.x * blockDim.x) {
        int x, y, zz;
        decode(i, v, x, y, zz);
        const long long q = v.pad_row(x, y, zz);
        float acc = 0.0f;
        for (int tap = 0; tap < NTAP; ++tap) {
            const long long qq = q + (long long)(tap / 9 - 1) * P2 + ((tap / 3) % 3 - 1) * W2 + (tap % 3 - 1);
            float f[CH];
            load_row32(h + qq * CH, f);  // the zero border supplies the padding
#pragma unroll
            for (int c = 0; c < CH; ++c) acc = fmaf(ws[c * NTAP + tap], f[c], acc);
        }
        if (zhat) zhat[i] = acc;
        if (z) z[i] = fmaf(so, acc, dinv[i] * r[i]);
    }
}

// Backward of C_out: dh[v][c] = sum_tap w[c][tap] * dzhat[v - s_tap] (BF16,
// interior rows), and dW_out[c][tap] += sum_v dzhat[v] * h[v + s_tap][c].
__global__ void out_conv_dgrad_kernel(const float* __restrict__ dz, const float* __restrict__ w, Vol v,
                                      __nv_bfloat16* __restrict__ dh) {
    __shared__ float ws[CH * NTAP];
    for (int i = threadIdx.x; i < CH * NTAP; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n(); i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        decode(i, v, x, y, z);
        float acc[CH];
#pragma unroll
        for (int c = 0; c < CH; ++c) acc[c] = 0.0f;
        for (int tap = 0; tap < NTAP; ++tap) {
            const int xx = x - (tap / 9 - 1), yy = y - ((tap / 3) % 3 - 1), zz = z - (tap % 3 - 1);
            if (xx < 0 || xx >= v.nx || yy < 0 || yy >= v.ny || zz < 0 || zz >= v.nz) continue;
            const float g = dz[((long long)xx * v.ny + yy) * v.nz + zz];
#pragma unroll
            for (int c = 0; c < CH; ++c) acc[c] = fmaf(ws[c * NTAP + tap], g, acc[c]);
        }
        store_row32(dh + v.pad_row(x, y, z) * CH, acc);
    }
}

__global__ void out_conv_wgrad_kernel(const float* __restrict__ dz, const __nv_bfloat16* __restrict__ h, Vol v,
                                      float* __restrict__ dw) {
    const int tap = blockIdx.y;
    const int W2 = v.nz + 2, P2 = (v.ny + 2) * W2;
    const long long shift = (long long)(tap / 9 - 1) * P2 + ((tap / 3) % 3 - 1) * W2 + (tap % 3 - 1);
    float acc[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) acc[c] = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n(); i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        decode(i, v, x, y, z);
        const float g = dz[i];
        float f[CH];
        load_row32(h + (v.pad_row(x, y, z) + shift) * CH, f);
#pragma unroll
        for (int c = 0; c < CH; ++c) acc[c] = fmaf(g, f[c], acc[c]);
    }
    __shared__ float red[CH][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
        float t = acc[c];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[c][warp] = t;
    }
    __syncthreads();
    if (threadIdx.x < CH) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        atomicAdd(&dw[threadIdx.x * NTAP + tap], t);
    }
}

// g = dh * [h > 0] over interior rows (BF16, padded layout).
__global__ void relu_mask_kernel(const __nv_bfloat16* __restrict__ dh, const __nv_bfloat16* __restrict__ h, Vol v,
                                 __nv_bfloat16* __restrict__ g) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < v.n(); i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        decode(i, v, x, y, z);
        const long long q = v.pad_row(x, y, z) * CH;
        float a[CH], b[CH];
        load_row32(dh + q, a);
        load_row32(h + q, b);
#pragma unroll
        for (int c = 0; c < CH; ++c) a[c] = b[c] > 0.0f ? a[c] : 0.0f;
        store_row32(g + q, a);
    }
}

// acc[0] += sum r^2, acc[1] += sum dinv (multi-block, FP64 atomics).
__global__ void pc_sums_kernel(const float* __restrict__ r, const float* __restrict__ dinv, long long n, double* acc) {
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        a += (double)r[i] * (double)r[i];
        b += (double)dinv[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __shared__ double ra[8], rb[8];
    if ((threadIdx.x & 31) == 0) {
        ra[threadIdx.x >> 5] = a;
        rb[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += ra[w];
            b += rb[w];
        }
        atomicAdd(acc, a);
        atomicAdd(acc + 1, b);
    }
}

// s[0] = 1 / rms(r), s[1] = rms(r) * mean(dinv)
__global__ void pc_finalize_kernel(const double* acc, long long n, float* s) {
    const double rms = sqrt(acc[0] / (double)n);
    s[0] = rms > 0.0 ? (float)(1.0 / rms) : 0.0f;
    s[1] = (float)(rms * (acc[1] / (double)n));
}

// a = s_in * sqrt(dinv) * r
__global__ void pc_scale_in_kernel(const float* __restrict__ r, const float* __restrict__ dinv, const float* s,
                                   long long n, float* __restrict__ a) {
    const float si = s[0];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] = si * sqrtf(dinv[i]) * r[i];
}

// z = dinv * r + (1 / s_in) * sqrt(dinv) * y
__global__ void pc_combine_kernel(const float* __restrict__ y, const float* __restrict__ r,
                                  const float* __restrict__ dinv, const float* s, long long n, float* __restrict__ z) {
    const float si = s[0];
    const float inv = si > 0.0f ? 1.0f / si : 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        z[i] = fmaf(inv * sqrtf(dinv[i]), y[i], dinv[i] * r[i]);
}

unsigned grid_for(long long n, int cap = 152 * 16) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, cap));
}

}  // namespace
}  // namespace stg

using namespace stg;

extern "C" {

int st_pc_in_conv(const float* r, const float* dinv, const float* scale, const float* w, void* h, int64_t nx,
                  int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(r && dinv && scale && w && h, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    in_conv_kernel<<<grid_for(v.n()), 256, 0, (cudaStream_t)stream>>>(r, dinv, scale, w, v,
                                                                      static_cast<__nv_bfloat16*>(h));
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_in_conv_wgrad(const float* r, const float* dinv, const float* scale, const void* g, float* dw, int64_t nx,
                        int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(r && dinv && scale && g && dw, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    in_conv_wgrad_kernel<<<dim3(grid_for(v.n(), 64), NTAP), 256, 0, (cudaStream_t)stream>>>(
        r, dinv, scale, static_cast<const __nv_bfloat16*>(g), v, dw);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_out_conv(const void* h, const float* w, const float* r, const float* dinv, const float* s_out, float* zhat,
                   float* z, int64_t nx, int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(h && w && (!z || (r && dinv && s_out)), ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    out_conv_kernel<<<grid_for(v.n()), 256, 0, (cudaStream_t)stream>>>(static_cast<const __nv_bfloat16*>(h), w, v, r,
                                                                       dinv, s_out, zhat, z);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_out_conv_bwd(const float* dzhat, const void* h, const float* w, void* dh, float* dw, int64_t nx, int64_t ny,
                       int64_t nz, void* stream) {
    ST_CHECK(dzhat && h && w && dh && dw, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    cudaStream_t st = (cudaStream_t)stream;
    out_conv_dgrad_kernel<<<grid_for(v.n()), 256, 0, st>>>(dzhat, w, v, static_cast<__nv_bfloat16*>(dh));
    count_launch();
    out_conv_wgrad_kernel<<<dim3(grid_for(v.n(), 64), NTAP), 256, 0, st>>>(dzhat, static_cast<const __nv_bfloat16*>(h),
                                                                            v, dw);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_relu_mask(const void* dh, const void* h, void* g, int64_t nx, int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(dh && h && g, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    relu_mask_kernel<<<grid_for(v.n()), 256, 0, (cudaStream_t)stream>>>(static_cast<const __nv_bfloat16*>(dh),
                                                                        static_cast<const __nv_bfloat16*>(h), v,
                                                                        static_cast<__nv_bfloat16*>(g));
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_scales(const float* r, const float* dinv, double* acc, float* scales, int64_t n, void* stream) {
    ST_CHECK(r && dinv && acc && scales, ST_ERR_ARG, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    ST_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), st));
    pc_sums_kernel<<<grid_for(n, 152 * 4), 256, 0, st>>>(r, dinv, n, acc);
    count_launch();
    pc_finalize_kernel<<<1, 1, 0, st>>>(acc, n, scales);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_scale_in(const float* r, const float* dinv, const float* scales, float* a, int64_t n, void* stream) {
    ST_CHECK(r && dinv && scales && a, ST_ERR_ARG, "null argument");
    pc_scale_in_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(r, dinv, scales, n, a);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_combine(const float* y, const float* r, const float* dinv, const float* scales, float* z, int64_t n,
                  void* stream) {
    ST_CHECK(y && r && dinv && scales && z, ST_ERR_ARG, "null argument");
    pc_combine_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(y, r, dinv, scales, n, z);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_tconv1(const float* a, const float* w, void* h, int64_t nx, int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(a && w && h, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    out_conv_dgrad_kernel<<<grid_for(v.n()), 256, 0, (cudaStream_t)stream>>>(a, w, v, static_cast<__nv_bfloat16*>(h));
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_pc_conv1_wgrad(const float* dz, const void* h, float* dw, int64_t nx, int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(dz && h && dw, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    out_conv_wgrad_kernel<<<dim3(grid_for(v.n(), 64), NTAP), 256, 0, (cudaStream_t)stream>>>(
        dz, static_cast<const __nv_bfloat16*>(h), v, dw);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- network handle
// The trained preconditioner as one native object (weights packed once,
// activations allocated once), applied by st_pcnet_apply inside the native
// flexible CG. It is the symmetric positive (semi)definite form
//     z = D r + S G^T G S r,   D = diag(dinv), S = sqrt(D),
//     G = (I + conv_K) ... (I + conv_1) C^T,   C^T: 1 -> 32 channels,
// so G^T = C (I + conv_1^T) ... (I + conv_K^T): the tensor-core kernel with
// the transposed packing and the residual added. The input is scaled by
// 1 / rms(r) and the output back, which keeps z linear in r.

struct st_pcnet {
    int device = 0;
    int nx = 0, ny = 0, nz = 0, layers = 0;
    float* w_c = nullptr;      // C: [32][27]
    void* packed = nullptr;    // layers x 55,296 bytes (conv_k)
    void* packed_t = nullptr;  // layers x 55,296 bytes (conv_k^T)
    void* u = nullptr;         // two padded BF16 volumes (ping-pong)
    float* a = nullptr;        // scaled input / output, n floats
    double* acc = nullptr;
    float* scales = nullptr;
    size_t vol_bytes = 0;
};

namespace stg {
long long pcnet_points(const st_pcnet* p) { return (long long)p->nx * p->ny * p->nz; }
}  // namespace stg

extern "C" {

int st_pcnet_create(int64_t nx, int64_t ny, int64_t nz, int layers, int device, st_pcnet** out) {
    ST_CHECK(out && nx > 0 && ny > 0 && nz > 0 && layers >= 0 && layers <= 64, ST_ERR_ARG, "bad network shape");
    ST_CUDA(cudaSetDevice(device));
    st_pcnet* p = new st_pcnet();
    p->device = device;
    p->nx = (int)nx;
    p->ny = (int)ny;
    p->nz = (int)nz;
    p->layers = layers;
    p->vol_bytes = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2) * CH * 2;
    const size_t wb = (size_t)std::max(layers, 1) * NTAP * CH * CH * 2;
    const size_t n = (size_t)(nx * ny * nz);
    const bool ok = cudaMalloc(&p->w_c, CH * NTAP * 4) == cudaSuccess && cudaMalloc(&p->packed, wb) == cudaSuccess &&
                    cudaMalloc(&p->packed_t, wb) == cudaSuccess &&
                    cudaMalloc(&p->u, 2 * p->vol_bytes) == cudaSuccess &&
                    cudaMalloc(&p->a, n * sizeof(float)) == cudaSuccess &&
                    cudaMalloc(&p->acc, 2 * sizeof(double)) == cudaSuccess &&
                    cudaMalloc(&p->scales, 2 * sizeof(float)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cudaFree(p->w_c);
        cudaFree(p->packed);
        cudaFree(p->packed_t);
        cudaFree(p->u);
        cudaFree(p->a);
        cudaFree(p->acc);
        cudaFree(p->scales);
        delete p;
        set_error("device allocation for the preconditioner network failed");
        return ST_ERR_ALLOC;
    }
    ST_CUDA(cudaMemset(p->u, 0, 2 * p->vol_bytes));
    ST_CUDA(cudaMemset(p->w_c, 0, CH * NTAP * 4));
    ST_CUDA(cudaMemset(p->packed, 0, wb));
    ST_CUDA(cudaMemset(p->packed_t, 0, wb));
    *out = p;
    return ST_OK;
}

int st_pcnet_destroy(st_pcnet* p) {
    if (!p) return ST_OK;
    cudaSetDevice(p->device);
    cudaDeviceSynchronize();
    cudaFree(p->w_c);
    cudaFree(p->packed);
    cudaFree(p->packed_t);
    cudaFree(p->u);
    cudaFree(p->a);
    cudaFree(p->acc);
    cudaFree(p->scales);
    delete p;
    return ST_OK;
}

// w_c: device FP32 [32][27]; w_k: `layers` consecutive [32][32][27] FP32 blocks.
int st_pcnet_set_weights(st_pcnet* p, const float* w_c, const float* w_k) {
    ST_CHECK(p && w_c && (p->layers == 0 || w_k), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(p->device));
    ST_CUDA(cudaMemcpy(p->w_c, w_c, CH * NTAP * 4, cudaMemcpyDeviceToDevice));
    for (int k = 0; k < p->layers; ++k) {
        const float* w = w_k + (size_t)k * CH * CH * NTAP;
        const size_t off = (size_t)k * NTAP * CH * CH * 2;
        ST_TRY(st_conv3d_pack_weights(w, static_cast<char*>(p->packed) + off, 0, nullptr));
        ST_TRY(st_conv3d_pack_weights(w, static_cast<char*>(p->packed_t) + off, 1, nullptr));
    }
    ST_CUDA(cudaDeviceSynchronize());
    return ST_OK;
}

int st_pcnet_apply(st_pcnet* p, const float* r, const float* dinv, float* z, void* stream) {
    ST_CHECK(p && r && dinv && z, ST_ERR_ARG, "null argument");
    const long long n = (long long)p->nx * p->ny * p->nz;
    char* u0 = static_cast<char*>(p->u);
    char* u1 = u0 + p->vol_bytes;
    ST_TRY(st_pc_scales(r, dinv, p->acc, p->scales, n, stream));
    ST_TRY(st_pc_scale_in(r, dinv, p->scales, p->a, n, stream));
    ST_TRY(st_pc_tconv1(p->a, p->w_c, u0, p->nx, p->ny, p->nz, stream));
    const size_t wsz = (size_t)NTAP * CH * CH * 2;
    for (int k = 0; k < p->layers; ++k) {  // u <- (I + conv_k) u
        ST_TRY(st_conv3d_bf16(u0, static_cast<char*>(p->packed) + k * wsz, nullptr, u0, u1, 0, p->nx, p->ny, p->nz, 0,
                              stream));
        std::swap(u0, u1);
    }
    for (int k = p->layers - 1; k >= 0; --k) {  // u <- (I + conv_k^T) u
        ST_TRY(st_conv3d_bf16(u0, static_cast<char*>(p->packed_t) + k * wsz, nullptr, u0, u1, 0, p->nx, p->ny,
                              p->nz, 0, stream));
        std::swap(u0, u1);
    }
    ST_TRY(st_pc_out_conv(u0, p->w_c, nullptr, nullptr, nullptr, p->a, nullptr, p->nx, p->ny, p->nz, stream));
    return st_pc_combine(p->a, r, dinv, p->scales, z, n, stream);
}

}  // extern "C"
