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

// dW[co][ci][tap] += sum_v g[v][co] * x[v + s_tap][ci] for a 32 -> 32 layer.
// Block (range, tap): 256 threads, thread t owns co = t / 8 and ci = 4 (t % 8)
// .. +3; 64-voxel chunks of g and of the shifted x are staged in shared memory.
__global__ void __launch_bounds__(256) conv32_wgrad_kernel(const __nv_bfloat16* __restrict__ x,
                                                           const __nv_bfloat16* __restrict__ g, Vol v,
                                                           float* __restrict__ dw) {
    constexpr int CHUNK = 64;
    __shared__ float gs[CHUNK][CH + 1];
    __shared__ float xs[CHUNK][CH + 1];
    const int tap = blockIdx.y;
    const int W2 = v.nz + 2, P2 = (v.ny + 2) * W2;
    const long long shift = (long long)(tap / 9 - 1) * P2 + ((tap / 3) % 3 - 1) * W2 + (tap % 3 - 1);
    const int co = threadIdx.x >> 3, ci0 = (threadIdx.x & 7) * 4;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const long long n = v.n();
    const long long per = (n + gridDim.x - 1) / gridDim.x;
    const long long i0 = blockIdx.x * per, i1 = min(n, i0 + per);
    for (long long c0 = i0; c0 < i1; c0 += CHUNK) {
        // stage: 64 voxels x 32 channels of g and of x shifted by the tap
        for (int e = threadIdx.x; e < CHUNK * 4; e += blockDim.x) {
            const int vi = e >> 2, part = e & 3;
            const long long i = c0 + vi;
            float gg[8], xx[8];
            if (i < i1) {
                int px, py, pz;
                decode(i, v, px, py, pz);
                const long long q = v.pad_row(px, py, pz);
                const uint4 ug = reinterpret_cast<const uint4*>(g + q * CH)[part];
                const uint4 ux = reinterpret_cast<const uint4*>(x + (q + shift) * CH)[part];
                const __nv_bfloat162* bg = reinterpret_cast<const __nv_bfloat162*>(&ug);
                const __nv_bfloat162* bx = reinterpret_cast<const __nv_bfloat162*>(&ux);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float2 a = __bfloat1622float2(bg[k]), b = __bfloat1622float2(bx[k]);
                    gg[2 * k] = a.x;
                    gg[2 * k + 1] = a.y;
                    xx[2 * k] = b.x;
                    xx[2 * k + 1] = b.y;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) gg[k] = xx[k] = 0.0f;
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                gs[vi][part * 8 + k] = gg[k];
                xs[vi][part * 8 + k] = xx[k];
            }
        }
        __syncthreads();
#pragma unroll 8
        for (int vi = 0; vi < CHUNK; ++vi) {
            const float a = gs[vi][co];
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] = fmaf(a, xs[vi][ci0 + k], acc[k]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) atomicAdd(&dw[((size_t)co * CH + ci0 + k) * NTAP + tap], acc[k]);
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

int st_conv3d_wgrad(const void* x, const void* g, float* dw, int64_t nx, int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(x && g && dw, ST_ERR_ARG, "null argument");
    const Vol v{(int)nx, (int)ny, (int)nz};
    conv32_wgrad_kernel<<<dim3(grid_for(v.n(), 48), NTAP), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const __nv_bfloat16*>(x), static_cast<const __nv_bfloat16*>(g), v, dw);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

}  // extern "C"
