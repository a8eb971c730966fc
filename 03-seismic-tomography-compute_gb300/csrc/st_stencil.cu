// Fused 7-point acoustic propagator step for sm_103a.
//
// One kernel computes, for every interior point of one time step,
//     out = 2u - D*prev + c * L u          (guards and clamp as the reference)
// which is WaveEquationSolver::step_forward (solver/wave_equation.cpp:56-76:
// fd_7point_operator_safe :299-405, apply_sponge_layer :262-297 and the
// buffer swap :61-62) with the sponge applied to `prev` on read instead of
// being written back: the reference damps current and previous after the
// update and before the swap, so its previous field is always D times the
// undamped current of the step before. c = v^2 dt^2 is precomputed.
//
// The same kernel is the exact discrete adjoint: for mu = c * lambda the
// transposed recursion lambda_{t-1} = (2I + L C) lambda_t - D lambda_{t+1}
// becomes mu_{t-1} = (2I + C L) mu_t - D mu_{t+1}, i.e. this operator, with
// the receiver forcing scaled by c. Epilogues fused into the write:
//   - receiver sampling of the update (before injection) on a receiver grid,
//   - point-source injection of the next sample (inject_source :39-54),
//   - adjoint forcing c * r at the receivers,
//   - BF16/FP16/FP32 snapshot store of the centre field with a per-snapshot
//     scale (|max| tracked with one atomic per CTA),
//   - zero-lag cross-correlation imaging image += f*a, illum += f*f with
//     a = mu / c (RTMEngine::apply_image_condition, rtm/rtm_engine.cpp:24-57).
//
// Data movement: each CTA owns a TY x TZ (y,z) tile and marches along x (the
// slowest axis), staging every x-plane of u (with a one-cell y/z halo), prev
// and c in shared memory with TMA (cp.async.bulk.tensor, no multicast) in a
// 4-deep mbarrier ring; u at x-1/x/x+1 rides in a register queue. HBM traffic
// is 16 B per point (read u, prev, c; write out), plus the epilogue's bytes.
#include "st_kernels.cuh"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <mutex>

namespace stg {

namespace {

constexpr int TZ = FD_TZ;
constexpr int TY = FD_TY;
constexpr int TZ4 = TZ / 4;
constexpr int NTHREADS = TZ4 * TY;  // 256
constexpr int STAGES = 4;
constexpr int CUR_W = TZ + 8;
constexpr int CUR_H = TY + 2;
constexpr int CUR_BYTES = CUR_W * CUR_H * 4;
constexpr int CUR_BYTES_PAD = ((CUR_BYTES + 127) / 128) * 128;
constexpr int CTR_BYTES = TZ * TY * 4;
constexpr int STAGE_BYTES = CUR_BYTES_PAD + 2 * CTR_BYTES;
constexpr int STAGE_TX = CUR_BYTES + 2 * CTR_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 128;
constexpr int MIN_BLOCKS = 4;
constexpr unsigned FULL = 0xffffffffu;

template <int K>
__device__ __forceinline__ float snap_load(const void* p, long long i) {
    if constexpr (K == SNAP_BF16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(p)[i]);
    else if constexpr (K == SNAP_FP16) return __half2float(reinterpret_cast<const __half*>(p)[i]);
    else return reinterpret_cast<const float*>(p)[i];
}

template <int K>
__device__ __forceinline__ void snap_store(void* p, long long i, float v) {
    if constexpr (K == SNAP_BF16) reinterpret_cast<__nv_bfloat16*>(p)[i] = __float2bfloat16_rn(v);
    else if constexpr (K == SNAP_FP16) reinterpret_cast<__half*>(p)[i] = __float2half_rn(v);
    else reinterpret_cast<float*>(p)[i] = v;
}

// Four consecutive values (8 B aligned for 16-bit kinds, 16 B for FP32).
template <int K>
__device__ __forceinline__ void snap_store4(void* p, long long i, float4 v) {
    if constexpr (K == SNAP_BF16) {
        __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<unsigned*>(&a);
        w.y = *reinterpret_cast<unsigned*>(&b);
        *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(p) + i) = w;
    } else if constexpr (K == SNAP_FP16) {
        __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<unsigned*>(&a);
        w.y = *reinterpret_cast<unsigned*>(&b);
        *reinterpret_cast<uint2*>(reinterpret_cast<__half*>(p) + i) = w;
    } else {
        *reinterpret_cast<float4*>(reinterpret_cast<float*>(p) + i) = v;
    }
}

template <int K>
__device__ __forceinline__ float4 snap_load4(const void* p, long long i) {
    if constexpr (K == SNAP_BF16) {
        uint2 w = *reinterpret_cast<const uint2*>(reinterpret_cast<const __nv_bfloat16*>(p) + i);
        __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&w.x), b = *reinterpret_cast<__nv_bfloat162*>(&w.y);
        float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
        return make_float4(fa.x, fa.y, fb.x, fb.y);
    } else if constexpr (K == SNAP_FP16) {
        uint2 w = *reinterpret_cast<const uint2*>(reinterpret_cast<const __half*>(p) + i);
        __half2 a = *reinterpret_cast<__half2*>(&w.x), b = *reinterpret_cast<__half2*>(&w.y);
        float2 fa = __half22float2(a), fb = __half22float2(b);
        return make_float4(fa.x, fa.y, fb.x, fb.y);
    } else {
        return *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(p) + i);
    }
}

__device__ __forceinline__ float f4get(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}
__device__ __forceinline__ void f4set(float4& v, int k, float x) {
    if (k == 0) v.x = x;
    else if (k == 1) v.y = x;
    else if (k == 2) v.z = x;
    else v.w = x;
}

// The reference update of one point with its NaN/Inf guards
// (wave_equation.cpp:342-399). `upd` is the damped previous value.
__device__ __forceinline__ float point_update(float u, float upd, float xm, float xp, float ym, float yp, float zm,
                                              float zp, float c, float ax, float ay, float az, float amp,
                                              bool& fired) {
    const float sx = xp + xm, sy = yp + ym, sz = zp + zm;
    const float probe = (sx + sy) + (sz + u) + upd;
    if (isfinite(probe)) {
        // all eight inputs are finite (any NaN/Inf would propagate into probe)
        const float lap = fmaf(-2.0f, u, sx) * ax + fmaf(-2.0f, u, sy) * ay + fmaf(-2.0f, u, sz) * az;
        float nv = fmaf(2.0f, u, -upd) + c * lap;
        if (!isfinite(nv)) {
            nv = u;
            fired = true;
        }
        return fminf(fmaxf(nv, -amp), amp);
    }
    // slow path: a non-finite input, or a finite sum that overflowed
    if (!isfinite(u) || !isfinite(upd)) {
        fired = true;
        return 0.0f;
    }
    if (!isfinite(xm) || !isfinite(xp) || !isfinite(ym) || !isfinite(yp) || !isfinite(zm) || !isfinite(zp)) {
        fired = true;
        return u;
    }
    const float lap = ((xp - 2.0f * u) + xm) * ax + ((yp - 2.0f * u) + ym) * ay + ((zp - 2.0f * u) + zm) * az;
    float nv = (2.0f * u - upd) + c * lap;
    if (!isfinite(nv)) {
        nv = u;
        fired = true;
    }
    return fminf(fmaxf(nv, -amp), amp);
}

template <int SNAP_OUT, int SNAP_IN, bool IMAGE>
__global__ void __launch_bounds__(NTHREADS, MIN_BLOCKS)
    fd_step_kernel(const __grid_constant__ CUtensorMap map_cur, const __grid_constant__ CUtensorMap map_prev,
                   const __grid_constant__ CUtensorMap map_c, const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    float* red = reinterpret_cast<float*>(smem + STAGES * STAGE_BYTES + 64);

    const int tid = threadIdx.x;
    const int tz4 = tid % TZ4;
    const int ty = tid / TZ4;
    const int z0 = blockIdx.x * TZ;
    const int y0 = blockIdx.y * TY;
    const int xa = blockIdx.z * a.x_chunk;
    const int xb = min(xa + a.x_chunk, a.nx);
    if (xa >= xb) return;  // uniform over the CTA
    const int nplanes = xb - xa + 2;

    const int iy = y0 + ty;
    const int iz0 = z0 + 4 * tz4;
    const int zvalid = min(4, a.nz - iz0);
    const bool active = (iy < a.ny) && (zvalid > 0);

    // sponge distances: y part now, z part per element, x part per plane
    const int dy = min(iy, a.ny - 1 - iy);
    int dz4[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) dz4[k] = min(iz0 + k, a.nz - 1 - (iz0 + k));

    // receiver bookkeeping for this thread's (y, z-group)
    int rk = -1, iry = -1;
    if ((a.seis_row || a.force_row) && active) {
        const int kk = a.rz - iz0;
        const int yy = iy - a.ry0;
        if (kk >= 0 && kk < zvalid && yy >= 0 && yy % a.rsy == 0 && yy / a.rsy < a.rny) {
            rk = kk;
            iry = yy / a.rsy;
        }
    }

    float snap_inv = 0.0f;
    if constexpr (SNAP_OUT != SNAP_NONE) {
        const float m = __uint_as_float(*a.amax_cur);
        snap_inv = m > 0.0f ? SNAP_QMAX / m : 0.0f;
    }
    float snap_in_scale = 1.0f;
    if constexpr (IMAGE) {
        const float m = __uint_as_float(*a.amax_in);
        snap_in_scale = m / SNAP_QMAX;
    }

    auto cur_tile = [&](int s) { return reinterpret_cast<float*>(smem + s * STAGE_BYTES); };
    auto prev_tile = [&](int s) { return reinterpret_cast<float*>(smem + s * STAGE_BYTES + CUR_BYTES_PAD); };
    auto c_tile = [&](int s) {
        return reinterpret_cast<float*>(smem + s * STAGE_BYTES + CUR_BYTES_PAD + CTR_BYTES);
    };

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    // plane index i in [0, nplanes) is interior x = xa - 1 + i, device x = xa + i
    auto issue = [&](int i) {
        const int s = i % STAGES;
        const int xd = xa + i;
        mbar_arrive_expect_tx(&bar[s], STAGE_TX);
        tma_load_3d(cur_tile(s), &map_cur, &bar[s], z0, y0, xd);
        tma_load_3d(prev_tile(s), &map_prev, &bar[s], z0 + Layout::ZOFF, y0 + 1, xd);
        tma_load_3d(c_tile(s), &map_c, &bar[s], z0 + Layout::ZOFF, y0 + 1, xd);
    };
    int issued = 0;
    if (tid == 0) {
        issued = min(STAGES, nplanes);
        for (int i = 0; i < issued; ++i) issue(i);
    }

    const int crow = (ty + 1) * CUR_W + 4 * tz4 + 4;  // centre float4 of this thread in a cur tile
    const int ctr = ty * TZ + 4 * tz4;                 // its float4 in prev / c tiles
    float4 um = make_float4(0.f, 0.f, 0.f, 0.f), u0 = um, up = um;
    float amax_local = 0.0f;
    bool fired = false;
    int timed_out = 0;
    int i = 0;

    for (; i < nplanes; ++i) {
        const int s = i % STAGES;
        if (!mbar_wait_bounded(&bar[s], (i / STAGES) & 1, a.timeout_ns)) timed_out = 1;
        up = *reinterpret_cast<const float4*>(cur_tile(s) + crow);
        if (i >= 2) {
            const int sp = (i - 1) % STAGES;
            const int x = xa + i - 2;
            const float* T = cur_tile(sp);
            const float4 ym = *reinterpret_cast<const float4*>(T + crow - CUR_W);
            const float4 yp = *reinterpret_cast<const float4*>(T + crow + CUR_W);
            float zm0 = __shfl_up_sync(FULL, u0.w, 1, TZ4);
            float zp3 = __shfl_down_sync(FULL, u0.x, 1, TZ4);
            if (tz4 == 0) zm0 = T[crow - 1];
            if (tz4 == TZ4 - 1) zp3 = T[crow + 4];
            const float4 pv = *reinterpret_cast<const float4*>(prev_tile(sp) + ctr);
            const float4 cv = *reinterpret_cast<const float4*>(c_tile(sp) + ctr);
            const int dxy = min(dy, min(x, a.nx - 1 - x));
            const long long obase = (long long)(x + 1) * a.plane + (long long)(iy + 1) * a.NZP + iz0 + Layout::ZOFF;
            const long long cbase = ((long long)x * a.ny + iy) * a.nz + iz0;  // compact interior index
            int irx = -1;
            if (rk >= 0) {
                const int xx = x - a.rx0;
                if (xx >= 0 && xx % a.rsx == 0 && xx / a.rsx < a.rnx) irx = xx / a.rsx;
            }
            float4 res;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float u = f4get(u0, k);
                const float zm = k == 0 ? zm0 : f4get(u0, k - 1);
                const float zp = k == 3 ? zp3 : f4get(u0, k + 1);
                const int d = min(dxy, dz4[k]);
                const float D = (d >= 0 && d < a.sw) ? __ldg(a.dtab + d) : 1.0f;
                const float c = f4get(cv, k);
                float nv = point_update(u, D * f4get(pv, k), f4get(um, k), f4get(up, k), f4get(ym, k), f4get(yp, k),
                                        zm, zp, c, a.ax, a.ay, a.az, a.amp, fired);
                if (k == rk && irx >= 0) {
                    const int q = irx * a.rny + iry;
                    if (a.seis_row) a.seis_row[q] = nv;
                    if (a.force_row) nv += c * a.force_row[q];
                }
                if (obase + k == a.inj_idx) nv += a.inj_val;
                f4set(res, k, nv);
            }
            if (active) {
                if (zvalid == 4) {
                    *reinterpret_cast<float4*>(a.out + obase) = res;
                } else {
                    for (int k = 0; k < zvalid; ++k) a.out[obase + k] = f4get(res, k);
                }
                if constexpr (SNAP_OUT != SNAP_NONE) {
                    float4 q = make_float4(u0.x * snap_inv, u0.y * snap_inv, u0.z * snap_inv, u0.w * snap_inv);
                    if (zvalid == 4 && (a.nz & 3) == 0) {
                        snap_store4<SNAP_OUT>(a.snap_out, cbase, q);
                    } else {
                        for (int k = 0; k < zvalid; ++k) snap_store<SNAP_OUT>(a.snap_out, cbase + k, f4get(q, k));
                    }
                    for (int k = 0; k < zvalid; ++k) amax_local = fmaxf(amax_local, fabsf(f4get(res, k)));
                }
                if constexpr (IMAGE) {
                    const bool vec = zvalid == 4 && (a.nz & 3) == 0;
                    float4 fv;
                    if (vec) fv = snap_load4<SNAP_IN>(a.snap_in, cbase);
                    float4 im = vec ? *reinterpret_cast<const float4*>(a.image + cbase) : make_float4(0, 0, 0, 0);
                    float4 il = vec ? *reinterpret_cast<const float4*>(a.illum + cbase) : make_float4(0, 0, 0, 0);
                    for (int k = 0; k < zvalid; ++k) {
                        float f = (vec ? f4get(fv, k) : snap_load<SNAP_IN>(a.snap_in, cbase + k)) * snap_in_scale;
                        float ad = f4get(u0, k) / f4get(cv, k);
                        if (!isfinite(f)) f = 0.0f;
                        if (!isfinite(ad)) ad = 0.0f;
                        if (vec) {
                            f4set(im, k, fmaf(f, ad, f4get(im, k)));
                            f4set(il, k, fmaf(f, f, f4get(il, k)));
                        } else {
                            a.image[cbase + k] += f * ad;
                            a.illum[cbase + k] += f * f;
                        }
                    }
                    if (vec) {
                        *reinterpret_cast<float4*>(a.image + cbase) = im;
                        *reinterpret_cast<float4*>(a.illum + cbase) = il;
                    }
                }
            }
        }
        um = u0;
        u0 = up;
        // every thread is done with the slot of plane i-1: refill it
        if (__syncthreads_or(timed_out)) break;
        if (tid == 0 && i >= 1 && issued < nplanes) issue(issued++);
    }

    if (i < nplanes) {
        // A wait gave up: drain the copies still in flight (bounded), then leave.
        if (tid == 0) {
            for (int j = i; j < issued; ++j) mbar_wait_bounded(&bar[j % STAGES], (j / STAGES) & 1, a.timeout_ns);
            atomicOr(a.flags, FLAG_TIMEOUT);
        }
        __syncthreads();
        return;
    }
    if (fired) atomicOr(a.flags, FLAG_GUARD);
    if constexpr (SNAP_OUT != SNAP_NONE) {
        float m = amax_local;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
        if ((tid & 31) == 0) red[tid >> 5] = m;
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < NTHREADS / 32; ++w) m = fmaxf(m, red[w]);
            atomicMax(a.amax_next, __float_as_uint(m));
        }
    }
}

template <int SO, int SI, bool IM>
int launch_variant(dim3 grid, const CUtensorMap& mcur, const CUtensorMap& mprev, const CUtensorMap& mc,
                   const StepArgs& a, cudaStream_t st) {
    static bool configured = false;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!configured) {
            ST_CUDA(cudaFuncSetAttribute(fd_step_kernel<SO, SI, IM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES));
            configured = true;
        }
    }
    fd_step_kernel<SO, SI, IM><<<grid, NTHREADS, SMEM_BYTES, st>>>(mcur, mprev, mc, a);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// ---------------------------------------------------------------- small kernels

__global__ void add_point_kernel(float* f, long long idx, float val, unsigned* amax_slot) {
    const float v = f[idx] + val;
    f[idx] = v;
    if (amax_slot) atomicMax(amax_slot, __float_as_uint(fabsf(v)));
}

__global__ void gather_kernel(const float* f, const long long* idx, int n, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = f[idx[i]];
}

__global__ void scatter_scaled_kernel(float* f, const long long* idx, int n, const float* val, const float* c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const long long j = idx[i];
        f[j] += (c ? c[j] : 1.0f) * val[i];
    }
}

__device__ __forceinline__ float sponge_at(const Layout& L, const float* dtab, int sw, long long xd, long long yd,
                                           long long zr) {
    // zr: reference padded z index; padded cells use the reference's distance rule
    const long long ix = xd - 1, iy = yd - 1, iz = zr - 1;
    long long d = sw;
    d = min(d, ix);
    d = min(d, L.nx - 1 - ix);
    d = min(d, iy);
    d = min(d, L.ny - 1 - iy);
    d = min(d, iz);
    d = min(d, L.nz - 1 - iz);
    return (d >= 0 && d < sw) ? dtab[d] : 1.0f;
}

// Reference layout (FP64, pitch nz+2) -> device layout (FP32, pitch NZP).
__global__ void ref_to_dev_kernel(const double* __restrict__ src, float* __restrict__ dst, Layout L,
                                  const float* dtab, int sw, int undamp_pow) {
    const long long total = L.elems;
    const long long NZh = L.nz + 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long xd = e / L.plane;
        const long long r = e - xd * L.plane;
        const long long yd = r / L.NZP;
        const long long zd = r - yd * L.NZP;
        const long long zr = zd - (Layout::ZOFF - 1);
        float v = 0.0f;
        if (zr >= 0 && zr < NZh) {
            double s = src[(xd * L.NYh + yd) * NZh + zr];
            if (undamp_pow > 0) {
                const double D = (double)sponge_at(L, dtab, sw, xd, yd, zr);
                for (int p = 0; p < undamp_pow; ++p) s = s / D;
            }
            v = (float)s;
        }
        dst[e] = v;
    }
}

// Device layout -> reference layout, optionally times D^damp_pow.
__global__ void dev_to_ref_kernel(const float* __restrict__ src, double* __restrict__ dst, Layout L,
                                  const float* dtab, int sw, int damp_pow) {
    const long long NZh = L.nz + 2;
    const long long total = L.NXh * L.NYh * NZh;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long xd = e / (L.NYh * NZh);
        const long long r = e - xd * (L.NYh * NZh);
        const long long yd = r / NZh;
        const long long zr = r - yd * NZh;
        double v = (double)src[xd * L.plane + yd * L.NZP + zr + (Layout::ZOFF - 1)];
        if (damp_pow > 0) {
            const double D = (double)sponge_at(L, dtab, sw, xd, yd, zr);
            for (int p = 0; p < damp_pow; ++p) v *= D;
        }
        dst[e] = v;
    }
}

// c = v^2 dt^2 damp^2 with the reference's velocity fallback (v <= 0 or
// non-finite -> 1500 m/s, wave_equation.cpp:375-378), device layout.
__global__ void vel_to_coeff_kernel(const double* __restrict__ vel, float* __restrict__ c, Layout L,
                                    double dt2damp) {
    const long long total = L.elems;
    const long long NZh = L.nz + 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long xd = e / L.plane;
        const long long r = e - xd * L.plane;
        const long long yd = r / L.NZP;
        const long long zd = r - yd * L.NZP;
        const long long zr = zd - (Layout::ZOFF - 1);
        float out = 0.0f;
        if (zr >= 0 && zr < NZh) {
            double v = vel[(xd * L.NYh + yd) * NZh + zr];
            if (!isfinite(v) || v <= 0.0) v = 1500.0;
            out = (float)(v * v * dt2damp);
        }
        c[e] = out;
    }
}

__global__ void count_nonfinite_kernel(const float* __restrict__ f, long long n, unsigned long long* out) {
    unsigned long long cnt = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        cnt += !isfinite(f[i]);
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, cnt);
}

__global__ void sumsq_finite_kernel(const float* __restrict__ f, long long n, double* out) {
    __shared__ double part[32];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = f[i];
        if (isfinite(v)) s += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        atomicAdd(out, t);
    }
}

// Interior copy with non-finite values replaced by 0 (save_snapshot, wave_equation.cpp:463-480).
__global__ void interior_copy_kernel(const float* __restrict__ f, Layout L, float* __restrict__ out) {
    const long long total = L.nx * L.ny * L.nz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long ix = e / (L.ny * L.nz);
        const long long r = e - ix * (L.ny * L.nz);
        const long long iy = r / L.nz;
        const long long iz = r - iy * L.nz;
        const float v = f[L.at(ix, iy, iz)];
        out[e] = isfinite(v) ? v : 0.0f;
    }
}

// RTMEngine::finalize_image (rtm/rtm_engine.cpp:170-182).
__global__ void finalize_image_kernel(const float* __restrict__ image, const float* __restrict__ illum,
                                      float* __restrict__ refl, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float il = illum[i];
        refl[i] = il > 1e-10f ? image[i] / il : 0.0f;
    }
}

int grid_for(long long n, int threads = 256) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)num_sms() * 8;
    return (int)std::max<long long>(1, std::min(b, cap));
}

}  // namespace

// ---------------------------------------------------------------- host side

int build_stencil_map_cur(CUtensorMap* m, const float* base, const Layout& L) {
    return make_field_map(m, base, L, TZ + 8, TY + 2);
}
int build_stencil_map_ctr(CUtensorMap* m, const float* base, const Layout& L) {
    return make_field_map(m, base, L, TZ, TY);
}

int fd_step_grid_chunks(const Layout& L) {
    const long long gx = (L.nz + TZ - 1) / TZ, gy = (L.ny + TY - 1) / TY;
    // one resident wave: every CTA marches its x-chunk from start to end
    const long long target = (long long)num_sms() * MIN_BLOCKS;
    long long chunks = target / (gx * gy);
    chunks = std::max<long long>(1, std::min<long long>(chunks, L.nx));
    return (int)chunks;
}

int launch_fd_step(const Layout& L, const CUtensorMap& mcur, const CUtensorMap& mprev, const CUtensorMap& mc,
                   StepArgs a, int snap_out, int snap_in, bool image, cudaStream_t st) {
    const int chunks = fd_step_grid_chunks(L);
    a.x_chunk = (int)((L.nx + chunks - 1) / chunks);
    const int nch = (int)((L.nx + a.x_chunk - 1) / a.x_chunk);
    dim3 grid((unsigned)((L.nz + TZ - 1) / TZ), (unsigned)((L.ny + TY - 1) / TY), (unsigned)nch);
    a.nx = (int)L.nx;
    a.ny = (int)L.ny;
    a.nz = (int)L.nz;
    a.NZP = (int)L.NZP;
    a.plane = L.plane;
    if (a.timeout_ns == 0) a.timeout_ns = 2000000000ull;
    if (image) {
        ST_CHECK(snap_out == SNAP_NONE, ST_ERR_ARG, "imaging step cannot also store snapshots");
        switch (snap_in) {
            case SNAP_BF16: return launch_variant<SNAP_NONE, SNAP_BF16, true>(grid, mcur, mprev, mc, a, st);
            case SNAP_FP16: return launch_variant<SNAP_NONE, SNAP_FP16, true>(grid, mcur, mprev, mc, a, st);
            case SNAP_FP32: return launch_variant<SNAP_NONE, SNAP_FP32, true>(grid, mcur, mprev, mc, a, st);
            default: ST_CHECK(false, ST_ERR_ARG, "imaging step needs a snapshot kind");
        }
    }
    switch (snap_out) {
        case SNAP_NONE: return launch_variant<SNAP_NONE, SNAP_NONE, false>(grid, mcur, mprev, mc, a, st);
        case SNAP_BF16: return launch_variant<SNAP_BF16, SNAP_NONE, false>(grid, mcur, mprev, mc, a, st);
        case SNAP_FP16: return launch_variant<SNAP_FP16, SNAP_NONE, false>(grid, mcur, mprev, mc, a, st);
        case SNAP_FP32: return launch_variant<SNAP_FP32, SNAP_NONE, false>(grid, mcur, mprev, mc, a, st);
        default: ST_CHECK(false, ST_ERR_ARG, "bad snapshot kind %d", snap_out);
    }
}

int launch_add_point(float* f, long long idx, float val, unsigned* amax_slot, cudaStream_t st) {
    add_point_kernel<<<1, 1, 0, st>>>(f, idx, val, amax_slot);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_gather(const float* f, const long long* idx, int n, float* out, cudaStream_t st) {
    if (n <= 0) return ST_OK;
    gather_kernel<<<(n + 255) / 256, 256, 0, st>>>(f, idx, n, out);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_scatter_scaled(float* f, const long long* idx, int n, const float* val, const float* c, cudaStream_t st) {
    if (n <= 0) return ST_OK;
    scatter_scaled_kernel<<<(n + 255) / 256, 256, 0, st>>>(f, idx, n, val, c);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_ref_to_dev(const double* src, float* dst, const Layout& L, cudaStream_t st) {
    ref_to_dev_kernel<<<grid_for(L.elems), 256, 0, st>>>(src, dst, L, nullptr, 0, 0);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_ref_to_dev_undamp(const double* src, float* dst, const Layout& L, const float* dtab, int sw, int pow,
                             cudaStream_t st) {
    ref_to_dev_kernel<<<grid_for(L.elems), 256, 0, st>>>(src, dst, L, dtab, sw, pow);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_dev_to_ref(const float* src, double* dst, const Layout& L, const float* dtab, int sw, int damp_pow,
                      cudaStream_t st) {
    const long long n = L.NXh * L.NYh * (L.nz + 2);
    dev_to_ref_kernel<<<grid_for(n), 256, 0, st>>>(src, dst, L, dtab, sw, damp_pow);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_vel_to_coeff(const double* vel_ref, float* c, const Layout& L, double dt2damp, cudaStream_t st) {
    vel_to_coeff_kernel<<<grid_for(L.elems), 256, 0, st>>>(vel_ref, c, L, dt2damp);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_count_nonfinite(const float* f, long long n, unsigned long long* out, cudaStream_t st) {
    ST_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long), st));
    count_nonfinite_kernel<<<grid_for(n), 256, 0, st>>>(f, n, out);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_sumsq_finite(const float* f, long long n, double* out, cudaStream_t st) {
    ST_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    sumsq_finite_kernel<<<grid_for(n), 256, 0, st>>>(f, n, out);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_interior_copy(const float* f, const Layout& L, float* out, cudaStream_t st) {
    interior_copy_kernel<<<grid_for(L.nx * L.ny * L.nz), 256, 0, st>>>(f, L, out);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int launch_finalize_image(const float* image, const float* illum, float* refl, long long n, cudaStream_t st) {
    finalize_image_kernel<<<grid_for(n), 256, 0, st>>>(image, illum, refl, n);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

// ---------------------------------------------------------------- launch counter

namespace {
std::atomic<long long> g_launches{0};
}
void count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------- tensor maps

int get_encode_tiled(EncodeTiledFn* out) {
    static EncodeTiledFn fn = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        ST_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        ST_CHECK(q == cudaDriverEntryPointSuccess && p, ST_ERR_CUDA, "cuTensorMapEncodeTiled not available");
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    *out = fn;
    return ST_OK;
}

int make_field_map(CUtensorMap* map, const float* base, const Layout& L, int bz, int by) {
    EncodeTiledFn enc = nullptr;
    ST_TRY(get_encode_tiled(&enc));
    ST_CHECK((reinterpret_cast<uintptr_t>(base) & 15) == 0, ST_ERR_ARG, "field base not 16-byte aligned");
    cuuint64_t dims[3] = {(cuuint64_t)L.NZP, (cuuint64_t)L.NYh, (cuuint64_t)L.NXh};
    cuuint64_t strides[2] = {(cuuint64_t)L.NZP * 4, (cuuint64_t)L.plane * 4};
    cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)by, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    ST_CHECK(r == CUDA_SUCCESS, ST_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return ST_OK;
}

}  // namespace stg
