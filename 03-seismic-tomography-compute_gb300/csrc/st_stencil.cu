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
//     a = mu / c (RTMEngine::apply_image_condition, rtm/rtm_engine.cpp:24-57),
//   - the adjoint-state gradient grad_c += (mu / c) * L S of a forward
//     snapshot S staged through TMA with its halo.
//
// Stable sponge (opt-in, StepArgs::stable_sponge): the reference rule
// u_{n+1} = 2u_n - D u_{n-1} + c L u_n grows exponentially for smooth modes in
// a wide sponge (characteristic roots 1 +- sqrt(1 - D) when c L u is small;
// the default 20-cell, 0.015 sponge diverges within a few hundred steps).
// The Cerjan form damps the new field instead:
//     out = D * (2u - D*prev + c L u)        (prev = the undamped u_{n-1})
// whose roots have modulus D < 1. Its adjoint is again this operator for
// mu = c * D * lambda, with forcing c * D * r entering before the damping.
//
// Data movement: each CTA owns a (16 or 32) x 64 (y,z) tile and marches along
// x (the slowest axis), staging every x-plane of u (with a one-cell y/z halo),
// prev and c in shared memory with TMA (cp.async.bulk.tensor, no multicast) in
// a 3- or 4-deep mbarrier ring; u at x-1/x/x+1 rides in a register queue. HBM
// traffic is 16 B per point (read u, prev, c; write out) plus the epilogue's.
#include "st_kernels.cuh"

#include <algorithm>
#include <cfloat>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <mutex>
#include <type_traits>

namespace stg {

namespace {

constexpr int TZ = FD_TZ;                     // 64 interior z per tile
constexpr int TZ4 = TZ / 4;                   // threads along z (4 points each)
constexpr int NTHREADS = TZ4 * 16;            // 256 threads: 16 thread rows x 16 z-groups
constexpr int CUR_W = TZ + 8;
constexpr int DTAB_MAX = 512;                 // sponge widths up to this use a shared-memory table
constexpr int EXTRA_BYTES = 128 + DTAB_MAX * 4;
constexpr int SM_SMEM = 232448;               // shared memory per SM (227 KB usable per CTA)
constexpr unsigned FULL = 0xffffffffu;

// EPI_IMAGE_T: imaging with its operands (snapshot, image, illumination tiles)
// staged through the TMA ring instead of loaded at use. EPI_MASK: a forward
// step that also applies the terrain's per-column z limits (StepArgs::zlim);
// kept apart from EPI_NONE so the plain forward step carries no mask code.
enum Epilogue : int { EPI_NONE = 0, EPI_IMAGE = 1, EPI_GRAD = 2, EPI_IMAGE_T = 3, EPI_MASK = 4 };
constexpr bool is_image(int e) { return e == EPI_IMAGE || e == EPI_IMAGE_T; }
constexpr bool is_forward(int e) { return e == EPI_NONE || e == EPI_MASK; }

// Per-variant tiling. Forward variants give each thread 2 adjacent rows
// (32-row tiles, 2 CTAs per SM): fewer instructions per point. The imaging
// and gradient variants, whose epilogues read and write global memory
// directly, give each thread 1 row (16-row tiles) so more warps per SM hide
// those accesses. The gradient variant also stages the forward snapshot tile
// with its halo (box starting 16 bytes left of the tile), in a 3-deep ring.
// The staged imaging variant adds the snapshot, image and illumination tiles
// of each plane to the stage (3-deep ring).
template <int EPI, int SNAP_IN>
struct Geo {
    static constexpr int RPT = is_forward(EPI) ? 2 : 1;  // rows per thread
    static constexpr int TYV = 16 * RPT;                 // tile rows
    static constexpr int CUR_H = TYV + 2;
    static constexpr int CUR_BYTES = CUR_W * CUR_H * 4;
    static constexpr int CUR_BYTES_PAD = ((CUR_BYTES + 127) / 128) * 128;
    static constexpr int CTR_BYTES = TZ * TYV * 4;
    static constexpr int STAGES = (EPI == EPI_GRAD || EPI == EPI_IMAGE_T) ? 3 : 4;
    static constexpr int SES = (EPI == EPI_GRAD || EPI == EPI_IMAGE_T) ? snap_bytes(SNAP_IN) : 0;
    static constexpr int SW = EPI == EPI_GRAD ? (SES == 2 ? TZ + 16 : TZ + 8) : (EPI == EPI_IMAGE_T ? TZ : 0);
    static constexpr int SOFF = EPI == EPI_GRAD ? (SES == 2 ? 8 : 4) : 0;
    static constexpr int SNAP_H = EPI == EPI_GRAD ? CUR_H : TYV;
    static constexpr int SNAP_TILE = SW * SNAP_H * SES;
    static constexpr int SNAP_TILE_PAD = ((SNAP_TILE + 127) / 128) * 128;
    static constexpr int ACC_BYTES = EPI == EPI_IMAGE_T ? 2 * CTR_BYTES : 0;  // image + illumination tiles
    static constexpr int STAGE_BYTES = CUR_BYTES_PAD + 2 * CTR_BYTES + SNAP_TILE_PAD + ACC_BYTES;
    static constexpr int STAGE_TX = CUR_BYTES + 2 * CTR_BYTES + SNAP_TILE + ACC_BYTES;
    static constexpr int SMEM = STAGES * STAGE_BYTES + EXTRA_BYTES;
    static constexpr int FIT = SM_SMEM / (SMEM + 1024);
    static constexpr int MINB = FIT < 4 ? FIT : 4;       // resident CTAs per SM
};

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

// Four consecutive snapshot values: 8 B for the 16-bit kinds, 16 B for FP32.
template <int K>
struct Snap4 {
    using T = typename std::conditional<K == SNAP_FP32, float4, uint2>::type;
};

template <int K>
__device__ __forceinline__ void snap_store4(void* p, long long i, const float v[4]) {
    if constexpr (K == SNAP_BF16) {
        __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]), b = __floats2bfloat162_rn(v[2], v[3]);
        uint2 w;
        w.x = *reinterpret_cast<unsigned*>(&a);
        w.y = *reinterpret_cast<unsigned*>(&b);
        *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(p) + i) = w;
    } else if constexpr (K == SNAP_FP16) {
        __half2 a = __floats2half2_rn(v[0], v[1]), b = __floats2half2_rn(v[2], v[3]);
        uint2 w;
        w.x = *reinterpret_cast<unsigned*>(&a);
        w.y = *reinterpret_cast<unsigned*>(&b);
        *reinterpret_cast<uint2*>(reinterpret_cast<__half*>(p) + i) = w;
    } else {
        *reinterpret_cast<float4*>(reinterpret_cast<float*>(p) + i) = make_float4(v[0], v[1], v[2], v[3]);
    }
}

template <int K>
__device__ __forceinline__ typename Snap4<K>::T snap_raw4(const void* p, long long i) {
    if constexpr (K == SNAP_FP32) return *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(p) + i);
    else return *reinterpret_cast<const uint2*>(reinterpret_cast<const unsigned short*>(p) + i);
}

template <int K>
__device__ __forceinline__ void snap_unpack4(const typename Snap4<K>::T& w, float f[4]) {
    if constexpr (K == SNAP_BF16) {
        uint2 ww = w;
        const float2 a = __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&ww.x));
        const float2 b = __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&ww.y));
        f[0] = a.x; f[1] = a.y; f[2] = b.x; f[3] = b.y;
    } else if constexpr (K == SNAP_FP16) {
        uint2 ww = w;
        const float2 a = __half22float2(*reinterpret_cast<__half2*>(&ww.x));
        const float2 b = __half22float2(*reinterpret_cast<__half2*>(&ww.y));
        f[0] = a.x; f[1] = a.y; f[2] = b.x; f[3] = b.y;
    } else {
        f[0] = w.x; f[1] = w.y; f[2] = w.z; f[3] = w.w;
    }
}

// Shared-memory snapshot value (element offset e of a tile) as float.
template <int K>
__device__ __forceinline__ float snap_smem1(const unsigned char* tile, int e) {
    if constexpr (K == SNAP_BF16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(tile)[e]);
    else if constexpr (K == SNAP_FP16) return __half2float(reinterpret_cast<const __half*>(tile)[e]);
    else return reinterpret_cast<const float*>(tile)[e];
}

// Four consecutive shared-memory snapshot values at element offset e (aligned).
template <int K>
__device__ __forceinline__ void snap_smem4(const unsigned char* tile, int e, float f[4]) {
    if constexpr (K == SNAP_FP32) {
        const float4 v = *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(tile) + e);
        f[0] = v.x; f[1] = v.y; f[2] = v.z; f[3] = v.w;
    } else {
        const uint2 w = *reinterpret_cast<const uint2*>(reinterpret_cast<const unsigned short*>(tile) + e);
        snap_unpack4<K>(w, f);
    }
}

__device__ __forceinline__ void f4_to(const float4& v, float a[4]) {
    a[0] = v.x;
    a[1] = v.y;
    a[2] = v.z;
    a[3] = v.w;
}

// The update of one point: out = 2u - upd + c * L u, upd = D * prev.
__device__ __forceinline__ float update_fast(float u, float upd, float xm, float xp, float ym, float yp, float zm,
                                             float zp, float c, float ax, float ay, float az) {
    const float lap = fmaf(-2.0f, u, xp + xm) * ax + fmaf(-2.0f, u, yp + ym) * ay + fmaf(-2.0f, u, zp + zm) * az;
    return fmaf(c, lap, fmaf(2.0f, u, -upd));
}

// The reference's guarded update (wave_equation.cpp:342-399), taken only when
// the fast result is non-finite or beyond the amplitude limit. A non-finite
// input always makes the fast result non-finite (c, 1/d^2 > 0), so the fast
// path is exact whenever it is taken. GINL: inlined at the call site (the
// two-step kernels measured faster so); otherwise one out-of-line copy
// shared by the call sites.
template <bool GINL = false>
__device__ __forceinline__ float update_guarded(float u, float upd, float xm, float xp, float ym, float yp, float zm,
                                                float zp, float c, float ax, float ay, float az, float amp,
                                                int* fired);
__device__ __forceinline__ float guarded_body(float u, float upd, float xm, float xp, float ym, float yp, float zm,
                                              float zp, float c, float ax, float ay, float az, float amp,
                                              int* fired) {
    if (!isfinite(u) || !isfinite(upd)) {
        *fired = 1;
        return 0.0f;
    }
    if (!isfinite(xm) || !isfinite(xp) || !isfinite(ym) || !isfinite(yp) || !isfinite(zm) || !isfinite(zp)) {
        *fired = 1;
        return u;
    }
    float nv = update_fast(u, upd, xm, xp, ym, yp, zm, zp, c, ax, ay, az);
    if (!isfinite(nv)) {
        nv = u;
        *fired = 1;
    }
    return fminf(fmaxf(nv, -amp), amp);
}
__device__ __noinline__ float guarded_call(float u, float upd, float xm, float xp, float ym, float yp, float zm,
                                           float zp, float c, float ax, float ay, float az, float amp, int* fired) {
    return guarded_body(u, upd, xm, xp, ym, yp, zm, zp, c, ax, ay, az, amp, fired);
}
template <bool GINL>
__device__ __forceinline__ float update_guarded(float u, float upd, float xm, float xp, float ym, float yp, float zm,
                                                float zp, float c, float ax, float ay, float az, float amp,
                                                int* fired) {
    if constexpr (GINL) return guarded_body(u, upd, xm, xp, ym, yp, zm, zp, c, ax, ay, az, amp, fired);
    else return guarded_call(u, upd, xm, xp, ym, yp, zm, zp, c, ax, ay, az, amp, fired);
}

// Per-row bookkeeping of one thread (4 consecutive z of one y row).
struct RowCtx {
    int iy;
    bool active;
    int dy;      // sponge distance along y
    int iry;     // receiver y index, -1 if the row holds no receiver
    bool inj;    // the fused injection point lies in this row
};

// Update of the 4 points of one row of plane x and its fused epilogue.
// fin: imaging -> dequantised forward snapshot; gradient -> L(snapshot) (dequantised).
template <int SNAP_OUT, int SNAP_IN, int EPI>
__device__ __forceinline__ void process_row(const StepArgs& a, const RowCtx& R, int x, int zvalid, const int dz[4],
                                            bool zfar, int dxx, const float* dtab, const float um[4],
                                            const float u0[4], const float up[4], const float ym[4],
                                            const float yp[4], float zm0, float zp3, const float pv[4],
                                            const float cv[4], int rk, int irx, int inj_k, float snap_inv,
                                            float& amax, int* fired, long long obase, long long cbase,
                                            const float fin[4], const float4& acc0, const float4& acc1,
                                            bool vec_acc) {
    float D[4];
    const int dxy = min(R.dy, dxx);
    if (zfar && dxy >= a.sw) {
#pragma unroll
        for (int k = 0; k < 4; ++k) D[k] = 1.0f;
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int d = min(dxy, dz[k]);
            D[k] = (d >= 0 && d < a.sw) ? dtab[d] : 1.0f;
        }
    }
    float res[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float zm = k == 0 ? zm0 : u0[k - 1];
        const float zp = k == 3 ? zp3 : u0[k + 1];
        const float upd = D[k] * pv[k];
        float nv = update_fast(u0[k], upd, um[k], up[k], ym[k], yp[k], zm, zp, cv[k], a.ax, a.ay, a.az);
        if (!(fabsf(nv) <= a.amp))
            nv = update_guarded(u0[k], upd, um[k], up[k], ym[k], yp[k], zm, zp, cv[k], a.ax, a.ay, a.az, a.amp,
                                fired);
        res[k] = nv;
    }
    // Receivers: the adjoint forcing enters before the damping of the new
    // field (stable sponge), the forward samples read the stored value. The
    // two never meet in one step.
    const bool rec_here = rk >= 0 && irx >= 0 && R.iry >= 0;
    const int q = rec_here ? irx * a.rny + R.iry : 0;
    if (rec_here && a.force_row) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k == rk) res[k] = fmaf(cv[k], a.force_row[q], res[k]);
    }
    if (a.stable_sponge) {
#pragma unroll
        for (int k = 0; k < 4; ++k) res[k] *= D[k];
    }
    if constexpr (EPI == EPI_MASK) {  // terrain masks: the column's points above its z limit hold 0
        const long long col = (long long)x * a.ny + R.iy;
        const int zl = a.zlim[col] - (int)(cbase - col * a.nz);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < zl) res[k] = 0.0f;
    }
    if (rec_here && a.seis_row) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k == rk) a.seis_row[q] = res[k];
    }
    if (R.inj && x == a.inj_x) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k == inj_k) res[k] += a.inj_val;
    }
    if (!R.active) return;
    if (zvalid == 4) {
        *reinterpret_cast<float4*>(a.out + obase) = make_float4(res[0], res[1], res[2], res[3]);
    } else {
        for (int k = 0; k < zvalid; ++k) a.out[obase + k] = res[k];
    }
    if constexpr (SNAP_OUT != SNAP_NONE) {
        float q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = u0[k] * snap_inv;
        if (zvalid == 4 && (a.nz & 3) == 0) {
            snap_store4<SNAP_OUT>(a.snap_out, cbase, q);
        } else {
            for (int k = 0; k < zvalid; ++k) snap_store<SNAP_OUT>(a.snap_out, cbase + k, q[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < zvalid) amax = fmaxf(amax, fabsf(res[k]));
    }
    if constexpr (is_image(EPI)) {
        if (vec_acc) {
            float im[4], il[4];
            f4_to(acc0, im);
            f4_to(acc1, il);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float f = fin[k];
                float ad = __fdividef(u0[k], a.stable_sponge ? cv[k] * D[k] : cv[k]);
                if (!isfinite(f)) f = 0.0f;
                if (!isfinite(ad)) ad = 0.0f;
                im[k] = fmaf(f, ad, im[k]);
                il[k] = fmaf(f, f, il[k]);
            }
            *reinterpret_cast<float4*>(a.image + cbase) = make_float4(im[0], im[1], im[2], im[3]);
            *reinterpret_cast<float4*>(a.illum + cbase) = make_float4(il[0], il[1], il[2], il[3]);
        } else {
            const float sc = __uint_as_float(*a.amax_in) / SNAP_QMAX;
            for (int k = 0; k < zvalid; ++k) {
                float f = snap_load<SNAP_IN>(a.snap_in, cbase + k) * sc;
                float ad = __fdividef(u0[k], a.stable_sponge ? cv[k] * D[k] : cv[k]);
                if (!isfinite(f)) f = 0.0f;
                if (!isfinite(ad)) ad = 0.0f;
                a.image[cbase + k] += f * ad;
                a.illum[cbase + k] += f * f;
            }
        }
    }
    if constexpr (EPI == EPI_GRAD) {
        if (vec_acc) {
            float g[4];
            f4_to(acc0, g);
#pragma unroll
            for (int k = 0; k < 4; ++k) g[k] = fmaf(__fdividef(u0[k], cv[k]), fin[k], g[k]);
            *reinterpret_cast<float4*>(a.grad + cbase) = make_float4(g[0], g[1], g[2], g[3]);
        } else {
            for (int k = 0; k < zvalid; ++k) a.grad[cbase + k] += __fdividef(u0[k], cv[k]) * fin[k];
        }
    }
}

template <int SNAP_OUT, int SNAP_IN, int EPI>
__global__ void __launch_bounds__(NTHREADS, (Geo<EPI, SNAP_IN>::MINB))
    fd_step_kernel(const __grid_constant__ CUtensorMap map_cur, const __grid_constant__ CUtensorMap map_prev,
                   const __grid_constant__ CUtensorMap map_c, const __grid_constant__ CUtensorMap map_snap,
                   const __grid_constant__ CUtensorMap map_img, const __grid_constant__ CUtensorMap map_ill,
                   const StepArgs a) {
    using G = Geo<EPI, SNAP_IN>;
    constexpr int STAGES = G::STAGES;
    constexpr int RPT = G::RPT;
    constexpr int TYV = G::TYV;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + STAGES * G::STAGE_BYTES);
    float* red = reinterpret_cast<float*>(smem + STAGES * G::STAGE_BYTES + 64);
    float* dtab_s = reinterpret_cast<float*>(smem + STAGES * G::STAGE_BYTES + 128);

    const int tid = threadIdx.x;
    const int tz4 = tid % TZ4;
    const int yp2 = tid / TZ4;  // thread row within the tile (owns rows RPT*yp2 ..)
    const int z0 = blockIdx.x * TZ;
    const int y0 = blockIdx.y * TYV;
    const int xa = blockIdx.z * a.x_chunk;
    const int xb = min(xa + a.x_chunk, a.nx);
    if (xa >= xb) return;  // uniform over the CTA
    const int nplanes = xb - xa + 2;

    const int iz0 = z0 + 4 * tz4;
    const int zvalid = min(4, a.nz - iz0);
    int dz[4];
    bool zfar = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        dz[k] = min(iz0 + k, a.nz - 1 - (iz0 + k));
        zfar = zfar && dz[k] >= a.sw;
    }
    RowCtx RA, RB;
    RA.iy = y0 + RPT * yp2;
    RB.iy = RA.iy + 1;
    RA.active = RA.iy < a.ny && zvalid > 0;
    RB.active = RPT == 2 && RB.iy < a.ny && zvalid > 0;
    RA.dy = min(RA.iy, a.ny - 1 - RA.iy);
    RB.dy = min(RB.iy, a.ny - 1 - RB.iy);
    int rk = -1;
    RA.iry = RB.iry = -1;
    if (a.seis_row || a.force_row) {
        const int kk = a.rz - iz0;
        if (kk >= 0 && kk < zvalid) rk = kk;
        const int ya = RA.iy - a.ry0, yb = RB.iy - a.ry0;
        if (RA.active && ya >= 0 && ya % a.rsy == 0 && ya / a.rsy < a.rny) RA.iry = ya / a.rsy;
        if (RPT == 2 && RB.active && yb >= 0 && yb % a.rsy == 0 && yb / a.rsy < a.rny) RB.iry = yb / a.rsy;
    }
    const int inj_k = (a.inj_x >= 0) ? a.inj_z - iz0 : -1;
    RA.inj = a.inj_x >= 0 && a.inj_y == RA.iy && inj_k >= 0 && inj_k < zvalid;
    RB.inj = RPT == 2 && a.inj_x >= 0 && a.inj_y == RB.iy && inj_k >= 0 && inj_k < zvalid;

    float snap_inv = 0.0f;
    if constexpr (SNAP_OUT != SNAP_NONE) {
        const float m = __uint_as_float(*a.amax_cur);
        snap_inv = m > 0.0f ? SNAP_QMAX / m : 0.0f;
    }
    float snap_scale = 1.0f;
    const bool vec_acc = !is_forward(EPI) && (a.nz & 3) == 0 && zvalid == 4;
    if constexpr (!is_forward(EPI)) snap_scale = __uint_as_float(*a.amax_in) / SNAP_QMAX;

    const bool tab_smem = a.sw <= DTAB_MAX;
    if (tab_smem)
        for (int i = tid; i < a.sw; i += NTHREADS) dtab_s[i] = a.dtab[i];
    const float* dtab = tab_smem ? dtab_s : a.dtab;

    auto cur_tile = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES); };
    auto prev_tile = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::CUR_BYTES_PAD); };
    auto c_tile = [&](int s) {
        return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::CUR_BYTES_PAD + G::CTR_BYTES);
    };
    auto snap_tile = [&](int s) {
        return reinterpret_cast<const unsigned char*>(smem + s * G::STAGE_BYTES + G::CUR_BYTES_PAD +
                                                      2 * G::CTR_BYTES);
    };
    auto img_tile = [&](int s) {
        return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::CUR_BYTES_PAD + 2 * G::CTR_BYTES +
                                        G::SNAP_TILE_PAD);
    };
    auto ill_tile = [&](int s) { return img_tile(s) + TZ * TYV; };

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    // plane index i in [0, nplanes) is interior x = xa - 1 + i, device x = xa + i
    auto issue = [&](int i) {
        const int s = i % STAGES;
        const int xd = xa + i;
        if (i + 1 == a.withhold) return;  // fault-path test hook: this stage never completes
        mbar_arrive_expect_tx(&bar[s], G::STAGE_TX);
        tma_load_3d(cur_tile(s), &map_cur, &bar[s], z0, y0, xd);
        tma_load_3d(prev_tile(s), &map_prev, &bar[s], z0 + Layout::ZOFF, y0 + 1, xd);
        tma_load_3d(c_tile(s), &map_c, &bar[s], z0 + Layout::ZOFF, y0 + 1, xd);
        if constexpr (EPI == EPI_GRAD)
            tma_load_4d(const_cast<unsigned char*>(snap_tile(s)), &map_snap, &bar[s], z0 - G::SOFF, y0 - 1, xd - 1,
                        a.snap_t);
        if constexpr (EPI == EPI_IMAGE_T) {
            // compact interior tiles of interior plane xd - 1 (zero outside the domain)
            tma_load_4d(const_cast<unsigned char*>(snap_tile(s)), &map_snap, &bar[s], z0, y0, xd - 1, a.snap_t);
            tma_load_3d(img_tile(s), &map_img, &bar[s], z0, y0, xd - 1);
            tma_load_3d(ill_tile(s), &map_ill, &bar[s], z0, y0, xd - 1);
        }
    };
    int issued = 0;
    if (tid == 0) {
        issued = min(STAGES, nplanes);
        for (int i = 0; i < issued; ++i) issue(i);
    }

    const int rowA = (RPT * yp2 + 1) * CUR_W + 4 * tz4 + 4;  // centre of row A in a cur tile
    const int rowB = rowA + CUR_W;
    const int ctrA = (RPT * yp2) * TZ + 4 * tz4;              // row A in prev / c tiles
    const int ctrB = ctrA + TZ;
    const int srowA = (RPT * yp2 + 1) * G::SW + 4 * tz4 + G::SOFF;  // row A in a snapshot tile
    float umA[4] = {0, 0, 0, 0}, u0A[4] = {0, 0, 0, 0}, umB[4] = {0, 0, 0, 0}, u0B[4] = {0, 0, 0, 0};
    float smA[4] = {0, 0, 0, 0};  // snapshot centres of plane x-1 (gradient)
    float amax_local = 0.0f;
    int fired = 0;
    int timed_out = 0;

    // epilogue operands of the next plane, loaded one plane ahead
    using SR = typename Snap4<(SNAP_IN == SNAP_NONE ? SNAP_FP32 : SNAP_IN)>::T;
    SR snA{}, snB{};
    float4 a0A{}, a0B{}, a1A{}, a1B{};
    // Imaging loads its operands at use (more resident warps hide them better
    // than holding them in registers a plane ahead); the gradient prefetches
    // its single accumulator.
    constexpr bool kPrefetch = EPI == EPI_GRAD;
    auto prefetch = [&](int x) {
        if constexpr (EPI == EPI_IMAGE || EPI == EPI_GRAD) {
            if (!vec_acc || x >= xb) return;
            const long long ca = ((long long)x * a.ny + RA.iy) * a.nz + iz0;
            const long long cb = ca + a.nz;
            if constexpr (EPI == EPI_IMAGE) {
                if (RA.active) {
                    snA = snap_raw4<SNAP_IN>(a.snap_in, ca);
                    a0A = *reinterpret_cast<const float4*>(a.image + ca);
                    a1A = *reinterpret_cast<const float4*>(a.illum + ca);
                }
                if (RPT == 2 && RB.active) {
                    snB = snap_raw4<SNAP_IN>(a.snap_in, cb);
                    a0B = *reinterpret_cast<const float4*>(a.image + cb);
                    a1B = *reinterpret_cast<const float4*>(a.illum + cb);
                }
            } else {
                if (RA.active) a0A = *reinterpret_cast<const float4*>(a.grad + ca);
                if (RPT == 2 && RB.active) a0B = *reinterpret_cast<const float4*>(a.grad + cb);
            }
        }
    };
    if constexpr (kPrefetch) prefetch(xa);

    int i = 0;
    for (; i < nplanes; ++i) {
        const int s = i % STAGES;
        if (!mbar_wait_bounded(&bar[s], (i / STAGES) & 1, a.timeout_ns)) timed_out = 1;
        float upA[4], upB[4] = {0, 0, 0, 0};
        f4_to(*reinterpret_cast<const float4*>(cur_tile(s) + rowA), upA);
        if constexpr (RPT == 2) f4_to(*reinterpret_cast<const float4*>(cur_tile(s) + rowB), upB);
        if (i >= 2) {
            const int sp = (i - 1) % STAGES;
            const int x = xa + i - 2;
            const float* T = cur_tile(sp);
            // y neighbours: row A's y- from the tile; with two rows, row A's y+ is
            // row B's centre and row B's y- is row A's centre
            float ymA[4], ypA[4], ypB[4] = {0, 0, 0, 0}, pvA[4], pvB[4] = {0, 0, 0, 0}, cvA[4],
                cvB[4] = {0, 0, 0, 0};
            f4_to(*reinterpret_cast<const float4*>(T + rowA - CUR_W), ymA);
            if constexpr (RPT == 2) {
                f4_to(*reinterpret_cast<const float4*>(T + rowB + CUR_W), ypB);
#pragma unroll
                for (int k = 0; k < 4; ++k) ypA[k] = u0B[k];
            } else {
                f4_to(*reinterpret_cast<const float4*>(T + rowA + CUR_W), ypA);
            }
            f4_to(*reinterpret_cast<const float4*>(prev_tile(sp) + ctrA), pvA);
            f4_to(*reinterpret_cast<const float4*>(c_tile(sp) + ctrA), cvA);
            if constexpr (RPT == 2) {
                f4_to(*reinterpret_cast<const float4*>(prev_tile(sp) + ctrB), pvB);
                f4_to(*reinterpret_cast<const float4*>(c_tile(sp) + ctrB), cvB);
            }
            float zmA = __shfl_up_sync(FULL, u0A[3], 1, TZ4);
            float zpA = __shfl_down_sync(FULL, u0A[0], 1, TZ4);
            float zmB = 0.0f, zpB = 0.0f;
            if constexpr (RPT == 2) {
                zmB = __shfl_up_sync(FULL, u0B[3], 1, TZ4);
                zpB = __shfl_down_sync(FULL, u0B[0], 1, TZ4);
            }
            if (tz4 == 0) {
                zmA = T[rowA - 1];
                if constexpr (RPT == 2) zmB = T[rowB - 1];
            }
            if (tz4 == TZ4 - 1) {
                zpA = T[rowA + 4];
                if constexpr (RPT == 2) zpB = T[rowB + 4];
            }
            const int dxx = min(x, a.nx - 1 - x);
            int irx = -1;
            if (rk >= 0) {
                const int xx = x - a.rx0;
                if (xx >= 0 && xx % a.rsx == 0 && xx / a.rsx < a.rnx) irx = xx / a.rsx;
            }
            const long long obA = (long long)(x + 1) * a.plane + (long long)(RA.iy + 1) * a.NZP + iz0 + Layout::ZOFF;
            const long long cbA = ((long long)x * a.ny + RA.iy) * a.nz + iz0;
            float finA[4] = {0, 0, 0, 0}, finB[4] = {0, 0, 0, 0};
            if constexpr (!kPrefetch) prefetch(x);  // operands of this plane, at use
            if constexpr (EPI == EPI_IMAGE_T) {
                // operands staged with the plane's tiles
                snap_smem4<SNAP_IN>(snap_tile(sp), ctrA, finA);
#pragma unroll
                for (int k = 0; k < 4; ++k) finA[k] *= snap_scale;
                a0A = *reinterpret_cast<const float4*>(img_tile(sp) + ctrA);
                a1A = *reinterpret_cast<const float4*>(ill_tile(sp) + ctrA);
            }
            if constexpr (EPI == EPI_IMAGE) {
                snap_unpack4<SNAP_IN>(snA, finA);
                if constexpr (RPT == 2) snap_unpack4<SNAP_IN>(snB, finB);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    finA[k] *= snap_scale;
                    finB[k] *= snap_scale;
                }
            }
            if constexpr (EPI == EPI_GRAD) {
                // 7-point Laplacian of the forward snapshot V_t (zero halo from the TMA fill);
                // the gradient variant runs one row per thread
                const unsigned char* S = snap_tile(sp);
                const unsigned char* Sn = snap_tile(s);
                float s0A[4], spA[4], symA[4], sypA[4];
                snap_smem4<SNAP_IN>(S, srowA, s0A);
                snap_smem4<SNAP_IN>(Sn, srowA, spA);
                snap_smem4<SNAP_IN>(S, srowA - G::SW, symA);
                snap_smem4<SNAP_IN>(S, srowA + G::SW, sypA);
                float szmA = __shfl_up_sync(FULL, s0A[3], 1, TZ4);
                float szpA = __shfl_down_sync(FULL, s0A[0], 1, TZ4);
                if (tz4 == 0) szmA = snap_smem1<SNAP_IN>(S, srowA - 1);
                if (tz4 == TZ4 - 1) szpA = snap_smem1<SNAP_IN>(S, srowA + 4);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float zm_ = k == 0 ? szmA : s0A[k - 1], zp_ = k == 3 ? szpA : s0A[k + 1];
                    finA[k] = snap_scale * (fmaf(-2.0f, s0A[k], spA[k] + smA[k]) * a.ax +
                                            fmaf(-2.0f, s0A[k], sypA[k] + symA[k]) * a.ay +
                                            fmaf(-2.0f, s0A[k], zp_ + zm_) * a.az);
                    smA[k] = s0A[k];
                }
            }
            const float4 a0A0 = a0A, a1A0 = a1A, a0B0 = a0B, a1B0 = a1B;
            if constexpr (kPrefetch) prefetch(x + 1);
            process_row<SNAP_OUT, SNAP_IN, EPI>(a, RA, x, zvalid, dz, zfar, dxx, dtab, umA, u0A, upA, ymA, ypA, zmA,
                                                zpA, pvA, cvA, rk, irx, inj_k, snap_inv, amax_local, &fired, obA,
                                                cbA, finA, a0A0, a1A0, vec_acc);
            if constexpr (RPT == 2)
                process_row<SNAP_OUT, SNAP_IN, EPI>(a, RB, x, zvalid, dz, zfar, dxx, dtab, umB, u0B, upB, u0A, ypB,
                                                    zmB, zpB, pvB, cvB, rk, irx, inj_k, snap_inv, amax_local, &fired,
                                                    obA + a.NZP, cbA + a.nz, finB, a0B0, a1B0, vec_acc);
        } else if constexpr (EPI == EPI_GRAD) {
            if (i == 1) {
                // snapshot centres of plane xa-1 (zero outside the domain)
                const unsigned char* S = snap_tile((i - 1) % STAGES);
                snap_smem4<SNAP_IN>(S, srowA, smA);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            umA[k] = u0A[k];
            u0A[k] = upA[k];
            umB[k] = u0B[k];
            u0B[k] = upB[k];
        }
        // every thread is done with the slot of plane i-1: refill it
        if (__syncthreads_or(timed_out)) break;
        if (tid == 0 && i >= 1 && issued < nplanes) issue(issued++);
    }

    if (i < nplanes) {
        // A wait gave up: drain the copies still in flight (bounded), then leave.
        if (tid == 0) {
            for (int j = i; j < issued; ++j)
                if (j + 1 != a.withhold) mbar_wait_bounded(&bar[j % STAGES], (j / STAGES) & 1, WAIT_DRAIN_NS);
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

template <int SO, int SI, int EPI>
int launch_variant(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                   const CUtensorMap& msnap, StepArgs a, cudaStream_t st, const CUtensorMap* mimg = nullptr,
                   const CUtensorMap* mill = nullptr) {
    using G = Geo<EPI, SI>;
    constexpr int SMEM = G::SMEM;
    constexpr int ti = G::RPT == 2 ? 1 : 0;  // which tile height the maps were built for
    static bool configured = false;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!configured) {
            ST_CUDA(cudaFuncSetAttribute(fd_step_kernel<SO, SI, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM));
            configured = true;
        }
    }
    // The forward variants run best as one wave of long x-chunks; the imaging
    // and gradient variants (one row per thread, more resident CTAs) keep more
    // loads in flight with at least four waves of shorter chunks.
    const int chunks = fd_step_grid_chunks(L, G::TYV, G::MINB, is_forward(EPI) ? 1 : 4);
    a.x_chunk = (int)((L.nx + chunks - 1) / chunks);
    const int nch = (int)((L.nx + a.x_chunk - 1) / a.x_chunk);
    dim3 grid((unsigned)((L.nz + TZ - 1) / TZ), (unsigned)((L.ny + G::TYV - 1) / G::TYV), (unsigned)nch);
    const CUtensorMap& mi = mimg ? *mimg : msnap;  // unused unless EPI == EPI_IMAGE_T
    const CUtensorMap& ml = mill ? *mill : msnap;
    fd_step_kernel<SO, SI, EPI><<<grid, NTHREADS, SMEM, st>>>(mcur.cur[ti], mprev.ctr[ti], mc.ctr[ti], msnap, mi, ml,
                                                             a);
    ::stg::count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

// ---------------------------------------------------------------- two time steps per launch
//
// fd_step2_kernel<MODE, SK> runs two time steps in one launch: sub-step A
// computes u' = step(u, u_prev) on the 16 x 64 tile plus a one-cell y/z ring
// (recomputed by every tile that needs it), sub-step B computes
// u'' = step(u', u) on the tile from the ring held in shared memory. Each
// point is updated by the same arithmetic, in the same order, as two launches
// of fd_step_kernel, so the results are bit-identical.
//
// MODE_ADJ (the RTM imaging pass; SK = the snapshot kind read): adjoint steps
// t and t-1 with the receiver forcing of each, and the imaging terms of both
// steps accumulated in one read-modify-write of the image and illumination:
// 40 bytes per point per launch instead of 2 x 34 (read lambda_t,
// lambda_{t+1}, c, two snapshots, image, illumination; write lambda',
// lambda'', image, illumination).
// MODE_FWD (SK = the snapshot kind stored, or SNAP_NONE): forward steps t and
// t+1 with the receiver sampling and source injection of each. The launch
// stores the snapshots of its two input fields, u_t and u_{t-1}, whose scales
// are complete by then; the snapshot of u_{t+1} is left to the next launch,
// which reads it as its previous field. |u'| and |u''| are max-reduced into
// the scales of steps t+1 and t+2. 24 bytes per point per launch with 16-bit
// snapshots instead of 2 x 18.
// MODE_GRAD (the FWI gradient pass; SK = the snapshot kind read): adjoint
// steps t and t-1 with the receiver forcing of each, and grad += (lambda / c)
// * L(snapshot) of both steps in one read-modify-write: 32 bytes per point
// per launch with 16-bit snapshots instead of 2 x 26.
//
// Planes i = 0 .. n+3 of a CTA's chunk [xa, xb) (n = xb - xa) are interior
// x = xa - 2 + i. Stage i of the TMA ring carries the current field of plane
// i (rows y0-2 .. y0+17), the previous field and c of plane i (rows y0-1 ..
// y0+16) and, one plane behind, the operands of the adjoint modes at interior
// x = xa - 3 + i: for imaging the two snapshot tiles and the image and
// illumination tiles, for the gradient the two snapshot tiles with a one-cell
// y/z halo (also for the planes either side of the chunk) and the gradient
// tile. Iteration i runs sub-step A on plane i-1 and sub-step B (with the
// stores) on plane i-2.
enum Step2Mode : int { MODE_ADJ = 0, MODE_FWD = 1, MODE_GRAD = 2 };

template <int MODE, int SK>
struct Geo2 {
    static constexpr bool IMG = MODE == MODE_ADJ;
    static constexpr bool GRD = MODE == MODE_GRAD;
    // gradient: snapshot tiles with a one-cell y/z halo (box from z0 - GSOFF,
    // rows y0-1 .. y0+16), as the one-step gradient kernel stages them
    static constexpr int GSW = snap_bytes(SK) == 2 ? TZ + 16 : TZ + 8;
    static constexpr int GSOFF = snap_bytes(SK) == 2 ? 8 : 4;
    static constexpr int TYV = 16;
    static constexpr int W = TZ + 8;            // z from z0 - 4
    static constexpr int CUR_H = TYV + 4;       // rows y0 - 2 .. y0 + 17
    static constexpr int RING_H = TYV + 2;      // rows y0 - 1 .. y0 + 16
    static constexpr int CUR_BYTES = W * CUR_H * 4;
    static constexpr int RING_BYTES = W * RING_H * 4;
    static constexpr int RING_PAD = ((RING_BYTES + 127) / 128) * 128;
    static constexpr int SNAP_TILE = IMG ? TZ * TYV * snap_bytes(SK) : (GRD ? GSW * RING_H * snap_bytes(SK) : 0);
    static constexpr int SNAP_PAD = ((SNAP_TILE + 127) / 128) * 128;
    static constexpr int CTR = (IMG || GRD) ? TZ * TYV * 4 : 0;
    static constexpr int OFF_PREV = ((CUR_BYTES + 127) / 128) * 128;
    static constexpr int OFF_C = OFF_PREV + RING_PAD;
    static constexpr int OFF_SA = OFF_C + RING_PAD;
    static constexpr int OFF_SB = OFF_SA + SNAP_PAD;
    static constexpr int OFF_IMG = OFF_SB + SNAP_PAD;
    static constexpr int OFF_ILL = OFF_IMG + CTR;
    static constexpr int STAGE_BYTES = OFF_ILL + (IMG ? CTR : 0);
    static constexpr int TX_FIELDS = CUR_BYTES + 2 * RING_BYTES;
    static constexpr int TX_SNAPS = 2 * SNAP_TILE;         // the two snapshot tiles
    static constexpr int TX_ACC = (IMG ? 2 : 1) * CTR;     // image + illumination, or gradient
    // the forward stage is small enough for five slots at two CTAs per SM:
    // three planes in flight instead of one (256^3: 0.0901 ms with 3 stages,
    // 0.0827 with 4, 0.0820 with 5, 0.0826 with 6). The imaging mode's
    // stage fits three; a fourth, with its imaging tiles in a ring of three
    // slots of their own, measured slower (0.1380 against 0.1283 ms).
    static constexpr int STAGES = MODE == MODE_FWD ? 5 : 3;
    static constexpr int SMEM = STAGES * STAGE_BYTES + 2 * RING_PAD + EXTRA_BYTES;
    static constexpr int FIT = SM_SMEM / (SMEM + 1024);
    // two resident CTAs per SM: three (80 registers) spilled in the forward
    // mode and measured 0.1009 against 0.0941 ms per pair at 256^3 (3 stages)
    static constexpr int MINB = FIT < 2 ? FIT : 2;
};

// Receiver row index of y (iry) or column index of x (irx) on the receiver
// grid, or -1.
__device__ __forceinline__ int rec_line(int v, int v0, int sv, int nv) {
    const int d = v - v0;
    if (d < 0 || d % sv) return -1;
    return d / sv < nv ? d / sv : -1;
}

__device__ __forceinline__ void ld4(const float* p, float v[4]) { f4_to(*reinterpret_cast<const float4*>(p), v); }
__device__ __forceinline__ void st4(float* p, const float v[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// Four point updates in fd_step_kernel's order, first part: the update (the
// guarded form where the fast one is out of range). The caller then adds the
// adjoint receiver forcing, applies the stable damping (stable_damp4) and, in
// the forward mode, samples the receivers and injects the source.
template <bool GINL>
__device__ __forceinline__ void update4(const StepArgs& a, const float u0[4], const float pv[4], const float um[4],
                                        const float up[4], const float ym[4], const float yp[4], float zm0, float zp3,
                                        const float cv[4], const float D[4], float res[4], int* fired) {
    float upd[4];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float zm = k == 0 ? zm0 : u0[k - 1];
        const float zp = k == 3 ? zp3 : u0[k + 1];
        upd[k] = D[k] * pv[k];
        res[k] = update_fast(u0[k], upd[k], um[k], up[k], ym[k], yp[k], zm, zp, cv[k], a.ax, a.ay, a.az);
        bad = bad || !(fabsf(res[k]) <= a.amp);
    }
    if (bad) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (fabsf(res[k]) <= a.amp) continue;
            const float zm = k == 0 ? zm0 : u0[k - 1];
            const float zp = k == 3 ? zp3 : u0[k + 1];
            res[k] = update_guarded<GINL>(u0[k], upd[k], um[k], up[k], ym[k], yp[k], zm, zp, cv[k], a.ax, a.ay, a.az,
                                          a.amp, fired);
        }
    }
}

// The stable sponge mode damps the new values as well.
__device__ __forceinline__ void stable_damp4(const StepArgs& a, const float D[4], float res[4]) {
    if (a.stable_sponge) {
#pragma unroll
        for (int k = 0; k < 4; ++k) res[k] *= D[k];
    }
}

// Sponge factors of a 4-point group: D(min(dx, dyz)) for each point, formed
// as min(D(dx), D(dyz)) from the plane's x factor Dx and the y/z factors Dyz
// the thread looked up once (the table is non-decreasing in the distance and
// at most 1, so this is bit for bit the same).
__device__ __forceinline__ void sponge4f(float Dx, const float Dyz[4], float D[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) D[k] = fminf(Dx, Dyz[k]);
}

// Laplacian of a snapshot at the four z of a centre group, scaled, with the
// one-step gradient kernel's expression: S / Sn are the halo tiles (width SW)
// of planes x / x+1 and srow the group's offset there, sm the group's values
// at plane x-1.
template <int K, int SW>
__device__ __forceinline__ void snap_lap4(const unsigned char* S, const unsigned char* Sn, int srow,
                                          const float sm[4], const StepArgs& a, float scale, float out[4]) {
    float s0[4], spn[4], sym[4], syp[4];
    snap_smem4<K>(S, srow, s0);
    snap_smem4<K>(Sn, srow, spn);
    snap_smem4<K>(S, srow - SW, sym);
    snap_smem4<K>(S, srow + SW, syp);
    const float zm0 = snap_smem1<K>(S, srow - 1), zp3 = snap_smem1<K>(S, srow + 4);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float zm_ = k == 0 ? zm0 : s0[k - 1], zp_ = k == 3 ? zp3 : s0[k + 1];
        out[k] = scale * (fmaf(-2.0f, s0[k], spn[k] + sm[k]) * a.ax + fmaf(-2.0f, s0[k], syp[k] + sym[k]) * a.ay +
                          fmaf(-2.0f, s0[k], zp_ + zm_) * a.az);
    }
}

// What one iteration of fd_step2_kernel's plane loop runs, fixed at compile
// time by the loop position. Sub-step A: A_NONE (the first two planes),
// A_EDGE (a halo plane beside the chunk: the grid test at run time, no
// sampling, snapshots or maxima), A_OWN (a plane of the chunk). Sub-step B:
// B_NONE (the first four planes), B_ON.
enum : int { A_NONE, A_EDGE, A_OWN };
enum : int { B_NONE, B_ON };
template <int PA_, int PB_>
struct PlaneKind {
    static constexpr int PA = PA_, PB = PB_;
};

template <int MODE, int SK>
__global__ void __launch_bounds__(NTHREADS, (Geo2<MODE, SK>::MINB))
    fd_step2_kernel(const __grid_constant__ CUtensorMap map_cur, const __grid_constant__ CUtensorMap map_prev,
                    const __grid_constant__ CUtensorMap map_c, const __grid_constant__ CUtensorMap map_snap,
                    const __grid_constant__ CUtensorMap map_img, const __grid_constant__ CUtensorMap map_ill,
                    const StepArgs a) {
    using G = Geo2<MODE, SK>;
    constexpr bool ADJ = MODE == MODE_ADJ;     // adjoint steps with imaging
    constexpr bool GRD = MODE == MODE_GRAD;    // adjoint steps with the gradient
    constexpr bool FWD = MODE == MODE_FWD;
    constexpr bool BACK = !FWD;                // receiver forcing, snapshots read
    constexpr bool SNAPS = FWD && SK != SNAP_NONE;
    constexpr bool GINL = true;                // the guarded update inlined
    constexpr int W = G::W;
    constexpr int STAGES = G::STAGES;
    extern __shared__ __align__(128) unsigned char smem[];
    float* lbuf = reinterpret_cast<float*>(smem + STAGES * G::STAGE_BYTES);  // two ring planes
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + STAGES * G::STAGE_BYTES + 2 * G::RING_PAD);
    float* red = reinterpret_cast<float*>(smem + STAGES * G::STAGE_BYTES + 2 * G::RING_PAD + 64);
    float* dtab_s = reinterpret_cast<float*>(smem + STAGES * G::STAGE_BYTES + 2 * G::RING_PAD + 128);

    const int tid = threadIdx.x;
    const int tz4 = tid % TZ4;
    const int yr = tid / TZ4;
    const int z0 = blockIdx.x * TZ;
    const int y0 = blockIdx.y * G::TYV;
    const int xa = blockIdx.z * a.x_chunk;
    const int xb = min(xa + a.x_chunk, a.nx);
    if (xa >= xb) return;  // uniform over the CTA
    const int nplanes = xb - xa + 4;

    // the thread's tasks: the centre group (row yc, z zc .. zc+3) and, for
    // threads 0 .. 159 (warps 0-4), one point of sub-step A's ring: threads
    // 0-63 row y0-1 and 64-127 row y0+16 at z0 + (tid & 63), threads 128-159
    // the points z0-1 (even) and z0+64 (odd) of row y0 + (tid - 128) / 2.
    // One point per lane keeps the extra work of any warp to one scalar
    // update, so no warp holds the others up at the plane barrier.
    const int warp = tid >> 5, lane = tid & 31;
    (void)warp;
    (void)lane;
    const int zc = z0 + 4 * tz4;
    const int yc = y0 + yr;
    const bool cin = yc < a.ny && zc < a.nz;
    constexpr int NRING = 2 * TZ + 2 * G::TYV;
    static_assert(NRING <= NTHREADS, "one ring point per thread");
    const bool has_ring = tid < NRING;
    int yq, zq;
    if (tid < 2 * TZ) {
        yq = tid < TZ ? y0 - 1 : y0 + G::TYV;
        zq = z0 + (tid & (TZ - 1));
    } else {
        const int q = tid - 2 * TZ;
        yq = y0 + (q >> 1);
        zq = (q & 1) ? z0 + TZ : z0 - 1;
    }
    const bool ringin = has_ring && yq >= 0 && yq < a.ny && zq >= 0 && zq < a.nz;
    // y/z distances to the nearest face (sponge), fixed over the march
    int dyz_c[4];
    const int dyc = min(yc, a.ny - 1 - yc);
#pragma unroll
    for (int k = 0; k < 4; ++k) dyz_c[k] = min(dyc, min(zc + k, a.nz - 1 - (zc + k)));
    const int dyz_q = min(min(yq, a.ny - 1 - yq), min(zq, a.nz - 1 - zq));
    // receivers: forcing (adjoint) at every task, sampling (forward) at the
    // centre only; rk: the receiver plane's point in the centre group
    const bool recs = BACK ? (a.force_row || a.force_row2) : (a.seis_row || a.seis_row2);
    const int rk = (recs && a.rz >= zc && a.rz < zc + 4) ? a.rz - zc : -1;
    const int iry_c = rk >= 0 ? rec_line(yc, a.ry0, a.rsy, a.rny) : -1;
    const int iry_q = BACK && recs && ringin && zq == a.rz ? rec_line(yq, a.ry0, a.rsy, a.rny) : -1;
    const bool any_rec = iry_c >= 0 || iry_q >= 0;
    // forward source injection (a.inj_steps bit 0: sub-step A, bit 1: B) at
    // point inj_kc of the centre group, or the ring point
    const bool inj = FWD && a.inj_x >= 0;
    const int inj_kc = (inj && a.inj_y == yc && a.inj_z >= zc && a.inj_z < zc + 4) ? a.inj_z - zc : -1;
    const bool inj_q = inj && has_ring && a.inj_y == yq && a.inj_z == zq;
    // the thread holds a receiver or the source point: the only threads that
    // run the per-plane receiver and source work
    const bool special = any_rec || inj_kc >= 0 || inj_q;

    const bool tab_smem = a.sw <= DTAB_MAX;
    if (tab_smem)
        for (int i = tid; i < a.sw; i += NTHREADS) dtab_s[i] = a.dtab[i];
    // x factor of a plane: the shared copy of the table when it has one
    // (addressed as shared memory, not through a generic pointer)
    auto x_factor = [&](int dx) -> float {
        if (dx >= a.sw) return 1.0f;
        return tab_smem ? dtab_s[dx] : __ldg(a.dtab + dx);
    };
    // The sponge factor of a point is D(min(dx, dyz)) = min(D(dx), D(dyz)):
    // the table grows with the distance, so the y/z factors are looked up once
    // (from the global table: the shared copy is complete only after the
    // barrier below) and each plane takes one lookup for x.
    // (distances below 0 belong to points outside the grid, never updated)
    float Dc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) Dc[k] = (dyz_c[k] >= 0 && dyz_c[k] < a.sw) ? a.dtab[dyz_c[k]] : 1.0f;
    const float Dq = (dyz_q >= 0 && dyz_q < a.sw) ? a.dtab[dyz_q] : 1.0f;
    // imaging: snapshot scales of steps t and t-1; forward: inverse scales of
    // the two stored snapshots (u_t and u_{t-1})
    float scale_a = 0.0f, scale_b = 0.0f;
    if constexpr (BACK) {
        scale_a = __uint_as_float(*a.amax_in) / SNAP_QMAX;
        scale_b = __uint_as_float(*a.amax_in2) / SNAP_QMAX;
    }
    if constexpr (SNAPS) {
        const float m = __uint_as_float(*a.amax_cur);
        scale_a = m > 0.0f ? SNAP_QMAX / m : 0.0f;
        if (a.snap_out2) {
            const float mp = __uint_as_float(*a.amax_cur2);
            scale_b = mp > 0.0f ? SNAP_QMAX / mp : 0.0f;
        }
    }

    auto st_cur = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES); };
    auto st_prev = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::OFF_PREV); };
    auto st_c = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::OFF_C); };
    auto st_sa = [&](int s) { return smem + s * G::STAGE_BYTES + G::OFF_SA; };
    auto st_sb = [&](int s) { return smem + s * G::STAGE_BYTES + G::OFF_SB; };
    auto st_img = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::OFF_IMG); };
    auto st_ill = [&](int s) { return reinterpret_cast<float*>(smem + s * G::STAGE_BYTES + G::OFF_ILL); };
    auto lb = [&](int i) { return lbuf + (i & 1) * (G::RING_PAD / 4); };

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int i) {
        const int s = i % STAGES;
        if (i + 1 == a.withhold) return;  // fault-path test hook: this stage never completes
        const int xd = xa - 1 + i;  // device x of interior plane xa - 2 + i
        const int xi = xa - 3 + i;  // interior plane of the imaging / gradient operands
        const bool acc = (ADJ || GRD) && xi >= xa && xi < xb;
        // the gradient's snapshot Laplacian also reads the planes either side
        const bool snp = ADJ ? acc : (GRD && xi >= xa - 1 && xi <= xb);
        mbar_arrive_expect_tx(&bar[s], G::TX_FIELDS + (snp ? G::TX_SNAPS : 0) + (acc ? G::TX_ACC : 0));
        tma_load_3d(st_cur(s), &map_cur, &bar[s], z0, y0 - 1, xd);
        tma_load_3d(st_prev(s), &map_prev, &bar[s], z0, y0, xd);
        tma_load_3d(st_c(s), &map_c, &bar[s], z0, y0, xd);
        if constexpr (ADJ) {
            if (acc) {
                tma_load_4d(st_sa(s), &map_snap, &bar[s], z0, y0, xi, a.snap_t);
                tma_load_4d(st_sb(s), &map_snap, &bar[s], z0, y0, xi, a.snap_t - 1);
                tma_load_3d(st_img(s), &map_img, &bar[s], z0, y0, xi);
                tma_load_3d(st_ill(s), &map_ill, &bar[s], z0, y0, xi);
            }
        }
        if constexpr (GRD) {
            // x = z0 - GSOFF is 16 bytes left of the tile (negative at z0 = 0:
            // a load, zero-filled there, as the rows beyond the grid)
            if (snp) {
                tma_load_4d(st_sa(s), &map_snap, &bar[s], z0 - G::GSOFF, y0 - 1, xi, a.snap_t);
                tma_load_4d(st_sb(s), &map_snap, &bar[s], z0 - G::GSOFF, y0 - 1, xi, a.snap_t - 1);
            }
            if (acc) tma_load_3d(st_img(s), &map_img, &bar[s], z0, y0, xi);
        }
    };
    int issued = 0;
    if (tid == 0) {
        issued = min(STAGES, nplanes);
        for (int i = 0; i < issued; ++i) issue(i);
    }

    const int tcen = (yr + 2) * W + 4 * tz4 + 4;                 // centre in a current-field tile
    const int tq = has_ring ? (yq - y0 + 2) * W + (zq - z0 + 4) : 0;  // ring point in a current-field tile
    const int rcen = tcen - W, rq = tq - W;                      // the same in ring-geometry tiles
    const int ccen = yr * TZ + 4 * tz4;                          // centre in the compact tiles
    const int gsrow = (yr + 1) * G::GSW + 4 * tz4 + G::GSOFF;    // centre in the gradient's snapshot tiles
    // current-field queues (x-1, x, x+1) of the centre group and of the ring
    // point, the u' queue of the centre (planes i-3, i-2, i-1) and c of the
    // centre at plane i-2. The queues have period 3 along x: in the forward
    // mode the plane loop is unrolled three times and each copy names the
    // slots in its own order, so the queues rotate by renaming, not by moves.
    float U[3][4] = {}, Qq[3] = {}, Lq[3][4] = {};
    float cprev[4] = {0, 0, 0, 0};
    float sm_a[4] = {0, 0, 0, 0}, sm_b[4] = {0, 0, 0, 0};  // gradient: snapshot centres at plane i-3
    int irx_prev = -1;  // receiver column of plane i-2
    float amax1 = 0.0f, amax2 = 0.0f;
    int fired = 0;
    int timed_out = 0;

    // stage of plane i (s), of plane i-1 (sp) and the phase parity of stage s,
    // kept by increment; 64-bit offsets of plane i-2's centre group in the
    // device-layout fields (ob) and in the compact volumes (cb), advanced by a
    // plane per iteration once sub-step B runs
    int s = 0, sp = STAGES - 1;
    unsigned parity = 0;
    long long ob = (long long)(xa + 1) * a.plane + (long long)(yc + 1) * a.NZP + zc + Layout::ZOFF;
    long long cb = ((long long)xa * a.ny + yc) * a.nz + zc;
    const long long cplane = (long long)a.ny * a.nz;
    int i = 0;
    // one plane; q0 / q1 / q2 are the queue slots of planes i-2 / i-1 / i
    // (for the u' queue: i-3 / i-2 / i-1); returns true when a wait gave up
    // cs / csp: the stage of plane i / i-1 (literals in the unrolled loops,
    // so every shared-memory address there is a constant offset); kind: a
    // PlaneKind, what the iteration runs
    auto plane = [&](auto kind, const int q0, const int q1, const int q2, const int cs, const int csp) -> bool {
        constexpr int PA = decltype(kind)::PA;
        constexpr int PB = decltype(kind)::PB;
        float(&um)[4] = U[q0];
        float(&up)[4] = U[q2];
        float& qm_ = Qq[q0];
        float& qp_ = Qq[q2];
        float(&lm)[4] = Lq[q0];
        float(&l0)[4] = Lq[q1];
        float(&lp)[4] = Lq[q2];
        if (!mbar_wait_bounded(&bar[cs], parity, a.timeout_ns)) timed_out = 1;
#pragma unroll
        for (int k = 0; k < 4; ++k) lp[k] = 0.0f;
        // qp_ is read only by the ring threads, which load it here
        ld4(st_cur(cs) + tcen, up);
        if (has_ring) qp_ = st_cur(cs)[tq];
        float cnow[4] = {0, 0, 0, 0};
        int irx = -1;
        constexpr bool runA = PA != A_NONE;
        constexpr bool runB = PB == B_ON;
        if (runA) {
            // sub-step A on plane i-1 (interior x = xa - 3 + i); it writes the
            // ring buffer of plane i-1, which no thread reads before the
            // barrier that ends this iteration
            const int x = xa - 3 + i;
            const bool xin = PA == A_OWN || (x >= 0 && x < a.nx);
            // this chunk's plane: sampling, snapshots, maxima
            const bool own = PA == A_OWN;
            (void)own;  // read by the forward mode only
            const int dx = min(x, a.nx - 1 - x);
            int irx_a = -1;  // receiver column of step t's receivers
            bool inj_a = false;
            if (special) {
                if (any_rec && xin) irx = rec_line(x, a.rx0, a.rsx, a.rnx);
                irx_a = (BACK ? a.force_row : a.seis_row) ? irx : -1;
                inj_a = inj && (a.inj_steps & 1) && x == a.inj_x;
            }
            const float* T = st_cur(csp);
            const float* P = st_prev(csp);
            const float* Cc = st_c(csp);
            float* Lw = lb(i - 1);
            const float Dx = xin ? x_factor(dx) : 1.0f;
            // centre
            ld4(Cc + rcen, cnow);
            if (xin && cin) {
                // the centre values of plane i-1: the queue slot loaded one iteration ago
                const float(&c0)[4] = U[q1];
                float pv[4], ym[4], yp[4], D[4];
                ld4(P + rcen, pv);
                ld4(T + tcen - W, ym);
                ld4(T + tcen + W, yp);
                sponge4f(Dx, Dc, D);
                update4<GINL>(a, c0, pv, um, up, ym, yp, T[tcen - 1], T[tcen + 4], cnow, D, lp, &fired);
                const bool rc = special && irx_a >= 0 && iry_c >= 0;
                const int q = rc ? irx_a * a.rny + iry_c : 0;
                if constexpr (BACK) {
                    if (rc) {
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (k == rk) lp[k] = fmaf(cnow[k], a.force_row[q], lp[k]);
                    }
                }
                stable_damp4(a, D, lp);
                if constexpr (FWD) {
                    if (special) {
                        if (own && rc) {
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                if (k == rk) a.seis_row[q] = lp[k];
                        }
                        if (inj_a) {
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                if (k == inj_kc) lp[k] += a.inj_val;
                        }
                    }
                    if constexpr (SNAPS) {
                        if (own) {
                            // plane x = xa - 3 + i: one plane past sub-step B's (cb),
                            // except at i = 3 where both name the chunk's first plane
                            const long long cbA = cb + (runB ? cplane : 0);
                            float qv[4];
#pragma unroll
                            for (int k = 0; k < 4; ++k) {
                                qv[k] = c0[k] * scale_a;
                                amax1 = fmaxf(amax1, fabsf(lp[k]));
                            }
                            snap_store4<SK>(a.snap_out, cbA, qv);
                            if (a.snap_out2) {
#pragma unroll
                                for (int k = 0; k < 4; ++k) qv[k] = pv[k] * scale_b;
                                snap_store4<SK>(a.snap_out2, cbA, qv);
                            }
                        }
                    }
                }
            }
            st4(Lw + rcen, lp);
            if (has_ring) {
                float res = 0.0f;
                if (xin && ringin) {
                    const float D = fminf(Dx, Dq);
                    const float u = Qq[q1], c = Cc[rq];  // u: loaded one iteration ago
                    const float upd = D * P[rq];
                    const float ym = T[tq - W], yp = T[tq + W], zm = T[tq - 1], zp = T[tq + 1];
                    res = update_fast(u, upd, qm_, qp_, ym, yp, zm, zp, c, a.ax, a.ay, a.az);
                    if (!(fabsf(res) <= a.amp))
                        res = update_guarded<GINL>(u, upd, qm_, qp_, ym, yp, zm, zp, c, a.ax, a.ay, a.az, a.amp,
                                                   &fired);
                    if (BACK && special && irx_a >= 0 && iry_q >= 0)
                        res = fmaf(c, a.force_row[irx_a * a.rny + iry_q], res);
                    if (a.stable_sponge) res *= D;
                    if (FWD && special && inj_a && inj_q) res += a.inj_val;
                }
                Lw[rq] = res;
            }
        }
        if (runB && cin) {
            // sub-step B and the stores on plane i-2 (interior x = xa - 4 + i),
            // from the ring buffer of plane i-2 (complete since the last barrier)
            const int x = xa - 4 + i;
            const float* Lr = lb(i - 2);
            const int dx = min(x, a.nx - 1 - x);
            float ym[4], yp[4], D[4], res[4];
            ld4(Lr + rcen - W, ym);
            ld4(Lr + rcen + W, yp);
            sponge4f(x_factor(dx), Dc, D);
            update4<GINL>(a, l0, um, lm, lp, ym, yp, Lr[rcen - 1], Lr[rcen + 4], cprev, D, res, &fired);
            const float* rows2 = BACK ? a.force_row2 : a.seis_row2;
            const bool rc = special && rows2 && irx_prev >= 0 && iry_c >= 0;
            const int q = rc ? irx_prev * a.rny + iry_c : 0;
            if constexpr (BACK) {
                if (rc) {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k == rk) res[k] = fmaf(cprev[k], a.force_row2[q], res[k]);
                }
            }
            stable_damp4(a, D, res);
            if constexpr (FWD) {
                if (special) {
                    if (rc) {
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (k == rk) a.seis_row2[q] = res[k];
                    }
                    if (inj && (a.inj_steps & 2) && x == a.inj_x) {
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (k == inj_kc) res[k] += a.inj_val2;
                    }
                }
                if constexpr (SNAPS) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) amax2 = fmaxf(amax2, fabsf(res[k]));
                }
            }
            st4(a.out + ob, l0);
            st4(a.out2 + ob, res);
            if constexpr (ADJ) {
                // imaging: step t pairs lambda_t with the snapshot of t, step t-1
                // pairs lambda' with the snapshot of t-1, in that order
                float fa[4], fb[4], im[4], il[4];
                snap_smem4<SK>(st_sa(csp), ccen, fa);
                snap_smem4<SK>(st_sb(csp), ccen, fb);
                ld4(st_img(csp) + ccen, im);
                ld4(st_ill(csp) + ccen, il);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float w = a.stable_sponge ? cprev[k] * D[k] : cprev[k];
                    float f = fa[k] * scale_a;
                    float ad = __fdividef(um[k], w);
                    if (!(fabsf(f) <= FLT_MAX)) f = 0.0f;  // not finite
                    if (!(fabsf(ad) <= FLT_MAX)) ad = 0.0f;
                    im[k] = fmaf(f, ad, im[k]);
                    il[k] = fmaf(f, f, il[k]);
                    f = fb[k] * scale_b;
                    ad = __fdividef(l0[k], w);
                    if (!(fabsf(f) <= FLT_MAX)) f = 0.0f;  // not finite
                    if (!(fabsf(ad) <= FLT_MAX)) ad = 0.0f;
                    im[k] = fmaf(f, ad, im[k]);
                    il[k] = fmaf(f, f, il[k]);
                }
                st4(a.image + cb, im);
                st4(a.illum + cb, il);
            }
            if constexpr (GRD) {
                // gradient: step t pairs lambda_t with L(snapshot of t), step t-1
                // pairs lambda' with L(snapshot of t-1), in that order
                float fa[4], fb[4], g[4];
                snap_lap4<SK, G::GSW>(st_sa(csp), st_sa(cs), gsrow, sm_a, a, scale_a, fa);
                snap_lap4<SK, G::GSW>(st_sb(csp), st_sb(cs), gsrow, sm_b, a, scale_b, fb);
                ld4(st_img(csp) + ccen, g);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    g[k] = fmaf(__fdividef(um[k], cprev[k]), fa[k], g[k]);
                    g[k] = fmaf(__fdividef(l0[k], cprev[k]), fb[k], g[k]);
                }
                st4(a.grad + cb, g);
            }
        }
        if constexpr (GRD) {
            // the snapshot centres of plane i-2 are the next plane's x-1 values
            if (i >= 3) {
                snap_smem4<SK>(st_sa(csp), gsrow, sm_a);
                snap_smem4<SK>(st_sb(csp), gsrow, sm_b);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) cprev[k] = cnow[k];
        irx_prev = irx;
        sp = s;
        if (++s == STAGES) {
            s = 0;
            parity ^= 1u;
        }
        if (runB) {
            ob += a.plane;
            cb += cplane;
        }
        // every thread is done with the slot of plane i-1 and the ring buffer
        // of plane i-2: refill the one, let the next iteration overwrite the other
        if (__syncthreads_or(timed_out)) return true;
        const bool refill = PA == A_NONE ? i >= 1 : true;
        if (tid == 0 && refill && issued < nplanes) issue(issued++);
        return false;
    };
    {
        // Every queue slot (and, with a 3-deep ring, every stage) is named by
        // a literal: the first four planes one by one, the planes where both
        // sub-steps run in a loop unrolled three times (the x-queues have
        // period 3 and rotate by renaming), then the last plane with its
        // queues moved to slots 0-2 and the stages from s / sp. A deeper ring
        // takes its stages from s / sp throughout.
        constexpr bool LIT = STAGES == 3;
        using KFill = PlaneKind<A_NONE, B_NONE>;
        using KHalo = PlaneKind<A_EDGE, B_NONE>;
        using KFirst = PlaneKind<A_OWN, B_NONE>;
        using KBoth = PlaneKind<A_OWN, B_ON>;
        using KLast = PlaneKind<A_EDGE, B_ON>;
        const int last = nplanes - 1;  // >= 4: a chunk holds at least one plane
        bool stop = plane(KFill{}, 0, 1, 2, LIT ? 0 : s, LIT ? 2 : sp);
        if (!stop) {
            ++i;
            stop = plane(KFill{}, 1, 2, 0, LIT ? 1 : s, LIT ? 0 : sp);
        }
        if (!stop) {
            ++i;
            stop = plane(KHalo{}, 2, 0, 1, LIT ? 2 : s, LIT ? 1 : sp);
        }
        if (!stop) {
            ++i;
            stop = plane(KFirst{}, 0, 1, 2, LIT ? 0 : s, LIT ? 2 : sp);
        }
        if (!stop) {
            ++i;
            int ph = 1;  // i % 3 at i = 4
            while (i < last) {
                if ((stop = plane(KBoth{}, 1, 2, 0, LIT ? 1 : s, LIT ? 0 : sp)) || ++i == last) {
                    ph = 2;
                    break;
                }
                if ((stop = plane(KBoth{}, 2, 0, 1, LIT ? 2 : s, LIT ? 1 : sp)) || ++i == last) {
                    ph = 0;
                    break;
                }
                if ((stop = plane(KBoth{}, 0, 1, 2, LIT ? 0 : s, LIT ? 2 : sp)) || ++i == last) {
                    ph = 1;
                    break;
                }
            }
            if (!stop) {
                // slots (p, p+1) of phase p hold planes i-2, i-1: move them to (0, 1)
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (ph == 1) {
                        U[0][k] = U[1][k];
                        U[1][k] = U[2][k];
                        Lq[0][k] = Lq[1][k];
                        Lq[1][k] = Lq[2][k];
                    } else if (ph == 2) {
                        const float tu = U[0][k], tl = Lq[0][k];
                        U[0][k] = U[2][k];
                        U[1][k] = tu;
                        Lq[0][k] = Lq[2][k];
                        Lq[1][k] = tl;
                    }
                }
                if (ph == 1) {
                    Qq[0] = Qq[1];
                    Qq[1] = Qq[2];
                } else if (ph == 2) {
                    const float tq_ = Qq[0];
                    Qq[0] = Qq[2];
                    Qq[1] = tq_;
                }
                if (!plane(KLast{}, 0, 1, 2, s, sp)) ++i;
            }
        }
    }

    if (i < nplanes) {
        // A wait gave up: drain the copies still in flight (bounded), then leave.
        if (tid == 0) {
            for (int j = i; j < issued; ++j)
                if (j + 1 != a.withhold) mbar_wait_bounded(&bar[j % STAGES], (j / STAGES) & 1, WAIT_DRAIN_NS);
            atomicOr(a.flags, FLAG_TIMEOUT);
        }
        __syncthreads();
        return;
    }
    if (fired) atomicOr(a.flags, FLAG_GUARD);
    if constexpr (SNAPS) {
        for (int o = 16; o > 0; o >>= 1) {
            amax1 = fmaxf(amax1, __shfl_xor_sync(FULL, amax1, o));
            amax2 = fmaxf(amax2, __shfl_xor_sync(FULL, amax2, o));
        }
        if (lane == 0) {
            red[warp] = amax1;
            red[NTHREADS / 32 + warp] = amax2;
        }
        __syncthreads();
        if (tid == 0) {
            float m1 = red[0], m2 = red[NTHREADS / 32];
            for (int w = 1; w < NTHREADS / 32; ++w) {
                m1 = fmaxf(m1, red[w]);
                m2 = fmaxf(m2, red[NTHREADS / 32 + w]);
            }
            atomicMax(a.amax_next, __float_as_uint(m1));
            atomicMax(a.amax_next2, __float_as_uint(m2));
        }
    }
}

template <int MODE, int SK>
int launch_step2_variant(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                         const ImageMaps* im, StepArgs a, cudaStream_t st) {
    using G = Geo2<MODE, SK>;
    static bool configured = false;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!configured) {
            ST_CUDA(cudaFuncSetAttribute(fd_step2_kernel<MODE, SK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         G::SMEM));
            configured = true;
        }
    }
    const int chunks = fd_step_grid_chunks(L, G::TYV, G::MINB, 1, 4);
    a.x_chunk = (int)((L.nx + chunks - 1) / chunks);
    const int nch = (int)((L.nx + a.x_chunk - 1) / a.x_chunk);
    dim3 grid((unsigned)((L.nz + TZ - 1) / TZ), (unsigned)((L.ny + G::TYV - 1) / G::TYV), (unsigned)nch);
    // the imaging maps are read only by the adjoint mode
    const CUtensorMap& ms = im ? im->snap : mc.cur[0];
    const CUtensorMap& mi = im ? im->image : mc.cur[0];
    const CUtensorMap& ml = im ? im->illum : mc.cur[0];
    fd_step2_kernel<MODE, SK><<<grid, NTHREADS, G::SMEM, st>>>(mcur.cur2, mprev.cur[0], mc.cur[0], ms, mi, ml, a);
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
// Snapshot of one field, as fd_step_kernel stores the snapshot of its centre
// field: v * (16384 / |max|) rounded to the store's kind, compact interior.
template <int K>
__global__ void snapshot_of_field_kernel(const float* __restrict__ f, Layout L, void* snap,
                                         const unsigned* amax) {
    const float m = __uint_as_float(*amax);
    const float inv = m > 0.0f ? SNAP_QMAX / m : 0.0f;
    const long long total = L.nx * L.ny * L.nz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long ix = e / (L.ny * L.nz);
        const long long r = e - ix * (L.ny * L.nz);
        const long long iy = r / L.nz;
        const long long iz = r - iy * L.nz;
        snap_store<K>(snap, e, f[L.at(ix, iy, iz)] * inv);
    }
}

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

int build_field_maps(FieldMaps* m, const float* base, const Layout& L) {
    for (int t = 0; t < 2; ++t) {
        const int rows = 16 << t;
        ST_TRY(make_field_map(&m->cur[t], base, L, TZ + 8, rows + 2));
        ST_TRY(make_field_map(&m->ctr[t], base, L, TZ, rows));
    }
    ST_TRY(make_field_map(&m->cur2, base, L, TZ + 8, 16 + 4));
    return ST_OK;
}

int fd_step_grid_chunks(const Layout& L, int tyv, int minb, int min_waves, int halo) {
    const long long gx = (L.nz + TZ - 1) / TZ, gy = (L.ny + tyv - 1) / tyv;
    const long long tiles = gx * gy;
    // tuning override: SEISMIC_GB300_XCHUNKS=<chunks> (1..nx)
    if (const char* env = std::getenv("SEISMIC_GB300_XCHUNKS")) {
        const long long v = std::atoll(env);
        if (v >= 1) return (int)std::min<long long>(v, L.nx);
    }
    // Split the x range into chunks so that the CTA count fills whole waves of
    // resident CTAs (SMs x resident CTAs per SM); each chunk re-reads `halo`
    // planes, a cost weighed in against shorter chunks.
    const double slots = (double)num_sms() * minb;
    long long best = 1;
    double best_eff = -1.0;
    const long long max_chunks = std::max<long long>(1, std::min<long long>(L.nx / 4, 256));
    const long long need = min_waves > 1 ? (long long)std::ceil(min_waves * slots / (double)tiles) : 1;
    const long long first = std::min<long long>(std::max<long long>(1, need), max_chunks);
    for (long long ch = first; ch <= max_chunks; ++ch) {
        const double waves = (double)(tiles * ch) / slots;
        const double fill = waves / std::ceil(waves);
        const double len = std::ceil((double)L.nx / (double)ch);
        const double eff = fill / (1.0 + (double)halo / len);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = ch;
        }
    }
    return (int)best;
}

int launch_fd_step(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                   StepArgs a, int snap_out, int snap_in, int epi, const CUtensorMap* msnap, cudaStream_t st,
                   const ImageMaps* imaps) {
    a.nx = (int)L.nx;
    a.ny = (int)L.ny;
    a.nz = (int)L.nz;
    a.NZP = (int)L.NZP;
    a.plane = L.plane;
    if (a.timeout_ns == 0) a.timeout_ns = 2000000000ull;
    ST_CHECK(!a.zlim || epi == EPI_NONE, ST_ERR_UNSUPPORTED, "terrain limits apply to plain forward steps only");
    const CUtensorMap& ms = msnap ? *msnap : mc.ctr[0];  // unused unless epi == gradient
    if (epi == EPI_IMAGE && imaps) {
        // operands staged by TMA: snapshot store map (box {64, 16}), image and illumination maps
        ST_CHECK(snap_out == SNAP_NONE, ST_ERR_ARG, "imaging step cannot also store snapshots");
        switch (snap_in) {
            case SNAP_BF16:
                return launch_variant<SNAP_NONE, SNAP_BF16, EPI_IMAGE_T>(L, mcur, mprev, mc, imaps->snap, a, st,
                                                                         &imaps->image, &imaps->illum);
            case SNAP_FP16:
                return launch_variant<SNAP_NONE, SNAP_FP16, EPI_IMAGE_T>(L, mcur, mprev, mc, imaps->snap, a, st,
                                                                         &imaps->image, &imaps->illum);
            case SNAP_FP32:
                return launch_variant<SNAP_NONE, SNAP_FP32, EPI_IMAGE_T>(L, mcur, mprev, mc, imaps->snap, a, st,
                                                                         &imaps->image, &imaps->illum);
            default: ST_CHECK(false, ST_ERR_ARG, "imaging step needs a snapshot kind");
        }
    }
    if (epi == EPI_IMAGE) {
        ST_CHECK(snap_out == SNAP_NONE, ST_ERR_ARG, "imaging step cannot also store snapshots");
        switch (snap_in) {
            case SNAP_BF16: return launch_variant<SNAP_NONE, SNAP_BF16, EPI_IMAGE>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_FP16: return launch_variant<SNAP_NONE, SNAP_FP16, EPI_IMAGE>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_FP32: return launch_variant<SNAP_NONE, SNAP_FP32, EPI_IMAGE>(L, mcur, mprev, mc, ms, a, st);
            default: ST_CHECK(false, ST_ERR_ARG, "imaging step needs a snapshot kind");
        }
    }
    if (epi == EPI_GRAD) {
        ST_CHECK(snap_out == SNAP_NONE && msnap, ST_ERR_ARG, "gradient step needs a snapshot map and no store");
        switch (snap_in) {
            case SNAP_BF16: return launch_variant<SNAP_NONE, SNAP_BF16, EPI_GRAD>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_FP16: return launch_variant<SNAP_NONE, SNAP_FP16, EPI_GRAD>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_FP32: return launch_variant<SNAP_NONE, SNAP_FP32, EPI_GRAD>(L, mcur, mprev, mc, ms, a, st);
            default: ST_CHECK(false, ST_ERR_ARG, "gradient step needs a snapshot kind");
        }
    }
    if (a.zlim) {
        switch (snap_out) {
            case SNAP_NONE: return launch_variant<SNAP_NONE, SNAP_NONE, EPI_MASK>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_BF16: return launch_variant<SNAP_BF16, SNAP_NONE, EPI_MASK>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_FP16: return launch_variant<SNAP_FP16, SNAP_NONE, EPI_MASK>(L, mcur, mprev, mc, ms, a, st);
            case SNAP_FP32: return launch_variant<SNAP_FP32, SNAP_NONE, EPI_MASK>(L, mcur, mprev, mc, ms, a, st);
            default: ST_CHECK(false, ST_ERR_ARG, "bad snapshot kind %d", snap_out);
        }
    }
    switch (snap_out) {
        case SNAP_NONE: return launch_variant<SNAP_NONE, SNAP_NONE, EPI_NONE>(L, mcur, mprev, mc, ms, a, st);
        case SNAP_BF16: return launch_variant<SNAP_BF16, SNAP_NONE, EPI_NONE>(L, mcur, mprev, mc, ms, a, st);
        case SNAP_FP16: return launch_variant<SNAP_FP16, SNAP_NONE, EPI_NONE>(L, mcur, mprev, mc, ms, a, st);
        case SNAP_FP32: return launch_variant<SNAP_FP32, SNAP_NONE, EPI_NONE>(L, mcur, mprev, mc, ms, a, st);
        default: ST_CHECK(false, ST_ERR_ARG, "bad snapshot kind %d", snap_out);
    }
}

int launch_fd_step2_image(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                          StepArgs a, int snap_in, const ImageMaps& imaps, cudaStream_t st) {
    a.nx = (int)L.nx;
    a.ny = (int)L.ny;
    a.nz = (int)L.nz;
    a.NZP = (int)L.NZP;
    a.plane = L.plane;
    if (a.timeout_ns == 0) a.timeout_ns = 2000000000ull;
    ST_CHECK(image_maps_supported(snap_in, L), ST_ERR_UNSUPPORTED, "two-step imaging needs staged image maps");
    ST_CHECK(a.out && a.out2 && a.image && a.illum && a.amax_in && a.amax_in2 && a.snap_t >= 1, ST_ERR_ARG,
             "two-step imaging: missing operands");
    ST_CHECK(!a.zlim && !a.seis_row && !a.snap_out && a.inj_x < 0, ST_ERR_UNSUPPORTED,
             "two-step imaging: adjoint steps only");
    switch (snap_in) {
        case SNAP_BF16: return launch_step2_variant<MODE_ADJ, SNAP_BF16>(L, mcur, mprev, mc, &imaps, a, st);
        case SNAP_FP16: return launch_step2_variant<MODE_ADJ, SNAP_FP16>(L, mcur, mprev, mc, &imaps, a, st);
        case SNAP_FP32: return launch_step2_variant<MODE_ADJ, SNAP_FP32>(L, mcur, mprev, mc, &imaps, a, st);
        default: ST_CHECK(false, ST_ERR_ARG, "imaging step needs a snapshot kind");
    }
}

int launch_fd_step2_grad(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                         StepArgs a, int snap_in, const CUtensorMap& msnap, const CUtensorMap& mgrad,
                         cudaStream_t st) {
    a.nx = (int)L.nx;
    a.ny = (int)L.ny;
    a.nz = (int)L.nz;
    a.NZP = (int)L.NZP;
    a.plane = L.plane;
    if (a.timeout_ns == 0) a.timeout_ns = 2000000000ull;
    ST_CHECK(L.nz % 4 == 0, ST_ERR_UNSUPPORTED, "two-step gradient needs nz %% 4 == 0");
    ST_CHECK(a.out && a.out2 && a.grad && a.amax_in && a.amax_in2 && a.snap_t >= 1, ST_ERR_ARG,
             "two-step gradient: missing operands");
    ST_CHECK(!a.zlim && !a.seis_row && !a.snap_out && a.inj_x < 0 && !a.image, ST_ERR_UNSUPPORTED,
             "two-step gradient: adjoint steps only");
    ImageMaps m;
    m.snap = msnap;
    m.image = mgrad;
    m.illum = mgrad;
    switch (snap_in) {
        case SNAP_BF16: return launch_step2_variant<MODE_GRAD, SNAP_BF16>(L, mcur, mprev, mc, &m, a, st);
        case SNAP_FP16: return launch_step2_variant<MODE_GRAD, SNAP_FP16>(L, mcur, mprev, mc, &m, a, st);
        case SNAP_FP32: return launch_step2_variant<MODE_GRAD, SNAP_FP32>(L, mcur, mprev, mc, &m, a, st);
        default: ST_CHECK(false, ST_ERR_ARG, "gradient step needs a snapshot kind");
    }
}

int launch_fd_step2_forward(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                            StepArgs a, int snap_out, cudaStream_t st) {
    a.nx = (int)L.nx;
    a.ny = (int)L.ny;
    a.nz = (int)L.nz;
    a.NZP = (int)L.NZP;
    a.plane = L.plane;
    if (a.timeout_ns == 0) a.timeout_ns = 2000000000ull;
    ST_CHECK(a.out && a.out2, ST_ERR_ARG, "two-step forward: missing outputs");
    ST_CHECK(!a.zlim && !a.force_row && !a.force_row2 && !a.image && !a.grad, ST_ERR_UNSUPPORTED,
             "two-step forward: forward steps without terrain only");
    ST_CHECK(L.nz % 4 == 0, ST_ERR_UNSUPPORTED, "two-step forward needs nz %% 4 == 0");
    ST_CHECK(snap_out == SNAP_NONE || (a.snap_out && a.amax_cur && a.amax_next && a.amax_next2 &&
                                       (!a.snap_out2 || a.amax_cur2)),
             ST_ERR_ARG, "two-step forward: missing snapshot operands");
    switch (snap_out) {
        case SNAP_NONE: return launch_step2_variant<MODE_FWD, SNAP_NONE>(L, mcur, mprev, mc, nullptr, a, st);
        case SNAP_BF16: return launch_step2_variant<MODE_FWD, SNAP_BF16>(L, mcur, mprev, mc, nullptr, a, st);
        case SNAP_FP16: return launch_step2_variant<MODE_FWD, SNAP_FP16>(L, mcur, mprev, mc, nullptr, a, st);
        case SNAP_FP32: return launch_step2_variant<MODE_FWD, SNAP_FP32>(L, mcur, mprev, mc, nullptr, a, st);
        default: ST_CHECK(false, ST_ERR_ARG, "bad snapshot kind %d", snap_out);
    }
}

int build_image_maps(ImageMaps* m, const void* snaps, int kind, long long nt, const float* image,
                     const float* illum, const Layout& L) {
    ST_CHECK(image_maps_supported(kind, L), ST_ERR_UNSUPPORTED, "staged imaging needs nz * %d bytes divisible by 16",
             snap_bytes(kind));
    ST_TRY(make_snap_map(&m->snap, snaps, kind, L, nt, TZ, 16));
    ST_TRY(make_compact_map(&m->image, image, L, TZ, 16));
    ST_TRY(make_compact_map(&m->illum, illum, L, TZ, 16));
    return ST_OK;
}

bool image_maps_supported(int kind, const Layout& L) {
    const int es = snap_bytes(kind);
    return es > 0 && (L.nz * es) % 16 == 0 && (L.nz % 4) == 0;
}

// 3-D map over a compact interior FP32 volume [nx][ny][nz], box {bz, by, 1}.
int make_compact_map(CUtensorMap* map, const float* base, const Layout& L, int bz, int by) {
    EncodeTiledFn enc = nullptr;
    ST_TRY(get_encode_tiled(&enc));
    ST_CHECK((reinterpret_cast<uintptr_t>(base) & 15) == 0, ST_ERR_ARG, "volume base not 16-byte aligned");
    ST_CHECK((L.nz * 4) % 16 == 0, ST_ERR_ARG, "compact volume rows must be multiples of 16 bytes");
    cuuint64_t dims[3] = {(cuuint64_t)L.nz, (cuuint64_t)L.ny, (cuuint64_t)L.nx};
    cuuint64_t strides[2] = {(cuuint64_t)L.nz * 4, (cuuint64_t)(L.ny * L.nz) * 4};
    cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)by, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    ST_CHECK(r == CUDA_SUCCESS, ST_ERR_CUDA, "cuTensorMapEncodeTiled (compact volume) failed (%d)", (int)r);
    return ST_OK;
}

int build_snap_map_grad(CUtensorMap* m, const void* base, int kind, const Layout& L, long long nt) {
    // the gradient variant uses 16-row tiles (one row per thread)
    const int bz = snap_bytes(kind) == 2 ? TZ + 16 : TZ + 8;
    return make_snap_map(m, base, kind, L, nt, bz, 16 + 2);
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

int launch_snapshot_of_field(const float* f, const Layout& L, void* snap, int kind, const unsigned* amax,
                             cudaStream_t st) {
    const int g = grid_for(L.nx * L.ny * L.nz);
    switch (kind) {
        case SNAP_BF16: snapshot_of_field_kernel<SNAP_BF16><<<g, 256, 0, st>>>(f, L, snap, amax); break;
        case SNAP_FP16: snapshot_of_field_kernel<SNAP_FP16><<<g, 256, 0, st>>>(f, L, snap, amax); break;
        case SNAP_FP32: snapshot_of_field_kernel<SNAP_FP32><<<g, 256, 0, st>>>(f, L, snap, amax); break;
        default: ST_CHECK(false, ST_ERR_ARG, "bad snapshot kind %d", kind);
    }
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

int make_snap_map(CUtensorMap* map, const void* base, int kind, const Layout& L, long long nt, int bz, int by) {
    EncodeTiledFn enc = nullptr;
    ST_TRY(get_encode_tiled(&enc));
    const int es = snap_bytes(kind);
    ST_CHECK(es > 0, ST_ERR_ARG, "bad snapshot kind %d", kind);
    ST_CHECK((reinterpret_cast<uintptr_t>(base) & 15) == 0, ST_ERR_ARG, "snapshot store not 16-byte aligned");
    ST_CHECK((L.nz * es) % 16 == 0, ST_ERR_UNSUPPORTED,
             "gradient snapshots need nz*%d bytes to be a multiple of 16 (nz=%lld)", es, (long long)L.nz);
    const CUtensorMapDataType dt = kind == SNAP_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                   : kind == SNAP_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                       : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    cuuint64_t dims[4] = {(cuuint64_t)L.nz, (cuuint64_t)L.ny, (cuuint64_t)L.nx, (cuuint64_t)std::max<long long>(nt, 1)};
    cuuint64_t strides[3] = {(cuuint64_t)(L.nz * es), (cuuint64_t)(L.ny * L.nz * es),
                             (cuuint64_t)(L.nx * L.ny * L.nz * es)};
    cuuint32_t box[4] = {(cuuint32_t)bz, (cuuint32_t)by, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = enc(map, dt, 4, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    ST_CHECK(r == CUDA_SUCCESS, ST_ERR_CUDA, "cuTensorMapEncodeTiled (snapshots) failed (%d)", (int)r);
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
