// 3x3x3 convolution of a 32-channel volume on the 5th-generation tensor
// cores (tcgen05), the building block of the learned CG preconditioner.
//
// Layout. A volume of D x H x W voxels is stored padded and channels-last:
// [(D+2) (H+2) (W+2)][32] BF16 (64 bytes per voxel), zero on the one-voxel
// border. Flattening the padded volume to rows q = (d*(H+2) + h)*(W+2) + w
// turns every tap (kd, kh, kw) of the stencil into a constant row shift
// s = (kd-1) PL + (kh-1)(W+2) + (kw-1), PL = (H+2)(W+2), and the zero border
// supplies the convolution's zero padding. So for a tile of 128 consecutive
// rows of one plane, out[128 x 32] = sum over 27 taps of
// in[rows + s][128 x 32] . W_tap[32 x 32]^T: an implicit GEMM with M = 128
// voxels, N = 32 output channels and K = 27 x 32.
//
// Data path per CTA (persistent, one per SM, 6 warps). The work is cut into
// units: one in-plane tile position (128 rows) for a run of consecutive
// planes d0..d1-1, so a CTA marches along d and every plane window it loads
// serves three consecutive tiles (taps kd = 2, 1, 0):
//   warp 0  TMA producer: loads the 128 + 2(W+3)-row window of each plane the
//           unit needs (d0 .. d1+1 in padded planes) as 16-byte channel-block
//           columns ([cb][row][8 channels], no swizzle) into a ring of four
//           window slots, a slot refilled once its last tile's MMAs are done;
//   warp 1  allocates 64 TMEM columns (two FP32 accumulators of 128 x 32) and
//           issues 54 tcgen05.mma.kind::f16 (BF16 x BF16 -> FP32, M=128,
//           N=32, K=16) per tile: every tap is a 16-byte-aligned start row
//           inside the windows, read in the canonical no-swizzle K-major
//           layout (8-row x 16-byte core matrices: LBO = channel-block
//           stride, SBO = 128 bytes); the weights (55,296 bytes, packed in the
//           same layout) stay resident in shared memory;
//   warps 2-5  epilogue: tcgen05.ld of the accumulator, + bias, + optional
//           residual input, optional ReLU, BF16 (or FP32) store of the row,
//           zero on border rows so the output keeps the padded convention.
// Every mbarrier wait is bounded by a %globaltimer deadline: on expiry the
// kernel records CONV_FLAG_TIMEOUT, drains its own copies and MMAs (bounded
// too), frees TMEM and returns.
#include "st_common.cuh"

#include <algorithm>
#include <mutex>

namespace stg {
namespace {

constexpr int CH = 32;
constexpr int TM = 128;
constexpr int NTAP = 27;
constexpr int W_BYTES = NTAP * CH * CH * 2;  // 55,296: [tap][cb][co][8 ci]
// plane-window slots: three in use by a tile, the rest loading ahead; the
// host takes MAX_SLOT where it fits in shared memory, else MIN_SLOT (six
// measured 3% faster than four on a 100^3 volume, eight no faster than six)
constexpr int MIN_SLOT = 4, MAX_SLOT = 6;
constexpr int CONV_THREADS = 192;
constexpr int TMEM_COLS = 64;
constexpr int SMEM_LIMIT = 232448 - 1024;
constexpr unsigned CONV_FLAG_TIMEOUT = 1u;

struct ConvArgs {
    const void* w;          // packed weights (global, 16-byte aligned)
    const float* bias;      // [32] or null
    const __nv_bfloat16* add;  // residual input, padded layout, or null
    void* out;              // padded layout, BF16 or FP32
    int out_f32;
    int D, H, W;
    int relu;
    int rows_box, nload;    // TMA box rows and boxes per window column
    int tiles_per_plane;    // in-plane tile positions (units' columns)
    int dchunk, units;      // planes per unit, units = tiles_per_plane * ceil(D / dchunk)
    unsigned* flags;
    unsigned long long timeout_ns;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ int read_abort(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor, canonical K-major layout without swizzle:
// start address, leading (K-direction) and stride (M/N-direction) byte
// offsets between 8-row x 16-byte core matrices, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 32, M = 128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(CH >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct ConvSmem {
    uint64_t full[MAX_SLOT], empty[MAX_SLOT], tfull[2], tempty[2], wbar;
    uint32_t tmem_base;
    int abort;
};

// Unit u: in-plane tile column u % tiles_per_plane, planes [d0, d1).
struct ConvUnit {
    int col, d0, d1;
};
__device__ __forceinline__ ConvUnit unit_of(const ConvArgs& a, int u) {
    ConvUnit r;
    r.col = u % a.tiles_per_plane;
    r.d0 = (u / a.tiles_per_plane) * a.dchunk;
    r.d1 = min(a.D, r.d0 + a.dchunk);
    return r;
}

template <int NSLOT>
__global__ void __launch_bounds__(CONV_THREADS, 1)
    conv3d_tc_kernel(const __grid_constant__ CUtensorMap m0, const __grid_constant__ CUtensorMap m1,
                     const __grid_constant__ CUtensorMap m2, const __grid_constant__ CUtensorMap m3,
                     const ConvArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // every TMA destination below is a multiple of 128 bytes from this base
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    const int W2 = a.W + 2;
    const int PL = (a.H + 2) * W2;
    const int win_rows = a.rows_box * a.nload;          // rows per (kd, cb) column
    const uint32_t lbo_a = (uint32_t)win_rows * 16u;    // channel-block stride
    const uint32_t slot_bytes = 4u * lbo_a;           // one plane window, 4 channel-block columns
    unsigned char* wsm = smem;                           // weights
    unsigned char* slots = smem + W_BYTES;               // 128-byte aligned (W_BYTES = 54 KB)
    ConvSmem* cs = reinterpret_cast<ConvSmem*>(slots + NSLOT * slot_bytes);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t lim = a.timeout_ns;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NSLOT; ++s) {
            mbar_init(&cs->full[s], 1);
            mbar_init(&cs->empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&cs->tfull[s], 1);
            mbar_init(&cs->tempty[s], 128);
        }
        mbar_init(&cs->wbar, 1);
        cs->abort = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&cs->tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = cs->tmem_base;
    const CUtensorMap* maps[4] = {&m0, &m1, &m2, &m3};

    // Window fills are numbered g = 0, 1, ... in the CTA's unit order; fill g
    // goes to slot g % NSLOT. A unit of planes [d0, d1) takes d1 - d0 + 2 fills
    // (padded planes d0 .. d1 + 1); its k-th tile reads fills g0 + k + kd.
    if (warp == 0) {
        if (lane == 0) {
            mbar_arrive_expect_tx(&cs->wbar, W_BYTES);
            bulk_load(wsm, a.w, W_BYTES, &cs->wbar);
            int g = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < a.units && !stop; u += gridDim.x) {
                const ConvUnit U = unit_of(a, u);
                const int p0 = U.col * TM;
                const int nfill = U.d1 - U.d0 + 2;
                for (int j = 0; j < nfill; ++j, ++g) {
                    const int slot = g % NSLOT;
                    if (g >= NSLOT && !mbar_wait_bounded(&cs->empty[slot], ((g / NSLOT) - 1) & 1, lim)) {
                        atomicOr(a.flags, CONV_FLAG_TIMEOUT);
                        cs->abort = 1;
                        stop = true;
                        break;
                    }
                    if (read_abort(&cs->abort)) {
                        stop = true;
                        break;
                    }
                    unsigned char* sb = slots + slot * slot_bytes;
                    const int q0 = (U.d0 + j) * PL + p0 - (W2 + 1);
                    mbar_arrive_expect_tx(&cs->full[slot], 4u * (uint32_t)a.nload * (uint32_t)a.rows_box * 16u);
                    for (int cb = 0; cb < 4; ++cb)
                        for (int l = 0; l < a.nload; ++l)
                            tma_load_2d(sb + cb * lbo_a + l * a.rows_box * 16, maps[cb], &cs->full[slot], 0,
                                        q0 + l * a.rows_box);
                }
            }
            // drain: every issued window has landed before the CTA may exit
            for (int f = (g > NSLOT ? g - NSLOT : 0); f < g; ++f)
                if (!mbar_wait_bounded(&cs->full[f % NSLOT], (f / NSLOT) & 1, lim > WAIT_DRAIN_NS ? lim : WAIT_DRAIN_NS))
                    atomicOr(a.flags, CONV_FLAG_TIMEOUT);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            bool ok = mbar_wait_bounded(&cs->wbar, 0, lim);
            int committed = 0, i = 0, g0 = 0;
            const uint32_t wb = smem_u32(wsm);
            for (int u = blockIdx.x; ok && u < a.units; u += gridDim.x) {
                const ConvUnit U = unit_of(a, u);
                const int nt = U.d1 - U.d0;
                for (int k = 0; ok && k < nt; ++k, ++i) {
                    const int acc = i & 1;
                    if (i >= 2 && !mbar_wait_bounded(&cs->tempty[acc], ((i >> 1) & 1) ^ 1, lim)) {
                        ok = false;
                        break;
                    }
                    uint32_t sbase[3];
                    for (int kd = 0; kd < 3; ++kd) {
                        const int f = g0 + k + kd;
                        if (!mbar_wait_bounded(&cs->full[f % NSLOT], (f / NSLOT) & 1, lim)) ok = false;
                        sbase[kd] = smem_u32(slots + (f % NSLOT) * slot_bytes);
                    }
                    if (!ok || read_abort(&cs->abort)) {
                        ok = ok && !read_abort(&cs->abort);
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d_tmem = tmem + (uint32_t)(acc * CH);
                    for (int kd = 0; kd < 3; ++kd)
                        for (int kh = 0; kh < 3; ++kh)
                            for (int kw = 0; kw < 3; ++kw) {
                                const int tap = (kd * 3 + kh) * 3 + kw;
                                const uint32_t roff = (uint32_t)(W2 + 1 + (kh - 1) * W2 + (kw - 1)) * 16u;
#pragma unroll
                                for (int ks = 0; ks < 2; ++ks) {
                                    const uint64_t ad = smem_desc(sbase[kd] + (uint32_t)(2 * ks) * lbo_a + roff, lbo_a,
                                                                  128u);
                                    const uint64_t bd = smem_desc(wb + (uint32_t)tap * 2048u + (uint32_t)ks * 1024u,
                                                                  512u, 128u);
                                    mma_bf16(d_tmem, ad, bd, (tap | ks) != 0);
                                }
                            }
                    mma_commit(&cs->tfull[acc]);
                    // the window of plane d (tap kd = 0) has served its last tile; at
                    // the unit's end so have the two after it
                    mma_commit(&cs->empty[(g0 + k) % NSLOT]);
                    if (k == nt - 1) {
                        mma_commit(&cs->empty[(g0 + k + 1) % NSLOT]);
                        mma_commit(&cs->empty[(g0 + k + 2) % NSLOT]);
                    }
                    ++committed;
                }
                g0 += nt + 2;
            }
            if (!ok) {
                atomicOr(a.flags, CONV_FLAG_TIMEOUT);
                cs->abort = 1;
            }
            // drain: the last commit tracks every MMA this thread issued
            if (committed > 0) {
                const int last = committed - 1;
                if (!mbar_wait_bounded(&cs->tfull[last & 1], (last >> 1) & 1, lim > WAIT_DRAIN_NS ? lim : WAIT_DRAIN_NS))
                    atomicOr(a.flags, CONV_FLAG_TIMEOUT);
            }
        }
    } else {
        // epilogue: warps 2..5 own TMEM lane quarters (warp % 4)
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        float bias[CH];
#pragma unroll
        for (int c = 0; c < CH; ++c) bias[c] = a.bias ? a.bias[c] : 0.0f;
        int i = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < a.units && !stop; u += gridDim.x) {
            const ConvUnit U = unit_of(a, u);
            for (int d = U.d0; d < U.d1; ++d, ++i) {
                const int acc = i & 1;
                // warp-uniform outcome: the TMEM load below is a warp-collective
                const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&cs->tfull[acc], (i >> 1) & 1, lim));
                if (!ok) {
                    if (lane == 0) atomicOr(a.flags, CONV_FLAG_TIMEOUT);
                    cs->abort = 1;
                    stop = true;
                    break;
                }
                tc_fence_after();
                float v[CH];
                tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * CH), v);
                tc_fence_before();
                mbar_arrive(&cs->tempty[acc]);
                const int p = U.col * TM + row;
                if (p >= PL) continue;
                const int h = p / W2, w = p - h * W2;
                const bool inside = h >= 1 && h <= a.H && w >= 1 && w <= a.W;
                const long long q = (long long)(d + 1) * PL + p;
                if (inside) {
                    if (a.add) {
                        const uint4* ap = reinterpret_cast<const uint4*>(a.add + q * CH);
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const uint4 uu = ap[j];
                            const __nv_bfloat162* b2 = reinterpret_cast<const __nv_bfloat162*>(&uu);
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const float2 f = __bfloat1622float2(b2[e]);
                                v[8 * j + 2 * e] += f.x;
                                v[8 * j + 2 * e + 1] += f.y;
                            }
                        }
                    }
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        v[c] += bias[c];
                        if (a.relu) v[c] = fmaxf(v[c], 0.0f);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < CH; ++c) v[c] = 0.0f;
                }
                if (a.out_f32) {
                    float4* op = reinterpret_cast<float4*>(static_cast<float*>(a.out) + q * CH);
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        op[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                } else {
                    uint4* op = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(a.out) + q * CH);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        uint4 uu;
                        __nv_bfloat162* b2 = reinterpret_cast<__nv_bfloat162*>(&uu);
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            b2[e] = __floats2bfloat162_rn(v[8 * j + 2 * e], v[8 * j + 2 * e + 1]);
                        op[j] = uu;
                    }
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// [co][ci][kd][kh][kw] FP32 (the usual conv weight order) -> packed BF16
// [tap][cb][co][8 ci]. transpose: the weights of the input gradient, i.e. the
// taps mirrored and in/out channels swapped.
__global__ void pack_weights_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ out, int transpose) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NTAP * CH * CH) return;
    const int tap = i / (CH * CH), r = i % (CH * CH), cb = r / (8 * CH), r2 = r % (8 * CH), co = r2 / 8,
              ci = cb * 8 + r2 % 8;
    float v;
    if (transpose) v = w[((size_t)ci * CH + co) * NTAP + (NTAP - 1 - tap)];
    else v = w[((size_t)co * CH + ci) * NTAP + tap];
    out[i] = __float2bfloat16_rn(v);
}

int num_sms_conv() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// One 2-D map per 8-channel block over the padded volume viewed as
// [rows][32 channels]: box {8 channels, rows_box rows}.
int make_conv_map(CUtensorMap* map, const __nv_bfloat16* base, long long rows, int cb, int rows_box) {
    EncodeTiledFn enc = nullptr;
    ST_TRY(get_encode_tiled(&enc));
    cuuint64_t dims[2] = {8, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)CH * 2};
    cuuint32_t box[2] = {8, (cuuint32_t)rows_box};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base + cb * 8), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    ST_CHECK(r == CUDA_SUCCESS, ST_ERR_CUDA, "cuTensorMapEncodeTiled (conv) failed (%d)", (int)r);
    return ST_OK;
}

// ---------------------------------------------------------------- weight gradient
// dW[co][ci][tap] += sum over interior voxels v of g[v][co] x[v + s_tap][ci]
// for a 32 -> 32 layer, on the tensor cores: an implicit GEMM with
// M = (tap, ci) in 7 tiles of 4 taps x 32 input channels (the last tile has 3
// taps), N = 32 output channels and K = the padded volume's rows q, split
// over CTAs (each CTA one M tile and one K range; FP32 atomics add the
// partial tiles). g's border rows are zeroed on the way in, so a K step may
// run over them; x's border is zero by the padded convention, and rows past
// the volume arrive as zeros from the TMA bounds fill.
//
// Per K step of 64 rows the TMA brings [64 rows][32 ch] tiles of x (one per
// tap of the tile, shifted by the tap's row offset) and of g into a ring of
// raw stages. Channels-last rows are channel-contiguous, but both operands
// of the contraction over q must be K-major (q contiguous): warps 2-5
// transpose the tiles 8x8 at a time with ldmatrix.trans / stmatrix into the
// canonical no-swizzle K-major layout (8 rows x 16-byte core matrices; A:
// LBO 2048 between K blocks, SBO 128 between M blocks; B: LBO 512, SBO 128)
// of an operand stage; warp 1 issues four tcgen05.mma (M=128, N=32, K=16) per
// step into a 32-column TMEM accumulator; warps 2-5 then read it back
// (tcgen05.ld) and add it to dW. Every wait is bounded as in the forward conv.
constexpr int WG_KSTEP = 64;
constexpr int WG_TILES = 7;
constexpr int WG_NRAW = 3;
constexpr int WG_NOP = 2;
constexpr int WG_RAW_TILE = WG_KSTEP * CH * 2;  // 4096
constexpr int WG_RAW_BYTES = 5 * WG_RAW_TILE;   // four x tiles + the g tile
constexpr int WG_A_BYTES = TM * WG_KSTEP * 2;   // 16384
constexpr int WG_B_BYTES = CH * WG_KSTEP * 2;   // 4096
constexpr int WG_OP_BYTES = WG_A_BYTES + WG_B_BYTES;
constexpr int WG_THREADS = 192;
constexpr int WG_TMEM_COLS = 32;

struct WgradArgs {
    float* dw;
    int D, H, W;
    long long rows;  // (D+2)(H+2)(W+2)
    int ksteps;      // ceil(rows / 64)
    int splits;      // CTAs per M tile
    unsigned* flags;
    unsigned long long timeout_ns;
};

struct WgradSmem {
    uint64_t raw_full[WG_NRAW], raw_empty[WG_NRAW], op_full[WG_NOP], op_empty[WG_NOP], done;
    uint32_t tmem_base;
    int abort;
};

__device__ __forceinline__ void ldsm_x4_trans(uint32_t addr, uint32_t r[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr)
                 : "memory");
}
__device__ __forceinline__ void stsm_x4(uint32_t addr, const uint32_t r[4]) {
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3])
                 : "memory");
}
__device__ __forceinline__ void named_sync_128() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__global__ void __launch_bounds__(WG_THREADS, 1)
    conv32_wgrad_tc_kernel(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap mg,
                           const WgradArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char* raw = smem;
    unsigned char* ops = smem + WG_NRAW * WG_RAW_BYTES;
    WgradSmem* cs = reinterpret_cast<WgradSmem*>(ops + WG_NOP * WG_OP_BYTES);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x % WG_TILES, split = blockIdx.x / WG_TILES;
    const int ntap = tile == WG_TILES - 1 ? NTAP - 4 * (WG_TILES - 1) : 4;
    const int k0 = (int)((long long)a.ksteps * split / a.splits);
    const int nk = (int)((long long)a.ksteps * (split + 1) / a.splits) - k0;
    const int W2 = a.W + 2;
    const int PL = (a.H + 2) * W2;
    const uint64_t lim = a.timeout_ns;
    const uint64_t dlim = lim > WAIT_DRAIN_NS ? lim : WAIT_DRAIN_NS;

    if (threadIdx.x == 0) {
        for (int s = 0; s < WG_NRAW; ++s) {
            mbar_init(&cs->raw_full[s], 1);
            mbar_init(&cs->raw_empty[s], 128);
        }
        for (int s = 0; s < WG_NOP; ++s) {
            mbar_init(&cs->op_full[s], 128);
            mbar_init(&cs->op_empty[s], 1);
        }
        mbar_init(&cs->done, 1);
        cs->abort = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&cs->tmem_base)),
                     "r"(WG_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = cs->tmem_base;

    if (warp == 0) {
        if (lane == 0) {
            int k = 0;
            for (; k < nk; ++k) {
                const int s = k % WG_NRAW;
                if (k >= WG_NRAW && !mbar_wait_bounded(&cs->raw_empty[s], ((k / WG_NRAW) - 1) & 1, lim)) {
                    atomicOr(a.flags, CONV_FLAG_TIMEOUT);
                    cs->abort = 1;
                    break;
                }
                if (read_abort(&cs->abort)) break;
                const int q0 = (k0 + k) * WG_KSTEP;
                unsigned char* rb = raw + s * WG_RAW_BYTES;
                mbar_arrive_expect_tx(&cs->raw_full[s], (uint32_t)(ntap + 1) * WG_RAW_TILE);
                for (int t = 0; t < ntap; ++t) {
                    const int tap = 4 * tile + t;
                    const int shift = (tap / 9 - 1) * PL + ((tap / 3) % 3 - 1) * W2 + (tap % 3 - 1);
                    tma_load_2d(rb + t * WG_RAW_TILE, &mx, &cs->raw_full[s], 0, q0 + shift);
                }
                tma_load_2d(rb + 4 * WG_RAW_TILE, &mg, &cs->raw_full[s], 0, q0);
            }
            // drain: every issued stage has landed before the CTA may exit
            for (int f = (k > WG_NRAW ? k - WG_NRAW : 0); f < k; ++f)
                if (!mbar_wait_bounded(&cs->raw_full[f % WG_NRAW], (f / WG_NRAW) & 1, dlim))
                    atomicOr(a.flags, CONV_FLAG_TIMEOUT);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int k = 0;
            for (; k < nk; ++k) {
                const int o = k % WG_NOP;
                if (!mbar_wait_bounded(&cs->op_full[o], (k / WG_NOP) & 1, lim) || read_abort(&cs->abort)) {
                    atomicOr(a.flags, CONV_FLAG_TIMEOUT);
                    cs->abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t ab = smem_u32(ops + o * WG_OP_BYTES), bb = ab + WG_A_BYTES;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    mma_bf16(tmem, smem_desc(ab + (uint32_t)j * 4096u, 2048u, 128u),
                             smem_desc(bb + (uint32_t)j * 1024u, 512u, 128u), (k | j) != 0);
                mma_commit(&cs->op_empty[o]);
            }
            // the last commit tracks every MMA issued: the accumulator is final
            // (and, after an abort, no MMA is left running when TMEM is freed)
            if (k > 0) {
                mma_commit(&cs->done);
                if (!mbar_wait_bounded(&cs->done, 0, dlim)) atomicOr(a.flags, CONV_FLAG_TIMEOUT);
            }
        }
    } else {
        // warps 2-5: transposes, then the epilogue. The four warps meet at a
        // named barrier every step, so none leaves the loop early: after a
        // failed wait (or another warp's abort) a warp stops waiting and
        // working but still takes every barrier.
        const int tt = threadIdx.x - 64, tw = warp - 2;
        // this lane's row of each of the warp's ten groups of four 8 x 8 blocks
        // (groups tw, tw + 4, ...; A: 4 taps x 8 row blocks x 4 channel blocks,
        // B: 8 x 4): source offset in a raw stage, destination offset in an
        // operand stage. The raw tiles arrive 64-byte swizzled (16-byte chunk c
        // of row v at chunk c ^ ((v >> 1) & 3)), so the eight rows an ldmatrix
        // reads fall in eight different bank groups.
        constexpr uint32_t SKIP = 0xffffffffu;
        uint32_t so[10], dof[10];
        {
            const int r = lane & 7;
#pragma unroll
            for (int j = 0; j < 10; ++j) {
                const int b = (tw + 4 * j) * 4 + (lane >> 3);
                int t, vb, cb;
                uint32_t dst;
                if (b < 128) {
                    t = b >> 5;
                    vb = (b & 31) >> 2;
                    cb = b & 3;
                    dst = (uint32_t)(vb * 2048 + (t * 4 + cb) * 128 + r * 16);
                } else {
                    t = 4;
                    vb = (b - 128) >> 2;
                    cb = (b - 128) & 3;
                    dst = (uint32_t)(WG_A_BYTES + vb * 512 + cb * 128 + r * 16);
                }
                const int row = vb * 8 + r;
                so[j] = (b < 128 && t >= ntap) ? SKIP  // uniform over the group (32 blocks per tap)
                                               : (uint32_t)(t * WG_RAW_TILE + row * (CH * 2) + ((cb ^ ((row >> 1) & 3)) << 4));
                dof[j] = dst;
            }
        }
        bool ok = true;
        for (int k = 0; k < nk; ++k) {
            const int s = k % WG_NRAW, o = k % WG_NOP;
            if (ok) {
                bool w = !read_abort(&cs->abort) && mbar_wait_bounded(&cs->raw_full[s], (k / WG_NRAW) & 1, lim);
                if (w && k >= WG_NOP) w = mbar_wait_bounded(&cs->op_empty[o], ((k / WG_NOP) - 1) & 1, lim);
                // ldmatrix / stmatrix are warp-collective: a warp-uniform outcome
                if (!__all_sync(0xffffffffu, w && !read_abort(&cs->abort))) {
                    if (lane == 0) atomicOr(a.flags, CONV_FLAG_TIMEOUT);
                    cs->abort = 1;
                    ok = false;
                }
            }
            unsigned char* rb = raw + s * WG_RAW_BYTES;
            unsigned char* ob = ops + o * WG_OP_BYTES;
            if (ok && tt < WG_KSTEP) {
                // g rows outside the interior contribute nothing
                const long long q = (long long)(k0 + k) * WG_KSTEP + tt;
                const int d = (int)(q / PL), rem = (int)(q - (long long)d * PL), h = rem / W2, wv = rem - h * W2;
                const bool inside = d >= 1 && d <= a.D && h >= 1 && h <= a.H && wv >= 1 && wv <= a.W;
                if (!inside) {
                    uint4* row = reinterpret_cast<uint4*>(rb + 4 * WG_RAW_TILE + tt * (CH * 2));
#pragma unroll
                    for (int j = 0; j < 4; ++j) row[j] = make_uint4(0u, 0u, 0u, 0u);
                }
            }
            named_sync_128();
            if (!ok) continue;
            // four 8 x 8 blocks per ldmatrix / stmatrix pair; lane l addresses row
            // l % 8 of block l / 8 of the group
            const uint32_t rbu = smem_u32(rb), obu = smem_u32(ob);
#pragma unroll
            for (int j = 0; j < 10; ++j) {
                if (so[j] == SKIP) continue;
                uint32_t v4[4];
                ldsm_x4_trans(rbu + so[j], v4);
                stsm_x4(obu + dof[j], v4);
            }
            // generic-proxy writes read by the tensor cores, and a raw stage the
            // TMA overwrites next
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&cs->op_full[o]);
            mbar_arrive(&cs->raw_empty[s]);
        }
        if (ok && nk > 0) {
            const bool got = __all_sync(0xffffffffu, mbar_wait_bounded(&cs->done, 0, dlim));
            if (!got) {
                if (lane == 0) atomicOr(a.flags, CONV_FLAG_TIMEOUT);
            } else {
                tc_fence_after();
                const int quarter = warp & 3;  // TMEM lanes 32 quarter .. : tap quarter of the tile, ci = lane
                float v[CH];
                tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16), v);
                tc_fence_before();
                if (quarter < ntap) {
                    const int tap = 4 * tile + quarter;
#pragma unroll
                    for (int co = 0; co < CH; ++co) atomicAdd(&a.dw[((size_t)co * CH + lane) * NTAP + tap], v[co]);
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(WG_TMEM_COLS)
                     : "memory");
    }
}

// The padded volume viewed as [rows][32 channels], box {32 channels, 64 rows},
// 64-byte swizzled in shared memory.
int make_wgrad_map(CUtensorMap* map, const __nv_bfloat16* base, long long rows) {
    EncodeTiledFn enc = nullptr;
    ST_TRY(get_encode_tiled(&enc));
    cuuint64_t dims[2] = {CH, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)CH * 2};
    cuuint32_t box[2] = {CH, WG_KSTEP};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    ST_CHECK(r == CUDA_SUCCESS, ST_ERR_CUDA, "cuTensorMapEncodeTiled (wgrad) failed (%d)", (int)r);
    return ST_OK;
}

__device__ unsigned g_conv_flags;

}  // namespace

}  // namespace stg

using namespace stg;

extern "C" {

int st_conv3d_pack_weights(const float* w, void* packed, int transpose, void* stream) {
    ST_CHECK(w && packed, ST_ERR_ARG, "null argument");
    ST_CHECK((reinterpret_cast<uintptr_t>(packed) & 15) == 0, ST_ERR_ARG, "packed weights not 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    pack_weights_kernel<<<(NTAP * CH * CH + 255) / 256, 256, 0, st>>>(w, static_cast<__nv_bfloat16*>(packed),
                                                                      transpose);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_conv3d_bf16(const void* in, const void* packed_w, const float* bias, const void* add, void* out, int out_fp32,
                   int64_t D, int64_t H, int64_t W, int relu, void* stream) {
    ST_CHECK(in && packed_w && out, ST_ERR_ARG, "null argument");
    ST_CHECK(D > 0 && H > 0 && W > 0, ST_ERR_ARG, "bad volume extents");
    ST_CHECK(in != out && (!add || add != out), ST_ERR_ARG, "output must not alias the inputs");
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    ST_CHECK(al16(in) && al16(packed_w) && al16(out) && (!add || al16(add)), ST_ERR_ARG,
             "conv buffers must be 16-byte aligned");
    const long long W2 = W + 2, PL = (H + 2) * W2, rows = (D + 2) * PL;
    ST_CHECK(rows < (1ll << 31), ST_ERR_ARG, "volume too large");
    // window column of one plane and channel block: win rows, loaded as nload
    // boxes of rows_box rows (<= 256, a multiple of 8 so that every TMA
    // destination stays 128-byte aligned)
    const long long win = TM + 2 * (W2 + 1);
    int nload = (int)((win + 255) / 256);
    int rows_box = (int)((((win + nload - 1) / nload) + 7) / 8 * 8);
    while (rows_box > 256) {
        ++nload;
        rows_box = (int)((((win + nload - 1) / nload) + 7) / 8 * 8);
    }
    auto smem_of = [&](int ns) {
        return (size_t)W_BYTES + (size_t)ns * 4 * 16 * nload * rows_box + sizeof(ConvSmem) + 128;
    };
    const int nslot = smem_of(MAX_SLOT) <= (size_t)SMEM_LIMIT ? MAX_SLOT : MIN_SLOT;
    const size_t smem = smem_of(nslot);
    ST_CHECK(smem <= (size_t)SMEM_LIMIT, ST_ERR_UNSUPPORTED, "volume width %lld too large for the conv tiles",
             (long long)W);
    const __nv_bfloat16* src = static_cast<const __nv_bfloat16*>(in);
    CUtensorMap maps[4];
    for (int cb = 0; cb < 4; ++cb) ST_TRY(make_conv_map(&maps[cb], src, rows, cb, rows_box));
    unsigned* flags = nullptr;
    ST_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&flags), g_conv_flags));
    ConvArgs a{};
    a.w = packed_w;
    a.bias = bias;
    a.add = static_cast<const __nv_bfloat16*>(add);
    a.out = out;
    a.out_f32 = out_fp32;
    a.D = (int)D;
    a.H = (int)H;
    a.W = (int)W;
    a.relu = relu;
    a.rows_box = rows_box;
    a.nload = nload;
    a.tiles_per_plane = (int)((PL + TM - 1) / TM);
    // planes per unit: the fewest rounds of units over the SMs, each unit
    // paying two extra window loads (its first two planes)
    const long long nsm = num_sms_conv();
    long long best_cost = -1;
    for (long long dc = 1; dc <= D; ++dc) {
        const long long units = (long long)a.tiles_per_plane * ((D + dc - 1) / dc);
        const long long rounds = (units + nsm - 1) / nsm;
        const long long cost = rounds * (dc + 2);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            a.dchunk = (int)dc;
        }
    }
    a.units = (int)((long long)a.tiles_per_plane * ((D + a.dchunk - 1) / a.dchunk));
    a.flags = flags;
    a.timeout_ns = 2000000000ull;
    auto kern = nslot == MAX_SLOT ? conv3d_tc_kernel<MAX_SLOT> : conv3d_tc_kernel<MIN_SLOT>;
    static std::mutex mu;
    static size_t configured[2] = {0, 0};
    {
        std::lock_guard<std::mutex> lk(mu);
        size_t& c = configured[nslot == MAX_SLOT ? 1 : 0];
        if (c < smem) {
            ST_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            c = smem;
        }
    }
    const int grid = std::min(a.units, num_sms_conv());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    kern<<<grid, CONV_THREADS, smem, st>>>(maps[0], maps[1], maps[2], maps[3], a);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_conv3d_wgrad(const void* x, const void* g, float* dw, int64_t nx, int64_t ny, int64_t nz, void* stream) {
    ST_CHECK(x && g && dw, ST_ERR_ARG, "null argument");
    ST_CHECK(nx > 0 && ny > 0 && nz > 0, ST_ERR_ARG, "bad volume extents");
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    ST_CHECK(al16(x) && al16(g), ST_ERR_ARG, "conv buffers must be 16-byte aligned");
    const long long rows = (nx + 2) * (ny + 2) * (nz + 2);
    ST_CHECK(rows + (ny + 2) * (nz + 2) + nz + 3 < (1ll << 31), ST_ERR_ARG, "volume too large");
    CUtensorMap mx, mg;
    ST_TRY(make_wgrad_map(&mx, static_cast<const __nv_bfloat16*>(x), rows));
    ST_TRY(make_wgrad_map(&mg, static_cast<const __nv_bfloat16*>(g), rows));
    unsigned* flags = nullptr;
    ST_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&flags), g_conv_flags));
    WgradArgs a{};
    a.dw = dw;
    a.D = (int)nx;
    a.H = (int)ny;
    a.W = (int)nz;
    a.rows = rows;
    a.ksteps = (int)((rows + WG_KSTEP - 1) / WG_KSTEP);
    // two CTAs per SM over the 7 M tiles, at least one K step each
    a.splits = (int)std::max<long long>(1, std::min<long long>(a.ksteps, (2LL * num_sms_conv() + WG_TILES - 1) / WG_TILES));
    a.flags = flags;
    a.timeout_ns = 2000000000ull;
    const size_t smem = (size_t)WG_NRAW * WG_RAW_BYTES + (size_t)WG_NOP * WG_OP_BYTES + sizeof(WgradSmem) + 1024;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [&] {
        attr = cudaFuncSetAttribute(conv32_wgrad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    ST_CUDA(attr);
    conv32_wgrad_tc_kernel<<<WG_TILES * a.splits, WG_THREADS, smem, static_cast<cudaStream_t>(stream)>>>(mx, mg, a);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int st_conv3d_check(void* stream) {
    unsigned h = 0;
    ST_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    ST_CUDA(cudaMemcpyFromSymbol(&h, g_conv_flags, sizeof(h)));
    const unsigned zero = 0;
    ST_CUDA(cudaMemcpyToSymbol(g_conv_flags, &zero, sizeof(zero)));
    ST_CHECK(!(h & CONV_FLAG_TIMEOUT), ST_ERR_TIMEOUT, "a conv3d wait timed out");
    return ST_OK;
}

}  // extern "C"
