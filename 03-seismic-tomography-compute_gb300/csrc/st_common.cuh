// Shared definitions of the GB300 seismic engine: device field layout,
// status codes, error reporting, and the inline-PTX TMA / mbarrier helpers
// used by the stencil kernels. sm_103a only.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "seismic_gb300.h"

namespace stg {

// ---------------------------------------------------------------- errors
// The last error message of the calling host thread (st_last_error()).
void set_error(const char* fmt, ...);
const char* last_error();

#define ST_CUDA(call)                                                                    \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            ::stg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return ST_ERR_CUDA;                                                          \
        }                                                                                \
    } while (0)

#define ST_CHECK(cond, code, ...)                \
    do {                                         \
        if (!(cond)) {                           \
            ::stg::set_error(__VA_ARGS__);       \
            return (code);                       \
        }                                        \
    } while (0)

#define ST_TRY(expr)                 \
    do {                             \
        int rc_ = (expr);            \
        if (rc_ < 0) return rc_;     \
    } while (0)

// Bits of the per-solver device status word.
enum : unsigned {
    FLAG_GUARD = 1u,    // a NaN/Inf guard of the update fired (NAN_DETECTED_AND_REPAIRED)
    FLAG_TIMEOUT = 2u,  // a bounded mbarrier wait gave up (pipeline fault)
};

// Number of kernels this library has launched in the process (every launch
// site calls count_launch right after its <<<>>>).
void count_launch(long long n = 1);
long long launch_count();

// ---------------------------------------------------------------- layout
// Device layout of one FP32 field. x and y carry the reference's one-cell
// halo (x slowest, z fastest, as core/grid.cpp:45-49); along z the interior
// starts at column ZOFF = 4 and rows are padded to NZP (a multiple of 8), so
// every row starts on a 32-byte boundary, every interior row on a 16-byte
// boundary, and TMA boxes can start on 16-byte-aligned z coordinates. The
// reference layout (pitch nz+2, interior at column 1) is converted at the
// boundary by st_field_upload / st_field_download.
struct Layout {
    int64_t nx, ny, nz;     // interior extents
    int64_t NXh, NYh, NZP;  // device extents
    int64_t plane;          // NYh * NZP
    int64_t elems;          // NXh * plane
    static constexpr int ZOFF = 4;
    __host__ __device__ int64_t at(int64_t ix, int64_t iy, int64_t iz) const {
        return (ix + 1) * plane + (iy + 1) * NZP + (iz + ZOFF);
    }
};

inline Layout make_layout(int64_t nx, int64_t ny, int64_t nz) {
    Layout L;
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.NXh = nx + 2;
    L.NYh = ny + 2;
    L.NZP = ((nz + 8 + 7) / 8) * 8;
    L.plane = L.NYh * L.NZP;
    L.elems = L.NXh * L.plane;
    return L;
}

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Spins on an mbarrier phase for at most ~limit_ns of GPU time. Returns false
// when the limit ran out (the caller records FLAG_TIMEOUT and unwinds).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    uint64_t t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > limit_ns) return false;
    }
}

// Limit of the waits that drain a kernel's copies in flight after another
// wait gave up: always the full default, whatever limit the pipeline ran with,
// so that no copy can land in shared memory after the CTA has exited.
constexpr uint64_t WAIT_DRAIN_NS = 2000000000ull;

// 3-D tiled TMA load of one box into shared memory, completing on `bar`.
// c0 is the innermost (z) coordinate and must be a multiple of 4 elements
// (16 bytes) for FP32 data; the launchers guarantee it.
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// 4-D tiled TMA load (snapshot store: z, y, x, t). Same alignment rule on c0.
__device__ __forceinline__ void tma_load_4d(void* smem_dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void st_global_cs_f4(float* p, float4 v) {
    asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ float4 ld_global_nc_f4(const float* p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

// ---------------------------------------------------------------- snapshots
// Storage kinds of forward snapshots (values per interior point).
enum SnapKind : int { SNAP_NONE = 0, SNAP_BF16 = 1, SNAP_FP16 = 2, SNAP_FP32 = 3 };

// Quantised values are x / scale with scale = absmax / QMAX: 2^14 keeps FP16
// well inside its range (max 65504) with headroom; BF16 has FP32's exponent
// range, so its scale only normalises magnitudes.
constexpr float SNAP_QMAX = 16384.0f;

__host__ __device__ constexpr int snap_bytes(int kind) {
    return kind == SNAP_BF16 || kind == SNAP_FP16 ? 2 : (kind == SNAP_FP32 ? 4 : 0);
}

// ---------------------------------------------------------------- driver API
// cuTensorMapEncodeTiled, resolved once through the runtime's driver entry
// point so the library does not link libcuda directly.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
int get_encode_tiled(EncodeTiledFn* out);

// 4-D tensor map over a snapshot store of nt compact interior fields
// [t][x][y][z] of `kind` with box {bz, by, 1, 1}; needs nz * element size to
// be a multiple of 16 bytes (TMA stride rule).
int make_snap_map(CUtensorMap* map, const void* base, int kind, const Layout& L, long long nt, int bz, int by);

// Builds a 3-D FP32 tensor map over a device field of layout L with box
// {bz, by, 1} (innermost first).
int make_field_map(CUtensorMap* map, const float* base, const Layout& L, int bz, int by);

}  // namespace stg
