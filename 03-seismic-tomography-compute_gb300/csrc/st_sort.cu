// Exclusive prefix sum (int64) and stable LSD radix sort (u64 keys, u32
// payloads) used by the CSR builder.
#include "st_sort.cuh"

namespace stg {
namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* warp_sums, long long* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        long long s = lane < nw ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;  // inclusive warp prefix
    }
    __syncthreads();
    const long long base = warp > 0 ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    return base + x - v;
}

__global__ void scan_reduce_kernel(const long long* __restrict__ in, long long n, long long* __restrict__ part) {
    __shared__ long long ws[32];
    const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    long long s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += in[base + k];
    long long tot;
    block_exclusive_scan(s, ws, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void scan_down_kernel(const long long* __restrict__ in, long long n, const long long* __restrict__ part,
                                 long long* __restrict__ out) {
    __shared__ long long ws[32];
    const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    long long v[SCAN_ITEMS];
    long long s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    long long off = block_exclusive_scan(s, ws, nullptr) + (part ? part[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
}

__global__ void copy_last_total_kernel(const long long* in, const long long* out, long long n, long long* total) {
    *total = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

// ---------------------------------------------------------------- radix sort
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_DIGITS = 256;

__global__ void rs_hist_kernel(const unsigned long long* __restrict__ keys, long long n, int shift, long long ntiles,
                               long long* __restrict__ hist) {
    __shared__ int cnt[RS_DIGITS];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * RS_TILE;
    for (int j = 0; j < RS_ITEMS; ++j) {
        const long long i = base + j * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xff], 1);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void rs_scatter_kernel(const unsigned long long* __restrict__ keys, const unsigned* __restrict__ vals,
                                  long long n, int shift, long long ntiles, const long long* __restrict__ offs,
                                  unsigned long long* __restrict__ okeys, unsigned* __restrict__ ovals) {
    __shared__ int running[RS_DIGITS];
    __shared__ int wcnt[RS_THREADS / 32][RS_DIGITS];
    __shared__ long long tile_off[RS_DIGITS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    running[tid] = 0;
    tile_off[tid] = offs[(long long)tid * ntiles + blockIdx.x];
    for (int w = 0; w < RS_THREADS / 32; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * RS_TILE;
    const unsigned lt = (1u << lane) - 1;
    for (int j = 0; j < RS_ITEMS; ++j) {
        const long long i = base + j * RS_THREADS + tid;
        const bool valid = i < n;
        unsigned long long k = 0;
        unsigned v = 0;
        int d = -1;
        if (valid) {
            k = keys[i];
            v = vals[i];
            d = (int)((k >> shift) & 0xff);
        }
        const unsigned peers = __match_any_sync(FULL, d);
        const int rank_w = __popc(peers & lt);
        const bool leader = valid && rank_w == 0;
        if (leader) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int r = rank_w;
            for (int w = 0; w < warp; ++w) r += wcnt[w][d];
            const long long pos = tile_off[d] + running[d] + r;
            okeys[pos] = k;
            ovals[pos] = v;
        }
        __syncthreads();
        if (leader) {
            atomicAdd(&running[d], __popc(peers));
            wcnt[warp][d] = 0;
        }
        __syncthreads();
    }
}

long long tiles_of(long long n, long long tile) { return (n + tile - 1) / tile; }

}  // namespace

size_t scan_tmp_bytes(long long n) {
    size_t bytes = 0;
    long long m = n;
    while (m > SCAN_TILE) {
        m = tiles_of(m, SCAN_TILE);
        bytes += (size_t)(2 * m + 1) * sizeof(long long);
    }
    return bytes + 64;
}

int exclusive_scan_i64(const long long* in, long long* out, long long n, long long* total, void* tmp,
                       cudaStream_t st) {
    if (n <= 0) {
        if (total) ST_CUDA(cudaMemsetAsync(total, 0, sizeof(long long), st));
        return ST_OK;
    }
    const long long nb = tiles_of(n, SCAN_TILE);
    if (nb == 1) {
        scan_down_kernel<<<1, SCAN_THREADS, 0, st>>>(in, n, nullptr, out);
        count_launch();
    } else {
        long long* part = static_cast<long long*>(tmp);
        long long* part_scan = part + nb;
        void* rest = part_scan + nb + 1;
        scan_reduce_kernel<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, part);
        count_launch();
        ST_CUDA(cudaGetLastError());
        ST_TRY(exclusive_scan_i64(part, part_scan, nb, nullptr, rest, st));
        scan_down_kernel<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, part_scan, out);
        count_launch();
    }
    ST_CUDA(cudaGetLastError());
    if (total) {
        copy_last_total_kernel<<<1, 1, 0, st>>>(in, out, n, total);
        count_launch();
        ST_CUDA(cudaGetLastError());
    }
    return ST_OK;
}

size_t radix_tmp_bytes(long long n) {
    const long long nt = std::max<long long>(1, tiles_of(n, RS_TILE));
    const long long h = nt * RS_DIGITS;
    return (size_t)(2 * h) * sizeof(long long) + scan_tmp_bytes(h) + 256;
}

int radix_sort_u64(unsigned long long* keys, unsigned* vals, unsigned long long* alt_keys, unsigned* alt_vals,
                   long long n, int bits, void* tmp, cudaStream_t st) {
    if (n <= 1 || bits <= 0) return ST_OK;
    const long long ntiles = tiles_of(n, RS_TILE);
    const long long h = ntiles * RS_DIGITS;
    long long* hist = static_cast<long long*>(tmp);
    long long* offs = hist + h;
    void* scan_tmp = offs + h;
    unsigned long long *ka = keys, *kb = alt_keys;
    unsigned *va = vals, *vb = alt_vals;
    const int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        rs_hist_kernel<<<(unsigned)ntiles, RS_THREADS, 0, st>>>(ka, n, shift, ntiles, hist);
        count_launch();
        ST_CUDA(cudaGetLastError());
        ST_TRY(exclusive_scan_i64(hist, offs, h, nullptr, scan_tmp, st));
        rs_scatter_kernel<<<(unsigned)ntiles, RS_THREADS, 0, st>>>(ka, va, n, shift, ntiles, offs, kb, vb);
        count_launch();
        ST_CUDA(cudaGetLastError());
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        ST_CUDA(cudaMemcpyAsync(keys, ka, (size_t)n * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
        ST_CUDA(cudaMemcpyAsync(vals, va, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
    }
    return ST_OK;
}

}  // namespace stg
