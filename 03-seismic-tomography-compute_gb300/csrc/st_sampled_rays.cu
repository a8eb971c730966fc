// Midpoint-sampled straight rays: the traveltime forward model and gradient
// of the reference's Python inversion driver (AdjointStateInversion.
// _forward_model / _compute_gradient, seismic_tomography/inversion.py:
// 329-433) as device kernels over a sample list built once per pick set.
//
// Build (st_ray_picks_create):
//   1. pick_geometry_kernel: per pick, the snapped source and station cells,
//      the distance, n = max(int(dist / (5 dx)), 2) and ds = dist / n.
//   2. exclusive scan of the sample counts -> per-pick offsets.
//   3. pick_samples_kernel (one warp per pick, lanes over samples): the cell
//      of every sample, in the reference's (pick, sample) order.
//   4. a stable radix sort of the samples by cell: within a cell the samples
//      stay in (pick, sample) order, which is the order in which the
//      reference's loop adds them into gradient[cell]; plus a histogram scan
//      for the per-cell offsets.
// Forward: one thread per pick adds its samples sequentially (the
// reference's order). Gradient: one thread per cell adds its samples in the
// sorted order. Both kernels are bound by the FP64 pipe (one correctly
// rounded division per sample); threads take picks and cells in order of
// their sample counts, so the lanes of a warp run loops of similar length
// and the FP64 pipe is not spent on masked-off lanes. All FP64 arithmetic is written with explicitly rounded
// intrinsics (no contraction into FMA), so each value is the reference's
// expression evaluated in IEEE double: the results match it bit for bit
// given the same source-station distances.
#include "st_sort.cuh"
#include "st_sparse.cuh"

#include <algorithm>
#include <cmath>
#include <memory>

struct st_ray_picks {
    int device = 0;
    cudaStream_t stream = nullptr;
    st_ray_model model{};
    long long n_picks = 0, n_samples = 0, n_cells = 0;
    double* ds = nullptr;         // [n_picks] sample length
    double* dist = nullptr;       // [n_picks] source-station distance
    double* weight = nullptr;     // [n_picks]
    long long* off = nullptr;     // [n_picks + 1] sample offsets (invalid picks: none)
    int* cell = nullptr;          // [n_samples] cell of each sample, pick-major
    long long* cell_ptr = nullptr;  // [n_cells + 1] offsets into t_pick
    int* t_pick = nullptr;        // [n_samples] pick of each sample, cell-major
    int* pick_order = nullptr;    // [n_picks] picks by descending sample count
    int* cell_order = nullptr;    // [n_cells] cells by descending sample count
    double* stage_vp = nullptr;   // host-call staging: [n_cells]
    double* stage_res = nullptr;  // [n_picks]
    double* stage_out = nullptr;  // [max(n_cells, n_picks)]
    ~st_ray_picks() {
        cudaFree(ds);
        cudaFree(dist);
        cudaFree(weight);
        cudaFree(off);
        cudaFree(cell);
        cudaFree(cell_ptr);
        cudaFree(t_pick);
        cudaFree(pick_order);
        cudaFree(cell_order);
        cudaFree(stage_vp);
        cudaFree(stage_res);
        cudaFree(stage_out);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace stg {
namespace {

constexpr long long kMaxSteps = 1ll << 24;

struct PickGrid {
    long long n[3];
    double d[3];
    double o[3];
};

// int((p - o) / d) clamped to [0, n - 1] (inversion.py:344-350). Python's
// int() truncates toward zero, so everything below 1 lands on cell 0.
__device__ inline long long snap(double p, double o, double d, long long n) {
    const double q = __ddiv_rn(__dsub_rn(p, o), d);
    if (q < 1.0) return 0;
    if (q >= (double)(n - 1)) return n - 1;
    return (long long)q;
}

__global__ void pick_geometry_kernel(long long np, const double* __restrict__ src, const double* __restrict__ sta,
                                     const double* __restrict__ dist_in, const unsigned char* __restrict__ valid,
                                     PickGrid G, int* __restrict__ cells, double* __restrict__ dist,
                                     double* __restrict__ ds, long long* __restrict__ count, int* __restrict__ err) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np;
         i += (long long)gridDim.x * blockDim.x) {
        const double* s = src + 3 * i;
        const double* r = sta + 3 * i;
        double dd;
        if (dist_in) {
            dd = dist_in[i];
        } else {
            const double ex = __dsub_rn(s[0], r[0]), ey = __dsub_rn(s[1], r[1]), ez = __dsub_rn(s[2], r[2]);
            dd = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
        }
        for (int a = 0; a < 3; ++a) {
            cells[6 * i + a] = (int)snap(s[a], G.o[a], G.d[a], G.n[a]);
            cells[6 * i + 3 + a] = (int)snap(r[a], G.o[a], G.d[a], G.n[a]);
        }
        // n = max(int(dist / (dx * 5)), 2) (inversion.py:352)
        const double q = __ddiv_rn(dd, __dmul_rn(G.d[0], 5.0));
        long long n = 0;
        if (!valid || valid[i]) {
            if (!(q < (double)kMaxSteps)) {  // also catches a non-finite distance
                atomicExch(err, 1);
            } else {
                n = q < 3.0 ? 2 : (long long)q;
            }
        }
        count[i] = n;
        dist[i] = dd;
        ds[i] = n ? __ddiv_rn(dd, (double)n) : 0.0;
    }
}

// One warp per pick: cell of sample k = (int(c0 + frac (c1 - c0)) per axis,
// frac = (k + 0.5) / n (inversion.py:355-364; the clamp there is a no-op
// because the value lies between two in-grid cells).
__global__ void pick_samples_kernel(long long np, const int* __restrict__ cells, const long long* __restrict__ off,
                                    PickGrid G, int* __restrict__ cell, unsigned long long* __restrict__ key,
                                    unsigned* __restrict__ payload, unsigned* __restrict__ spick) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; i < np; i += warps) {
        const long long o = off[i];
        const long long n = off[i + 1] - o;
        if (n == 0) continue;
        const int* c = cells + 6 * i;
        const double dn = (double)n;
        for (long long k = lane; k < n; k += 32) {
            const double frac = __ddiv_rn(__dadd_rn((double)k, 0.5), dn);
            long long idx = 0;
            for (int a = 0; a < 3; ++a) {
                long long v = (long long)__dadd_rn((double)c[a], __dmul_rn(frac, (double)(c[3 + a] - c[a])));
                v = v < 0 ? 0 : (v > G.n[a] - 1 ? G.n[a] - 1 : v);
                idx = idx * G.n[a] + v;
            }
            cell[o + k] = (int)idx;
            key[o + k] = (unsigned long long)idx;
            payload[o + k] = (unsigned)(o + k);
            spick[o + k] = (unsigned)i;
        }
    }
}

__global__ void cell_histogram_kernel(const int* __restrict__ cell, long long ns, unsigned long long* cnt) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ns;
         k += (long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + cell[k], 1ull);
}

// keys[j] = 2^32 - 1 - count of item j, vals[j] = j: an ascending sort
// lists the items by descending sample count (the count-ordered schedules
// start the longest loops first, so the light ones fill the tail).
template <class T>
__global__ void count_keys_kernel(const T* __restrict__ cnt, long long n, unsigned long long* __restrict__ keys,
                                  unsigned* __restrict__ vals) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
         j += (long long)gridDim.x * blockDim.x) {
        keys[j] = 0xffffffffull - (unsigned long long)cnt[j];
        vals[j] = (unsigned)j;
    }
}

__global__ void iota_kernel(int* __restrict__ a, long long n) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
         j += (long long)gridDim.x * blockDim.x)
        a[j] = (int)j;
}

__global__ void gather_pick_kernel(const unsigned* __restrict__ order, const unsigned* __restrict__ spick,
                                   long long ns, int* __restrict__ t_pick) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ns;
         k += (long long)gridDim.x * blockDim.x)
        t_pick[k] = (int)spick[order[k]];
}

__device__ inline bool valid_velocity(double v) { return isfinite(v) && v > 0.0; }

// _forward_model (inversion.py:329-381), one thread per pick, the samples
// added in order. The loads and divisions of four samples are issued
// together (they are independent); only the additions keep the reference's
// order.
__global__ void ray_forward_kernel(long long np, const int* __restrict__ order, const long long* __restrict__ off,
                                   const int* __restrict__ cell, const double* __restrict__ ds,
                                   const double* __restrict__ dist, const double* __restrict__ vp,
                                   double* __restrict__ times) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < np;
         j += (long long)gridDim.x * blockDim.x) {
        const long long i = order[j];
        const long long b = off[i], e = off[i + 1];
        const double d = ds[i];
        double t = 0.0;
        long long k = b;
        for (; k + 4 <= e; k += 4) {
            double term[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                double v = __ldg(vp + __ldg(cell + k + j));
                if (!valid_velocity(v)) v = 1500.0;
                term[j] = __ddiv_rn(d, v);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (isfinite(term[j])) t = __dadd_rn(t, term[j]);
        }
        for (; k < e; ++k) {
            double v = __ldg(vp + __ldg(cell + k));
            if (!valid_velocity(v)) v = 1500.0;
            const double term = __ddiv_rn(d, v);
            if (isfinite(term)) t = __dadd_rn(t, term);
        }
        if (b < e && (!isfinite(t) || t < 0.0)) t = __ddiv_rn(dist[i], 6000.0);
        times[i] = t;
    }
}

// _compute_gradient (inversion.py:383-433), one thread per cell, its samples
// in (pick, sample) order: g += (r * (-ds / (v * v))) * w. Terms of four
// samples are formed together; the additions keep the order.
__device__ inline double grad_term(int i, double vv, const double* __restrict__ ds, const double* __restrict__ weight,
                                   const double* __restrict__ res, bool* ok) {
    const double r = __ldg(res + i);
    const double f = __ddiv_rn(-__ldg(ds + i), vv);
    *ok = isfinite(r) && isfinite(f);
    return __dmul_rn(__dmul_rn(r, f), __ldg(weight + i));
}

__global__ void ray_gradient_kernel(long long nc, const int* __restrict__ order,
                                    const long long* __restrict__ cell_ptr, const int* __restrict__ t_pick,
                                    const double* __restrict__ ds, const double* __restrict__ weight,
                                    const double* __restrict__ vp, const double* __restrict__ res,
                                    double* __restrict__ g) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nc;
         j += (long long)gridDim.x * blockDim.x) {
        const long long c = order[j];
        const long long b = cell_ptr[c], e = cell_ptr[c + 1];
        const double v = vp[c];
        double acc = 0.0;
        if (b < e && valid_velocity(v)) {
            const double vv = __dmul_rn(v, v);
            long long k = b;
            for (; k + 4 <= e; k += 4) {
                double term[4];
                bool ok[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) term[j] = grad_term(__ldg(t_pick + k + j), vv, ds, weight, res, ok + j);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (ok[j]) acc = __dadd_rn(acc, term[j]);
            }
            for (; k < e; ++k) {
                bool ok;
                const double term = grad_term(__ldg(t_pick + k), vv, ds, weight, res, &ok);
                if (ok) acc = __dadd_rn(acc, term);
            }
        }
        g[c] = acc;
    }
}

// (pick, cell, ds) triplets of every sample, for the sampled-ray CSR.
__global__ void ray_triplet_kernel(long long np, const long long* __restrict__ off, const int* __restrict__ cell,
                                   const double* __restrict__ ds, long long* __restrict__ rows,
                                   long long* __restrict__ cols, double* __restrict__ vals) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; i < np; i += warps) {
        const long long b = off[i], e = off[i + 1];
        const double d = ds[i];
        for (long long k = b + lane; k < e; k += 32) {
            rows[k] = i;
            cols[k] = cell[k];
            vals[k] = d;
        }
    }
}

unsigned blocks_for(long long n, int per_block) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + per_block - 1) / per_block, 152LL * 32));
}

int bits_for(long long n) {
    int b = 1;
    while ((1ll << b) < n) ++b;
    return b;
}

}  // namespace

int build_sampled_ray_csr(const st_ray_picks* p, DevCsr* out, long long* nnz, cudaStream_t st) {
    DeviceBuffers bufs;
    const long long ns = std::max<long long>(p->n_samples, 1);
    auto* r = static_cast<long long*>(bufs.get((size_t)ns * 8));
    auto* c = static_cast<long long*>(bufs.get((size_t)ns * 8));
    auto* v = static_cast<double*>(bufs.get((size_t)ns * 8));
    if (!r || !c || !v) return bufs.fail();
    if (p->n_samples > 0) {
        ray_triplet_kernel<<<blocks_for(p->n_picks * 32, 256), 256, 0, st>>>(p->n_picks, p->off, p->cell, p->ds, r,
                                                                             c, v);
        count_launch();
        ST_CUDA(cudaGetLastError());
    }
    if (nnz) *nnz = p->n_samples;
    return build_csr<long long, double>(p->n_picks, p->n_cells, p->n_samples, r, c, v, false, out, st);
}

}  // namespace stg

using namespace stg;

namespace {

int build_samples(st_ray_picks* p, const double* src, const double* sta, const double* dist,
                  const unsigned char* valid) {
    cudaStream_t st = p->stream;
    const long long np = p->n_picks;
    PickGrid G{{p->model.nx, p->model.ny, p->model.nz},
               {p->model.dx, p->model.dy, p->model.dz},
               {p->model.origin_x, p->model.origin_y, p->model.origin_z}};
    DeviceBuffers bufs;
    const long long npp = std::max<long long>(np, 1);
    auto* d_src = static_cast<double*>(bufs.get((size_t)npp * 24));
    auto* d_sta = static_cast<double*>(bufs.get((size_t)npp * 24));
    auto* d_dist = dist ? static_cast<double*>(bufs.get((size_t)npp * 8)) : nullptr;
    auto* d_valid = valid ? static_cast<unsigned char*>(bufs.get((size_t)npp)) : nullptr;
    auto* cells = static_cast<int*>(bufs.get((size_t)npp * 24));
    auto* count = static_cast<long long*>(bufs.get((size_t)(npp + 1) * 8));
    auto* err = static_cast<int*>(bufs.get(sizeof(int)));
    void* stmp = bufs.get(scan_tmp_bytes(std::max<long long>(std::max(np, p->n_cells), 1)));
    if (!d_src || !d_sta || (dist && !d_dist) || (valid && !d_valid) || !cells || !count || !err || !stmp)
        return bufs.fail();
    ST_CUDA(cudaMalloc(&p->off, (size_t)(npp + 1) * 8));
    ST_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    ST_CUDA(cudaMemsetAsync(p->off, 0, (size_t)(npp + 1) * 8, st));
    long long total = 0;
    if (np > 0) {
        ST_CUDA(cudaMemcpyAsync(d_src, src, (size_t)np * 24, cudaMemcpyHostToDevice, st));
        ST_CUDA(cudaMemcpyAsync(d_sta, sta, (size_t)np * 24, cudaMemcpyHostToDevice, st));
        if (dist) ST_CUDA(cudaMemcpyAsync(d_dist, dist, (size_t)np * 8, cudaMemcpyHostToDevice, st));
        if (valid) ST_CUDA(cudaMemcpyAsync(d_valid, valid, (size_t)np, cudaMemcpyHostToDevice, st));
        pick_geometry_kernel<<<blocks_for(np, 256), 256, 0, st>>>(np, d_src, d_sta, d_dist, d_valid, G, cells,
                                                                  p->dist, p->ds, count, err);
        count_launch();
        ST_CUDA(cudaGetLastError());
        ST_TRY(exclusive_scan_i64(count, p->off, np, p->off + np, stmp, st));
        int herr = 0;
        ST_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaMemcpyAsync(&total, p->off + np, sizeof(long long), cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
        ST_CHECK(!herr, ST_ERR_ARG, "a pick's ray has more than %lld samples (or a non-finite distance)", kMaxSteps);
        ST_CHECK(total < (1ll << 32), ST_ERR_ARG, "%lld samples exceed the 2^32 limit of one pick set", total);
    }
    p->n_samples = total;
    const long long ns = std::max<long long>(total, 1);
    ST_CUDA(cudaMalloc(&p->cell, (size_t)ns * 4));
    ST_CUDA(cudaMalloc(&p->t_pick, (size_t)ns * 4));
    ST_CUDA(cudaMalloc(&p->cell_ptr, (size_t)(p->n_cells + 1) * 8));
    ST_CUDA(cudaMemsetAsync(p->cell_ptr, 0, (size_t)(p->n_cells + 1) * 8, st));
    ST_CUDA(cudaMalloc(&p->pick_order, (size_t)npp * 4));
    ST_CUDA(cudaMalloc(&p->cell_order, (size_t)p->n_cells * 4));
    if (total == 0) {  // no samples: identity schedules
        iota_kernel<<<blocks_for(npp, 256), 256, 0, st>>>(p->pick_order, npp);
        count_launch();
        iota_kernel<<<blocks_for(p->n_cells, 256), 256, 0, st>>>(p->cell_order, p->n_cells);
        count_launch();
        ST_CUDA(cudaGetLastError());
        ST_CUDA(cudaStreamSynchronize(st));
        return ST_OK;
    }
    auto* key = static_cast<unsigned long long*>(bufs.get((size_t)ns * 8));
    auto* key2 = static_cast<unsigned long long*>(bufs.get((size_t)ns * 8));
    auto* pay = static_cast<unsigned*>(bufs.get((size_t)ns * 4));
    auto* pay2 = static_cast<unsigned*>(bufs.get((size_t)ns * 4));
    auto* spick = static_cast<unsigned*>(bufs.get((size_t)ns * 4));
    auto* cnt = static_cast<unsigned long long*>(bufs.get((size_t)(p->n_cells + 1) * 8));
    void* rtmp = bufs.get(radix_tmp_bytes(total));
    if (!key || !key2 || !pay || !pay2 || !spick || !cnt || !rtmp) return bufs.fail();
    pick_samples_kernel<<<blocks_for(np * 32, 256), 256, 0, st>>>(np, cells, p->off, G, p->cell, key, pay, spick);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_CUDA(cudaMemsetAsync(cnt, 0, (size_t)(p->n_cells + 1) * 8, st));
    cell_histogram_kernel<<<blocks_for(total, 256), 256, 0, st>>>(p->cell, total, cnt);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_TRY(exclusive_scan_i64(reinterpret_cast<const long long*>(cnt), p->cell_ptr, p->n_cells,
                              p->cell_ptr + p->n_cells, stmp, st));
    ST_TRY(radix_sort_u64(key, pay, key2, pay2, total, bits_for(p->n_cells), rtmp, st));
    gather_pick_kernel<<<blocks_for(total, 256), 256, 0, st>>>(pay, spick, total, p->t_pick);
    count_launch();
    ST_CUDA(cudaGetLastError());
    // count-ordered schedules: reuse the sample-sort buffers when they are
    // large enough (n_picks and n_cells may exceed the sample count)
    const long long nmax = std::max(np, p->n_cells);
    unsigned long long *ok = key, *ok2 = key2;
    unsigned *ov = pay, *ov2 = pay2;
    void* otmp = rtmp;
    if (nmax > total) {
        ok = static_cast<unsigned long long*>(bufs.get((size_t)nmax * 8));
        ok2 = static_cast<unsigned long long*>(bufs.get((size_t)nmax * 8));
        ov = static_cast<unsigned*>(bufs.get((size_t)nmax * 4));
        ov2 = static_cast<unsigned*>(bufs.get((size_t)nmax * 4));
        otmp = bufs.get(radix_tmp_bytes(nmax));
        if (!ok || !ok2 || !ov || !ov2 || !otmp) return bufs.fail();
    }
    count_keys_kernel<<<blocks_for(np, 256), 256, 0, st>>>(count, np, ok, ov);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_TRY(radix_sort_u64(ok, ov, ok2, ov2, np, 32, otmp, st));
    ST_CUDA(cudaMemcpyAsync(p->pick_order, ov, (size_t)np * 4, cudaMemcpyDeviceToDevice, st));
    count_keys_kernel<<<blocks_for(p->n_cells, 256), 256, 0, st>>>(cnt, p->n_cells, ok, ov);
    count_launch();
    ST_CUDA(cudaGetLastError());
    ST_TRY(radix_sort_u64(ok, ov, ok2, ov2, p->n_cells, 32, otmp, st));
    ST_CUDA(cudaMemcpyAsync(p->cell_order, ov, (size_t)p->n_cells * 4, cudaMemcpyDeviceToDevice, st));
    ST_CUDA(cudaStreamSynchronize(st));
    return ST_OK;
}

}  // namespace

extern "C" {

int st_ray_picks_create(int device, const st_ray_model* model, int64_t n_picks, const double* src_xyz,
                        const double* sta_xyz, const double* dist, const double* weight, const uint8_t* valid,
                        st_ray_picks** out) {
    ST_CHECK(model && out && (n_picks == 0 || (src_xyz && sta_xyz && weight)), ST_ERR_ARG, "null argument");
    *out = nullptr;
    ST_CHECK(n_picks >= 0 && n_picks < (1ll << 31), ST_ERR_ARG, "pick count out of range (%lld)",
             (long long)n_picks);
    ST_CHECK(model->nx > 0 && model->ny > 0 && model->nz > 0, ST_ERR_ARG, "bad model extents");
    ST_CHECK(model->nx * model->ny * model->nz < (1ll << 31), ST_ERR_ARG, "cell count must fit int32");
    const double sp[3] = {model->dx, model->dy, model->dz};
    const double org[3] = {model->origin_x, model->origin_y, model->origin_z};
    for (int a = 0; a < 3; ++a) {
        ST_CHECK(std::isfinite(sp[a]) && sp[a] > 0.0, ST_ERR_ARG, "cell spacing must be positive and finite");
        ST_CHECK(std::isfinite(org[a]), ST_ERR_ARG, "model origin must be finite");
    }
    for (int64_t i = 0; i < n_picks; ++i) {
        if (valid && !valid[i]) continue;
        for (int a = 0; a < 3; ++a)
            ST_CHECK(std::isfinite(src_xyz[3 * i + a]) && std::isfinite(sta_xyz[3 * i + a]), ST_ERR_ARG,
                     "pick %lld has a non-finite source or station coordinate", (long long)i);
        if (dist)
            ST_CHECK(std::isfinite(dist[i]) && dist[i] >= 0.0, ST_ERR_ARG,
                     "pick %lld: distance must be finite and non-negative", (long long)i);
    }
    int ndev = 0;
    ST_CUDA(cudaGetDeviceCount(&ndev));
    ST_CHECK(device >= 0 && device < ndev, ST_ERR_ARG, "device %d out of range", device);
    ST_CUDA(cudaSetDevice(device));
    std::unique_ptr<st_ray_picks> p(new st_ray_picks());
    p->device = device;
    p->model = *model;
    p->n_picks = n_picks;
    p->n_cells = model->nx * model->ny * model->nz;
    ST_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    const long long npp = std::max<long long>(n_picks, 1);
    ST_CUDA(cudaMalloc(&p->ds, (size_t)npp * 8));
    ST_CUDA(cudaMalloc(&p->dist, (size_t)npp * 8));
    ST_CUDA(cudaMalloc(&p->weight, (size_t)npp * 8));
    ST_CUDA(cudaMalloc(&p->stage_vp, (size_t)p->n_cells * 8));
    ST_CUDA(cudaMalloc(&p->stage_res, (size_t)npp * 8));
    ST_CUDA(cudaMalloc(&p->stage_out, (size_t)std::max(npp, p->n_cells) * 8));
    if (n_picks)
        ST_CUDA(cudaMemcpyAsync(p->weight, weight, (size_t)n_picks * 8, cudaMemcpyHostToDevice, p->stream));
    ST_TRY(build_samples(p.get(), src_xyz, sta_xyz, dist, valid));
    *out = p.release();
    return ST_OK;
}

int st_ray_picks_destroy(st_ray_picks* p) {
    if (!p) return ST_OK;
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    delete p;
    return ST_OK;
}

int st_ray_picks_info(st_ray_picks* p, int64_t out[3]) {
    ST_CHECK(p && out, ST_ERR_ARG, "null argument");
    out[0] = p->n_picks;
    out[1] = p->n_samples;
    out[2] = p->n_cells;
    return ST_OK;
}

int st_ray_picks_stream(st_ray_picks* p, void** out) {
    ST_CHECK(p && out, ST_ERR_ARG, "null argument");
    *out = p->stream;
    return ST_OK;
}

int st_ray_picks_forward_model(st_ray_picks* p, const double* vp, int on_device, double* times) {
    ST_CHECK(p && vp && (times || p->n_picks == 0), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(p->device));
    cudaStream_t st = p->stream;
    const double* dvp = vp;
    double* dt = times;
    if (!on_device) {
        ST_CUDA(cudaMemcpyAsync(p->stage_vp, vp, (size_t)p->n_cells * 8, cudaMemcpyHostToDevice, st));
        dvp = p->stage_vp;
        dt = p->stage_out;
    }
    if (p->n_picks > 0) {
        ray_forward_kernel<<<blocks_for(p->n_picks, 128), 128, 0, st>>>(p->n_picks, p->pick_order, p->off, p->cell,
                                                                        p->ds, p->dist, dvp, dt);
        count_launch();
        ST_CUDA(cudaGetLastError());
    }
    if (!on_device) {
        if (p->n_picks)
            ST_CUDA(cudaMemcpyAsync(times, dt, (size_t)p->n_picks * 8, cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
    }
    return ST_OK;
}

int st_ray_picks_compute_gradient(st_ray_picks* p, const double* vp, const double* residuals, int on_device,
                                  double* gradient) {
    ST_CHECK(p && vp && gradient && (residuals || p->n_picks == 0), ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(p->device));
    cudaStream_t st = p->stream;
    const double* dvp = vp;
    const double* dres = residuals;
    double* dg = gradient;
    if (!on_device) {
        ST_CUDA(cudaMemcpyAsync(p->stage_vp, vp, (size_t)p->n_cells * 8, cudaMemcpyHostToDevice, st));
        if (p->n_picks)
            ST_CUDA(cudaMemcpyAsync(p->stage_res, residuals, (size_t)p->n_picks * 8, cudaMemcpyHostToDevice, st));
        dvp = p->stage_vp;
        dres = p->stage_res;
        dg = p->stage_out;
    }
    ray_gradient_kernel<<<blocks_for(p->n_cells, 128), 128, 0, st>>>(p->n_cells, p->cell_order, p->cell_ptr,
                                                                     p->t_pick, p->ds, p->weight, dvp, dres, dg);
    count_launch();
    ST_CUDA(cudaGetLastError());
    if (!on_device) {
        ST_CUDA(cudaMemcpyAsync(gradient, dg, (size_t)p->n_cells * 8, cudaMemcpyDeviceToHost, st));
        ST_CUDA(cudaStreamSynchronize(st));
    }
    return ST_OK;
}

}  // extern "C"
