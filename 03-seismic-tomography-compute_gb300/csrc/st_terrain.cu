// Irregular seafloor terrain: seismic::TerrainBoundary (solver/boundary.h,
// solver/boundary.cpp) with its field operations on the GPU, and the
// per-column z limits the propagator applies after every step when a
// terrain is attached to a solver (st_solver_set_terrain).
//
// The bathymetry grid (nx * ny depths) is host data, built the reference's
// way (flat water depth, generate_synthetic_bathymetry, or
// set_bathymetry_data points) and mirrored to the device. The field
// operations take the reference's halo-padded layout (FP64) on the host or
// the device; their FP64 arithmetic is written with explicitly rounded
// intrinsics so each value is the source expression evaluated in IEEE
// double.
#include "st_solver_impl.cuh"

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

struct st_terrain {
    st_grid_params p{};
    double water_depth = 0.0;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<double> bathy;  // [nx * ny], column (ix, iy) at ix * ny + iy
    ~st_terrain() {
        if (stream) cudaStreamDestroy(stream);
    }
    int64_t nx() const { return p.nx_global; }
    int64_t ny() const { return p.ny_global; }
    int64_t nz() const { return p.nz_global; }
    int hw() const { return p.halo_width; }
    int64_t padded() const { return (nx() + 2 * hw()) * (ny() + 2 * hw()) * (nz() + 2 * hw()); }
    // seafloor_depth / seafloor_index (boundary.cpp:71-86)
    double depth(int64_t gx, int64_t gy) const {
        if (gx < 0 || gx >= nx() || gy < 0 || gy >= ny()) return water_depth;
        return bathy[gx * ny() + gy];
    }
    int64_t index(int64_t gx, int64_t gy) const { return static_cast<int64_t>(depth(gx, gy) / p.dz); }
};

namespace stg {
namespace {

struct PadGrid {
    int64_t nx, ny, nz;  // interior
    int hw;
    int64_t NYh, NZh, total;
};

PadGrid pad_grid(const st_terrain* t) {
    PadGrid g{t->nx(), t->ny(), t->nz(), t->hw(), 0, 0, 0};
    g.NYh = g.ny + 2 * g.hw;
    g.NZh = g.nz + 2 * g.hw;
    g.total = t->padded();
    return g;
}

unsigned blocks_for(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16));
}

// update_velocity_mask (boundary.cpp:158-186): water above the seafloor,
// below it sediment_vp (1 + 0.3 (depth below the seafloor) / 5000) capped
// at 8500. sfi = per-column seafloor index.
__global__ void velocity_mask_kernel(double* v, PadGrid g, const long long* sfi, double dz, double water_vp,
                                     double sediment_vp) {
    const long long n = g.nx * g.ny * g.nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long ix = k / (g.ny * g.nz), rem = k % (g.ny * g.nz), iy = rem / g.nz, iz = rem % g.nz;
        const long long sf = sfi[ix * g.ny + iy];
        const long long idx = ((ix + g.hw) * g.NYh + (iy + g.hw)) * g.NZh + (iz + g.hw);
        double val;
        if (iz < sf) {
            val = water_vp;
        } else {
            const double grad = __dadd_rn(1.0, __dmul_rn(0.3, __ddiv_rn(__dmul_rn((double)(iz - sf), dz), 5000.0)));
            const double sv = __dmul_rn(sediment_vp, grad);
            val = 8500.0 < sv ? 8500.0 : sv;  // std::min(velocity, 8500.0)
        }
        v[idx] = val;
    }
}

// build_boundary_mask (boundary.cpp:188-214): 1 below the seafloor
// (origin_z + gz dz >= depth), 2 in the water, 0 in the halo.
__global__ void boundary_mask_kernel(unsigned char* m, PadGrid g, const double* depth, double oz, double dz) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < g.total;
         k += (long long)gridDim.x * blockDim.x) {
        const long long X = k / (g.NYh * g.NZh), rem = k % (g.NYh * g.NZh), Y = rem / g.NZh, Z = rem % g.NZh;
        const long long ix = X - g.hw, iy = Y - g.hw, iz = Z - g.hw;
        unsigned char v = 0;
        if (ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny && iz >= 0 && iz < g.nz) {
            const double z = __dadd_rn(oz, __dmul_rn((double)iz, dz));
            v = z >= depth[ix * g.ny + iy] ? 1 : 2;
        }
        m[k] = v;
    }
}

// apply_free_surface_bc (boundary.cpp:88-100): the first interior z plane.
__global__ void free_surface_kernel(double* f, PadGrid g) {
    const long long n = g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long ix = k / g.ny, iy = k % g.ny;
        f[((ix + g.hw) * g.NYh + (iy + g.hw)) * g.NZh + g.hw] = 0.0;
    }
}

// apply_seafloor_bc (boundary.cpp:102-124): per interior column, the flat
// index range [base + hw, base + hw + sf) of the array, as the reference
// writes it (a seafloor below the grid runs on into the following cells,
// bounded only by the array's end).
__global__ void seafloor_kernel(double* f, PadGrid g, const long long* sfi) {
    const long long n = g.nx * g.ny;
    for (long long c = blockIdx.x; c < n; c += gridDim.x) {
        const long long ix = c / g.ny, iy = c % g.ny;
        const long long base = ((ix + g.hw) * g.NYh + (iy + g.hw)) * g.NZh + g.hw;
        const long long lim = base + sfi[c];
        const long long end = lim < g.total ? lim : g.total;
        for (long long i = base + threadIdx.x; i < end; i += blockDim.x) f[i] = 0.0;
    }
}

// apply_absorbing_bc (boundary.cpp:126-156): interior points within
// sponge_width of a face are scaled by 1 - damping (sw - d)^2 / sw^2.
__global__ void absorbing_kernel(double* f, PadGrid g, int sw, double damping) {
    const long long n = g.nx * g.ny * g.nz;
    const double sw2 = (double)(sw * sw);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long ix = k / (g.ny * g.nz), rem = k % (g.ny * g.nz), iy = rem / g.nz, iz = rem % g.nz;
        long long d = min(iz, g.nz - 1 - iz);
        d = min(d, min(ix, g.nx - 1 - ix));
        d = min(d, min(iy, g.ny - 1 - iy));
        if (d < sw && d >= 0) {
            const double s = (double)sw - (double)d;
            const double factor = __dsub_rn(1.0, __ddiv_rn(__dmul_rn(__dmul_rn(damping, s), s), sw2));
            const long long idx = ((ix + g.hw) * g.NYh + (iy + g.hw)) * g.NZh + (iz + g.hw);
            f[idx] = __dmul_rn(f[idx], factor);
        }
    }
}

// Runs `launch(device_ptr)` on a field given on the host (copied in and out)
// or on the device (in place), on the terrain's stream, and waits for it.
template <class T, class F>
int on_field(st_terrain* t, T* field, int on_device, bool copy_in, F launch) {
    ST_CHECK(t && field, ST_ERR_ARG, "null argument");
    ST_CUDA(cudaSetDevice(t->device));
    const size_t bytes = (size_t)t->padded() * sizeof(T);
    T* d = field;
    if (!on_device) {
        ST_CUDA(cudaMallocAsync(&d, bytes, t->stream));
        if (copy_in) ST_CUDA(cudaMemcpyAsync(d, field, bytes, cudaMemcpyHostToDevice, t->stream));
    }
    int rc = launch(d);
    if (!on_device) {
        if (rc == ST_OK) rc = cudaMemcpyAsync(field, d, bytes, cudaMemcpyDeviceToHost, t->stream) == cudaSuccess
                                  ? ST_OK : ST_ERR_CUDA;
        cudaFreeAsync(d, t->stream);
    }
    ST_CUDA(cudaStreamSynchronize(t->stream));
    return rc;
}

// Device copy of a per-column host array (freed with the stream).
template <class T>
T* upload_columns(st_terrain* t, const std::vector<T>& h) {
    T* d = nullptr;
    if (cudaMallocAsync(&d, h.size() * sizeof(T), t->stream) != cudaSuccess) return nullptr;
    if (cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, t->stream) != cudaSuccess) {
        cudaFreeAsync(d, t->stream);
        return nullptr;
    }
    return d;
}

std::vector<long long> seafloor_indices(const st_terrain* t) {
    std::vector<long long> s((size_t)(t->nx() * t->ny()));
    for (int64_t ix = 0; ix < t->nx(); ++ix)
        for (int64_t iy = 0; iy < t->ny(); ++iy) s[(size_t)(ix * t->ny() + iy)] = t->index(ix, iy);
    return s;
}

}  // namespace
}  // namespace stg

using namespace stg;

extern "C" {

int st_terrain_create(const st_grid_params* grid, double water_depth, int device, st_terrain** out) {
    ST_CHECK(grid && out, ST_ERR_ARG, "null argument");
    *out = nullptr;
    ST_CHECK(grid->nx_global > 0 && grid->ny_global > 0 && grid->nz_global > 0 && grid->halo_width >= 0,
             ST_ERR_ARG, "bad terrain grid");
    ST_CHECK(grid->dz > 0.0 && grid->dx > 0.0 && grid->dy > 0.0, ST_ERR_ARG, "grid spacing must be positive");
    std::unique_ptr<st_terrain> t(new st_terrain());
    t->p = *grid;
    t->water_depth = water_depth;
    t->device = device;
    // TerrainBoundary::TerrainBoundary (boundary.cpp:8-14): flat water depth
    t->bathy.assign((size_t)(grid->nx_global * grid->ny_global), water_depth);
    ST_CUDA(cudaSetDevice(device));
    ST_CUDA(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking));
    *out = t.release();
    return ST_OK;
}

int st_terrain_destroy(st_terrain* t) {
    if (!t) return ST_OK;
    cudaSetDevice(t->device);
    cudaStreamSynchronize(t->stream);
    delete t;
    return ST_OK;
}

int st_terrain_set_bathymetry_data(st_terrain* t, const st_bathymetry_point* pts, int64_t n) {
    ST_CHECK(t && (pts || n == 0) && n >= 0, ST_ERR_ARG, "bad bathymetry points");
    // set_bathymetry_data (boundary.cpp:16-32): the cell of each point, points
    // outside the grid ignored, later points win
    for (int64_t k = 0; k < n; ++k) {
        const double qx = (pts[k].x - t->p.origin_x) / t->p.dx;
        const double qy = (pts[k].y - t->p.origin_y) / t->p.dy;
        if (!(qx > -1.0 && qx < (double)t->nx() && qy > -1.0 && qy < (double)t->ny())) continue;
        const int64_t ix = static_cast<int64_t>(qx), iy = static_cast<int64_t>(qy);
        if (ix >= 0 && ix < t->nx() && iy >= 0 && iy < t->ny()) t->bathy[(size_t)(ix * t->ny() + iy)] = pts[k].depth;
    }
    return ST_OK;
}

int st_terrain_generate_synthetic_bathymetry(st_terrain* t, double gradient, double roughness) {
    ST_CHECK(t, ST_ERR_ARG, "null argument");
    // generate_synthetic_bathymetry (boundary.cpp:34-57), on the host
    const double pi = 3.14159265358979323846;
    for (int64_t ix = 0; ix < t->nx(); ++ix)
        for (int64_t iy = 0; iy < t->ny(); ++iy) {
            const double x = ix * t->p.dx, y = iy * t->p.dy;
            double d = t->water_depth + gradient * x +
                       roughness * std::sin(2.0 * pi * x / 5000.0) * std::cos(2.0 * pi * y / 7000.0) +
                       roughness * 0.5 * std::sin(4.0 * pi * x / 3000.0);
            d = std::min(std::max(d, 500.0), 8000.0);
            t->bathy[(size_t)(ix * t->ny() + iy)] = d;
        }
    return ST_OK;
}

int st_terrain_bathymetry(st_terrain* t, double* out) {
    ST_CHECK(t && out, ST_ERR_ARG, "null argument");
    std::copy(t->bathy.begin(), t->bathy.end(), out);
    return ST_OK;
}

int st_terrain_seafloor(st_terrain* t, int64_t gx, int64_t gy, double* depth, int64_t* index) {
    ST_CHECK(t, ST_ERR_ARG, "null argument");
    if (depth) *depth = t->depth(gx, gy);
    if (index) *index = t->index(gx, gy);
    return ST_OK;
}

int st_terrain_update_velocity_mask(st_terrain* t, double* velocity, int on_device, double water_vp,
                                    double sediment_vp) {
    return on_field(t, velocity, on_device, true, [&](double* d) {
        long long* sfi = upload_columns(t, seafloor_indices(t));
        ST_CHECK(sfi, ST_ERR_ALLOC, "terrain column table");
        const PadGrid g = pad_grid(t);
        velocity_mask_kernel<<<blocks_for(g.nx * g.ny * g.nz), 256, 0, t->stream>>>(d, g, sfi, t->p.dz, water_vp,
                                                                                     sediment_vp);
        count_launch();
        const cudaError_t e = cudaGetLastError();
        cudaFreeAsync(sfi, t->stream);
        ST_CUDA(e);
        return ST_OK;
    });
}

int st_terrain_build_boundary_mask(st_terrain* t, uint8_t* mask, int on_device) {
    return on_field(t, mask, on_device, false, [&](uint8_t* d) {
        double* dep = upload_columns(t, t->bathy);
        ST_CHECK(dep, ST_ERR_ALLOC, "terrain column table");
        const PadGrid g = pad_grid(t);
        boundary_mask_kernel<<<blocks_for(g.total), 256, 0, t->stream>>>(d, g, dep, t->p.origin_z, t->p.dz);
        count_launch();
        const cudaError_t e = cudaGetLastError();
        cudaFreeAsync(dep, t->stream);
        ST_CUDA(e);
        return ST_OK;
    });
}

int st_terrain_apply_free_surface_bc(st_terrain* t, double* field, int on_device) {
    return on_field(t, field, on_device, true, [&](double* d) {
        const PadGrid g = pad_grid(t);
        free_surface_kernel<<<blocks_for(g.nx * g.ny), 256, 0, t->stream>>>(d, g);
        count_launch();
        ST_CUDA(cudaGetLastError());
        return ST_OK;
    });
}

int st_terrain_apply_seafloor_bc(st_terrain* t, double* field, int on_device) {
    return on_field(t, field, on_device, true, [&](double* d) {
        long long* sfi = upload_columns(t, seafloor_indices(t));
        ST_CHECK(sfi, ST_ERR_ALLOC, "terrain column table");
        const PadGrid g = pad_grid(t);
        seafloor_kernel<<<(unsigned)std::min<long long>(g.nx * g.ny, 152LL * 32), 128, 0, t->stream>>>(d, g, sfi);
        count_launch();
        const cudaError_t e = cudaGetLastError();
        cudaFreeAsync(sfi, t->stream);
        ST_CUDA(e);
        return ST_OK;
    });
}

int st_terrain_apply_absorbing_bc(st_terrain* t, double* field, int on_device, int sponge_width, double damping) {
    return on_field(t, field, on_device, true, [&](double* d) {
        const PadGrid g = pad_grid(t);
        absorbing_kernel<<<blocks_for(g.nx * g.ny * g.nz), 256, 0, t->stream>>>(d, g, sponge_width, damping);
        count_launch();
        ST_CUDA(cudaGetLastError());
        return ST_OK;
    });
}

int st_generate_bathymetry(int64_t nx, int64_t ny, double dx, double dy, double origin_x, double origin_y,
                           double water_depth, double gradient, double roughness, double* out) {
    ST_CHECK(out && nx > 0 && ny > 0, ST_ERR_ARG, "bad bathymetry request");
    // the binding's generate_bathymetry (pybind/bindings.cpp:255-270): host only
    st_terrain t;
    t.p = st_grid_params{nx, ny, 1, dx, dy, 1.0, origin_x, origin_y, 0.0, 0};
    t.water_depth = water_depth;
    t.bathy.assign((size_t)(nx * ny), water_depth);
    ST_TRY(st_terrain_generate_synthetic_bathymetry(&t, gradient, roughness));
    std::copy(t.bathy.begin(), t.bathy.end(), out);
    return ST_OK;
}

int st_solver_set_terrain(st_solver* s, st_terrain* t, int flags) {
    ST_CHECK(s, ST_ERR_ARG, "null solver");
    ST_CUDA(cudaSetDevice(s->device));
    if (!t || !(flags & (ST_TERRAIN_FREE_SURFACE | ST_TERRAIN_SEAFLOOR))) {
        cudaFree(s->zlim);
        s->zlim = nullptr;
        return ST_OK;
    }
    ST_CHECK(t->nx() == s->L.nx && t->ny() == s->L.ny && t->nz() == s->L.nz, ST_ERR_ARG,
             "terrain grid does not match the solver's");
    std::vector<int> zl((size_t)(t->nx() * t->ny()));
    for (int64_t ix = 0; ix < t->nx(); ++ix)
        for (int64_t iy = 0; iy < t->ny(); ++iy) {
            int64_t z = (flags & ST_TERRAIN_FREE_SURFACE) ? 1 : 0;
            if (flags & ST_TERRAIN_SEAFLOOR) z = std::max(z, t->index(ix, iy));
            zl[(size_t)(ix * t->ny() + iy)] = (int)std::min<int64_t>(std::max<int64_t>(z, 0), t->nz());
        }
    if (!s->zlim) ST_CUDA(cudaMalloc(&s->zlim, zl.size() * sizeof(int)));
    ST_CUDA(cudaMemcpy(s->zlim, zl.data(), zl.size() * sizeof(int), cudaMemcpyHostToDevice));
    return ST_OK;
}

}  // extern "C"
