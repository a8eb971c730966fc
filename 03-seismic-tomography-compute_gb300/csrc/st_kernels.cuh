// Host-side declarations of the kernel launchers shared by the C-ABI files.
#pragma once

#include "st_common.cuh"

namespace stg {

// Arguments of one fused propagator step (fd_step_kernel). Field indices are
// device-layout indices; receiver numbering is q = irx * rny + iry.
struct StepArgs {
    float* out;              // field written: the update at every interior point
    int nx, ny, nz, NZP;
    long long plane;
    int x_chunk;             // x-planes marched by one CTA
    float ax, ay, az;        // 1/dx^2, 1/dy^2, 1/dz^2
    float amp;               // amplitude clamp (WaveEquationSolver::amplitude_limit_)
    int sw;                  // sponge width
    const float* dtab;       // sponge factor by distance, dtab[d] for 0 <= d < sw
    long long inj_idx;       // fused point injection into the written field, -1 = none
    float inj_val;
    int rz, rx0, rsx, rnx, ry0, rsy, rny;  // receiver grid on plane z = rz
    float* seis_row;         // receiver samples of the update (before injection/forcing), or null
    const float* force_row;  // adds c * force_row[q] at receiver q (adjoint forcing), or null
    void* snap_out;          // snapshot of this step's centre field (compact interior), or null
    const unsigned* amax_cur;  // |max| bits of the centre field (snapshot scale)
    unsigned* amax_next;     // |max| of the written field is atomically max-ed here
    const void* snap_in;     // forward snapshot paired with this step's centre field (imaging)
    const unsigned* amax_in;
    float* image;            // image += f * (centre / c)   (compact interior)
    float* illum;            // illum += f * f
    unsigned* flags;         // FLAG_GUARD / FLAG_TIMEOUT
    unsigned long long timeout_ns;
};

struct StencilMaps {
    CUtensorMap cur;   // box {TZ+8, TY+2, 1} at (z0, y0, x)
    CUtensorMap prev;  // box {TZ, TY, 1}
    CUtensorMap c;     // box {TZ, TY, 1}
};

// Tile geometry of the stencil kernels (shared with the map builders).
constexpr int FD_TZ = 64;
constexpr int FD_TY = 16;

int build_stencil_map_cur(CUtensorMap* m, const float* base, const Layout& L);
int build_stencil_map_ctr(CUtensorMap* m, const float* base, const Layout& L);

// Launch one fused step. snap_out / snap_in are SnapKind values; image selects
// the imaging epilogue. Returns ST_OK or a negative status.
int launch_fd_step(const Layout& L, const CUtensorMap& mcur, const CUtensorMap& mprev, const CUtensorMap& mc,
                   StepArgs a, int snap_out, int snap_in, bool image, cudaStream_t st);
int fd_step_grid_chunks(const Layout& L);

// Small kernels.
int launch_add_point(float* f, long long idx, float val, unsigned* amax_slot, cudaStream_t st);
int launch_gather(const float* f, const long long* idx, int n, float* out, cudaStream_t st);
int launch_ref_to_dev(const double* src, float* dst, const Layout& L, cudaStream_t st);
// dst (reference layout, FP64) = src (device layout) * (damp_pow > 0 ? D^damp_pow : 1)
int launch_dev_to_ref(const float* src, double* dst, const Layout& L, const float* dtab, int sw, int damp_pow,
                      cudaStream_t st);
// dst (device layout) = src (reference layout) / D^pow (inverse of the stored damping)
int launch_ref_to_dev_undamp(const double* src, float* dst, const Layout& L, const float* dtab, int sw, int pow,
                             cudaStream_t st);
int launch_vel_to_coeff(const double* vel_ref, float* c, const Layout& L, double dt2damp, cudaStream_t st);
int launch_count_nonfinite(const float* f, long long n, unsigned long long* out, cudaStream_t st);
int launch_sumsq_finite(const float* f, long long n, double* out, cudaStream_t st);
int launch_interior_copy(const float* f, const Layout& L, float* out, cudaStream_t st);
int launch_finalize_image(const float* image, const float* illum, float* refl, long long n, cudaStream_t st);
int launch_scatter_scaled(float* f, const long long* idx, int n, const float* val, const float* c,
                          cudaStream_t st);

}  // namespace stg
