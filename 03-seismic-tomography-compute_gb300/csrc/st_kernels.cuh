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
    int inj_x, inj_y, inj_z; // fused point injection into the written field (interior), inj_x = -1: none
    float inj_val;
    int rz, rx0, rsx, rnx, ry0, rsy, rny;  // receiver grid on plane z = rz
    float* seis_row;         // receiver samples of the update (before injection/forcing), or null
    const float* force_row;  // adds c * force_row[q] at receiver q (adjoint forcing), or null
    void* snap_out;          // snapshot of this step's centre field (compact interior), or null
    const unsigned* amax_cur;  // |max| bits of the centre field (snapshot scale)
    unsigned* amax_next;     // |max| of the written field is atomically max-ed here
    const void* snap_in;     // forward snapshot paired with this step's centre field (imaging)
    const unsigned* amax_in;
    float* image;            // image += f * (centre / c), centre / (c D) with the stable sponge
    float* illum;            // illum += f * f
    float* grad;             // gradient: grad += (centre / c) * L(snapshot)   (compact interior)
    int snap_t;              // gradient: time index of the snapshot in the store
    unsigned* flags;         // FLAG_GUARD / FLAG_TIMEOUT
    unsigned long long timeout_ns;  // limit of every bounded wait (0: the launcher's default, 2 s)
    int withhold;            // fault-path test hook: plane withhold - 1 of every CTA's march is never
                             // copied, so its waits run out (0: none)
    int stable_sponge;       // 1: out = D * (update + forcing) (damped new field), 0: the reference rule
    const int* zlim;         // terrain: per (x, y) column (x * ny + y), points with z < zlim are set to 0
                             // after the update (free surface / seafloor masks), or null
    // two-step launches only: the second step's output field; adjoint: its
    // forcing row and snapshot scale; forward: its receiver samples, source
    // injection (inj_steps bit 0: the first step injects inj_val, bit 1: the
    // second inj_val2, both at inj_x/y/z), the snapshot of the previous field
    // (snap_out2, scale amax_cur2) and the max of the second output (amax_next2)
    float* out2;
    const float* force_row2;
    const unsigned* amax_in2;
    float* seis_row2;
    int inj_steps;
    float inj_val2;
    void* snap_out2;
    const unsigned* amax_cur2;
    unsigned* amax_next2;
};

// Sponge factor of interior point (ix, iy, iz): D(d) for the distance d to the
// nearest face when d < sw, else 1 (apply_sponge_layer, wave_equation.cpp:262-297).
__device__ __forceinline__ float sponge_D(const Layout& L, const float* dtab, int sw, long long ix, long long iy,
                                          long long iz) {
    long long d = ix;
    d = min(d, L.nx - 1 - ix);
    d = min(d, iy);
    d = min(d, L.ny - 1 - iy);
    d = min(d, iz);
    d = min(d, L.nz - 1 - iz);
    return (d >= 0 && d < sw) ? dtab[d] : 1.0f;
}

// Tensor maps of one device field for the two tile heights of the stencil
// kernels ([0]: 16-row tiles, [1]: 32-row tiles): cur boxes {TZ+8, rows+2, 1}
// starting at (z0, y0, x), centre boxes {TZ, rows, 1}; cur2 is the two-step
// kernel's box {TZ+8, 16+4, 1} (a two-cell y halo).
struct FieldMaps {
    CUtensorMap cur[2];
    CUtensorMap ctr[2];
    CUtensorMap cur2;
};

// Tile width of the stencil kernels along z.
constexpr int FD_TZ = 64;

int build_field_maps(FieldMaps* m, const float* base, const Layout& L);
// x-chunks per CTA column for a tile height and resident CTAs per SM, with at
// least min_waves waves of resident CTAs when the grid allows it; each chunk
// re-reads halo extra x-planes.
int fd_step_grid_chunks(const Layout& L, int tyv, int minb, int min_waves, int halo = 2);

// Maps of the staged imaging variant: the snapshot store (box {64, 16} at
// (z, y, x, t)) and the compact image / illumination volumes (box {64, 16}).
struct ImageMaps {
    CUtensorMap snap, image, illum;
};
bool image_maps_supported(int kind, const Layout& L);
int build_image_maps(ImageMaps* m, const void* snaps, int kind, long long nt, const float* image,
                     const float* illum, const Layout& L);
int make_compact_map(CUtensorMap* map, const float* base, const Layout& L, int bz, int by);

// Launch one fused step. snap_out / snap_in are SnapKind values; epi: 0 = none,
// 1 = imaging (operands staged by TMA when imaps is given, StepArgs::snap_t
// then indexes the store; loaded at use from snap_in otherwise), 2 = gradient
// (needs msnap, the snapshot store's map).
int launch_fd_step(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                   StepArgs a, int snap_out, int snap_in, int epi, const CUtensorMap* msnap, cudaStream_t st,
                   const ImageMaps* imaps = nullptr);
// Launch two adjoint steps with fused imaging (fd_step2_kernel, adjoint mode): reads
// cur = lambda_t and prev = lambda_{t+1}, writes a.out = lambda_{t-1}' (the
// output of step t) and a.out2 = the output of step t-1, from snapshots
// a.snap_t and a.snap_t - 1 (scales a.amax_in, a.amax_in2) and the receiver
// forcing rows a.force_row (step t) and a.force_row2 (step t-1). Needs
// staged image maps (nz % 4 == 0).
int launch_fd_step2_image(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                          StepArgs a, int snap_in, const ImageMaps& imaps, cudaStream_t st);
// Launch two adjoint steps with the gradient epilogue (fd_step2_kernel,
// gradient mode): as launch_fd_step2_image, but a.grad (compact interior)
// accumulates (lambda / c) * L(snapshot) for both steps; msnap is the store's
// halo map (build_snap_map_grad), mgrad a compact map of a.grad (box {64, 16}).
int launch_fd_step2_grad(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                         StepArgs a, int snap_in, const CUtensorMap& msnap, const CUtensorMap& mgrad,
                         cudaStream_t st);
// Launch two forward steps t, t+1 (fd_step2_kernel, forward mode): reads
// cur = u_t, prev = u_{t-1}; writes a.out = u_{t+1}, a.out2 = u_{t+2};
// samples a.seis_row / a.seis_row2; injects per a.inj_steps; with snapshots
// stores u_t to a.snap_out (scale a.amax_cur) and u_{t-1} to a.snap_out2
// (scale a.amax_cur2, when not null) and max-reduces |u_{t+1}|, |u_{t+2}|
// into a.amax_next, a.amax_next2. Needs nz % 4 == 0.
int launch_fd_step2_forward(const Layout& L, const FieldMaps& mcur, const FieldMaps& mprev, const FieldMaps& mc,
                            StepArgs a, int snap_out, cudaStream_t st);
// 4-D map over a snapshot store for the gradient step's halo tile.
int build_snap_map_grad(CUtensorMap* m, const void* base, int kind, const Layout& L, long long nt);

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
// Snapshot of field f (device layout) with scale amax, as the stepping kernels store it.
int launch_snapshot_of_field(const float* f, const Layout& L, void* snap, int kind, const unsigned* amax,
                             cudaStream_t st);
int launch_finalize_image(const float* image, const float* illum, float* refl, long long n, cudaStream_t st);
int launch_scatter_scaled(float* f, const long long* idx, int n, const float* val, const float* c,
                          cudaStream_t st);

}  // namespace stg
