// C entry points over the reference's own public C++ API, compiled together
// with the reference sources (solver/wave_equation.cpp, rtm/rtm_engine.cpp,
// sparse/csr_matrix.cpp, core/*.cpp) into oracle/_ref/libseismic_ref.so by
// oracle/build_ref.sh. Test infrastructure only: it pins the C restatement in
// oracle/seismic_oracle.c and generates the golden fixtures under tests/golden/.
// Nothing in the product links or loads it.
#include "solver/wave_equation.h"
#include "rtm/rtm_engine.h"
#include "sparse/csr_matrix.h"
#include "core/config.h"
#include "core/fault_tolerance.h"

#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

namespace {

struct RefWorld {
    int argc = 1;
    char arg0[8] = "oracle";
    char* argv_store[2] = {arg0, nullptr};
    char** argv = argv_store;
    std::unique_ptr<seismic::MpiContext> mpi;
    RefWorld() { mpi = std::make_unique<seismic::MpiContext>(argc, argv); }
};

RefWorld& world() {
    static RefWorld w;
    return w;
}

seismic::GridParams make_params(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz) {
    seismic::GridParams p{};
    p.nx_global = nx;
    p.ny_global = ny;
    p.nz_global = nz;
    p.dx = dx;
    p.dy = dy;
    p.dz = dz;
    p.halo_width = 1;
    return p;
}

seismic::SolverConfig make_config(double dt, int nt, int sponge_width, double sponge_damping, int snapshot_interval) {
    seismic::SolverConfig c{};
    c.frequency = 2.0;
    c.dt = dt;
    c.nt = nt;
    c.water_depth = 4000.0;
    c.seafloor_gradient = 0.05;
    c.sponge_width = sponge_width;
    c.sponge_damping = sponge_damping;
    c.snapshot_interval = snapshot_interval;
    c.output_dir = "./output";
    return c;
}

std::unique_ptr<seismic::CSRMatrix> g_csr;

}  // namespace

extern "C" {

// Steps the reference solver `nsteps` times. Before step t every source s
// gets inject_source(src_xyz[s], {src_w[t*n_src+s]}) (wave_equation.cpp:39-54);
// then step_forward(t) (or step_adjoint(t) when use_adjoint), whose status is
// stored in statuses[t]; then every receiver r samples field().current into
// seis[t*nrec+r]. The final current/previous padded fields are copied out.
int ref_run_steps(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz,
                  double dt, int sponge_width, double sponge_damping,
                  const double* vel_padded, int n_src, const int64_t* src_xyz, const double* src_w,
                  int nrec, const int64_t* rec_xyz, double* seis, int nsteps, int use_adjoint,
                  int* statuses, double* out_current, double* out_previous) {
    auto& w = world();
    int coords[3] = {0, 0, 0};
    int dims[3] = {1, 1, 1};
    seismic::CartesianGrid grid(make_params(nx, ny, nz, dx, dy, dz), coords, dims);
    seismic::WaveEquationSolver solver(*w.mpi, grid, make_config(dt, nsteps, sponge_width, sponge_damping, 100));
    const int64_t n = grid.local().total_cells_with_halo;
    solver.set_velocity_field(vel_padded, n);
    const int64_t nyh = grid.local().ny_with_halo, nzh = grid.local().nz_with_halo;
    for (int t = 0; t < nsteps; ++t) {
        for (int s = 0; s < n_src; ++s) {
            std::vector<double> wv = {src_w[(int64_t)t * n_src + s]};
            solver.inject_source(src_xyz[3 * s], src_xyz[3 * s + 1], src_xyz[3 * s + 2], wv);
        }
        seismic::StepResult r = use_adjoint ? solver.step_adjoint(t) : solver.step_forward(t);
        statuses[t] = static_cast<int>(r);
        const auto& cur = solver.field().current;
        for (int q = 0; q < nrec; ++q) {
            int64_t idx = (rec_xyz[3 * q] + 1) * nyh * nzh + (rec_xyz[3 * q + 1] + 1) * nzh + (rec_xyz[3 * q + 2] + 1);
            seis[(int64_t)t * nrec + q] = cur[idx];
        }
    }
    std::memcpy(out_current, solver.field().current.data(), n * sizeof(double));
    std::memcpy(out_previous, solver.field().previous.data(), n * sizeof(double));
    return 0;
}

// The reference's forward_propagate (wave_equation.cpp:100-152): centre source,
// CFL check, snapshots every snapshot_interval steps. result[0..3] = status,
// total_nan_encountered, total_cells_repaired, timesteps_completed;
// result[4] = completed_successfully; result[5] = snapshot doubles stored.
int ref_forward_propagate(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz,
                          double dt, int nt, int sponge_width, double sponge_damping, int snapshot_interval,
                          const double* vel_padded, const double* wavelet, int64_t nw,
                          double* out_current, double* out_previous, double* out_snapshots,
                          int64_t snap_cap, int64_t* result) {
    auto& w = world();
    int coords[3] = {0, 0, 0};
    int dims[3] = {1, 1, 1};
    seismic::CartesianGrid grid(make_params(nx, ny, nz, dx, dy, dz), coords, dims);
    seismic::WaveEquationSolver solver(*w.mpi, grid,
                                       make_config(dt, nt, sponge_width, sponge_damping, snapshot_interval));
    const int64_t n = grid.local().total_cells_with_halo;
    solver.set_velocity_field(vel_padded, n);
    std::vector<double> wav(wavelet, wavelet + nw);
    seismic::PropagationResult pr = solver.forward_propagate(wav);
    result[0] = static_cast<int64_t>(pr.status);
    result[1] = pr.total_nan_encountered;
    result[2] = pr.total_cells_repaired;
    result[3] = pr.timesteps_completed;
    result[4] = pr.completed_successfully ? 1 : 0;
    const auto& snaps = solver.field().snapshots;
    result[5] = static_cast<int64_t>(snaps.size());
    std::memcpy(out_current, solver.field().current.data(), n * sizeof(double));
    std::memcpy(out_previous, solver.field().previous.data(), n * sizeof(double));
    int64_t m = std::min<int64_t>(snap_cap, static_cast<int64_t>(snaps.size()));
    if (m > 0) std::memcpy(out_snapshots, snaps.data(), m * sizeof(double));
    return 0;
}

// RTMEngine::apply_image_condition over nsteps pairs of halo-padded fields,
// then finalize_image (rtm/rtm_engine.cpp:24-57,170-182).
int ref_rtm_image(int64_t nx, int64_t ny, int64_t nz, int nsteps, const double* fwd, const double* adj,
                  double* image, double* illum, double* refl) {
    seismic::RTMEngine eng(nx, ny, nz, 10.0, 10.0, 10.0, 1);
    const int64_t nyh = ny + 2, nzh = nz + 2, np = (nx + 2) * nyh * nzh;
    for (int t = 0; t < nsteps; ++t)
        eng.apply_image_condition(fwd + (int64_t)t * np, adj + (int64_t)t * np, nyh, nzh, t);
    eng.finalize_image();
    const auto& r = eng.result();
    std::memcpy(image, r.image.data(), r.image.size() * sizeof(double));
    std::memcpy(illum, r.illumination.data(), r.illumination.size() * sizeof(double));
    std::memcpy(refl, r.reflectivity.data(), r.reflectivity.size() * sizeof(double));
    return 0;
}

// CSRMatrix::build_from_triplets (sparse/csr_matrix.cpp:25-72). The shipped
// pad_to_alignment under-allocates whenever it fires, so callers pass only
// inputs where every merged row has >= 8 entries (padding then never fires).
int64_t ref_csr_build(int64_t rows, int64_t cols, int64_t n, const int64_t* r, const int64_t* c, const double* v) {
    std::vector<seismic::SparseEntry> e(n);
    for (int64_t i = 0; i < n; ++i) e[i] = {r[i], c[i], v[i]};
    g_csr = std::make_unique<seismic::CSRMatrix>();
    g_csr->build_from_triplets(rows, cols, e);
    return g_csr->nnz();
}

int ref_csr_get(int64_t* row_ptr, int64_t* col, double* val) {
    if (!g_csr) return -1;
    std::memcpy(row_ptr, g_csr->row_ptr().data(), (g_csr->rows() + 1) * sizeof(int64_t));
    std::memcpy(col, g_csr->col_ind().data(), g_csr->nnz() * sizeof(int64_t));
    std::memcpy(val, g_csr->values().data(), g_csr->nnz() * sizeof(double));
    return 0;
}

// CSRMatrix::spmv (sparse/csr_matrix.cpp:118-149) on the last built matrix.
int ref_csr_spmv(const double* x, int64_t nxv, double* y) {
    if (!g_csr) return -1;
    seismic::AlignedVector<double> xv(nxv);
    for (int64_t i = 0; i < nxv; ++i) xv[i] = x[i];
    auto yv = g_csr->spmv(xv);
    for (int64_t i = 0; i < g_csr->rows(); ++i) y[i] = yv[i];
    return 0;
}

// FaultTolerance::repair_field_nan / clamp_field / count_nan_inf
// (core/fault_tolerance.cpp:72-157).
int ref_repair_field_nan(double* data, int64_t count, int64_t nx, int64_t ny, int64_t nz, int hw, double repl) {
    seismic::FaultTolerance ft(MPI_COMM_SELF, 0, 1);
    ft.repair_field_nan(data, count, nx, ny, nz, hw, repl);
    return 0;
}
int64_t ref_count_nan_inf(const double* data, int64_t count) {
    return seismic::FaultTolerance::count_nan_inf(data, count);
}
int ref_clamp_field(double* data, int64_t count, double lo, double hi) {
    seismic::FaultTolerance::clamp_field(data, count, lo, hi);
    return 0;
}

// load_config (core/config.cpp:9-94). out[0..] = frequency, dt, nt, water_depth,
// seafloor_gradient, sponge_width, sponge_damping, snapshot_interval,
// vp_min, vp_max, initial_vp, initial_vs, initial_rho, max_iterations,
// step_length, gradient_smoothing_sigma, regularization_lambda.
int ref_load_config(const char* path, double* out) {
    seismic::TomographyConfig c = seismic::load_config(path);
    double v[] = {c.solver.frequency, c.solver.dt, (double)c.solver.nt, c.solver.water_depth,
                  c.solver.seafloor_gradient, (double)c.solver.sponge_width, c.solver.sponge_damping,
                  (double)c.solver.snapshot_interval, c.model.vp_min, c.model.vp_max, c.model.initial_vp,
                  c.model.initial_vs, c.model.initial_rho, (double)c.inversion.max_iterations,
                  c.inversion.step_length, c.inversion.gradient_smoothing_sigma,
                  c.inversion.regularization_lambda};
    std::memcpy(out, v, sizeof(v));
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- slices
#include "rtm/mmap_writer.h"

extern "C" {

// RTMEngine::extract_slices (rtm/rtm_engine.cpp:59-81) with a callback that
// collects every CapturedSlice: meta[4 * k ..] = axis, index, dim0, dim1;
// vals = forward, adjoint and ic slices of each capture, concatenated.
// Returns the number of slices, or -1 when cap is too small.
int ref_extract_slices(int64_t nx, int64_t ny, int64_t nz, int n_specs, const int* axes, const int64_t* index,
                       const double* fwd, const double* adj, const double* ic, int64_t timestep, int64_t cap,
                       double* vals, int64_t* meta) {
    seismic::RTMEngine eng(nx, ny, nz, 10.0, 10.0, 10.0, 1);
    std::vector<seismic::SliceSpec> specs;
    for (int k = 0; k < n_specs; ++k) specs.push_back({static_cast<seismic::SliceAxis>(axes[k]), index[k], 1});
    eng.set_slice_specs(specs);
    std::vector<seismic::RTMEngine::CapturedSlice> got;
    eng.set_slice_callback([&got](const seismic::RTMEngine::CapturedSlice& s) { got.push_back(s); });
    eng.extract_slices(fwd, adj, ic, ny + 2, nz + 2, timestep);
    int64_t o = 0;
    for (size_t k = 0; k < got.size(); ++k) {
        const auto& s = got[k];
        meta[4 * k] = static_cast<int64_t>(s.axis);
        meta[4 * k + 1] = s.index;
        meta[4 * k + 2] = s.dim0;
        meta[4 * k + 3] = s.dim1;
        const int64_t n = s.dim0 * s.dim1;
        if (o + 3 * n > cap) return -1;
        std::memcpy(vals + o, s.forward_slice.data(), n * sizeof(double));
        std::memcpy(vals + o + n, s.adjoint_slice.data(), n * sizeof(double));
        std::memcpy(vals + o + 2 * n, s.ic_slice.data(), n * sizeof(double));
        o += 3 * n;
    }
    return static_cast<int>(got.size());
}

// MmapSnapshotWriter (rtm/mmap_writer.cpp:36-183): open(path, max_bytes),
// write_frame for each of the n frames (data concatenated, sizes[k] bytes),
// close. stats = frames_written, frames_dropped, total_bytes_written,
// mmap_cycles; returns the number of frames write_frame accepted.
int ref_mmap_write(const char* path, int64_t max_bytes, int n, const uint8_t* data, const int64_t* sizes,
                   int64_t* stats) {
    seismic::MmapSnapshotWriter w;
    if (!w.open(path, max_bytes)) return -1;
    int ok = 0;
    int64_t o = 0;
    for (int k = 0; k < n; ++k) {
        ok += w.write_frame(data + o, sizes[k]) ? 1 : 0;
        o += sizes[k];
    }
    const auto s = w.stats();
    stats[0] = s.frames_written;
    stats[1] = s.frames_dropped_buffer_full;
    stats[2] = s.total_bytes_written;
    stats[3] = s.mmap_cycles;
    w.close();
    return ok;
}

// MmapSnapshotWriter::read_frame / count_frames (rtm/mmap_writer.cpp:241-331).
int64_t ref_mmap_read_frame(const char* path, int64_t index, uint8_t* out, int64_t cap) {
    std::vector<uint8_t> buf;
    if (!seismic::MmapSnapshotWriter::read_frame(path, index, buf)) return -1;
    if (static_cast<int64_t>(buf.size()) > cap) return -2;
    std::memcpy(out, buf.data(), buf.size());
    return static_cast<int64_t>(buf.size());
}
int64_t ref_mmap_count_frames(const char* path) { return seismic::MmapSnapshotWriter::count_frames(path); }

}  // extern "C"

// ---------------------------------------------------------------- terrain
#include "solver/boundary.h"

extern "C" {

// TerrainBoundary (solver/boundary.cpp) on a single-rank grid with halo hw:
// the bathymetry (flat, generate_synthetic_bathymetry(gradient, roughness)
// when synthetic, then set_bathymetry_data(points) for n_points (x, y, depth)
// triples), seafloor_index per column, update_velocity_mask on `velocity`,
// build_boundary_mask into `mask`, and apply_free_surface_bc /
// apply_seafloor_bc / apply_absorbing_bc on three halo-padded fields (in
// place). Every array in the reference's (nx+2hw)(ny+2hw)(nz+2hw) layout.
int ref_terrain(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, double ox, double oy,
                double oz, int hw, double water_depth, int synthetic, double gradient, double roughness,
                int n_points, const double* points, double* bathy, int64_t* sf_index, double water_vp,
                double sediment_vp, double* velocity, uint8_t* mask, double* f_free, double* f_sea, double* f_abs,
                int sponge_width, double damping) {
    seismic::GridParams p{nx, ny, nz, dx, dy, dz, ox, oy, oz, hw};
    const int coords[3] = {0, 0, 0}, dims[3] = {1, 1, 1};
    seismic::CartesianGrid grid(p, coords, dims);
    seismic::TerrainBoundary tb(grid, water_depth);
    if (synthetic) tb.generate_synthetic_bathymetry(gradient, roughness);
    std::vector<seismic::BathymetryPoint> pts;
    for (int k = 0; k < n_points; ++k) pts.push_back({points[3 * k], points[3 * k + 1], points[3 * k + 2]});
    if (n_points) tb.set_bathymetry_data(pts);
    std::memcpy(bathy, tb.bathymetry().data(), nx * ny * sizeof(double));
    for (int64_t ix = 0; ix < nx; ++ix)
        for (int64_t iy = 0; iy < ny; ++iy) sf_index[ix * ny + iy] = tb.seafloor_index(ix, iy);
    const auto& loc = grid.local();
    const int64_t n = loc.total_cells_with_halo;
    std::vector<double> v(velocity, velocity + n);
    tb.update_velocity_mask(v, water_vp, sediment_vp);
    std::memcpy(velocity, v.data(), n * sizeof(double));
    tb.build_boundary_mask(loc, hw);
    std::memcpy(mask, tb.mask().data(), n);
    std::vector<double> a(f_free, f_free + n), b(f_sea, f_sea + n), c(f_abs, f_abs + n);
    tb.apply_free_surface_bc(a, loc, hw);
    tb.apply_seafloor_bc(b, loc, hw);
    tb.apply_absorbing_bc(c, loc, hw, sponge_width, damping);
    std::memcpy(f_free, a.data(), n * sizeof(double));
    std::memcpy(f_sea, b.data(), n * sizeof(double));
    std::memcpy(f_abs, c.data(), n * sizeof(double));
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- sparse ops
// Built against the patched scratch copy of sparse/ (oracle/build_ref.sh lists
// the three fixes); every call below runs the reference's own code on it.
#include "sparse/sparse_ops.h"

namespace {
seismic::AlignedVector<double> to_aligned(const double* p, int64_t n) {
    seismic::AlignedVector<double> v(n);
    for (int64_t i = 0; i < n; ++i) v[i] = p[i];
    return v;
}
}  // namespace

extern "C" {

// CSRMatrix::build_fd_stencil_7point (sparse/csr_matrix.cpp:74-116) into the
// current matrix (its build_from_triplets pads every row to a multiple of 8,
// the fixed pad_to_alignment). Returns nnz.
int64_t ref_csr_fd_stencil(int64_t nx, int64_t ny, int64_t nz, const double* vel, double dx, double dy, double dz,
                           double dt) {
    g_csr = std::make_unique<seismic::CSRMatrix>();
    g_csr->build_fd_stencil_7point(nx, ny, nz, vel, dx, dy, dz, dt);
    return g_csr->nnz();
}

// CSRMatrix::spmv_transpose (sparse/csr_matrix.cpp:151-166) on the current
// matrix; with the zero-fill fix its accumulator starts at 0.
int ref_csr_spmv_t(const double* x, int64_t nxv, double* y) {
    if (!g_csr) return -1;
    auto yv = g_csr->spmv_transpose(to_aligned(x, nxv));
    for (int64_t j = 0; j < g_csr->cols(); ++j) y[j] = yv[j];
    return 0;
}

// SparseOps::build_hessian_approx (sparse/sparse_ops.cpp:204-210): the current
// matrix is replaced by the returned copy with reg added to its diagonal.
int64_t ref_hessian_approx(double reg) {
    if (!g_csr) return -1;
    auto h = std::make_unique<seismic::CSRMatrix>(seismic::SparseOps::build_hessian_approx(*g_csr, reg));
    g_csr = std::move(h);
    return g_csr->nnz();
}

// SparseOps::conjugate_gradient (jacobi == 0) or jacobi_preconditioned_cg
// (jacobi != 0) (sparse/sparse_ops.cpp:8-113) on the current matrix.
int ref_cg(int jacobi, const double* b, int64_t n, int max_iter, double tol, double* x) {
    if (!g_csr) return -1;
    auto bv = to_aligned(b, n);
    auto xv = jacobi ? seismic::SparseOps::jacobi_preconditioned_cg(*g_csr, bv, max_iter, tol)
                     : seismic::SparseOps::conjugate_gradient(*g_csr, bv, max_iter, tol);
    for (int64_t i = 0; i < g_csr->rows(); ++i) x[i] = xv[i];
    return 0;
}

// SparseOps::dot_product (sparse/sparse_ops.cpp:172-187).
double ref_dot(const double* a, const double* b, int64_t n) {
    return seismic::SparseOps::dot_product(to_aligned(a, n), to_aligned(b, n));
}

// SparseOps::smooth_gradient (sparse/sparse_ops.cpp:115-158).
int ref_smooth_gradient(const double* g, int64_t nx, int64_t ny, int64_t nz, double sigma, double* out) {
    std::vector<double> gv(g, g + nx * ny * nz);
    auto r = seismic::SparseOps::smooth_gradient(gv, nx, ny, nz, sigma);
    std::memcpy(out, r.data(), r.size() * sizeof(double));
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- solver RTM driver, sponge, adjoint_propagate
extern "C" {

// The reference's adjoint_propagate (wave_equation.cpp:154-194) on a fresh
// solver, after forward_propagate(fwd_wavelet) on the same solver when
// n_fwd > 0 (adjoint_propagate does not reset the fields). result[0..4] =
// status, total_nan_encountered, total_cells_repaired, timesteps_completed,
// completed_successfully.
int ref_adjoint_propagate(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, double dt, int nt,
                          int sponge_width, double sponge_damping, const double* vel_padded, const double* fwd_wavelet,
                          int64_t n_fwd, const double* residual, int64_t n_res, double* out_current,
                          double* out_previous, int64_t* result) {
    auto& w = world();
    int coords[3] = {0, 0, 0};
    int dims[3] = {1, 1, 1};
    seismic::CartesianGrid grid(make_params(nx, ny, nz, dx, dy, dz), coords, dims);
    seismic::WaveEquationSolver solver(*w.mpi, grid, make_config(dt, nt, sponge_width, sponge_damping, 100000));
    const int64_t n = grid.local().total_cells_with_halo;
    solver.set_velocity_field(vel_padded, n);
    if (n_fwd > 0) solver.forward_propagate(std::vector<double>(fwd_wavelet, fwd_wavelet + n_fwd));
    seismic::PropagationResult pr = solver.adjoint_propagate(std::vector<double>(residual, residual + n_res));
    result[0] = static_cast<int64_t>(pr.status);
    result[1] = pr.total_nan_encountered;
    result[2] = pr.total_cells_repaired;
    result[3] = pr.timesteps_completed;
    result[4] = pr.completed_successfully ? 1 : 0;
    std::memcpy(out_current, solver.field().current.data(), n * sizeof(double));
    std::memcpy(out_previous, solver.field().previous.data(), n * sizeof(double));
    return 0;
}

// The RTM building blocks of the solver (wave_equation.cpp:508-619) and a
// standalone apply_sponge_layer (:262-297). configure_rtm(enable_rtm, default
// slice specs, ring_capacity); then for t < nsteps: inject_source(centre,
// {w[t]}); step_forward(t); when ops[t] & 1 store_forward_wavefield_for_rtm(t);
// when ops[t] & 2 apply_rtm_step(t, ops[t] & 4); when ops[t] & 8
// apply_sponge_layer(). Afterwards finalize_image(): image / illum / refl
// (interior), the fields, counts[0..1] = snapshots_captured / dropped.
int ref_rtm_building_blocks(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, double dt,
                            int sponge_width, double sponge_damping, const double* vel_padded, const double* w,
                            int nsteps, const int* ops, int64_t ring_capacity, double* image, double* illum,
                            double* refl, double* out_current, double* out_previous, int64_t* counts) {
    auto& wd = world();
    int coords[3] = {0, 0, 0};
    int dims[3] = {1, 1, 1};
    seismic::CartesianGrid grid(make_params(nx, ny, nz, dx, dy, dz), coords, dims);
    seismic::WaveEquationSolver solver(*wd.mpi, grid, make_config(dt, nsteps, sponge_width, sponge_damping, 100000));
    const int64_t n = grid.local().total_cells_with_halo;
    solver.set_velocity_field(vel_padded, n);
    seismic::RTMConfig rc;
    rc.enable_rtm = true;
    rc.ring_buffer_capacity = static_cast<size_t>(ring_capacity);
    solver.configure_rtm(rc);
    for (int t = 0; t < nsteps; ++t) {
        solver.inject_source(nx / 2, ny / 2, nz / 2, {w[t]});
        solver.step_forward(t);
        if (ops[t] & 1) solver.store_forward_wavefield_for_rtm(t);
        if (ops[t] & 2) solver.apply_rtm_step(t, (ops[t] & 4) != 0);
        if (ops[t] & 8) solver.apply_sponge_layer();
    }
    solver.rtm_engine()->finalize_image();
    const auto& r = solver.rtm_engine()->result();
    std::memcpy(image, r.image.data(), r.image.size() * sizeof(double));
    std::memcpy(illum, r.illumination.data(), r.illumination.size() * sizeof(double));
    std::memcpy(refl, r.reflectivity.data(), r.reflectivity.size() * sizeof(double));
    std::memcpy(out_current, solver.field().current.data(), n * sizeof(double));
    std::memcpy(out_previous, solver.field().previous.data(), n * sizeof(double));
    counts[0] = solver.snapshots_captured();
    counts[1] = solver.snapshots_dropped();
    return 0;
}

}  // extern "C"
