// seismic_gb300.hpp -- source-compatible C++ face of the reference's hot-path
// classes (13262233692/03-seismic-tomography-compute, src/cpp), implemented
// over the C ABI in seismic_gb300.h. Header-only; link libseismic_gb300.so.
//
// Differences a caller of the reference sees:
//  - MpiContext is a single-rank stand-in (one device-resident domain, no
//    halo exchange); CartesianGrid decomposes over one rank.
//  - Field, snapshot and image vectors are FP64 host copies of device state:
//    field() downloads them; after writing through mutable_field() the next
//    device operation uploads them.
//  - Failures of the device library throw seismic::DeviceError (the reference
//    aborts or returns silently); StepResult codes are returned as there.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "seismic_gb300.h"

namespace seismic {

struct DeviceError : std::runtime_error {
    explicit DeviceError(int code) : std::runtime_error(std::string("seismic_gb300: ") + st_last_error()), code(code) {}
    int code;
};

inline int check(int rc) {
    if (rc < 0) throw DeviceError(rc);
    return rc;
}

// ---------------------------------------------------------------- core/grid.h:9-68
struct GridParams {
    int64_t nx_global, ny_global, nz_global;
    double dx, dy, dz;
    double origin_x, origin_y, origin_z;
    int halo_width;
};

struct LocalGrid {
    int64_t nx_local, ny_local, nz_local;
    int64_t nx_with_halo, ny_with_halo, nz_with_halo;
    int64_t offset_x, offset_y, offset_z;
    int64_t total_cells, total_cells_with_halo;
};

class CartesianGrid {
   public:
    CartesianGrid(const GridParams& params, const int mpi_coords[3], const int mpi_dims[3]) : params_(params) {
        auto axis = [](int64_t n, int ranks, int coord, int64_t& nl, int64_t& off) {
            const int64_t base = n / ranks, rem = n % ranks;
            off = (int64_t)coord * base + std::min<int64_t>(coord, rem);
            nl = base + (coord < rem ? 1 : 0);
        };
        axis(params.nx_global, mpi_dims[0], mpi_coords[0], local_.nx_local, local_.offset_x);
        axis(params.ny_global, mpi_dims[1], mpi_coords[1], local_.ny_local, local_.offset_y);
        axis(params.nz_global, mpi_dims[2], mpi_coords[2], local_.nz_local, local_.offset_z);
        const int hw = params.halo_width;
        local_.nx_with_halo = local_.nx_local + 2 * hw;
        local_.ny_with_halo = local_.ny_local + 2 * hw;
        local_.nz_with_halo = local_.nz_local + 2 * hw;
        local_.total_cells = local_.nx_local * local_.ny_local * local_.nz_local;
        local_.total_cells_with_halo = local_.nx_with_halo * local_.ny_with_halo * local_.nz_with_halo;
    }
    int64_t local_index(int64_t ix, int64_t iy, int64_t iz) const {
        return ix * local_.ny_local * local_.nz_local + iy * local_.nz_local + iz;
    }
    int64_t local_index_with_halo(int64_t ix, int64_t iy, int64_t iz) const {
        return ix * local_.ny_with_halo * local_.nz_with_halo + iy * local_.nz_with_halo + iz;
    }
    bool is_interior(int64_t lx, int64_t ly, int64_t lz) const {
        return lx >= 0 && lx < local_.nx_local && ly >= 0 && ly < local_.ny_local && lz >= 0 && lz < local_.nz_local;
    }
    const GridParams& params() const { return params_; }
    const LocalGrid& local() const { return local_; }
    double x_coord(int64_t ix) const { return params_.origin_x + (local_.offset_x + ix) * params_.dx; }
    double y_coord(int64_t iy) const { return params_.origin_y + (local_.offset_y + iy) * params_.dy; }
    double z_coord(int64_t iz) const { return params_.origin_z + (local_.offset_z + iz) * params_.dz; }

   private:
    GridParams params_;
    LocalGrid local_{};
};

// ---------------------------------------------------------------- core/mpi_context.h:10-57
struct MpiConfig {
    int rank = 0, size = 1, local_rank = 0;
    int cart_comm = 0;
    int dims[3] = {1, 1, 1};
    int coords[3] = {0, 0, 0};
    int neighbors[6] = {-2, -2, -2, -2, -2, -2};  // no neighbours: MPI_PROC_NULL
};

// Single-rank stand-in: every reduction returns its local value.
class MpiContext {
   public:
    MpiContext(int& argc, char**& argv) {
        (void)argc;
        (void)argv;
    }
    MpiContext(const MpiContext&) = delete;
    MpiContext& operator=(const MpiContext&) = delete;
    const MpiConfig& config() const { return cfg_; }
    void barrier() const {}
    double allreduce_max(double v) const { return v; }
    double allreduce_sum(double v) const { return v; }
    int allreduce_max_int(int v) const { return v; }
    int64_t allreduce_sum_int64(int64_t v) const { return v; }

   private:
    MpiConfig cfg_;
};

// ---------------------------------------------------------------- core/config.h:9-53
struct SolverConfig {
    double frequency = 2.0, dt = 0.001;
    int nt = 5000;
    double water_depth = 4000.0, seafloor_gradient = 0.05;
    int sponge_width = 20;
    double sponge_damping = 0.015;
    int snapshot_interval = 100;
    std::string output_dir = "./output";
};
struct ModelConfig {
    double vp_min = 1450.0, vp_max = 8500.0, vs_min = 0.0, vs_max = 5000.0, rho_min = 1000.0, rho_max = 3300.0;
    double initial_vp = 1500.0, initial_vs = 0.0, initial_rho = 2200.0;
};
struct InversionConfig {
    int max_iterations = 50;
    double step_length = 0.01, gradient_smoothing_sigma = 2.0, regularization_lambda = 1e-4, misfit_tolerance = 1e-6;
    std::string misfit_type = "cross_correlation";
    int gradient_precondition = 1, line_search_max = 10;
    double line_search_factor = 0.5;
};
struct TomographyConfig {
    SolverConfig solver;
    ModelConfig model;
    InversionConfig inversion;
    std::map<std::string, std::string> obs_stations;
    std::vector<double> source_positions;
};

// load_config (core/config.cpp:9-94): defaults, two-level "section:" /
// "key: value" lines, unknown sections and keys ignored.
inline TomographyConfig load_config(const std::string& yaml_path) {
    TomographyConfig cfg;
    std::ifstream ifs(yaml_path);
    if (!ifs.is_open()) return cfg;
    std::string line, section;
    const char* ws = " \t\r\n";
    while (std::getline(ifs, line)) {
        line.erase(0, line.find_first_not_of(ws));
        line.erase(line.find_last_not_of(ws) + 1);
        if (line.empty() || line[0] == '#') continue;
        if (line.back() == ':') {
            section = line.substr(0, line.size() - 1);
            continue;
        }
        const auto pos = line.find(':');
        if (pos == std::string::npos) continue;
        std::string key = line.substr(0, pos), val = line.substr(pos + 1);
        key.erase(0, key.find_first_not_of(" \t"));
        key.erase(key.find_last_not_of(" \t") + 1);
        val.erase(0, val.find_first_not_of(" \t"));
        val.erase(val.find_last_not_of(" \t") + 1);
        auto& s = cfg.solver;
        auto& m = cfg.model;
        auto& v = cfg.inversion;
        if (section == "solver") {
            if (key == "frequency") s.frequency = std::stod(val);
            else if (key == "dt") s.dt = std::stod(val);
            else if (key == "nt") s.nt = std::stoi(val);
            else if (key == "water_depth") s.water_depth = std::stod(val);
            else if (key == "sponge_width") s.sponge_width = std::stoi(val);
            else if (key == "sponge_damping") s.sponge_damping = std::stod(val);
        } else if (section == "model") {
            if (key == "vp_min") m.vp_min = std::stod(val);
            else if (key == "vp_max") m.vp_max = std::stod(val);
            else if (key == "initial_vp") m.initial_vp = std::stod(val);
            else if (key == "initial_vs") m.initial_vs = std::stod(val);
            else if (key == "initial_rho") m.initial_rho = std::stod(val);
        } else if (section == "inversion") {
            if (key == "max_iterations") v.max_iterations = std::stoi(val);
            else if (key == "step_length") v.step_length = std::stod(val);
            else if (key == "gradient_smoothing_sigma") v.gradient_smoothing_sigma = std::stod(val);
            else if (key == "regularization_lambda") v.regularization_lambda = std::stod(val);
            else if (key == "misfit_type") v.misfit_type = val;
        }
    }
    return cfg;
}

// ---------------------------------------------------------------- rtm/rtm_engine.h:12-23
enum class SliceAxis { X = 0, Y = 1, Z = 2, VOLUME = 3 };
// index < 0 = the middle plane of that axis.
struct SliceSpec {
    SliceAxis axis;
    int64_t index;
    int64_t stride;
};

// ---------------------------------------------------------------- rtm/rtm_engine.h:25-96
struct RTMImageCondition {
    std::vector<double> image, illumination, reflectivity;
};

class RTMEngine {
   public:
    RTMEngine(int64_t nx, int64_t ny, int64_t nz, double dx, double dy, double dz, int halo_width, int device = 0)
        : nx_(nx), ny_(ny), nz_(nz) {
        check(st_rtm_engine_create(nx, ny, nz, dx, dy, dz, halo_width, device, &h_));
    }
    ~RTMEngine() {
        if (owned_) st_rtm_engine_destroy(h_);
    }
    RTMEngine(const RTMEngine&) = delete;
    RTMEngine& operator=(const RTMEngine&) = delete;
    void apply_image_condition(const double* fwd, const double* adj, int64_t ny, int64_t nz, int64_t step) {
        check(st_rtm_engine_apply_image_condition(h_, fwd, adj, ny, nz, step));
    }
    void finalize_image() { check(st_rtm_engine_finalize_image(h_)); }
    void reset_image() { check(st_rtm_engine_reset_image(h_)); }
    const RTMImageCondition& result() const {
        auto& r = const_cast<RTMImageCondition&>(res_);
        const size_t n = (size_t)total_cells();
        r.image.resize(n);
        r.illumination.resize(n);
        r.reflectivity.resize(n);
        check(st_rtm_engine_result(h_, r.image.data(), r.illumination.data(), r.reflectivity.data()));
        return res_;
    }
    int64_t nx() const { return nx_; }
    int64_t ny() const { return ny_; }
    int64_t nz() const { return nz_; }
    int64_t total_cells() const { return nx_ * ny_ * nz_; }
    void set_slice_specs(const std::vector<SliceSpec>& specs) { specs_ = specs; }
    const std::vector<SliceSpec>& slice_specs() const { return specs_; }

   private:
    friend class WaveEquationSolver;
    // The engine a solver owns (WaveEquationSolver::rtm_engine()).
    RTMEngine(st_rtm_engine* borrowed, int64_t nx, int64_t ny, int64_t nz)
        : h_(borrowed), nx_(nx), ny_(ny), nz_(nz), owned_(false) {}
    st_rtm_engine* h_ = nullptr;
    int64_t nx_, ny_, nz_;
    bool owned_ = true;
    RTMImageCondition res_;
    std::vector<SliceSpec> specs_;
};

// ---------------------------------------------------------------- core/fault_tolerance.h:13-97
enum class HealthStatus : int {
    HEALTHY = 0,
    NAN_DETECTED = 1,
    INF_DETECTED = 2,
    CFL_VIOLATION = 3,
    DIVERGENCE = 4,
    COMM_FAILURE = 5
};

// One rank: the global checks are the local ones. The object a solver's
// fault_tolerance() returns reads and sets the statistics and settings the
// solver's steps use; a standalone object keeps its own settings. The field
// helpers run on the GPU in FP64 on host arrays.
class FaultTolerance {
   public:
    struct FaultStats {
        int64_t total_nan_count;
        int64_t total_inf_count;
        int64_t cells_repaired;
        int64_t timesteps_recovered;
        int global_abort_count;
    };
    explicit FaultTolerance(int comm = 0, int rank = 0, int size = 1) { (void)comm, (void)rank, (void)size; }

    int global_health_check(HealthStatus local_status) const { return static_cast<int>(local_status); }
    int global_health_check_field(const double* data, int64_t count) const {
        return count_nan_inf(data, count) > 0 ? 1 : 0;
    }
    int broadcast_error(int local_error) const { return local_error; }
    // fault_tolerance.cpp:49-70
    bool verify_cfl_condition(const double* velocity, int64_t count, double dx, double dy, double dz, double dt,
                              double cfl_limit = 0.5) const {
        double vmax = 0.0;
        for (int64_t i = 0; i < count; ++i)
            if (std::isfinite(velocity[i]) && velocity[i] > vmax) vmax = velocity[i];
        return std::max({vmax * dt / dx, vmax * dt / dy, vmax * dt / dz}) <= cfl_limit;
    }
    static int64_t count_nan_inf(const double* data, int64_t count) {
        int64_t n = 0;
        check(st_field_count_nonfinite(data, count, 0, &n));
        return n;
    }
    static bool is_valid_double(double v) { return std::isfinite(v); }
    static double safe_clamp(double v, double lo, double hi) {
        return std::isfinite(v) ? std::max(lo, std::min(v, hi)) : 0.0;
    }
    static void clamp_field(double* data, int64_t count, double lo, double hi) {
        check(st_field_clamp(data, count, lo, hi, 0));
    }
    void repair_field_nan(double* data, int64_t count, int64_t nx, int64_t ny, int64_t nz, int halo_width,
                          double replace_value = 0.0) const {
        check(st_field_repair_nan(data, count, nx, ny, nz, halo_width, replace_value, 0));
    }
    const FaultStats& stats() const {
        if (h_) {
            st_fault_stats st{};
            check(st_solver_fault_stats(h_, &st));
            stats_ = FaultStats{st.total_nan_count, st.total_inf_count, st.cells_repaired, st.timesteps_recovered,
                                st.global_abort_count};
        }
        return stats_;
    }
    void reset_stats() {
        stats_ = FaultStats{};
        if (h_) check(st_solver_reset_fault_stats(h_));
    }
    void set_max_repair_attempts(int n) { set(ST_FT_MAX_REPAIR_ATTEMPTS, n, max_repair_, 1.0, 1e9); }
    int max_repair_attempts() const { return (int)get(ST_FT_MAX_REPAIR_ATTEMPTS, max_repair_); }
    void set_amplitude_limit(double v) { set(ST_FT_AMPLITUDE_LIMIT, v, amp_, 1.0, HUGE_VAL); }
    double amplitude_limit() const { return get(ST_FT_AMPLITUDE_LIMIT, amp_); }
    void set_cfl_safety_factor(double v) { set(ST_FT_CFL_SAFETY_FACTOR, v, cfl_, 0.01, 0.99); }
    double cfl_safety_factor() const { return get(ST_FT_CFL_SAFETY_FACTOR, cfl_); }

   private:
    friend class WaveEquationSolver;
    void set(int which, double v, double& local, double lo, double hi) {
        if (h_) check(st_solver_set_fault_param(h_, which, v));
        else local = (int)which == ST_FT_MAX_REPAIR_ATTEMPTS ? std::floor(std::max(lo, std::min(v, hi)))
                                                             : std::max(lo, std::min(v, hi));
    }
    double get(int which, double local) const {
        if (!h_) return local;
        double v = 0.0;
        check(st_solver_fault_param(h_, which, &v));
        return v;
    }
    st_solver* h_ = nullptr;
    double max_repair_ = 3, amp_ = 1e10, cfl_ = 0.49;
    mutable FaultStats stats_{};
};

// ---------------------------------------------------------------- solver/wave_equation.h:16-144
struct WaveField {
    std::vector<double> current, previous, next, velocity, snapshots;
};

enum class StepResult { OK = 0, NAN_DETECTED_AND_REPAIRED = 1, CFL_VIOLATION = 2, FATAL_DIVERGENCE = 3 };

struct PropagationResult {
    StepResult status;
    int64_t total_nan_encountered;
    int64_t total_cells_repaired;
    int timesteps_completed;
    bool completed_successfully;
};

// RTMConfig (wave_equation.h:39-48), plus the inputs of the true RTM that
// run_rtm performs here (no reference counterpart): receivers of the residual
// traces (nx*ny == 0: every interior cell of the plane z = 0), the forward
// snapshot storage (ST_SNAP_NONE = BF16 with a per-snapshot scale) and
// binomial checkpointing (segment length in steps; 0 = store every step).
struct RTMConfig {
    bool enable_rtm = false;
    bool enable_snapshots = false;
    int snapshot_interval = 50;
    bool enable_mmap_writer = false;
    std::string mmap_filename = "rtm_snapshots.dat";
    int64_t mmap_max_bytes = 2LL * 1024LL * 1024LL * 1024LL;
    size_t ring_buffer_capacity = 1024;
    std::vector<SliceSpec> slice_specs;
    st_receiver_grid receivers{0, 1, 0, 0, 1, 0, 0};
    int snap_kind = ST_SNAP_NONE;
    int checkpoint_segment = 0;
};

class WaveEquationSolver {
   public:
    WaveEquationSolver(const MpiContext& mpi, const CartesianGrid& grid, const SolverConfig& config, int device = 0)
        : mpi_(mpi), grid_(grid), config_(config) {
        const GridParams& p = grid.params();
        st_grid_params gp{grid.local().nx_local, grid.local().ny_local, grid.local().nz_local, p.dx, p.dy, p.dz,
                          p.origin_x, p.origin_y, p.origin_z, p.halo_width};
        st_solver_config sc{config.frequency, config.dt, config.nt, config.water_depth, config.seafloor_gradient,
                            config.sponge_width, config.sponge_damping, config.snapshot_interval};
        check(st_solver_create(&gp, &sc, device, &h_));
        ft_.h_ = h_;
    }
    ~WaveEquationSolver() {
        engine_.reset();
        st_solver_destroy(h_);
    }
    WaveEquationSolver(const WaveEquationSolver&) = delete;
    WaveEquationSolver& operator=(const WaveEquationSolver&) = delete;

    void initialize_velocity(double vp0) { sync(); check(st_solver_initialize_velocity(h_, vp0)); }
    void set_velocity_field(const double* vp, int64_t count) { sync(); check(st_solver_set_velocity_field(h_, vp, count)); }
    void inject_source(int64_t ix, int64_t iy, int64_t iz, const std::vector<double>& w) {
        sync();
        check(st_solver_inject_source(h_, ix, iy, iz, w.data(), (int64_t)w.size()));
    }
    StepResult step_forward(int t) { sync(); return StepResult(check(st_solver_step_forward(h_, t))); }
    StepResult step_adjoint(int t) { sync(); return StepResult(check(st_solver_step_adjoint(h_, t))); }
    PropagationResult forward_propagate(const std::vector<double>& w) {
        return prop(st_solver_forward_propagate, w);
    }
    PropagationResult adjoint_propagate(const std::vector<double>& r) {
        return prop(st_solver_adjoint_propagate, r);
    }
    void exchange_halo(WaveField&) {}  // one domain: the halo ring stays zero
    // current and previous times the sponge factor over the sponge band (wave_equation.cpp:262-297)
    void apply_sponge_layer() {
        sync();
        check(st_solver_apply_sponge_layer(h_));
    }
    const WaveField& field() const {
        const_cast<WaveEquationSolver*>(this)->download();
        return field_;
    }
    WaveField& mutable_field() {
        download();
        dirty_ = true;
        return field_;
    }
    const CartesianGrid& grid() const { return grid_; }
    void save_snapshot(int t) { sync(); check(st_solver_save_snapshot(h_, t)); }
    void clear_snapshots() { sync(); check(st_solver_clear_snapshots(h_)); }
    double compute_energy() const {
        const_cast<WaveEquationSolver*>(this)->sync();
        double e = 0.0;
        check(st_solver_compute_energy(h_, &e));
        return e;
    }
    void reset_field() { dirty_ = false; check(st_solver_reset_field(h_)); }
    bool verify_cfl() const {
        int ok = 0;
        check(st_solver_verify_cfl(h_, &ok));
        return ok != 0;
    }
    void set_amplitude_limit(double limit) { check(st_solver_set_amplitude_limit(h_, limit)); }
    double amplitude_limit() const {
        double v = 0.0;
        check(st_solver_amplitude_limit(h_, &v));
        return v;
    }
    int64_t nan_count_current() const {
        const_cast<WaveEquationSolver*>(this)->sync();
        int64_t n = 0;
        check(st_solver_nan_count_current(h_, &n));
        return n;
    }
    FaultTolerance& fault_tolerance() { return ft_; }
    const FaultTolerance& fault_tolerance() const { return ft_; }
    const FaultTolerance::FaultStats& fault_stats() const { return ft_.stats(); }

    // ---- RTM driver (wave_equation.h:96-110, wave_equation.cpp:508-688)
    void configure_rtm(const RTMConfig& cfg) {
        sync();
        std::vector<st_slice_spec> specs;
        for (const auto& sp : cfg.slice_specs) specs.push_back({(int32_t)sp.axis, sp.index, sp.stride});
        st_rtm_config c{};
        c.enable_rtm = cfg.enable_rtm;
        c.enable_snapshots = cfg.enable_snapshots;
        c.snapshot_interval = cfg.snapshot_interval;
        c.enable_mmap_writer = cfg.enable_mmap_writer;
        c.mmap_filename = cfg.mmap_filename.c_str();
        c.mmap_max_bytes = cfg.mmap_max_bytes;
        c.ring_buffer_capacity = (int64_t)cfg.ring_buffer_capacity;
        c.slice_specs = specs.empty() ? nullptr : specs.data();
        c.n_slice_specs = (int)specs.size();
        c.receivers = cfg.receivers;
        c.snap_kind = cfg.snap_kind;
        c.checkpoint_segment = cfg.checkpoint_segment;
        engine_.reset();
        check(st_solver_configure_rtm(h_, &c));
        rtm_cfg_ = cfg;
        st_rtm_engine* e = nullptr;
        check(st_solver_rtm_engine(h_, &e));
        if (e) {
            const LocalGrid& l = grid_.local();
            engine_.reset(new RTMEngine(e, l.nx_local, l.ny_local, l.nz_local));
            engine_->set_slice_specs(cfg.slice_specs);
        }
    }
    const RTMConfig& rtm_config() const { return rtm_cfg_; }
    // nullptr while RTM is disabled; owned by the solver
    RTMEngine* rtm_engine() { return engine_.get(); }
    // The GPU slice stream plays both the ring buffer and the mmap writer
    // (nullptr without enable_mmap_writer); use st_slice_stream_* on it.
    st_slice_stream* snapshot_buffer() {
        st_slice_stream* p = nullptr;
        check(st_solver_rtm_slice_stream(h_, &p));
        return p;
    }
    st_slice_stream* mmap_writer() { return snapshot_buffer(); }
    // True RTM: source at the domain centre; receiver_residuals [nt][nrec]
    // time-major on rtm_config().receivers. rtm_engine()->result() holds the
    // image afterwards.
    PropagationResult run_rtm(const std::vector<double>& source_wavelet, const std::vector<double>& receiver_residuals) {
        sync();
        st_propagation_result r{};
        check(st_solver_run_rtm(h_, source_wavelet.data(), (int64_t)source_wavelet.size(), receiver_residuals.data(),
                                (int64_t)receiver_residuals.size(), &r));
        return PropagationResult{StepResult(r.status), r.total_nan_encountered, r.total_cells_repaired,
                                 r.timesteps_completed, r.completed_successfully != 0};
    }
    int64_t snapshots_captured() const {
        int64_t c = 0;
        check(st_solver_rtm_snapshot_counts(h_, &c, nullptr));
        return c;
    }
    int64_t snapshots_dropped() const {
        int64_t d = 0;
        check(st_solver_rtm_snapshot_counts(h_, nullptr, &d));
        return d;
    }
    void store_forward_wavefield_for_rtm(int timestep) {
        sync();
        check(st_solver_store_forward_wavefield_for_rtm(h_, timestep));
    }
    void apply_rtm_step(int timestep, bool with_snapshot) {
        sync();
        check(st_solver_apply_rtm_step(h_, timestep, with_snapshot ? 1 : 0));
    }
    st_solver* handle() { return h_; }

   private:
    template <class F>
    PropagationResult prop(F fn, const std::vector<double>& w) {
        sync();
        st_propagation_result r{};
        check(fn(h_, w.data(), (int64_t)w.size(), &r));
        return PropagationResult{StepResult(r.status), r.total_nan_encountered, r.total_cells_repaired,
                                 r.timesteps_completed, r.completed_successfully != 0};
    }
    void download() {
        const int64_t n = grid_.local().total_cells_with_halo;
        for (auto* v : {&field_.current, &field_.previous, &field_.next, &field_.velocity}) v->resize((size_t)n);
        check(st_solver_get_field(h_, ST_FIELD_CURRENT, field_.current.data(), n));
        check(st_solver_get_field(h_, ST_FIELD_PREVIOUS, field_.previous.data(), n));
        check(st_solver_get_field(h_, ST_FIELD_NEXT, field_.next.data(), n));
        check(st_solver_get_field(h_, ST_FIELD_VELOCITY, field_.velocity.data(), n));
        int64_t ns = 0;
        check(st_solver_snapshot_values(h_, &ns));
        field_.snapshots.resize((size_t)ns);
        if (ns) check(st_solver_get_snapshots(h_, field_.snapshots.data(), ns));
    }
    void sync() {
        if (!dirty_) return;
        dirty_ = false;
        const int64_t n = grid_.local().total_cells_with_halo;
        check(st_solver_set_field(h_, ST_FIELD_CURRENT, field_.current.data(), n));
        check(st_solver_set_field(h_, ST_FIELD_PREVIOUS, field_.previous.data(), n));
        check(st_solver_set_field(h_, ST_FIELD_NEXT, field_.next.data(), n));
        check(st_solver_set_velocity_field(h_, field_.velocity.data(), (int64_t)field_.velocity.size()));
    }
    const MpiContext& mpi_;
    const CartesianGrid& grid_;
    SolverConfig config_;
    st_solver* h_ = nullptr;
    WaveField field_;
    bool dirty_ = false;
    FaultTolerance ft_;
    RTMConfig rtm_cfg_;
    std::unique_ptr<RTMEngine> engine_;
};

// ---------------------------------------------------------------- solver/boundary.h:9-52
struct BathymetryPoint {
    double x, y, depth;
};

// TerrainBoundary over the GPU library: the bathymetry is built on the host,
// the field operations run on the device (host vectors are copied in and
// out). The grid must outlive the object, as in the reference.
class TerrainBoundary {
   public:
    TerrainBoundary(const CartesianGrid& grid, double water_depth, int device = 0) : grid_(grid) {
        const GridParams& g = grid.params();
        const st_grid_params p{g.nx_global, g.ny_global, g.nz_global, g.dx, g.dy, g.dz,
                               g.origin_x, g.origin_y, g.origin_z, g.halo_width};
        check(st_terrain_create(&p, water_depth, device, &h_));
    }
    ~TerrainBoundary() { st_terrain_destroy(h_); }
    TerrainBoundary(const TerrainBoundary&) = delete;
    TerrainBoundary& operator=(const TerrainBoundary&) = delete;

    void set_bathymetry_data(const std::vector<BathymetryPoint>& data) {
        std::vector<st_bathymetry_point> pts(data.size());
        for (size_t k = 0; k < data.size(); ++k) pts[k] = {data[k].x, data[k].y, data[k].depth};
        check(st_terrain_set_bathymetry_data(h_, pts.data(), (int64_t)pts.size()));
    }
    void generate_synthetic_bathymetry(double gradient, double roughness) {
        check(st_terrain_generate_synthetic_bathymetry(h_, gradient, roughness));
    }
    bool is_subsurface(int64_t gx, int64_t gy, int64_t gz) const {
        return grid_.params().origin_z + gz * grid_.params().dz >= seafloor_depth(gx, gy);
    }
    bool is_water(int64_t gx, int64_t gy, int64_t gz) const { return !is_subsurface(gx, gy, gz); }
    double seafloor_depth(int64_t gx, int64_t gy) const {
        double d = 0.0;
        check(st_terrain_seafloor(h_, gx, gy, &d, nullptr));
        return d;
    }
    int64_t seafloor_index(int64_t gx, int64_t gy) const {
        int64_t i = 0;
        check(st_terrain_seafloor(h_, gx, gy, nullptr, &i));
        return i;
    }
    // The reference's signatures take the local grid and halo width; one
    // device domain has the grid's own.
    void apply_free_surface_bc(std::vector<double>& field, const LocalGrid&, int) {
        check(st_terrain_apply_free_surface_bc(h_, sized(field), 0));
    }
    void apply_seafloor_bc(std::vector<double>& field, const LocalGrid&, int) {
        check(st_terrain_apply_seafloor_bc(h_, sized(field), 0));
    }
    void apply_absorbing_bc(std::vector<double>& field, const LocalGrid&, int, int sponge_width, double damping) {
        check(st_terrain_apply_absorbing_bc(h_, sized(field), 0, sponge_width, damping));
    }
    void update_velocity_mask(std::vector<double>& velocity, double water_vp, double sediment_vp) const {
        check(st_terrain_update_velocity_mask(h_, sized(velocity), 0, water_vp, sediment_vp));
    }
    const std::vector<double>& bathymetry() const {
        bathy_.resize((size_t)(grid_.params().nx_global * grid_.params().ny_global));
        check(st_terrain_bathymetry(h_, bathy_.data()));
        return bathy_;
    }
    void build_boundary_mask(const LocalGrid&, int) {
        mask_.assign((size_t)grid_.local().total_cells_with_halo, 0);
        check(st_terrain_build_boundary_mask(h_, mask_.data(), 0));
    }
    const std::vector<uint8_t>& mask() const { return mask_; }
    st_terrain* handle() const { return h_; }

   private:
    double* sized(std::vector<double>& f) const {
        if ((int64_t)f.size() < grid_.local().total_cells_with_halo) throw std::invalid_argument("field too small");
        return f.data();
    }
    const CartesianGrid& grid_;
    st_terrain* h_ = nullptr;
    mutable std::vector<double> bathy_;
    std::vector<uint8_t> mask_;
};

// ---------------------------------------------------------------- rtm/mmap_writer.h:24-124
constexpr int64_t DEFAULT_MMAP_MAX_BYTES = 4LL * 1024LL * 1024LL * 1024LL;
constexpr int64_t MMAP_FILE_MAGIC = 0x52544D534E4150LL;

// The slice-ring file writer (the library's C++ writer, the reference's file
// format); frames are serialized slices, e.g. from st_capture_slice_frames.
class MmapSnapshotWriter {
   public:
    struct Stats {
        int64_t frames_written, frames_dropped_buffer_full, total_bytes_written, mmap_cycles;
    };
    MmapSnapshotWriter() = default;
    ~MmapSnapshotWriter() { close(); }
    MmapSnapshotWriter(const MmapSnapshotWriter&) = delete;
    MmapSnapshotWriter& operator=(const MmapSnapshotWriter&) = delete;

    bool open(const std::string& filename, int64_t max_bytes = DEFAULT_MMAP_MAX_BYTES) {
        close();
        if (st_mmap_writer_open(filename.c_str(), max_bytes, &h_) != 0) return false;
        filename_ = filename;
        max_bytes_ = max_bytes;
        return true;
    }
    void close() {
        if (h_) st_mmap_writer_close(h_);
        h_ = nullptr;
    }
    bool is_open() const { return h_ != nullptr; }
    bool write_frame(const uint8_t* frame_data, int64_t frame_size) {
        return h_ && frame_data && frame_size > 0 && st_mmap_writer_write_frame(h_, frame_data, frame_size) == 0;
    }
    int64_t frame_count() const { return info()[0]; }
    int64_t write_offset() const { return info()[1]; }
    int64_t used_bytes() const { return write_offset(); }
    int64_t capacity_bytes() const { return max_bytes_; }
    Stats stats() const {
        const auto i = info();
        return Stats{i[3], i[4], i[5], i[6]};
    }
    std::string filename() const { return filename_; }
    static bool read_frame(const std::string& filename, int64_t frame_index, std::vector<uint8_t>& out_data) {
        int64_t n = 0;
        if (st_mmap_read_frame(filename.c_str(), frame_index, nullptr, 0, &n) != 0) return false;
        out_data.resize((size_t)n);
        return st_mmap_read_frame(filename.c_str(), frame_index, out_data.data(), n, &n) == 0;
    }
    static int64_t count_frames(const std::string& filename) {
        int64_t n = -1;
        return st_mmap_count_frames(filename.c_str(), &n) == 0 ? n : -1;
    }

   private:
    std::vector<int64_t> info() const {
        std::vector<int64_t> out(7, 0);
        if (h_) check(st_mmap_writer_info(h_, out.data()));
        return out;
    }
    st_mmap_writer* h_ = nullptr;
    std::string filename_;
    int64_t max_bytes_ = 0;
};

// ---------------------------------------------------------------- sparse/aligned_alloc.h:25-91
// 64-byte aligned vector; new elements are always value-initialised (the
// reference's AlignedVector(n, 0.0) leaves them uninitialised) and copies are
// allowed (its copy constructor is deleted, which breaks sparse_ops.cpp).
template <typename T>
class AlignedVector {
   public:
    AlignedVector() = default;
    explicit AlignedVector(size_t n, T value = T()) { resize(n, value); }
    AlignedVector(const AlignedVector& o) { *this = o; }
    AlignedVector& operator=(const AlignedVector& o) {
        if (this != &o) {
            resize(o.size_);
            std::copy(o.data_.get(), o.data_.get() + o.size_, data_.get());
        }
        return *this;
    }
    AlignedVector(AlignedVector&&) noexcept = default;
    AlignedVector& operator=(AlignedVector&&) noexcept = default;
    void resize(size_t n, T value = T()) {
        if (n > cap_) {
            std::unique_ptr<T[], Free> nd(static_cast<T*>(::operator new[](n * sizeof(T), std::align_val_t(64))));
            for (size_t i = 0; i < n; ++i) nd[i] = i < size_ ? data_[i] : value;
            data_ = std::move(nd);
            cap_ = n;
        } else {
            for (size_t i = size_; i < n; ++i) data_[i] = value;
        }
        size_ = n;
    }
    T& operator[](size_t i) { return data_[i]; }
    const T& operator[](size_t i) const { return data_[i]; }
    T* data() { return data_.get(); }
    const T* data() const { return data_.get(); }
    size_t size() const { return size_; }
    bool empty() const { return size_ == 0; }

   private:
    struct Free {
        void operator()(T* p) const { ::operator delete[](p, std::align_val_t(64)); }
    };
    std::unique_ptr<T[], Free> data_;
    size_t size_ = 0, cap_ = 0;
};

// ---------------------------------------------------------------- sparse/csr_matrix.h:11-71
struct SparseEntry {
    int64_t row;
    int64_t col;
    double value;
};

class CSRMatrix {
   public:
    CSRMatrix(int device = 0) { check(st_csr_create(0, 0, 0, device, &h_)); }
    CSRMatrix(int64_t rows, int64_t cols, int64_t nnz, int device = 0) {
        check(st_csr_create(rows, cols, nnz, device, &h_));
    }
    CSRMatrix(const CSRMatrix& o) { check(st_csr_clone(o.h_, &h_)); }
    CSRMatrix& operator=(const CSRMatrix& o) {
        if (this != &o) {
            st_csr* c = nullptr;
            check(st_csr_clone(o.h_, &c));
            st_csr_destroy(h_);
            h_ = c;
        }
        return *this;
    }
    ~CSRMatrix() { st_csr_destroy(h_); }

    void build_from_triplets(int64_t rows, int64_t cols, const std::vector<SparseEntry>& e, bool pad = false) {
        std::vector<int64_t> r(e.size()), c(e.size());
        std::vector<double> v(e.size());
        for (size_t i = 0; i < e.size(); ++i) {
            r[i] = e[i].row;
            c[i] = e[i].col;
            v[i] = e[i].value;
        }
        check(st_csr_build_from_triplets(h_, rows, cols, (int64_t)e.size(), r.data(), c.data(), v.data(), pad));
    }
    void build_fd_stencil_7point(int64_t nx, int64_t ny, int64_t nz, const double* velocity, double dx, double dy,
                                 double dz, double dt) {
        check(st_csr_build_fd_stencil_7point(h_, nx, ny, nz, velocity, dx, dy, dz, dt, 0));
    }
    AlignedVector<double> spmv(const AlignedVector<double>& x) const {
        AlignedVector<double> y((size_t)rows());
        check(st_csr_spmv(h_, x.data(), (int64_t)x.size(), y.data()));
        return y;
    }
    AlignedVector<double> spmv_transpose(const AlignedVector<double>& x) const {
        AlignedVector<double> y((size_t)cols());
        check(st_csr_spmv_transpose(h_, x.data(), (int64_t)x.size(), y.data()));
        return y;
    }
    int64_t rows() const { return shape()[0]; }
    int64_t cols() const { return shape()[1]; }
    int64_t nnz() const { return shape()[2]; }
    AlignedVector<int64_t> row_ptr() const {
        AlignedVector<int64_t> r((size_t)rows() + 1);
        check(st_csr_get(h_, r.data(), nullptr, nullptr));
        return r;
    }
    AlignedVector<int64_t> col_ind() const {
        AlignedVector<int64_t> c((size_t)nnz());
        check(st_csr_get(h_, nullptr, c.data(), nullptr));
        return c;
    }
    AlignedVector<double> values() const {
        AlignedVector<double> v((size_t)nnz());
        check(st_csr_get(h_, nullptr, nullptr, v.data()));
        return v;
    }
    double frobenius_norm() const {
        double f = 0.0;
        check(st_csr_frobenius_norm(h_, &f));
        return f;
    }
    void scale(double a) { check(st_csr_scale(h_, a)); }
    void add_diagonal(double a) { check(st_csr_add_diagonal(h_, a)); }
    void optimize_cache_blocking(int64_t = 8) {}  // the GPU SpMV assigns rows to thread groups itself
    st_csr* handle() const { return h_; }

   private:
    std::vector<int64_t> shape() const {
        std::vector<int64_t> s(3);
        check(st_csr_shape(h_, s.data()));
        return s;
    }
    st_csr* h_ = nullptr;
};

// ---------------------------------------------------------------- sparse/sparse_ops.h:9-48
class SparseOps {
   public:
    static AlignedVector<double> conjugate_gradient(const CSRMatrix& A, const AlignedVector<double>& b, int max_iter,
                                                    double tolerance) {
        return cg(A, b, max_iter, tolerance, 0);
    }
    static AlignedVector<double> jacobi_preconditioned_cg(const CSRMatrix& A, const AlignedVector<double>& b,
                                                          int max_iter, double tolerance) {
        return cg(A, b, max_iter, tolerance, 1);
    }
    static std::vector<double> smooth_gradient(const std::vector<double>& g, int64_t nx, int64_t ny, int64_t nz,
                                               double sigma) {
        std::vector<double> out((size_t)(nx * ny * nz), 0.0);
        check(st_smooth_gradient(g.data(), (int64_t)g.size(), nx, ny, nz, sigma, 0, out.data()));
        return out;
    }
    static double dot_product(const AlignedVector<double>& a, const AlignedVector<double>& b) {
        double d = 0.0;
        check(st_dot(a.data(), b.data(), (int64_t)std::min(a.size(), b.size()), 0, &d));
        return d;
    }
    static double l2_norm(const AlignedVector<double>& a) { return std::sqrt(dot_product(a, a)); }
    static AlignedVector<double> axpy(double alpha, const AlignedVector<double>& x, const AlignedVector<double>& y) {
        const size_t n = std::min(x.size(), y.size());
        AlignedVector<double> r(n);
        for (size_t i = 0; i < n; ++i) r[i] = alpha * x[i] + y[i];
        return r;
    }
    static CSRMatrix build_hessian_approx(const CSRMatrix& forward_operator, double regularization) {
        CSRMatrix H(forward_operator);
        H.add_diagonal(regularization);
        return H;
    }

   private:
    static AlignedVector<double> cg(const CSRMatrix& A, const AlignedVector<double>& b, int max_iter, double tol,
                                    int jacobi) {
        AlignedVector<double> x((size_t)A.rows());
        int it = 0;
        double rel = 0.0;
        check(st_cg(A.handle(), b.data(), (int64_t)b.size(), max_iter, tol, jacobi, x.data(), &it, &rel));
        return x;
    }
};

}  // namespace seismic
