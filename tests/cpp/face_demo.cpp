// Exercise of the header-only seismic:: C++ face (include/seismic_gb300.hpp)
// the way a caller of the reference's classes would use it; prints figures
// that tests/test_cpp_face.py compares with the Python face.
#include <cmath>
#include <cstdio>
#include <vector>

#include "seismic_gb300.hpp"

int main(int argc, char** argv) {
    seismic::MpiContext mpi(argc, argv);
    seismic::TomographyConfig cfg =
        argc > 1 && argv[1][0] ? seismic::load_config(argv[1]) : seismic::TomographyConfig{};
    cfg.solver.dt = 0.001;
    cfg.solver.sponge_width = 4;
    cfg.solver.sponge_damping = 0.015;
    seismic::GridParams gp{20, 18, 22, 10.0, 10.0, 10.0, 0.0, 0.0, 0.0, 1};
    int coords[3] = {0, 0, 0}, dims[3] = {1, 1, 1};
    seismic::CartesianGrid grid(gp, coords, dims);
    seismic::WaveEquationSolver solver(mpi, grid, cfg.solver);
    solver.initialize_velocity(2500.0);
    for (int t = 0; t < 30; ++t) {
        solver.inject_source(10, 9, 5, {std::sin(0.3 * t)});
        solver.step_forward(t);
    }
    const seismic::WaveField& f = solver.field();
    double e = 0.0;
    for (double v : f.current) e += v * v;
    std::printf("energy %.17g %.17g\n", solver.compute_energy(), e);
    std::printf("cfl %d\n", solver.verify_cfl() ? 1 : 0);
    std::printf("mpi %g\n", mpi.allreduce_sum(2.0));

    seismic::RTMEngine rtm(20, 18, 22, 10.0, 10.0, 10.0, 1);
    rtm.apply_image_condition(f.current.data(), f.previous.data(), 20, 24, 0);
    rtm.finalize_image();
    double img = 0.0;
    for (double v : rtm.result().image) img += v;
    std::printf("image %.17g\n", img);

    seismic::CSRMatrix A;
    std::vector<double> vel(8 * 8 * 8, 2000.0);
    A.build_fd_stencil_7point(8, 8, 8, vel.data(), 10.0, 10.0, 10.0, 0.00125);
    seismic::AlignedVector<double> b(512, 1.0);
    seismic::AlignedVector<double> x = seismic::SparseOps::jacobi_preconditioned_cg(A, b, 500, 1e-8);
    seismic::AlignedVector<double> ax = A.spmv(x);
    double r = 0.0, bb = 0.0;
    for (size_t i = 0; i < 512; ++i) {
        r += (ax[i] - b[i]) * (ax[i] - b[i]);
        bb += b[i] * b[i];
    }
    std::printf("cg_rel %.3e\n", std::sqrt(r / bb));
    std::printf("nnz %lld %lld\n", (long long)A.nnz(), (long long)A.rows());
    std::printf("dot %.17g\n", seismic::SparseOps::dot_product(b, x));

    // terrain: bathymetry from points, the water-column velocity and the seafloor condition
    seismic::TerrainBoundary terrain(grid, 50.0);
    terrain.set_bathymetry_data({{15.0, 15.0, 120.0}, {105.0, 95.0, 30.0}});
    std::vector<double> tv(grid.local().total_cells_with_halo, 0.0);
    terrain.update_velocity_mask(tv, 1500.0, 3000.0);
    std::vector<double> tf(grid.local().total_cells_with_halo, 1.0);
    terrain.apply_seafloor_bc(tf, grid.local(), 1);
    double tsum = 0.0, fsum = 0.0;
    for (double v : tv) tsum += v;
    for (double v : tf) fsum += v;
    std::printf("terrain %lld %lld %.17g %.17g\n", (long long)terrain.seafloor_index(1, 1),
                (long long)terrain.seafloor_index(10, 9), tsum, fsum);

    // the slice ring: two frames through the writer, read back
    const char* ring = argc > 2 ? argv[2] : "face_demo_ring.dat";
    seismic::MmapSnapshotWriter w;
    const std::vector<uint8_t> f1(300, 7), f2(500, 9);
    const bool ok = w.open(ring, 4096) && w.write_frame(f1.data(), 300) && w.write_frame(f2.data(), 500);
    w.close();
    std::vector<uint8_t> back;
    const bool rd = seismic::MmapSnapshotWriter::read_frame(ring, 1, back);
    std::printf("ring %d %lld %d %lld\n", ok ? 1 : 0, (long long)seismic::MmapSnapshotWriter::count_frames(ring),
                rd ? 1 : 0, (long long)back.size());

    // the RTM driver and the rest of the solver face
    seismic::RTMConfig rc;
    rc.enable_rtm = true;
    rc.receivers = st_receiver_grid{0, 2, 10, 0, 2, 9, 0};
    rc.snap_kind = ST_SNAP_FP32;
    seismic::CartesianGrid grid2(gp, coords, dims);
    seismic::SolverConfig sc2 = cfg.solver;
    sc2.nt = 24;
    seismic::WaveEquationSolver rtm_solver(mpi, grid2, sc2);
    rtm_solver.initialize_velocity(2500.0);
    const seismic::PropagationResult off = rtm_solver.run_rtm({1.0}, {});
    rtm_solver.configure_rtm(rc);
    std::vector<double> wav(24), res(24 * 90);
    for (int t = 0; t < 24; ++t) wav[t] = std::sin(0.4 * t);
    for (size_t k = 0; k < res.size(); ++k) res[k] = 1e-3 * std::cos(0.1 * (double)k);
    const seismic::PropagationResult pr = rtm_solver.run_rtm(wav, res);
    double rimg = 0.0;
    for (double v : rtm_solver.rtm_engine()->result().image) rimg += v;
    std::printf("run_rtm %d %d %d %.17g\n", off.completed_successfully ? 1 : 0, (int)pr.status,
                pr.timesteps_completed, rimg);
    rtm_solver.reset_field();
    rtm_solver.rtm_engine()->reset_image();
    for (int t = 0; t < 10; ++t) {
        rtm_solver.inject_source(10, 9, 11, {wav[t]});
        rtm_solver.step_forward(t);
        if (t == 4) rtm_solver.store_forward_wavefield_for_rtm(t);
        rtm_solver.apply_rtm_step(t, t % 3 == 0);
    }
    rtm_solver.apply_sponge_layer();
    rtm_solver.rtm_engine()->finalize_image();
    double bimg = 0.0;
    for (double v : rtm_solver.rtm_engine()->result().image) bimg += v;
    std::printf("blocks %.17g %.17g %lld %lld\n", bimg, rtm_solver.compute_energy(),
                (long long)rtm_solver.snapshots_captured(), (long long)rtm_solver.snapshots_dropped());
    seismic::FaultTolerance& ft = rtm_solver.fault_tolerance();
    ft.set_cfl_safety_factor(2.0);
    ft.reset_stats();
    std::printf("fault %g %d %lld\n", ft.cfl_safety_factor(), ft.max_repair_attempts(),
                (long long)rtm_solver.fault_stats().cells_repaired);
    const seismic::PropagationResult ap = rtm_solver.adjoint_propagate({0.5, -0.25, 0.125});
    std::printf("adjoint %d %d %.17g\n", (int)ap.status, ap.timesteps_completed, rtm_solver.compute_energy());
    return 0;
}
