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
    return 0;
}
