"""GPU parity of the sparse path (CSR build, SpMV, CG / PCG / normal-equation
CG), the field-health helpers and the gradient smoothing, against the
reference fixtures and the FP64 oracle, through the C ABI.

Bars: CSR row_ptr / col_ind bit-exact; values equal to the FP32 rounding of
the reference's FP64 sums (1 FP32 ulp where the FD stencil's FP64
expressions may contract differently); SpMV relative error <= 1e-6 (FP32
values and accumulation); CG solutions within 1e-5 relative of the FP64
oracle's; fault helpers bit-exact; smoothing within 1e-12."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def se():
    import importlib.util
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(repo, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import seismic_engine
    return seismic_engine


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def test_build_matches_reference_fixture(se, golden_dir):
    g = np.load(os.path.join(golden_dir, "csr_small.npz"))
    m = se.CSRMatrix().build_from_triplets(int(g["rows"]), int(g["cols"]), g["r"], g["c"], g["v"])
    assert m.rows() == int(g["rows"]) and m.cols() == int(g["cols"]) and m.nnz() == g["col"].size
    np.testing.assert_array_equal(m.row_ptr(), g["row_ptr"])
    np.testing.assert_array_equal(m.col_ind(), g["col"])
    np.testing.assert_array_equal(m.values(), f32(g["val"]))
    y = m.spmv(g["x"])
    assert np.linalg.norm(y - g["y"]) <= 1e-6 * np.linalg.norm(g["y"])


@pytest.mark.parametrize("rows,cols,n,seed", [(3000, 2500, 200000, 0), (1, 70000, 150000, 1),
                                              (50000, 7, 90000, 2), (5, 5, 0, 3), (0, 4, 10, 4)])
def test_build_random_vs_oracle(se, oracle, rows, cols, n, seed):
    rng = np.random.default_rng(seed)
    r = rng.integers(-2, rows + 2, n)
    c = rng.integers(-2, cols + 2, n)
    dup = rng.integers(0, max(n, 1), n // 5) if n else np.zeros(0, np.int64)
    r = np.concatenate([r, r[dup]]) if n else r
    c = np.concatenate([c, c[dup]]) if n else c
    v = rng.standard_normal(r.size)
    m = se.CSRMatrix().build_from_triplets(rows, cols, r, c, v)
    rp, col, val = oracle.csr_build(rows, cols, r, c, v)
    np.testing.assert_array_equal(m.row_ptr(), rp)
    np.testing.assert_array_equal(m.col_ind(), col)
    np.testing.assert_array_equal(m.values(), f32(val))


def test_pad_mode_vs_oracle(se, oracle):
    rng = np.random.default_rng(5)
    n = 300
    r = rng.integers(0, n, 1500)
    c = rng.integers(0, n, 1500)
    v = rng.standard_normal(1500)
    m = se.CSRMatrix().build_from_triplets(n, n, r, c, v, pad=True)
    rp, col, val = oracle.csr_build(n, n, r, c, v, pad=True)
    assert rp[-1] % 8 == 0 and m.nnz() == rp[-1]
    np.testing.assert_array_equal(m.row_ptr(), rp)
    np.testing.assert_array_equal(m.col_ind(), col)
    np.testing.assert_array_equal(m.values(), f32(val))
    with pytest.raises(se.SeismicError):
        se.CSRMatrix().build_from_triplets(2 * n, n, r, c, v, pad=True)


def fd_triplets(nx, ny, nz, vel, dx, dy, dz, dt):
    """Triplets of build_fd_stencil_7point (csr_matrix.cpp:74-116) in its order."""
    idx2, idy2, idz2, dt2 = 1 / dx ** 2, 1 / dy ** 2, 1 / dz ** 2, dt * dt
    R, C, V = [], [], []
    for ix in range(nx):
        for iy in range(ny):
            for iz in range(nz):
                r = (ix * ny + iy) * nz + iz
                v2 = vel[r] * vel[r] * dt2
                R.append(r); C.append(r); V.append(-2.0 * v2 * (idx2 + idy2 + idz2) + 2.0)
                for ok, cc, w in ((ix > 0, r - ny * nz, idx2), (ix < nx - 1, r + ny * nz, idx2),
                                  (iy > 0, r - nz, idy2), (iy < ny - 1, r + nz, idy2),
                                  (iz > 0, r - 1, idz2), (iz < nz - 1, r + 1, idz2)):
                    if ok:
                        R.append(r); C.append(cc); V.append(v2 * w)
    return np.array(R), np.array(C), np.array(V)


def test_fd_stencil_vs_oracle(se, oracle):
    nx, ny, nz = 7, 6, 9
    rng = np.random.default_rng(6)
    vel = 1500 + 1000 * rng.random(nx * ny * nz)
    m = se.compute_fd_stencil(nx, ny, nz, vel, 10.0, 12.0, 9.0, 1e-3)
    R, Cc, V = fd_triplets(nx, ny, nz, vel, 10.0, 12.0, 9.0, 1e-3)
    rp, col, val = oracle.csr_build(nx * ny * nz, nx * ny * nz, R, Cc, V)
    np.testing.assert_array_equal(m.row_ptr(), rp)
    np.testing.assert_array_equal(m.col_ind(), col)
    np.testing.assert_allclose(m.values(), f32(val), rtol=2.0 ** -23, atol=0)


def test_spmv_and_transpose_vs_oracle(se, oracle):
    rng = np.random.default_rng(7)
    rows, cols, n = 20000, 9000, 600000
    r = rng.integers(0, rows, n)
    c = rng.integers(0, cols, n)
    v = rng.standard_normal(n).astype(np.float32).astype(np.float64)
    m = se.CSRMatrix().build_from_triplets(rows, cols, r, c, v)
    rp, col, val = oracle.csr_build(rows, cols, r, c, v)
    om = oracle.csr(rows, cols, rp, col, f32(val))
    x = rng.standard_normal(cols).astype(np.float32).astype(np.float64)
    xt = rng.standard_normal(rows).astype(np.float32).astype(np.float64)
    y, yr = m.spmv(x), oracle.spmv(om, x)
    assert np.linalg.norm(y - yr) <= 1e-6 * np.linalg.norm(yr)
    yt, ytr = m.spmv_transpose(xt), oracle.spmv_t(om, xt)
    assert np.linalg.norm(yt - ytr) <= 1e-6 * np.linalg.norm(ytr)
    assert abs(m.frobenius_norm() - np.linalg.norm(f32(val))) <= 1e-12 * np.linalg.norm(val)
    m.scale(0.5)
    np.testing.assert_array_equal(m.values(), f32(val) * 0.5)


def spd_fd(se, oracle, n=(14, 12, 16), seed=8):
    nx, ny, nz = n
    vel = np.full(nx * ny * nz, 2000.0)
    dt = 0.25 * 10.0 / 2000.0  # c = (v dt / d)^2 = 1/16: diagonally dominant, symmetric
    R, Cc, V = fd_triplets(nx, ny, nz, vel, 10.0, 10.0, 10.0, dt)
    rp, col, val = oracle.csr_build(nx * ny * nz, nx * ny * nz, R, Cc, V)
    m = se.compute_fd_stencil(nx, ny, nz, vel, 10.0, 10.0, 10.0, dt)
    return m, oracle.csr(nx * ny * nz, nx * ny * nz, rp, col, f32(val)), nx * ny * nz


def test_cg_and_pcg_vs_oracle(se, oracle):
    m, om, n = spd_fd(se, oracle)
    b = np.random.default_rng(9).standard_normal(n)
    for jac, fn in ((False, se.SparseOps.conjugate_gradient), (True, se.SparseOps.jacobi_preconditioned_cg)):
        x = fn(m, b, 500, 1e-6)
        it = se.SparseOps.last_iterations
        xr, itr, relr = oracle.cg(om, b, 500, 1e-6, jacobi=jac)
        assert abs(it - itr) <= 2, (it, itr)
        assert np.linalg.norm(x - xr) <= 1e-5 * np.linalg.norm(xr)
    # ||b|| < 1e-30 returns x0 = 0 with no iteration
    assert not se.SparseOps.conjugate_gradient(m, np.zeros(n)).any() and se.SparseOps.last_iterations == 0
    H = se.SparseOps.build_hessian_approx(m, 0.25)
    d0 = m.values()[m.col_ind() == np.repeat(np.arange(n), np.diff(m.row_ptr()))]
    d1 = H.values()[H.col_ind() == np.repeat(np.arange(n), np.diff(H.row_ptr()))]
    np.testing.assert_allclose(d1, f32(d0 + 0.25), rtol=2.0 ** -23)


def test_normal_equation_cg_vs_oracle(se, oracle):
    import torch
    rng = np.random.default_rng(10)
    rows, cols = 6000, 2000
    r = np.repeat(np.arange(rows), 12)
    c = rng.integers(0, cols, r.size)
    v = rng.random(r.size).astype(np.float32).astype(np.float64)
    m = se.CSRMatrix().build_from_triplets(rows, cols, r, c, v)
    rp, col, val = oracle.csr_build(rows, cols, r, c, v)
    om = oracle.csr(rows, cols, rp, col, f32(val))
    d = rng.standard_normal(rows).astype(np.float32)
    lam = 1e-2
    x = torch.zeros(cols, device="cuda")
    rhs = torch.zeros(cols, device="cuda")
    it, rel, true_rel = se.normal_cg_device(m, torch.from_numpy(d).cuda(), lam, x, 1000, 1e-6, True, rhs)
    xr, itr, relr, rhsr = oracle.normal_cg(om, d.astype(np.float64), lam, 1000, 1e-6, jacobi=True)
    assert rel < 1e-6 and true_rel < 1e-5
    assert abs(it - itr) <= 3, (it, itr)
    assert np.linalg.norm(rhs.cpu().numpy() - rhsr) <= 1e-6 * np.linalg.norm(rhsr)
    assert np.linalg.norm(x.cpu().numpy() - xr) <= 1e-5 * np.linalg.norm(xr)


def test_dot_product(se):
    rng = np.random.default_rng(11)
    a, b = rng.standard_normal(100003), rng.standard_normal(100003)
    assert abs(se.SparseOps.dot_product(a, b) - float(np.dot(a, b))) <= 1e-12 * np.abs(a * b).sum()


def test_fault_helpers_match_reference_fixture(se, golden_dir):
    g = np.load(os.path.join(golden_dir, "fault_small.npz"))
    nx, ny, nz = (int(v) for v in g["n"])
    assert se.check_field_health(g["field"]) == int(g["nan_count"])
    np.testing.assert_array_equal(se.clamp_field_safe(g["field"].copy(), -500.0, 500.0), g["clamped"])
    rep = se.repair_field_nan(g["field"].copy(), nx + 2, ny + 2, nz + 2, 1, 0.0)
    np.testing.assert_allclose(rep, g["repaired"], rtol=1e-15, atol=0)


def test_smooth_gradient_vs_oracle(se, oracle):
    rng = np.random.default_rng(12)
    nx, ny, nz = 11, 9, 13
    g = rng.standard_normal(nx * ny * nz)
    for sigma in (0.7, 1.0, 2.0):
        out = se.SparseOps.smooth_gradient(g, nx, ny, nz, sigma)
        ref = oracle.smooth_gradient(g, nx, ny, nz, sigma)
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-13)
    assert not se.SparseOps.smooth_gradient(np.ones(10), nx, ny, nz, 1.0).any()


def test_regularised_update_with_given_rhs(se):
    """(I + L^T L) x = g for the 7-point Laplacian L (built by the FD-stencil
    builder with unit coefficients and a diagonal shift) with the right-hand
    side given directly: against a dense FP64 solve."""
    import torch
    n = 10
    L = se.CSRMatrix()
    L.build_fd_stencil_7point(n, n, n, np.full(n ** 3, 1.0), 1.0, 1.0, 1.0, 1.0)
    L.add_diagonal(-2.0)
    rp, col, val = L.row_ptr(), L.col_ind(), L.values()
    Ld = np.zeros((n ** 3, n ** 3))
    for i in range(n ** 3):
        Ld[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    assert np.allclose(np.diag(Ld), -6.0) and np.allclose(Ld, Ld.T)
    g = np.random.default_rng(13).standard_normal(n ** 3)
    xs = np.linalg.solve(np.eye(n ** 3) + Ld.T @ Ld, g)
    x = torch.zeros(n ** 3, device="cuda")
    rhs = torch.from_numpy(g.astype(np.float32)).cuda()
    it, rel, true_rel = se.normal_cg_device(L, None, 1.0, x, 2000, 1e-7, True, rhs=rhs)
    assert true_rel < 5e-6  # FP32 vectors: the attainable true residual of this operator is about 1e-6
    assert np.linalg.norm(x.cpu().numpy() - xs) <= 1e-5 * np.linalg.norm(xs)


def _unpadded(rp, col, val):
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    keep = ~((col == rows) & (val == 0.0))
    return rows[keep], col[keep], val[keep]


def test_sparse_ops_match_reference_fixture(se, golden_dir):
    """The GPU sparse path against the reference's own sparse module
    (sparse_small.npz, from sparse/csr_matrix.cpp + sparse/sparse_ops.cpp
    built with the three fixes oracle/build_ref.sh lists): the padded FD
    stencil build, SpMV / SpMV^T, CG and Jacobi-PCG at tol 1e-6 (iterations
    within 1, 2 for plain CG on the SPD matrix; solutions within 1e-5
    relative: FP32 vectors, FP64 scalars),
    dot_product, smooth_gradient and build_hessian_approx."""
    g = np.load(os.path.join(golden_dir, "sparse_small.npz"))
    nx, ny, nz = (int(v) for v in g["fd_n"])
    dx, dy, dz, dt = (float(v) for v in g["fd_d"])
    n = nx * ny * nz
    fd = se.CSRMatrix().build_fd_stencil_7point(nx, ny, nz, g["fd_vel"], dx, dy, dz, dt, pad=True)
    np.testing.assert_array_equal(fd.row_ptr(), g["fd_row_ptr"])
    np.testing.assert_array_equal(fd.col_ind(), g["fd_col"])
    np.testing.assert_allclose(fd.values(), f32(g["fd_val"]), rtol=2.0 ** -23, atol=0)
    for got, ref in ((fd.spmv(g["fd_x"]), g["fd_y"]), (fd.spmv_transpose(g["fd_xt"]), g["fd_yt"])):
        assert np.linalg.norm(got - ref) <= 1e-6 * np.linalg.norm(ref)
    sr, sc, sv = _unpadded(g["spd_row_ptr"], g["spd_col"], g["spd_val"])
    spd = se.CSRMatrix().build_from_triplets(200, 200, sr, sc, sv, pad=True)
    np.testing.assert_array_equal(spd.row_ptr(), g["spd_row_ptr"])
    np.testing.assert_array_equal(spd.col_ind(), g["spd_col"])
    np.testing.assert_array_equal(spd.values(), f32(g["spd_val"]))
    assert np.linalg.norm(spd.spmv(g["spd_x"]) - g["spd_y"]) <= 1e-6 * np.linalg.norm(g["spd_y"])
    for name, m in (("fd", fd), ("spd", spd)):
        for jac, fn in ((0, se.SparseOps.conjugate_gradient), (1, se.SparseOps.jacobi_preconditioned_cg)):
            key = f"cg_{name}_{jac}_6"
            x = fn(m, g[f"{name}_b"], 10000, 1e-6)
            # plain CG on the SPD matrix amplifies rounding differences (the FP64
            # oracle's iterates already move 3e-9 from the reference build's by
            # iteration 34); in FP32 vectors it measured 50 iterations against 48
            slack = 2 if (name, jac) == ("spd", 0) else 1
            assert abs(se.SparseOps.last_iterations - int(g[key + "_iters"])) <= slack, (key,
                                                                                      se.SparseOps.last_iterations)
            assert np.linalg.norm(x - g[key + "_x"]) <= 1e-5 * np.linalg.norm(g[key + "_x"])
    assert np.array_equal(se.SparseOps.conjugate_gradient(fd, np.zeros(n), 100, 1e-6), g["cg_fd_zero_x"])
    offs = np.concatenate([[0], np.cumsum(g["dot_lens"])])
    for i in range(g["dot_lens"].size):
        a, b = g["dot_a"][offs[i]:offs[i + 1]], g["dot_b"][offs[i]:offs[i + 1]]
        assert abs(se.SparseOps.dot_product(a, b) - g["dot_out"][i]) <= 1e-14 * np.abs(a * b).sum()
    sn = tuple(int(v) for v in g["smooth_n"])
    for s, ref in zip(g["smooth_sigma"], g["smooth_out"]):
        np.testing.assert_allclose(se.SparseOps.smooth_gradient(g["smooth_g"], *sn, float(s)), ref,
                                   rtol=1e-12, atol=1e-13)
    H = se.SparseOps.build_hessian_approx(fd, 0.37)
    np.testing.assert_array_equal(H.row_ptr(), g["fd_row_ptr"])
    np.testing.assert_allclose(H.values(), f32(g["hess_fd_val"]), rtol=2.0 ** -23, atol=0)
    R = se.CSRMatrix().build_from_triplets(40, 30, g["hess_rand_r"], g["hess_rand_c"], g["hess_rand_v"])
    HR = se.SparseOps.build_hessian_approx(R, 0.37)
    np.testing.assert_array_equal(HR.row_ptr(), g["hess_rand_row_ptr"])
    np.testing.assert_array_equal(HR.col_ind(), g["hess_rand_col"])
    np.testing.assert_array_equal(HR.values(), f32(g["hess_rand_val"]))


@pytest.mark.parametrize("per_row", [3, 7, 14, 40, 200, 300, 600])
def test_spmv_and_cg_with_ragged_last_sweep(se, per_row):
    """Row counts that are not a multiple of the row groups in a warp (32 / G,
    G = 2..32 threads per row by mean row length), so some groups of a warp
    have no row in the last sweep: SpMV, SpMV^T and CG (whose SpMV fuses the
    FP64 <p, Ap> reduction) against dense FP64 numpy. Rows of about 200 and
    1200 entries run past the entries each lane holds (16 threads x 10, 32 x
    6) into the loop that takes the rest."""
    rng = np.random.default_rng(100 + per_row)
    n = 333 if per_row < 200 else 1001 if per_row < 600 else 1500
    k = max(per_row // 2, 1)
    r = np.repeat(np.arange(n), k)
    c = rng.integers(0, n, r.size)
    v = rng.uniform(-1.0, 1.0, r.size).astype(np.float32).astype(np.float64)
    A = np.zeros((n, n))
    np.add.at(A, (r, c), v)
    np.add.at(A, (c, r), v)
    np.fill_diagonal(A, np.abs(A).sum(axis=1) + 1.0)
    A = A.astype(np.float32).astype(np.float64)
    rr, cc = np.nonzero(A)
    m = se.CSRMatrix().build_from_triplets(n, n, rr, cc, A[rr, cc])
    x = rng.standard_normal(n)
    assert np.linalg.norm(m.spmv(x) - A @ x) <= 1e-6 * np.linalg.norm(A @ x)
    assert np.linalg.norm(m.spmv_transpose(x) - A.T @ x) <= 1e-6 * np.linalg.norm(A.T @ x)
    b = rng.standard_normal(n)
    xs = np.linalg.solve(A, b)
    for fn in (se.SparseOps.conjugate_gradient, se.SparseOps.jacobi_preconditioned_cg):
        got = fn(m, b, 1000, 1e-7)
        assert np.linalg.norm(got - xs) <= 1e-5 * np.linalg.norm(xs)
