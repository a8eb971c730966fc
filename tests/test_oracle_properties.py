"""Properties of the oracle's restated operations that the reference lacks
(the exact discrete adjoint and its gradient, the normal-equation solve) or
that do not compile as shipped (CG, PCG, smoothing)."""
import numpy as np
import pytest

from seismic_engine import workloads as wl


def small(oracle, n=(10, 9, 11), nt=40, sw=3, mode="reference"):
    w = wl.small_case(n=n, nt=nt, seed=5, sponge_width=sw)
    g = oracle.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping, sponge_mode=mode)
    return w, g


@pytest.mark.parametrize("mode", ["reference", "stable"])
def test_exact_adjoint_dot_product(oracle, mode):
    w, g = small(oracle, mode=mode)
    rng = np.random.default_rng(0)
    rec = w.shots[0].rec.coords()
    src = np.array([w.shots[0].src])
    s = rng.standard_normal((w.nt, 1))
    r = rng.standard_normal((w.nt, rec.shape[0]))
    vel = wl.to_reference_layout(w.vel)
    fwd = oracle.run(g, vel, w.nt, src, s, rec)
    adj = oracle.adjoint(g, vel, w.nt, rec, r, src_xyz=src)
    lhs = float(np.sum(fwd["seis"] * r))
    rhs = float(np.sum(s * adj["src_adj"]))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1e-300)


@pytest.mark.parametrize("mode", ["reference", "stable"])
def test_exact_adjoint_gradient_taylor(oracle, mode):
    """J(c) = 1/2 ||F(c) - d||^2; the oracle's grad_c must give second-order
    Taylor remainders along a random smooth direction."""
    w, g = small(oracle, n=(9, 8, 10), nt=30, sw=2, mode=mode)
    rng = np.random.default_rng(1)
    rec = w.shots[0].rec.coords()
    src = np.array([w.shots[0].src])
    wav = w.shots[0].wavelet[:, None]
    v0 = w.vel.copy()
    d_obs = oracle.run(g, wl.to_reference_layout(v0 * 1.03), w.nt, src, wav, rec)["seis"]

    def J(v):
        f = oracle.run(g, wl.to_reference_layout(v), w.nt, src, wav, rec, keep_states=True)
        res = f["seis"] - d_obs
        return 0.5 * float(np.sum(res * res)), f, res

    j0, f0, res0 = J(v0)
    adj = oracle.adjoint(g, wl.to_reference_layout(v0), w.nt, rec, res0, states=f0["states"], want_grad=True)
    grad_v = adj["grad_c"].reshape(v0.shape) * 2.0 * v0 * w.dt * w.dt
    dv = wl.smooth(rng.standard_normal(v0.shape), 1.5)
    dv *= 0.01 * np.abs(v0).max() / np.abs(dv).max()
    gd = float(np.sum(grad_v * dv))
    rems = []
    for k in range(4):
        h = 2.0 ** -k
        jh = J(v0 + h * dv)[0]
        rems.append(abs(jh - j0 - h * gd))
    ratios = [rems[i] / rems[i + 1] for i in range(3)]
    assert all(3.0 < q < 5.0 for q in ratios), (rems, ratios)


def test_cg_and_pcg_solve_spd_system(oracle):
    rng = np.random.default_rng(2)
    n = 60
    rows, cols, vals = [], [], []
    for i in range(n):
        for j in range(max(0, i - 2), min(n, i + 3)):
            v = 4.0 if i == j else -0.5 / (1 + abs(i - j))
            rows.append(i); cols.append(j); vals.append(v * (1 + 0.5 * (i == j) * (i % 3)))
    rp, col, val = oracle.csr_build(n, n, rows, cols, vals)
    m = oracle.csr(n, n, rp, col, val)
    A = np.zeros((n, n))
    for i in range(n):
        A[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    b = rng.standard_normal(n)
    xs = np.linalg.solve(A, b)
    for jac in (False, True):
        x, it, rel = oracle.cg(m, b, 500, 1e-12, jacobi=jac)
        assert rel < 1e-12 and it > 0
        np.testing.assert_allclose(x, xs, rtol=1e-9, atol=1e-10)


def test_cg_breaks_on_zero_rhs(oracle):
    rp, col, val = oracle.csr_build(3, 3, [0, 1, 2], [0, 1, 2], [1.0, 2.0, 3.0])
    m = oracle.csr(3, 3, rp, col, val)
    x, it, rel = oracle.cg(m, np.zeros(3), 10, 1e-8)
    assert it == 0 and not x.any()


def test_normal_equation_cg(oracle):
    rng = np.random.default_rng(3)
    rows, cols = 80, 30
    r = np.repeat(np.arange(rows), 6)
    c = rng.integers(0, cols, r.size)
    v = rng.random(r.size)
    rp, col, val = oracle.csr_build(rows, cols, r, c, v)
    m = oracle.csr(rows, cols, rp, col, val)
    d = rng.standard_normal(rows)
    lam = 1e-2
    x, it, rel, rhs = oracle.normal_cg(m, d, lam, 500, 1e-10, jacobi=True)
    A = np.zeros((rows, cols))
    for i in range(rows):
        np.add.at(A[i], col[rp[i]:rp[i + 1]], val[rp[i]:rp[i + 1]])
    xs = np.linalg.solve(A.T @ A + lam * np.eye(cols), A.T @ d)
    np.testing.assert_allclose(rhs, A.T @ d, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(x, xs, rtol=1e-7, atol=1e-8)
    np.testing.assert_allclose(oracle.normal_apply(m, lam, x), rhs, rtol=1e-8, atol=1e-8)


def test_smoothing_is_separable_and_normalised(oracle):
    rng = np.random.default_rng(4)
    nx, ny, nz, sigma = 7, 6, 8, 1.0
    g = rng.standard_normal(nx * ny * nz)
    out = oracle.smooth_gradient(g, nx, ny, nz, sigma)
    # separable restatement: per-axis truncated weights, per-point in-bounds normalisation
    rad = int(3 * sigma)
    G = g.reshape(nx, ny, nz)
    for ax, n in enumerate((nx, ny, nz)):
        W = np.zeros((n, n))
        for i in range(n):
            for j in range(max(0, i - rad), min(n, i + rad + 1)):
                W[i, j] = np.exp(-((i - j) ** 2) / (2 * sigma * sigma))
        W /= W.sum(1, keepdims=True)
        G = np.moveaxis(np.tensordot(W, np.moveaxis(G, ax, 0), axes=(1, 0)), 0, ax)
    np.testing.assert_allclose(out, G.ravel(), rtol=1e-12, atol=1e-12)
    const = oracle.smooth_gradient(np.full(nx * ny * nz, 3.5), nx, ny, nz, sigma)
    np.testing.assert_allclose(const, 3.5, rtol=1e-14)
    assert not oracle.smooth_gradient(np.ones(5), nx, ny, nz, sigma).any()


def test_fp32_floor_against_fp64(oracle):
    """The same arithmetic in FP32: states how far an FP32 implementation can
    sit from FP64 on the small case (the GPU tolerances build on this)."""
    w, g = small(oracle, n=(20, 18, 22), nt=120, sw=5)
    rec = w.shots[0].rec.coords()
    src = np.array([w.shots[0].src])
    vel = wl.to_reference_layout(w.vel)
    a = oracle.run(g, vel, w.nt, src, w.shots[0].wavelet[:, None], rec)
    b = oracle.run(g, vel, w.nt, src, w.shots[0].wavelet[:, None], rec, fp32=True)
    rel = np.linalg.norm(b["seis"] - a["seis"]) / np.linalg.norm(a["seis"])
    assert rel < 1e-5


def blob_run(oracle, mode, nt, n=40, sw=20):
    v = np.full((n, n, n), 3000.0)
    g = oracle.grid(n, n, n, 10.0, 10.0, 10.0, 0.001, sw, 0.015, sponge_mode=mode)
    x = np.arange(n + 2) - (n + 1) / 2
    blob = np.exp(-(x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2) / 8.0).reshape(-1)
    r = oracle.run(g, wl.to_reference_layout(v), nt, np.zeros((0, 3), np.int64), np.zeros((nt, 0)),
                   np.zeros((0, 3), np.int64), init_cur=blob, init_prev=blob)
    return float(np.abs(r["cur"]).max())


def test_reference_sponge_diverges_and_stable_sponge_decays(oracle):
    """The reference's sponge rule (damp current and previous after the update)
    amplifies smooth modes in a wide sponge: with the default 20 cells and
    0.015 a unit blob grows past 1e3 within 300 steps, no source involved. The
    stable (Cerjan) form decays."""
    assert blob_run(oracle, "reference", 300) > 1e3
    assert blob_run(oracle, "stable", 300) < 0.1
