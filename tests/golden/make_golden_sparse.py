"""Generates sparse_small.npz by running the reference's own sparse module
(sparse/csr_matrix.cpp and sparse/sparse_ops.cpp of
13262233692/03-seismic-tomography-compute, compiled by oracle/build_ref.sh from
a scratch copy that carries the three fixes listed there: an AlignedVector
copy constructor, zero-filled resize, and a large enough pad_to_alignment
allocation) on small seeded inputs.

    SEISMIC_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden_sparse.py

Contents (all FP64 reference outputs):
  fd_*      build_fd_stencil_7point on a 9x7x6 grid with a variable velocity;
            its build pads every row to a multiple of 8 entries (col = row,
            value 0), then spmv and spmv_transpose of seeded vectors
  spd_*     a seeded SPD matrix B^T B + 0.5 I (n = 200, about 30 entries per
            row) through build_from_triplets (padded as well); its
            triplets are the fixture's own unpadded CSR entries, shuffled
  cg_<m>_<j>_<t>
            conjugate_gradient (j = 0) and jacobi_preconditioned_cg (j = 1) on
            m = fd / spd at tol t = 6 (1e-6) and 10 (1e-10): the solution
            (max_iter = 10000), the iteration count (the smallest max_iter whose
            solution equals it bit for bit) and the iterates after
            max_iter = 1, 2, 3, 5, 8, 13, 21, 34 (those below the count)
  dot_*     dot_product on lengths 1, 2, 3, 4, 5, 7, 8, 1001, 2051
  smooth_*  smooth_gradient on a 13x9x11 grid at sigma 0.5, 1, 1.5, 2, 3
  hess_*    build_hessian_approx(0.37) on the fd matrix (values; the
            structure is fd_*'s), and on a random 40x30 matrix whose rows
            0, 5, 10, ... hold no diagonal entry
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from oracle import Reference, build_ref  # noqa: E402

FIB = (1, 2, 3, 5, 8, 13, 21, 34)


def cg_record(ref, b, jacobi, tol):
    x = ref.cg(b, 10000, tol, jacobi)
    k = 1
    iterates = []
    while True:
        xk = ref.cg(b, k, tol, jacobi)
        if np.array_equal(xk, x):
            break
        if k in FIB:
            iterates.append(xk)
        k += 1
        assert k < 10000
    ks = np.array([f for f in FIB if f < k], np.int64)
    return x, k, ks, np.array(iterates).reshape(len(ks), b.size)


def main():
    if build_ref() is None:
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    ref = Reference()
    rng = np.random.default_rng(4321)
    out = {}

    # -- FD stencil matrix (padded by the reference's own build)
    nx, ny, nz = 9, 7, 6
    n = nx * ny * nz
    vel = 2000.0 * (1.0 + 0.03 * rng.standard_normal(n))
    dx, dy, dz, dt = 10.0, 12.0, 9.0, 1.6e-3
    rp, col, val = ref.csr_fd_stencil(nx, ny, nz, vel, dx, dy, dz, dt)
    assert rp[-1] % 8 == 0 and rp[-1] > 7 * n  # padding fired
    x = rng.standard_normal(n)
    xt = rng.standard_normal(n)
    out.update(fd_n=np.array([nx, ny, nz]), fd_d=np.array([dx, dy, dz, dt]), fd_vel=vel, fd_row_ptr=rp,
               fd_col=col, fd_val=val, fd_x=x, fd_y=ref.csr_spmv(x, n), fd_xt=xt, fd_yt=ref.csr_spmv_t(xt, n))
    b_fd = rng.standard_normal(n)
    out["fd_b"] = b_fd
    for jac in (0, 1):
        for tol, tag in ((1e-6, 6), (1e-10, 10)):
            xs, k, ks, its = cg_record(ref, b_fd, jac, tol)
            out.update({f"cg_fd_{jac}_{tag}_x": xs, f"cg_fd_{jac}_{tag}_iters": k, f"cg_fd_{jac}_{tag}_ks": ks,
                        f"cg_fd_{jac}_{tag}_xk": its})
    out["cg_fd_zero_x"] = ref.cg(np.zeros(n), 100, 1e-6, False)

    # -- Hessian approximation of the FD matrix (rebuild it first: hessian_approx replaces it)
    ref.csr_fd_stencil(nx, ny, nz, vel, dx, dy, dz, dt)
    h_rp, h_col, h_val = ref.hessian_approx(0.37, n)
    assert np.array_equal(h_rp, rp) and np.array_equal(h_col, col)
    out.update(hess_fd_val=h_val)

    # -- random SPD matrix: B^T B + 0.5 I from triplets (duplicates merged by the build)
    m = 200
    kb = 5
    br = np.repeat(np.arange(m), kb)
    bc = rng.integers(0, m, br.size)
    bv = rng.standard_normal(br.size)
    B = np.zeros((m, m))
    np.add.at(B, (br, bc), bv)
    S = B.T @ B + 0.5 * np.eye(m)
    sr, sc = np.nonzero(S)
    sv = S[sr, sc]
    perm = rng.permutation(sr.size)
    sr, sc, sv = sr[perm].astype(np.int64), sc[perm].astype(np.int64), sv[perm]
    srp, scol, sval = ref.csr_build(m, m, sr, sc, sv)
    b_spd = rng.standard_normal(m)
    xs_ = rng.standard_normal(m)
    out.update(spd_row_ptr=srp, spd_col=scol, spd_val=sval, spd_b=b_spd,
               spd_x=xs_, spd_y=ref.csr_spmv(xs_, m))
    for jac in (0, 1):
        for tol, tag in ((1e-6, 6), (1e-10, 10)):
            xs, k, ks, its = cg_record(ref, b_spd, jac, tol)
            out.update({f"cg_spd_{jac}_{tag}_x": xs, f"cg_spd_{jac}_{tag}_iters": k, f"cg_spd_{jac}_{tag}_ks": ks,
                        f"cg_spd_{jac}_{tag}_xk": its})

    # -- Hessian approximation where some rows have no diagonal entry
    hr, hc, hv = [], [], []
    for r in range(40):
        cs = rng.choice(30, size=9, replace=False)
        if r % 4 == 1 and r < 30 and r not in cs:
            cs[0] = r
        for c in cs:
            if r % 5 == 0 and c == r:
                continue
            hr.append(r); hc.append(c); hv.append(float(rng.integers(-64, 64)) / 8.0)
    hr, hc, hv = np.array(hr, np.int64), np.array(hc, np.int64), np.array(hv)
    ref.csr_build(40, 30, hr, hc, hv)
    g_rp, g_col, g_val = ref.hessian_approx(0.37, 40)
    out.update(hess_rand_r=hr, hess_rand_c=hc, hess_rand_v=hv, hess_rand_row_ptr=g_rp, hess_rand_col=g_col,
               hess_rand_val=g_val)

    # -- dot_product on odd and short lengths
    lens = np.array([1, 2, 3, 4, 5, 7, 8, 1001, 2051], np.int64)
    da = rng.standard_normal(int(lens.sum()))
    db = rng.standard_normal(int(lens.sum()))
    offs = np.concatenate([[0], np.cumsum(lens)])
    dots = np.array([ref.dot(da[offs[i]:offs[i + 1]], db[offs[i]:offs[i + 1]]) for i in range(lens.size)])
    out.update(dot_lens=lens, dot_a=da, dot_b=db, dot_out=dots)

    # -- smooth_gradient on a non-cubic grid
    sn = np.array([13, 9, 11])
    g = rng.standard_normal(int(sn.prod()))
    sig = np.array([0.5, 1.0, 1.5, 2.0, 3.0])
    sm = np.array([ref.smooth_gradient(g, *(int(v) for v in sn), s) for s in sig])
    out.update(smooth_n=sn, smooth_g=g, smooth_sigma=sig, smooth_out=sm)

    np.savez_compressed(os.path.join(HERE, "sparse_small.npz"), **out)
    print("sparse_small.npz", os.path.getsize(os.path.join(HERE, "sparse_small.npz")))
    for key in sorted(k for k in out if k.endswith("_iters")):
        print(key, int(out[key]))


if __name__ == "__main__":
    main()
