/*
 * CPU oracle: a plain-C restatement of the reference's hot path
 * (13262233692/03-seismic-tomography-compute, src/cpp) plus FP64 restatements
 * of the operations the reference lacks (the exact discrete adjoint, the
 * normal-equation operator A^T A + lambda I). Every function cites the
 * reference code it follows.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU
 * legs of bench.py load this library, and only as the checker or the timed CPU
 * baseline. The product (the CUDA library) never links or calls it.
 *
 * Pinning: the propagator, RTM imaging, CSR build (with and without the
 * padding rule), SpMV / SpMV^T, the CG / Jacobi-PCG loops, dot_product and
 * the Gaussian smoothing here are checked against the reference's own C++
 * (built by oracle/build_ref.sh; sparse/ from a scratch copy with the three
 * minimal fixes listed there) through the committed fixtures in tests/golden/
 * (tests/golden/make_golden.py, make_golden_sparse.py) in
 * tests/test_oracle_golden.py. The exact adjoint and the normal-equation
 * operator have no reference counterpart: they are pinned by properties
 * (dot-product and Taylor tests).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t nx, ny, nz;   /* interior extents (halo width 1) */
    double dx, dy, dz, dt;
    int sponge_width;
    double sponge_damping;
    double amp_limit;     /* WaveEquationSolver amplitude_limit_, default 1e10 */
    double cfl_safety;    /* FaultTolerance cfl_safety_factor_, default 0.49 */
    int sponge_mode;      /* 0: the reference rule (damp current and previous after the update);
                             1: stable Cerjan form (damp the new field and the current) - not in the reference */
} orc_grid;

#define REAL double
#define SFX 64
#include "oracle_prop.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX 32
#include "oracle_prop.h"
#undef REAL
#undef SFX

static double vfix(double v) { return (isfinite(v) && v > 0.0) ? v : 1500.0; }

/* Effective update coefficient c = v^2 dt^2 (times the CFL damping factor^2
 * when the reference would apply it), wave_equation.cpp:316-387. */
static void coeff_c(const orc_grid* g, const double* vel, double* c) {
    const int64_t n = (g->nx + 2) * (g->ny + 2) * (g->nz + 2);
    const double vmax = orc64_vmax(g, vel);
    double cfl = vmax * g->dt / g->dx;
    if (vmax * g->dt / g->dy > cfl) cfl = vmax * g->dt / g->dy;
    if (vmax * g->dt / g->dz > cfl) cfl = vmax * g->dt / g->dz;
    double damp2 = 1.0;
    if (cfl > 1.0) {
        double dmin = fmin(g->dx, fmin(g->dy, g->dz));
        double f = fmin(1.0, g->cfl_safety / (vmax * g->dt / dmin));
        damp2 = f * f;
    }
    for (int64_t i = 0; i < n; ++i) {
        double v = vfix(vel[i]);
        c[i] = v * v * g->dt * g->dt * damp2;
    }
}

/*
 * Exact discrete adjoint (transpose) of the linear forward recursion that
 * orc64_run implements when no guard fires:
 *     V_t = cur after the injection of step t
 *     next_t = 2 V_t - D V_{t-1} + c * L V_t,   d_t = R next_t,
 * with L the 7-point Laplacian of fd_7point_operator_safe (zero halo) and D
 * the sponge of apply_sponge_layer applied to the previous field
 * (wave_equation.cpp:57-62,262-297,370-389). The reference has no such
 * operator (its step_adjoint is step_forward, :78-98). Backward in t:
 *     lam_t  = a_C + R^T r_t                      (adjoint of next_t)
 *     a_C'   = a_P + 2 lam_t + L(c * lam_t)       (adjoint of V_t)
 *     a_P'   = -D lam_t
 * Outputs (each optional):
 *   src_adj[t*n_src+s] = a_C'[src_s]   (= dJ/ds_t for J = <F s, r>)
 *   image  += V_t * lam_t,  illum += V_t^2   over the interior, with the
 *     finite-value guards of RTMEngine::apply_image_condition
 *     (rtm/rtm_engine.cpp:24-57), given the forward states V_t;
 *   grad_c += lam_t * L V_t   (interior; dJ/dc, c = v^2 dt^2).
 */
int orc64_adjoint(const orc_grid* g, const double* vel, int nt, int nrec, const int64_t* rec_xyz,
                  const double* resid, int n_src, const int64_t* src_xyz, double* src_adj,
                  const double* states, double* image, double* illum, double* grad_c) {
    const int64_t NXh = g->nx + 2, NYh = g->ny + 2, NZh = g->nz + 2, P = NYh * NZh, n = NXh * P;
    const double idx2 = 1.0 / (g->dx * g->dx), idy2 = 1.0 / (g->dy * g->dy), idz2 = 1.0 / (g->dz * g->dz);
    double* c = (double*)malloc((size_t)n * sizeof(double));
    double* D = (double*)malloc((size_t)n * sizeof(double));
    double* aC = (double*)calloc((size_t)n, sizeof(double));
    double* aP = (double*)calloc((size_t)n, sizeof(double));
    double* cl = (double*)calloc((size_t)n, sizeof(double));
    double* nC = (double*)calloc((size_t)n, sizeof(double));
    if (!c || !D || !aC || !aP || !cl || !nC) {
        free(c); free(D); free(aC); free(aP); free(cl); free(nC);
        return -3;
    }
    coeff_c(g, vel, c);
    for (int64_t ix = 0; ix < NXh; ++ix)
        for (int64_t iy = 0; iy < NYh; ++iy)
            for (int64_t iz = 0; iz < NZh; ++iz) D[(ix * NYh + iy) * NZh + iz] = orc64_sponge(g, ix, iy, iz);
    for (int t = nt - 1; t >= 0; --t) {
        for (int q = 0; q < nrec; ++q) {
            const int64_t i = (rec_xyz[3 * q] + 1) * P + (rec_xyz[3 * q + 1] + 1) * NZh + (rec_xyz[3 * q + 2] + 1);
            aC[i] += resid[(int64_t)t * nrec + q];
        }
        if (states && (image || illum || grad_c)) {
            const double* V = states + (int64_t)t * n;
#pragma omp parallel for collapse(2) schedule(static)
            for (int64_t ix = 1; ix <= g->nx; ++ix)
                for (int64_t iy = 1; iy <= g->ny; ++iy)
                    for (int64_t iz = 1; iz <= g->nz; ++iz) {
                        const int64_t k = ((ix - 1) * g->ny + (iy - 1)) * g->nz + (iz - 1);
                        const int64_t i = ix * P + iy * NZh + iz;
                        double f = isfinite(V[i]) ? V[i] : 0.0;
                        double a = isfinite(aC[i]) ? aC[i] : 0.0;
                        if (image) image[k] += f * a;
                        if (illum) illum[k] += f * f;
                        if (grad_c) {
                            double lap = (V[i + P] - 2.0 * V[i] + V[i - P]) * idx2 +
                                         (V[i + NZh] - 2.0 * V[i] + V[i - NZh]) * idy2 +
                                         (V[i + 1] - 2.0 * V[i] + V[i - 1]) * idz2;
                            grad_c[k] += (g->sponge_mode == 1 ? D[i] * aC[i] : aC[i]) * lap;
                        }
                    }
        }
        /* reference rule: (C, P) -> (2C - P + cLC, D C); transpose:
         *   aC <- 2 aC' + L(c aC') + D aP',  aP <- -aC'.
         * stable rule: (C, P) -> (D (2C - P + cLC), D C); with b = D aC':
         *   aC <- 2 b + L(c b) + D aP',  aP <- -b.
         * aP is kept premultiplied by D. */
        if (g->sponge_mode == 1) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) aC[i] *= D[i];
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            cl[i] = c[i] * aC[i];
            nC[i] = 0.0;
        }
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t ix = 1; ix <= g->nx; ++ix)
            for (int64_t iy = 1; iy <= g->ny; ++iy)
                for (int64_t iz = 1; iz <= g->nz; ++iz) {
                    const int64_t i = ix * P + iy * NZh + iz;
                    /* halo cells of cl are c*0 = 0: the Dirichlet ring */
                    double lap = (cl[i + P] - 2.0 * cl[i] + cl[i - P]) * idx2 +
                                 (cl[i + NZh] - 2.0 * cl[i] + cl[i - NZh]) * idy2 +
                                 (cl[i + 1] - 2.0 * cl[i] + cl[i - 1]) * idz2;
                    nC[i] = aP[i] + 2.0 * aC[i] + lap;
                }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) aP[i] = -D[i] * aC[i];
        double* tmp = aC;
        aC = nC;
        nC = tmp;
        if (src_adj)
            for (int s = 0; s < n_src; ++s) {
                const int64_t i = (src_xyz[3 * s] + 1) * P + (src_xyz[3 * s + 1] + 1) * NZh + (src_xyz[3 * s + 2] + 1);
                src_adj[(int64_t)t * n_src + s] = aC[i];
            }
    }
    free(c); free(D); free(aC); free(aP); free(cl); free(nC);
    return 0;
}

/* RTMEngine::apply_image_condition over nsteps pairs of padded fields, then
 * finalize_image (rtm/rtm_engine.cpp:24-57,170-182). */
int orc64_rtm_image(int64_t nx, int64_t ny, int64_t nz, int nsteps, const double* fwd, const double* adj,
                    double* image, double* illum, double* refl) {
    const int64_t NZh = nz + 2, P = (ny + 2) * NZh, np = (nx + 2) * P, n = nx * ny * nz;
    memset(image, 0, (size_t)n * sizeof(double));
    memset(illum, 0, (size_t)n * sizeof(double));
    for (int t = 0; t < nsteps; ++t) {
        const double* F = fwd + (int64_t)t * np;
        const double* A = adj + (int64_t)t * np;
        int64_t k = 0;
        for (int64_t ix = 0; ix < nx; ++ix)
            for (int64_t iy = 0; iy < ny; ++iy)
                for (int64_t iz = 0; iz < nz; ++iz, ++k) {
                    const int64_t i = (ix + 1) * P + (iy + 1) * NZh + iz + 1;
                    double f = isfinite(F[i]) ? F[i] : 0.0;
                    double a = isfinite(A[i]) ? A[i] : 0.0;
                    image[k] += f * a;
                    illum[k] += f * f;
                }
    }
    for (int64_t k = 0; k < n; ++k) refl[k] = illum[k] > 1e-10 ? image[k] / illum[k] : 0.0;
    return 0;
}

/* ---------------------------------------------------------------- sparse */

typedef struct {
    int64_t rows, cols, nnz;
    int64_t* row_ptr;
    int64_t* col;
    double* val;
} orc_csr;

typedef struct {
    int64_t col, order;
    double val;
} orc_ent;

static int ent_cmp(const void* a, const void* b) {
    const orc_ent* x = (const orc_ent*)a;
    const orc_ent* y = (const orc_ent*)b;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return x->order < y->order ? -1 : (x->order > y->order);
}

/*
 * CSRMatrix::build_from_triplets (sparse/csr_matrix.cpp:25-72): drop entries
 * outside [0,rows)x[0,cols) (:33), sort each row by column (:39-40), merge
 * equal columns by summing in sorted order (:42-50), prefix-sum row_ptr
 * (:62-69). Ties between equal (row,col) keep input order (the reference's
 * std::sort leaves their order unspecified; sums of exactly representable
 * duplicates do not depend on it). pad != 0 applies pad_to_alignment
 * (:223-264) with its allocation fixed: it fires at the first row i with
 * roundup8(row_ptr[i]) > row_ptr[i+1] and then pads every row to a multiple
 * of 8 entries with col = row, value 0. Returns NULL on allocation failure.
 */
orc_csr* orc_csr_build(int64_t rows, int64_t cols, int64_t n, const int64_t* r, const int64_t* c, const double* v,
                       int pad) {
    orc_csr* m = (orc_csr*)calloc(1, sizeof(orc_csr));
    int64_t* cnt = (int64_t*)calloc((size_t)rows + 1, sizeof(int64_t));
    if (!m || !cnt) { free(m); free(cnt); return NULL; }
    m->rows = rows;
    m->cols = cols;
    for (int64_t i = 0; i < n; ++i)
        if (r[i] >= 0 && r[i] < rows && c[i] >= 0 && c[i] < cols) cnt[r[i] + 1]++;
    for (int64_t i = 0; i < rows; ++i) cnt[i + 1] += cnt[i];
    orc_ent* e = (orc_ent*)malloc((size_t)(cnt[rows] > 0 ? cnt[rows] : 1) * sizeof(orc_ent));
    int64_t* pos = (int64_t*)malloc((size_t)(rows > 0 ? rows : 1) * sizeof(int64_t));
    if (!e || !pos) { free(m); free(cnt); free(e); free(pos); return NULL; }
    memcpy(pos, cnt, (size_t)rows * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i)
        if (r[i] >= 0 && r[i] < rows && c[i] >= 0 && c[i] < cols) {
            orc_ent* d = &e[pos[r[i]]++];
            d->col = c[i];
            d->order = i;
            d->val = v[i];
        }
    /* sort + merge each row in place; uniq[i] = merged count of row i */
    int64_t* rp = (int64_t*)calloc((size_t)rows + 1, sizeof(int64_t));
    if (!rp) { free(m); free(cnt); free(e); free(pos); return NULL; }
    for (int64_t i = 0; i < rows; ++i) {
        orc_ent* s = e + cnt[i];
        int64_t len = cnt[i + 1] - cnt[i], u = 0;
        qsort(s, (size_t)len, sizeof(orc_ent), ent_cmp);
        for (int64_t j = 0; j < len; ++j) {
            if (u > 0 && s[u - 1].col == s[j].col) s[u - 1].val += s[j].val;
            else s[u++] = s[j];
        }
        rp[i + 1] = rp[i] + u;
    }
    int do_pad = 0;
    if (pad)
        for (int64_t i = 0; i < rows; ++i)
            if (((rp[i] + 7) / 8) * 8 > rp[i + 1]) { do_pad = 1; break; }
    int64_t total = 0;
    for (int64_t i = 0; i < rows; ++i) {
        int64_t len = rp[i + 1] - rp[i];
        total += do_pad ? ((len + 7) / 8) * 8 : len;
    }
    m->row_ptr = (int64_t*)malloc(((size_t)rows + 1) * sizeof(int64_t));
    m->col = (int64_t*)malloc((size_t)(total > 0 ? total : 1) * sizeof(int64_t));
    m->val = (double*)malloc((size_t)(total > 0 ? total : 1) * sizeof(double));
    if (!m->row_ptr || !m->col || !m->val) {
        free(m->row_ptr); free(m->col); free(m->val); free(m); free(cnt); free(e); free(pos); free(rp);
        return NULL;
    }
    int64_t off = 0;
    m->row_ptr[0] = 0;
    for (int64_t i = 0; i < rows; ++i) {
        int64_t len = rp[i + 1] - rp[i];
        const orc_ent* s = e + cnt[i];
        for (int64_t j = 0; j < len; ++j) {
            m->col[off + j] = s[j].col;
            m->val[off + j] = s[j].val;
        }
        int64_t plen = do_pad ? ((len + 7) / 8) * 8 : len;
        for (int64_t j = len; j < plen; ++j) {
            m->col[off + j] = i;
            m->val[off + j] = 0.0;
        }
        off += plen;
        m->row_ptr[i + 1] = off;
    }
    m->nnz = off;
    free(cnt); free(e); free(pos); free(rp);
    return m;
}

void orc_csr_free(orc_csr* m) {
    if (!m) return;
    free(m->row_ptr); free(m->col); free(m->val); free(m);
}
int64_t orc_csr_nnz(const orc_csr* m) { return m->nnz; }
void orc_csr_copy(const orc_csr* m, int64_t* row_ptr, int64_t* col, double* val) {
    memcpy(row_ptr, m->row_ptr, ((size_t)m->rows + 1) * sizeof(int64_t));
    memcpy(col, m->col, (size_t)m->nnz * sizeof(int64_t));
    memcpy(val, m->val, (size_t)m->nnz * sizeof(double));
}

/* Wrap caller-owned CSR arrays (no copy) so the solvers below can run on a
 * matrix held elsewhere (e.g. the fixtures). */
orc_csr* orc_csr_wrap(int64_t rows, int64_t cols, int64_t* row_ptr, int64_t* col, double* val) {
    orc_csr* m = (orc_csr*)calloc(1, sizeof(orc_csr));
    if (!m) return NULL;
    m->rows = rows; m->cols = cols; m->nnz = row_ptr[rows];
    m->row_ptr = row_ptr; m->col = col; m->val = val;
    return m;
}
void orc_csr_unwrap(orc_csr* m) { free(m); }

/* CSRMatrix::spmv (csr_matrix.cpp:118-149): two interleaved partial sums per
 * row (even / odd positions), y = sum0 + sum1. Rows run in parallel when the
 * library is built with OpenMP; each row's arithmetic is unchanged. */
void orc_spmv(const orc_csr* m, const double* x, double* y) {
    const int64_t rows = m->rows;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < rows; ++i) {
        double s0 = 0.0, s1 = 0.0;
        int64_t p = m->row_ptr[i];
        const int64_t e = m->row_ptr[i + 1];
        for (; p + 1 < e; p += 2) {
            s0 += m->val[p] * x[m->col[p]];
            s1 += m->val[p + 1] * x[m->col[p + 1]];
        }
        for (; p < e; ++p) s0 += m->val[p] * x[m->col[p]];
        y[i] = s0 + s1;
    }
}

/* CSRMatrix::spmv_transpose (csr_matrix.cpp:151-166) with the accumulator
 * zeroed (the shipped AlignedVector(n, 0.0) leaves it uninitialised,
 * aligned_alloc.h:71-75): y[col] += val * x[row] in row order. */
void orc_spmv_t(const orc_csr* m, const double* x, double* y) {
    memset(y, 0, (size_t)m->cols * sizeof(double));
    for (int64_t i = 0; i < m->rows; ++i)
        for (int64_t p = m->row_ptr[i]; p < m->row_ptr[i + 1]; ++p) y[m->col[p]] += m->val[p] * x[i];
}

/* SparseOps::dot_product (sparse_ops.cpp:172-187): 4-way unrolled serial sum. */
double orc_dot(const double* a, const double* b, int64_t n) {
    double sum = 0.0;
    int64_t i = 0;
    for (; i + 3 < n; i += 4) sum += a[i] * b[i] + a[i + 1] * b[i + 1] + a[i + 2] * b[i + 2] + a[i + 3] * b[i + 3];
    for (; i < n; ++i) sum += a[i] * b[i];
    return sum;
}

/* Operator used by the Krylov loops: y = A x (square) or y = A^T(A x) + lam x
 * (normal equations of a rectangular A, the tomography system). */
typedef struct {
    const orc_csr* A;
    int normal;
    double lam;
    double* tmp;
} orc_op;

static void op_apply(const orc_op* op, const double* x, double* y) {
    if (!op->normal) {
        orc_spmv(op->A, x, y);
        return;
    }
    orc_spmv(op->A, x, op->tmp);
    orc_spmv_t(op->A, op->tmp, y);
    for (int64_t i = 0; i < op->A->cols; ++i) y[i] += op->lam * x[i];
}

/*
 * SparseOps::conjugate_gradient (sparse_ops.cpp:8-50) with x0 = 0 as intended
 * (the shipped AlignedVector leaves x uninitialised) when diag_inv == NULL,
 * SparseOps::jacobi_preconditioned_cg (:52-113) when diag_inv != NULL. Same
 * break rules: return x0 if ||b|| < 1e-30; stop if |pAp| < 1e-30; stop after
 * the update when sqrt(rr)/||b|| < tol. Returns the iterations performed.
 */
static int krylov(const orc_op* op, int64_t n, const double* b, int max_iter, double tol, const double* diag_inv,
                  double* x, double* final_rel) {
    double* r = (double*)malloc((size_t)n * sizeof(double));
    double* z = (double*)malloc((size_t)n * sizeof(double));
    double* p = (double*)malloc((size_t)n * sizeof(double));
    double* Ap = (double*)malloc((size_t)n * sizeof(double));
    memset(x, 0, (size_t)n * sizeof(double));
    memcpy(r, b, (size_t)n * sizeof(double));
    for (int64_t i = 0; i < n; ++i) z[i] = diag_inv ? diag_inv[i] * r[i] : r[i];
    memcpy(p, z, (size_t)n * sizeof(double));
    double rz_old = orc_dot(r, z, n);
    const double b_norm = sqrt(orc_dot(b, b, n));
    int it = 0;
    double rel = 1.0;
    if (b_norm < 1e-30) {
        free(r); free(z); free(p); free(Ap);
        if (final_rel) *final_rel = 0.0;
        return 0;
    }
    for (int iter = 0; iter < max_iter; ++iter) {
        op_apply(op, p, Ap);
        const double pAp = orc_dot(p, Ap, n);
        if (fabs(pAp) < 1e-30) break;
        const double alpha = rz_old / pAp;
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * Ap[i];
        }
        ++it;
        const double rr = orc_dot(r, r, n);
        rel = sqrt(rr) / b_norm;
        if (rel < tol) break;
        for (int64_t i = 0; i < n; ++i) z[i] = diag_inv ? diag_inv[i] * r[i] : r[i];
        const double rz_new = diag_inv ? orc_dot(r, z, n) : rr;
        const double beta = rz_new / rz_old;
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz_old = rz_new;
    }
    if (final_rel) *final_rel = rel;
    free(r); free(z); free(p); free(Ap);
    return it;
}

/* Jacobi diagonal of sparse_ops.cpp:60-73: 1/A_ii from the first entry with
 * col == row when |A_ii| > 1e-30, otherwise 1. */
void orc_jacobi_diag_inv(const orc_csr* A, double* diag_inv) {
    for (int64_t i = 0; i < A->rows; ++i) {
        diag_inv[i] = 1.0;
        for (int64_t p = A->row_ptr[i]; p < A->row_ptr[i + 1]; ++p)
            if (A->col[p] == i) {
                if (fabs(A->val[p]) > 1e-30) diag_inv[i] = 1.0 / A->val[p];
                break;
            }
    }
}

int orc_cg(const orc_csr* A, const double* b, int max_iter, double tol, int jacobi, double* x, double* final_rel) {
    orc_op op = {A, 0, 0.0, NULL};
    double* d = NULL;
    if (jacobi) {
        d = (double*)malloc((size_t)A->rows * sizeof(double));
        orc_jacobi_diag_inv(A, d);
    }
    int it = krylov(&op, A->rows, b, max_iter, tol, d, x, final_rel);
    free(d);
    return it;
}

/* Damped normal equations of the tomography system (no reference counterpart;
 * build_hessian_approx, sparse_ops.cpp:204-210, only adds lambda to existing
 * diagonal entries): (A^T A + lam I) x = A^T d, Jacobi-preconditioned by
 * diag = column sums of A^2 + lam when jacobi != 0. rhs = A^T d on return. */
int orc_normal_cg(const orc_csr* A, const double* d, double lam, int max_iter, double tol, int jacobi, double* x,
                  double* rhs, double* final_rel) {
    const int64_t n = A->cols;
    orc_op op = {A, 1, lam, (double*)malloc((size_t)A->rows * sizeof(double))};
    orc_spmv_t(A, d, rhs);
    double* dinv = NULL;
    if (jacobi) {
        dinv = (double*)calloc((size_t)n, sizeof(double));
        for (int64_t i = 0; i < A->rows; ++i)
            for (int64_t p = A->row_ptr[i]; p < A->row_ptr[i + 1]; ++p) dinv[A->col[p]] += A->val[p] * A->val[p];
        for (int64_t j = 0; j < n; ++j) dinv[j] = 1.0 / (dinv[j] + lam);
    }
    int it = krylov(&op, n, rhs, max_iter, tol, dinv, x, final_rel);
    free(dinv);
    free(op.tmp);
    return it;
}

/* y = (A^T A + lam I) x, for residual checks. */
void orc_normal_apply(const orc_csr* A, double lam, const double* x, double* y) {
    orc_op op = {A, 1, lam, (double*)malloc((size_t)A->rows * sizeof(double))};
    op_apply(&op, x, y);
    free(op.tmp);
}

/* SparseOps::smooth_gradient (sparse_ops.cpp:115-158): truncated Gaussian of
 * radius floor(3 sigma), normalised per point by the in-bounds weight sum. */
void orc_smooth_gradient(const double* g, int64_t nx, int64_t ny, int64_t nz, double sigma, double* out) {
    const int64_t radius = (int64_t)(3 * sigma);
    for (int64_t ix = 0; ix < nx; ++ix)
        for (int64_t iy = 0; iy < ny; ++iy)
            for (int64_t iz = 0; iz < nz; ++iz) {
                double sum = 0.0, wsum = 0.0;
                for (int64_t a = -radius; a <= radius; ++a)
                    for (int64_t b = -radius; b <= radius; ++b)
                        for (int64_t c = -radius; c <= radius; ++c) {
                            const int64_t jx = ix + a, jy = iy + b, jz = iz + c;
                            if (jx >= 0 && jx < nx && jy >= 0 && jy < ny && jz >= 0 && jz < nz) {
                                double w = exp(-(double)(a * a + b * b + c * c) / (2.0 * sigma * sigma));
                                sum += w * g[(jx * ny + jy) * nz + jz];
                                wsum += w;
                            }
                        }
                out[(ix * ny + iy) * nz + iz] = sum / wsum;
            }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* FaultTolerance::repair_field_nan / clamp_field / count_nan_inf
 * (core/fault_tolerance.cpp:72-157), exported for the fixture checks. */
int64_t orc64_repair_field_nan(double* d, int64_t count, int64_t nx, int64_t ny, int64_t nz, int hw, double repl) {
    return orc64_repair_nan(d, count, nx, ny, nz, hw, repl);
}
void orc64_clamp_field(double* d, int64_t count, double lo, double hi) {
    for (int64_t i = 0; i < count; ++i) d[i] = orc64_safe_clamp(d[i], lo, hi);
}
int64_t orc64_count_nan_inf(const double* d, int64_t count) {
    int64_t n = 0;
    for (int64_t i = 0; i < count; ++i) n += !isfinite(d[i]);
    return n;
}

/* ------------------------------------------------------------ ray matrix */
/* Straight-ray path lengths by exact voxel traversal (Amanatides & Woo 1987),
 * restated from the algorithm, not from the reference: the reference's
 * Python inversion (seismic_tomography/inversion.py:329-433) samples the same
 * straight rays at n = max(floor(dist / (5 dx)), 2) midpoints instead. The ray
 * p(t) = p0 + t (p1 - p0), t in [0, 1], is cut at the cell faces in order of
 * t, ties to x, then y, then z; segment length = (t_exit - t) * |p1 - p0| * h.
 * FP64, evaluated in source order (this file is built with
 * -ffp-contract=off), so the GPU path can match it bit for bit. Emits
 * (row, col, value) triplets; returns their count, or -1 when cap is too
 * small. Parity of this restatement is against the traversal definition, not
 * against reference output (the reference has no such builder). */
static double orc_t_exit(int c, int step, double p0, double d) {
    if (step == 0) return 1e300;
    const double face = (double)(step > 0 ? c + 1 : c);
    return (face - p0) / d;
}

int64_t orc_ray_triplets(int64_t nrays, const double* ends, int nx, int ny, int nz, double h, int64_t cap,
                         int64_t* rows, int64_t* cols, double* vals) {
    int64_t k = 0;
    const int n[3] = {nx, ny, nz};
    for (int64_t i = 0; i < nrays; ++i) {
        const double* e = ends + 6 * i;
        const double p0[3] = {e[0], e[1], e[2]};
        const double d[3] = {e[3] - e[0], e[4] - e[1], e[5] - e[2]};
        const double len = sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
        int c[3], step[3];
        double tm[3];
        for (int a = 0; a < 3; ++a) {
            int f = (int)floor(p0[a]);
            c[a] = f < 0 ? 0 : (f > n[a] - 1 ? n[a] - 1 : f);
            step[a] = d[a] > 0.0 ? 1 : (d[a] < 0.0 ? -1 : 0);
            tm[a] = orc_t_exit(c[a], step[a], p0[a], d[a]);
        }
        double t = 0.0;
        const int max_iter = nx + ny + nz + 3;
        for (int it = 0; it < max_iter; ++it) {
            const int ax = (tm[0] <= tm[1] && tm[0] <= tm[2]) ? 0 : (tm[1] <= tm[2] ? 1 : 2);
            const double tn = tm[ax];
            const double te = tn < 1.0 ? tn : 1.0;
            const double seg = ((te - t) * len) * h;
            if (seg > 0.0) {
                if (k >= cap) return -1;
                rows[k] = i;
                cols[k] = ((int64_t)c[0] * ny + c[1]) * nz + c[2];
                vals[k] = seg;
                ++k;
            }
            if (tn >= 1.0) break;
            t = tn;
            c[ax] += step[ax];
            if (c[ax] < 0 || c[ax] >= n[ax]) break;
            tm[ax] = orc_t_exit(c[ax], step[ax], p0[ax], d[ax]);
        }
    }
    return k;
}

/* ------------------------------------------------------- sampled rays */
/* Straight-ray traveltimes and their gradient as the reference's Python
 * inversion driver computes them (seismic_tomography/inversion.py:329-433):
 * the source and the station are snapped to cells (int((p - origin) / d),
 * clamped to the grid; :344-350); the ray is sampled at
 * n = max(int(dist / (5 dx)), 2) midpoints frac = (k + 0.5) / n, cell
 * c = int(c_src + frac * (c_sta - c_src)) per axis (:355-364), each sample
 * of length ds = dist / n. Forward (:329-381): t = sum ds / v in sample
 * order, an invalid velocity (non-finite or <= 0) read as 1500, a
 * non-finite term skipped, a non-finite or negative total replaced by
 * dist / 6000. Gradient (:383-433): g[cell] += (r * (-ds / (v * v))) * w in
 * pick, then sample order, picks with a non-finite residual and samples at
 * an invalid velocity skipped. Picks with valid[i] == 0 (unknown source or
 * station) get time 0 and no gradient. vp is (nx, ny, nz) C order, cell
 * (ix, iy, iz) -> (ix * ny + iy) * nz + iz. FP64 in source order (no
 * contractions). The reference's distance squares Python floats with
 * x ** 2 (libm pow), which can round one unit in the last place away from
 * the correctly rounded x * x used here; given the reference's distances
 * (dist != NULL) the results are the reference's bit for bit. */
static int64_t orc_snap(double p, double o, double d, int64_t n) {
    const double q = (p - o) / d;
    if (q < 1.0) return 0;
    if (q >= (double)(n - 1)) return n - 1;
    return (int64_t)q;
}

typedef struct {
    int64_t c0[3], c1[3];
    int64_t n_steps;
    double dist, ds;
} orc_pick_geo;

static orc_pick_geo orc_pick(const int64_t n[3], const double d[3], const double o[3], const double* s,
                             const double* r, const double* dist) {
    orc_pick_geo g;
    const double ex = s[0] - r[0], ey = s[1] - r[1], ez = s[2] - r[2];
    g.dist = dist ? *dist : sqrt((ex * ex + ey * ey) + ez * ez);
    for (int a = 0; a < 3; ++a) {
        g.c0[a] = orc_snap(s[a], o[a], d[a], n[a]);
        g.c1[a] = orc_snap(r[a], o[a], d[a], n[a]);
    }
    const double q = g.dist / (d[0] * 5.0);
    g.n_steps = q < 3.0 ? 2 : (int64_t)q;
    g.ds = g.dist / (double)g.n_steps;
    return g;
}

static int64_t orc_sample_cell(const orc_pick_geo* g, const int64_t n[3], int64_t k) {
    const double frac = ((double)k + 0.5) / (double)g->n_steps;
    int64_t c[3];
    for (int a = 0; a < 3; ++a) {
        int64_t v = (int64_t)((double)g->c0[a] + frac * (double)(g->c1[a] - g->c0[a]));
        c[a] = v < 0 ? 0 : (v > n[a] - 1 ? n[a] - 1 : v);
    }
    return (c[0] * n[1] + c[1]) * n[2] + c[2];
}

void orc_sampled_traveltimes(const int64_t n[3], const double d[3], const double o[3], int64_t n_picks,
                             const double* src, const double* sta, const double* dist, const uint8_t* valid,
                             const double* vp, double* times) {
    for (int64_t i = 0; i < n_picks; ++i) {
        times[i] = 0.0;
        if (valid && !valid[i]) continue;
        const orc_pick_geo g = orc_pick(n, d, o, src + 3 * i, sta + 3 * i, dist ? dist + i : NULL);
        double t = 0.0;
        for (int64_t k = 0; k < g.n_steps; ++k) {
            double v = vp[orc_sample_cell(&g, n, k)];
            if (!isfinite(v) || v <= 0.0) v = 1500.0;
            const double term = g.ds / v;
            if (!isfinite(term)) continue;
            t += term;
        }
        if (!isfinite(t) || t < 0.0) t = g.dist / 6000.0;
        times[i] = t;
    }
}

void orc_sampled_gradient(const int64_t n[3], const double d[3], const double o[3], int64_t n_picks,
                          const double* src, const double* sta, const double* dist, const uint8_t* valid,
                          const double* weight,
                          const double* vp, const double* resid, double* grad) {
    memset(grad, 0, sizeof(double) * (size_t)(n[0] * n[1] * n[2]));
    for (int64_t i = 0; i < n_picks; ++i) {
        if (valid && !valid[i]) continue;
        if (!isfinite(resid[i])) continue;
        const orc_pick_geo g = orc_pick(n, d, o, src + 3 * i, sta + 3 * i, dist ? dist + i : NULL);
        for (int64_t k = 0; k < g.n_steps; ++k) {
            const int64_t c = orc_sample_cell(&g, n, k);
            const double v = vp[c];
            if (!isfinite(v) || v <= 0.0) continue;
            const double f = -g.ds / (v * v);
            if (!isfinite(f)) continue;
            grad[c] += (resid[i] * f) * weight[i];
        }
    }
}

/* ------------------------------------------------------- slice frames */
/* RTMEngine::capture_single_slice (rtm/rtm_engine.cpp:83-168): the slice of
 * the halo-padded forward and adjoint fields (pitches nyp = ny + 2hw,
 * nzp = nz + 2hw) at interior index `index` along `axis` (0 = X: dim0 = ny,
 * dim1 = nz; 1 = Y: nx, nz; 2 = Z: nx, ny), non-finite values read as 0; the
 * image-condition slice is the first dim0 * dim1 values of `ic` (the
 * reference indexes ic with the slice's own 2-D index). Then
 * LockFreeSnapshotBuffer::serialize_slice (rtm/snapshot_buffer.cpp:102-153):
 * a 124-byte packed SliceFrameHeader in a 128-byte slot (the reference
 * copies 128 bytes from the 124-byte struct; bytes 124..127 are written 0
 * here), then the three FP64 slices; checksum (:207-229) over the payload:
 * s = rotl13(s ^ w) over little-endian 32-bit words, the trailing bytes
 * XORed in unrotated; sequence_id 0. Returns the frame size, or -1 when cap
 * is too small or the axis is not X, Y or Z. Parity of the serializer is
 * against this restatement of the source (the reference's
 * snapshot_buffer.cpp does not compile); the slice values are pinned to the
 * reference's RTMEngine::extract_slices. */
uint32_t orc_slice_checksum(const uint8_t* data, size_t size) {
    uint32_t sum = 0;
    const size_t n32 = size / 4, rest = size % 4;
    for (size_t i = 0; i < n32; ++i) {
        uint32_t w;
        memcpy(&w, data + 4 * i, 4);
        sum ^= w;
        sum = (sum << 13) | (sum >> 19);
    }
    if (rest) {
        uint32_t r = 0;
        for (size_t i = 0; i < rest; ++i) r |= (uint32_t)data[4 * n32 + i] << (8 * i);
        sum ^= r;
    }
    return sum;
}

static void put64(uint8_t* p, int64_t v) { memcpy(p, &v, 8); }

int64_t orc_slice_frame(int axis, int64_t index, int64_t nx, int64_t ny, int64_t nz, int hw, const double* fwd,
                        const double* adj, const double* ic, int64_t timestep, double timestamp, uint8_t* out,
                        int64_t cap) {
    int64_t d0, d1;
    if (axis == 0) { d0 = ny; d1 = nz; }
    else if (axis == 1) { d0 = nx; d1 = nz; }
    else if (axis == 2) { d0 = nx; d1 = ny; }
    else return -1;
    const int64_t n = d0 * d1, bytes = n * 8, size = 128 + 3 * bytes;
    if (size > cap) return -1;
    const int64_t nyp = ny + 2 * hw, nzp = nz + 2 * hw;
    double* f = (double*)malloc((size_t)bytes);
    double* a = (double*)malloc((size_t)bytes);
    double* c = (double*)malloc((size_t)bytes);
    for (int64_t i = 0; i < d0; ++i)
        for (int64_t j = 0; j < d1; ++j) {
            int64_t ix, iy, iz;
            if (axis == 0) { ix = index; iy = i; iz = j; }
            else if (axis == 1) { ix = i; iy = index; iz = j; }
            else { ix = i; iy = j; iz = index; }
            const int64_t src = (ix + hw) * nyp * nzp + (iy + hw) * nzp + (iz + hw);
            const int64_t dst = i * d1 + j;
            f[dst] = isfinite(fwd[src]) ? fwd[src] : 0.0;
            a[dst] = isfinite(adj[src]) ? adj[src] : 0.0;
            c[dst] = isfinite(ic[dst]) ? ic[dst] : 0.0;
        }
    memset(out, 0, 128);
    const uint64_t magic = 0x534C494345303031ULL;
    const int32_t ax = axis;
    memcpy(out + 0, &magic, 8);
    put64(out + 8, timestep);
    memcpy(out + 16, &ax, 4);
    put64(out + 20, index);
    put64(out + 28, d0);
    put64(out + 36, d1);
    put64(out + 44, size);
    put64(out + 52, 128);
    put64(out + 60, 128 + bytes);
    put64(out + 68, 128 + 2 * bytes);
    put64(out + 76, bytes);
    put64(out + 84, bytes);
    put64(out + 92, bytes);
    memcpy(out + 100, &timestamp, 8);
    put64(out + 108, 0);
    memcpy(out + 128, f, (size_t)bytes);
    memcpy(out + 128 + bytes, a, (size_t)bytes);
    memcpy(out + 128 + 2 * bytes, c, (size_t)bytes);
    const uint32_t cs = orc_slice_checksum(out + 128, (size_t)(3 * bytes));
    memcpy(out + 116, &cs, 4);
    free(f);
    free(a);
    free(c);
    return size;
}
