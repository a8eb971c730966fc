/*
 * Propagator part of the CPU oracle, instantiated twice by seismic_oracle.c:
 * REAL = double (the FP64 oracle) and REAL = float (the FP32 floor: the same
 * arithmetic in single precision, used to state how far any FP32
 * implementation can be expected to sit from FP64).
 *
 * TEST INFRASTRUCTURE ONLY: the product never links or calls this code.
 *
 * Layout (reference core/grid.cpp:45-49, halo_width = 1): a field is
 * (nx+2)*(ny+2)*(nz+2) values, idx = ix*NYh*NZh + iy*NZh + iz on padded
 * coordinates, z fastest. All functions take and return padded fields.
 */
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(CAT(orc, SFX), CAT(_, name))

static int FN(isvalid)(REAL v) { return isfinite(v); }

/* FaultTolerance::safe_clamp (core/fault_tolerance.cpp:86-89) */
static REAL FN(safe_clamp)(REAL v, REAL lo, REAL hi) {
    if (!isfinite(v)) return (REAL)0;
    return v < lo ? lo : (v > hi ? hi : v);
}

/* Largest finite velocity over the padded array
 * (WaveEquationSolver::compute_local_max_velocity, wave_equation.cpp:435-443). */
static double FN(vmax)(const orc_grid* g, const REAL* vel) {
    int64_t n = (g->nx + 2) * (g->ny + 2) * (g->nz + 2);
    double vmax = 0.0;
#pragma omp parallel for reduction(max : vmax) schedule(static)
    for (int64_t i = 0; i < n; ++i)
        if (isfinite(vel[i]) && (double)vel[i] > vmax) vmax = (double)vel[i];
    return vmax;
}

/* Sponge damping of one padded cell (apply_sponge_layer, wave_equation.cpp:262-297):
 * dist = min over the six faces of the interior distance, capped at sw; cells
 * with 0 <= dist < sw get D = 1 - damping*(sw-dist)^2/sw^2, others 1. */
static REAL FN(sponge)(const orc_grid* g, int64_t ix, int64_t iy, int64_t iz) {
    const int sw = g->sponge_width;
    const int64_t NXh = g->nx + 2, NYh = g->ny + 2, NZh = g->nz + 2;
    int d = sw;
    if (ix < 1 + sw && (int)(ix - 1) < d) d = (int)(ix - 1);
    if (ix >= NXh - 1 - sw && (int)(NXh - 1 - ix - 1) < d) d = (int)(NXh - 1 - ix - 1);
    if (iy < 1 + sw && (int)(iy - 1) < d) d = (int)(iy - 1);
    if (iy >= NYh - 1 - sw && (int)(NYh - 1 - iy - 1) < d) d = (int)(NYh - 1 - iy - 1);
    if (iz < 1 + sw && (int)(iz - 1) < d) d = (int)(iz - 1);
    if (iz >= NZh - 1 - sw && (int)(NZh - 1 - iz - 1) < d) d = (int)(NZh - 1 - iz - 1);
    if (d < sw && d >= 0) {
        double damp = 1.0 - g->sponge_damping * (sw - d) * (sw - d) / (sw * sw);
        return (REAL)damp;
    }
    return (REAL)1;
}

/* One reference operator pass (fd_7point_operator_safe, wave_equation.cpp:299-405):
 * writes the interior of nxt from cur/prev and returns 1 when a NaN/Inf guard
 * fired (NAN_DETECTED_AND_REPAIRED), else 0. */
static int FN(fd7)(const orc_grid* g, const REAL* vel, const REAL* cur, const REAL* prev, REAL* nxt) {
    const int64_t NYh = g->ny + 2, NZh = g->nz + 2, P = NYh * NZh;
    const REAL idx2 = (REAL)(1.0 / (g->dx * g->dx));
    const REAL idy2 = (REAL)(1.0 / (g->dy * g->dy));
    const REAL idz2 = (REAL)(1.0 / (g->dz * g->dz));
    const REAL dt2 = (REAL)(g->dt * g->dt);
    const double vmax = FN(vmax)(g, vel);
    const double cfl_x = vmax * g->dt / g->dx, cfl_y = vmax * g->dt / g->dy, cfl_z = vmax * g->dt / g->dz;
    double cfl_max = cfl_x > cfl_y ? cfl_x : cfl_y;
    if (cfl_z > cfl_max) cfl_max = cfl_z;
    const int cfl_violation = cfl_max > 1.0;
    REAL cfl_damp2 = (REAL)1;
    if (cfl_violation) {
        double dmin = g->dx < g->dy ? g->dx : g->dy;
        if (g->dz < dmin) dmin = g->dz;
        double ratio = vmax * g->dt / dmin;
        double f = g->cfl_safety / ratio;
        if (f > 1.0) f = 1.0;
        cfl_damp2 = (REAL)(f * f);
    }
    const REAL amp = (REAL)g->amp_limit;
    int fired = 0;
#pragma omp parallel for collapse(2) reduction(| : fired) schedule(static)
    for (int64_t ix = 1; ix <= g->nx; ++ix)
        for (int64_t iy = 1; iy <= g->ny; ++iy)
            for (int64_t iz = 1; iz <= g->nz; ++iz) {
                const int64_t c = ix * P + iy * NZh + iz;
                const REAL uc = cur[c], up = prev[c];
                if (!FN(isvalid)(uc) || !FN(isvalid)(up)) {
                    nxt[c] = (REAL)0;
                    fired = 1;
                    continue;
                }
                const REAL xp = cur[c + P], xm = cur[c - P], yp = cur[c + NZh], ym = cur[c - NZh];
                const REAL zp = cur[c + 1], zm = cur[c - 1];
                if (!FN(isvalid)(xp) || !FN(isvalid)(xm) || !FN(isvalid)(yp) || !FN(isvalid)(ym) ||
                    !FN(isvalid)(zp) || !FN(isvalid)(zm)) {
                    nxt[c] = uc;
                    fired = 1;
                    continue;
                }
                const REAL lap = (xp - (REAL)2 * uc + xm) * idx2 + (yp - (REAL)2 * uc + ym) * idy2 +
                                 (zp - (REAL)2 * uc + zm) * idz2;
                REAL v = vel[c];
                if (!FN(isvalid)(v) || v <= (REAL)0) v = (REAL)1500;
                REAL update = v * v * dt2 * lap;
                if (cfl_violation) update *= cfl_damp2;
                REAL nv = (REAL)2 * uc - up + update;
                if (!FN(isvalid)(nv)) {
                    nv = uc;
                    fired = 1;
                }
                nxt[c] = FN(safe_clamp)(nv, -amp, amp);
            }
    return fired;
}

/* FaultTolerance::repair_field_nan (core/fault_tolerance.cpp:98-157): interior
 * non-finite cells take the mean of their finite in-domain face neighbours
 * (or repl), then any remaining non-finite cell takes repl. nx/ny/nz here are
 * the padded extents, as in the reference signature. */
static int64_t FN(repair_nan)(REAL* d, int64_t count, int64_t nx, int64_t ny, int64_t nz, int hw, REAL repl) {
    const int64_t nynz = ny * nz;
    int64_t repaired = 0;
    for (int64_t ix = hw; ix < nx - hw; ++ix)
        for (int64_t iy = hw; iy < ny - hw; ++iy)
            for (int64_t iz = hw; iz < nz - hw; ++iz) {
                const int64_t i = ix * nynz + iy * nz + iz;
                if (isfinite(d[i])) continue;
                double sum = 0.0;
                int nv = 0;
                if (ix > hw && isfinite(d[i - nynz])) { sum += d[i - nynz]; ++nv; }
                if (ix < nx - hw - 1 && isfinite(d[i + nynz])) { sum += d[i + nynz]; ++nv; }
                if (iy > hw && isfinite(d[i - nz])) { sum += d[i - nz]; ++nv; }
                if (iy < ny - hw - 1 && isfinite(d[i + nz])) { sum += d[i + nz]; ++nv; }
                if (iz > hw && isfinite(d[i - 1])) { sum += d[i - 1]; ++nv; }
                if (iz < nz - hw - 1 && isfinite(d[i + 1])) { sum += d[i + 1]; ++nv; }
                d[i] = nv > 0 ? (REAL)(sum / nv) : repl;
                ++repaired;
            }
    for (int64_t i = 0; i < count; ++i)
        if (!isfinite(d[i])) { d[i] = repl; ++repaired; }
    return repaired;
}

/* Full reference step (step_forward == step_adjoint, wave_equation.cpp:56-98):
 * operator pass into *nxt, sponge on cur and prev (cur and nxt with
 * g->sponge_mode == 1, the stable form that is not in the reference), rotation
 * prev<-cur, cur<-nxt, nxt<-old prev, then the NaN health check with repair
 * (perform_health_check :407-424 -> FaultTolerance::attempt_recovery
 * fault_tolerance.cpp:198-257, 3 attempts). Returns the StepResult code. */
static int FN(step)(const orc_grid* g, const REAL* vel, REAL** cur, REAL** prev, REAL** nxt) {
    const int64_t NXh = g->nx + 2, NYh = g->ny + 2, NZh = g->nz + 2, n = NXh * NYh * NZh;
    int fired = FN(fd7)(g, vel, *cur, *prev, *nxt);
    REAL* C = *cur;
    /* reference: damp current and previous; stable mode: the new field and current */
    REAL* Pv = g->sponge_mode == 1 ? *nxt : *prev;
#pragma omp parallel for schedule(static)
    for (int64_t ix = 0; ix < NXh; ++ix)
        for (int64_t iy = 0; iy < NYh; ++iy)
            for (int64_t iz = 0; iz < NZh; ++iz) {
                const REAL D = FN(sponge)(g, ix, iy, iz);
                if (D != (REAL)1) {
                    const int64_t i = (ix * NYh + iy) * NZh + iz;
                    C[i] *= D;
                    Pv[i] *= D;
                }
            }
    REAL* t = *prev;
    *prev = *cur;
    *cur = *nxt;
    *nxt = t;
    int64_t nan = 0;
    const REAL* Cn = *cur;
#pragma omp parallel for reduction(+ : nan) schedule(static)
    for (int64_t i = 0; i < n; ++i) nan += !isfinite(Cn[i]);
    if (nan > 0) {
        const REAL amp = (REAL)g->amp_limit;
        int ok = 0;
        for (int attempt = 0; attempt < 3 && !ok; ++attempt) {
            FN(repair_nan)(*cur, n, NXh, NYh, NZh, 1, (REAL)0);
            FN(repair_nan)(*prev, n, NXh, NYh, NZh, 1, (REAL)0);
            for (int64_t i = 0; i < n; ++i) {
                (*cur)[i] = FN(safe_clamp)((*cur)[i], -amp, amp);
                (*prev)[i] = FN(safe_clamp)((*prev)[i], -amp, amp);
            }
            int64_t post = 0;
            for (int64_t i = 0; i < n; ++i) post += !isfinite((*cur)[i]);
            ok = post == 0;
        }
        return ok ? 1 : 3;
    }
    return fired ? 1 : 0;
}

/* Driver mirroring oracle/ref_harness.cpp:ref_run_steps: per step t, every
 * source s gets cur[src_s] += src_w[t*n_src+s] when finite (inject_source,
 * wave_equation.cpp:39-54), then one reference step, then each receiver r
 * samples the new current into seis[t*nrec+r]. Optionally stores the
 * post-injection current of every step (V_t, the forward state the fused
 * imaging and gradient kernels correlate with) into states[t*npad...].
 * init_cur / init_prev (may be NULL = zeros) set current / previous first. */
int FN(run)(const orc_grid* g, const REAL* vel, int nsteps, int n_src, const int64_t* src_xyz, const REAL* src_w,
            int nrec, const int64_t* rec_xyz, REAL* seis, int* statuses, REAL* out_cur, REAL* out_prev,
            REAL* states, const REAL* init_cur, const REAL* init_prev) {
    const int64_t NYh = g->ny + 2, NZh = g->nz + 2, n = (g->nx + 2) * NYh * NZh;
    REAL* b0 = (REAL*)calloc((size_t)n, sizeof(REAL));
    REAL* b1 = (REAL*)calloc((size_t)n, sizeof(REAL));
    REAL* b2 = (REAL*)calloc((size_t)n, sizeof(REAL));
    if (!b0 || !b1 || !b2) { free(b0); free(b1); free(b2); return -3; }
    if (init_cur) memcpy(b0, init_cur, (size_t)n * sizeof(REAL));
    if (init_prev) memcpy(b1, init_prev, (size_t)n * sizeof(REAL));
    REAL *cur = b0, *prev = b1, *nxt = b2;
    for (int t = 0; t < nsteps; ++t) {
        for (int s = 0; s < n_src; ++s) {
            const int64_t i = (src_xyz[3 * s] + 1) * NYh * NZh + (src_xyz[3 * s + 1] + 1) * NZh + (src_xyz[3 * s + 2] + 1);
            const REAL w = src_w[(int64_t)t * n_src + s];
            if (i >= 0 && i < n && isfinite(w)) cur[i] += w;
        }
        if (states) memcpy(states + (int64_t)t * n, cur, (size_t)n * sizeof(REAL));
        int st = FN(step)(g, vel, &cur, &prev, &nxt);
        if (statuses) statuses[t] = st;
        for (int q = 0; q < nrec; ++q) {
            const int64_t i = (rec_xyz[3 * q] + 1) * NYh * NZh + (rec_xyz[3 * q + 1] + 1) * NZh + (rec_xyz[3 * q + 2] + 1);
            seis[(int64_t)t * nrec + q] = cur[i];
        }
    }
    if (out_cur) memcpy(out_cur, cur, (size_t)n * sizeof(REAL));
    if (out_prev) memcpy(out_prev, prev, (size_t)n * sizeof(REAL));
    free(b0);
    free(b1);
    free(b2);
    return 0;
}

#undef FN
