/*
 * Precision-generic body of the tortuosity oracle.  Included twice by
 * tau_oracle.c, once with REAL=double / SFX(x)=x##_f64 and once with
 * REAL=float / SFX(x)=x##_f32, mirroring the reference's float/double template
 * instantiations (fastlib/src/volume/VolumeMeasures.cpp:348-349).
 *
 * TEST INFRASTRUCTURE ONLY: this is the CPU restatement the CUDA path is
 * checked against.  Nothing in the product links or calls it.
 */

/* ------------------------------------------------------------------------ */
/* Assembly: the stored 7-coefficient system.                                */
/* ------------------------------------------------------------------------ */

/*
 * Assemble A (7 stored coefficient arrays, layout A[d*N + i] with d in the
 * reference's Dir order X_POS,X_NEG,Y_POS,Y_NEG,Z_POS,Z_NEG,DIR_NONE), b and
 * the initial guess x0.
 *
 * Follows, per voxel:
 *   - domain value D = mask>0 ? d1 : d0          (LinearSystemDevice.cu:8-20,
 *                                                  Diffusion.cpp:94-96)
 *   - face D = (D(clamped nbr) + D) * 0.5         (Diffusion.cu:47-53,
 *                                                  Diffusion.cpp:119-125)
 *   - getSystemTopKernel coefficient/rhs/x0 rules (Diffusion.cuh:54-148)
 * with cellDim = (float)(1/maxDim) for all three axes and
 * faceArea[k] = cellDim[a]*cellDim[b] computed in double (Diffusion.cpp:16-35,
 * VolumeMeasures.cpp:68).
 */
static void SFX(assemble)(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz,
                          int dir, double d0, double d1, float cell_f,
                          REAL *A, REAL *b, REAL *x0)
{
    const int64_t N = nx * ny * nz;
    const int64_t res[3] = {nx, ny, nz};
    const int primary = dir_index(dir);
    const int sgn_dir = dir_sgn(dir);
    const double conc_begin = (sgn_dir == 1) ? 1.0 : 0.0;
    const double conc_end = (sgn_dir == 1) ? 0.0 : 1.0;
    const double cell_dim[3] = {(double)cell_f, (double)cell_f, (double)cell_f};
    const double face_area[3] = {cell_dim[1] * cell_dim[2], cell_dim[0] * cell_dim[2],
                                 cell_dim[0] * cell_dim[1]};

#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++) {
        for (int64_t y = 0; y < ny; y++) {
            for (int64_t x = 0; x < nx; x++) {
                const int64_t vox[3] = {x, y, z};
                const int64_t i = x + nx * (y + ny * z);
                const REAL Dc = (mask[i] > 0) ? (REAL)d1 : (REAL)d0;
                REAL Dface[6];
                for (int d = 0; d < 6; d++) {
                    const int k = dir_index(d);
                    const int s = dir_sgn(d);
                    int64_t p[3] = {x, y, z};
                    const int64_t nv = p[k] + s;
                    if (nv >= 0 && nv < res[k]) p[k] = nv; /* clampedIndex, Diffusion.cpp:51-62 */
                    const int64_t j = p[0] + nx * (p[1] + ny * p[2]);
                    const REAL Dn = (mask[j] > 0) ? (REAL)d1 : (REAL)d0;
                    Dface[d] = (Dn + Dc) * (REAL)0.5;
                }
                REAL coeffs[7];
                int use[7];
                coeffs[DIR_NONE_] = (REAL)0;
                use[DIR_NONE_] = 1;
                for (int d = 0; d < 6; d++) {
                    const int k = dir_index(d);
                    const int s = dir_sgn(d);
                    REAL cell_dist[3] = {(REAL)cell_dim[0], (REAL)cell_dim[1], (REAL)cell_dim[2]};
                    use[d] = 1;
                    if ((vox[k] == 0 && s == -1) || (vox[k] == res[k] - 1 && s == 1)) {
                        cell_dist[k] = (REAL)(cell_dim[k] * (REAL)0.5);
                        use[d] = 0;
                    }
                    /* (Dface * faceArea[k]) / cellDist[k]: Dface and cellDist are T,
                     * faceArea is double, so the product/quotient run in double. */
                    coeffs[d] = (REAL)(((double)Dface[d] * face_area[k]) / (double)cell_dist[k]);
                    if (use[d] || k == primary) coeffs[DIR_NONE_] -= coeffs[d];
                }
                const int64_t primary_res = res[primary];
                REAL rhs = (REAL)0;
                if (vox[primary] == 0) {
                    const int dneg = make_dir(primary, -1);
                    rhs = (REAL)((double)rhs - (double)coeffs[dneg] * conc_begin);
                } else if (vox[primary] == primary_res - 1) {
                    const int dpos = make_dir(primary, 1);
                    rhs = (REAL)((double)rhs - (double)coeffs[dpos] * conc_end);
                }
                b[i] = rhs;
                const int64_t pv = vox[primary];
                if (sgn_dir == 1)
                    x0[i] = (REAL)1.0f - ((REAL)pv / (REAL)(primary_res + 1));
                else
                    x0[i] = ((REAL)pv / (REAL)(primary_res + 1));
                for (int d = 0; d < 6; d++)
                    if (!use[d]) coeffs[d] = (REAL)0;
                for (int d = 0; d < 7; d++) A[(int64_t)d * N + i] = coeffs[d];
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Sparse products (LinearSystemDevice.cuh:29-49, 67-80).                    */
/* ------------------------------------------------------------------------ */

/* y = A x, summation order X+,X-,Y+,Y-,Z+,Z-,diag, zero coefficients skipped. */
static void SFX(spmv)(const REAL *A, int64_t nx, int64_t ny, int64_t nz, const REAL *x, REAL *y,
                      const REAL *b_or_null)
{
    const int64_t N = nx * ny * nz;
    const int64_t sy = nx, sz = nx * ny;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++) {
        for (int64_t yy = 0; yy < ny; yy++) {
            const int64_t row = nx * (yy + ny * z);
            for (int64_t xx = 0; xx < nx; xx++) {
                const int64_t I = row + xx;
                REAL sum = (REAL)0;
                REAL c;
                c = A[0 * N + I]; if (c != (REAL)0) sum += x[I + 1] * c;
                c = A[1 * N + I]; if (c != (REAL)0) sum += x[I - 1] * c;
                c = A[2 * N + I]; if (c != (REAL)0) sum += x[I + sy] * c;
                c = A[3 * N + I]; if (c != (REAL)0) sum += x[I - sy] * c;
                c = A[4 * N + I]; if (c != (REAL)0) sum += x[I + sz] * c;
                c = A[5 * N + I]; if (c != (REAL)0) sum += x[I - sz] * c;
                c = A[6 * N + I]; if (c != (REAL)0) sum += x[I] * c;
                y[I] = b_or_null ? (b_or_null[I] - sum) : sum;
            }
        }
    }
}

/* Deterministic dot product: fixed chunks summed in index order, chunk sums in
 * order.  The result does not depend on the OpenMP thread count. */
static REAL SFX(dot)(const REAL *a, const REAL *b, int64_t N)
{
    const int64_t chunk = 65536;
    const int64_t nchunks = (N + chunk - 1) / chunk;
    REAL *part = (REAL *)malloc(sizeof(REAL) * (size_t)(nchunks > 0 ? nchunks : 1));
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nchunks; c++) {
        const int64_t lo = c * chunk;
        const int64_t hi = (lo + chunk < N) ? lo + chunk : N;
        REAL s = (REAL)0;
        for (int64_t i = lo; i < hi; i++) s += a[i] * b[i];
        part[c] = s;
    }
    REAL s = (REAL)0;
    for (int64_t c = 0; c < nchunks; c++) s += part[c];
    free(part);
    return s;
}

/* ------------------------------------------------------------------------ */
/* Jacobi-PCG.                                                               */
/*   variant ORACLE_DEVICE: fastlib/src/cuda/CG.cu:21-169 (the default path)  */
/*   variant ORACLE_EIGEN : the published Eigen::ConjugateGradient recurrence  */
/*                          with DiagonalPreconditioner, as called from       */
/*                          fastlib/src/solver/CG.cpp:85-100                   */
/* ------------------------------------------------------------------------ */
static int SFX(cg)(const REAL *A, int64_t nx, int64_t ny, int64_t nz, const REAL *b, REAL *x,
                   REAL tol, uint64_t max_iter, int variant, uint64_t *iters_out, REAL *err_out)
{
    const int64_t N = nx * ny * nz;
    const REAL *diag = A + 6 * N;
    REAL *r = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *p = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *ap = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *zv = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    int status = ORACLE_NO_CONVERGENCE;
    uint64_t i = 0;

    SFX(spmv)(A, nx, ny, nz, x, r, b); /* r = b - A x */
    const REAL rhs_sq = SFX(dot)(b, b, N);

    if (variant == ORACLE_DEVICE) {
        if (rhs_sq == (REAL)0) {
            for (int64_t k = 0; k < N; k++) x[k] = (REAL)0;
            /* CG.cu:41-44 returns false without touching the outputs. */
            *iters_out = 0; *err_out = (REAL)0;
            status = ORACLE_NO_CONVERGENCE;
            goto done;
        }
        const REAL tol2 = tol * tol * rhs_sq;
        REAL rsq = SFX(dot)(r, r, N);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < N; k++) zv[k] = r[k] * (REAL)1.0 / diag[k];
        memcpy(p, zv, sizeof(REAL) * (size_t)N);
        REAL zr = SFX(dot)(r, zv, N);
        while (rsq > tol2 && i < max_iter) {
            SFX(spmv)(A, nx, ny, nz, p, ap, NULL);
            const REAL pap = SFX(dot)(p, ap, N);
            const REAL alpha = zr / pap;
            const REAL nalpha = -alpha;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) {
                x[k] += alpha * p[k];
                r[k] += nalpha * ap[k];
            }
            rsq = SFX(dot)(r, r, N);
            if (rsq <= tol2) break;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) zv[k] = r[k] * (REAL)1.0 / diag[k];
            const REAL old_zr = zr;
            zr = SFX(dot)(r, zv, N);
            const REAL beta = zr / old_zr;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) p[k] = p[k] * beta + zv[k];
            ++i;
            if (rsq > (REAL)10e+10) break; /* CG.cu:151-154 */
        }
        *iters_out = i;
        *err_out = (REAL)sqrt((double)(SFX(dot)(r, r, N) / rhs_sq));
        status = (rsq <= tol2) ? ORACLE_OK : ORACLE_NO_CONVERGENCE;
    } else {
        if (rhs_sq == (REAL)0) {
            for (int64_t k = 0; k < N; k++) x[k] = (REAL)0;
            *iters_out = 0; *err_out = (REAL)0;
            status = ORACLE_OK;
            goto done;
        }
        REAL threshold = tol * tol * rhs_sq;
        if (threshold < ORACLE_REAL_MIN) threshold = ORACLE_REAL_MIN;
        REAL rsq = SFX(dot)(r, r, N);
        if (rsq < threshold) {
            *iters_out = 0;
            *err_out = (REAL)sqrt((double)(rsq / rhs_sq));
            status = ORACLE_OK;
            goto done;
        }
        /* DiagonalPreconditioner: invdiag = 1/diag, solve = invdiag * r */
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < N; k++) p[k] = ((REAL)1 / diag[k]) * r[k];
        REAL abs_new = SFX(dot)(r, p, N);
        while (i < max_iter) {
            SFX(spmv)(A, nx, ny, nz, p, ap, NULL);
            const REAL alpha = abs_new / SFX(dot)(p, ap, N);
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) {
                x[k] += alpha * p[k];
                r[k] -= alpha * ap[k];
            }
            rsq = SFX(dot)(r, r, N);
            if (rsq < threshold) break;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) zv[k] = ((REAL)1 / diag[k]) * r[k];
            const REAL abs_old = abs_new;
            abs_new = SFX(dot)(r, zv, N);
            const REAL beta = abs_new / abs_old;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) p[k] = zv[k] + beta * p[k];
            i++;
        }
        const REAL err = (REAL)sqrt((double)(rsq / rhs_sq));
        *iters_out = i;
        *err_out = err;
        status = (err <= tol) ? ORACLE_OK : ORACLE_NO_CONVERGENCE;
    }
done:
    free(r); free(p); free(ap); free(zv);
    return status;
}

/* ------------------------------------------------------------------------ */
/* Right-Jacobi BiCGSTAB.                                                    */
/*   variant ORACLE_DEVICE: fastlib/src/cuda/BICGSTAB.cu:24-230               */
/*   variant ORACLE_EIGEN : the published Eigen::BiCGSTAB recurrence, as      */
/*                          called from fastlib/src/solver/BICGSTAB.cpp:80-94 */
/* ------------------------------------------------------------------------ */
static int SFX(bicgstab)(const REAL *A, int64_t nx, int64_t ny, int64_t nz, const REAL *b, REAL *x,
                         REAL tol, uint64_t max_iter, int variant, uint64_t *iters_out,
                         REAL *err_out)
{
    const int64_t N = nx * ny * nz;
    const REAL *diag = A + 6 * N;
    REAL *r0 = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *r = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *p = (REAL *)calloc((size_t)N, sizeof(REAL));
    REAL *v = (REAL *)calloc((size_t)N, sizeof(REAL));
    REAL *s = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *t = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *y = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *zz = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    int status = ORACLE_NO_CONVERGENCE;

    SFX(spmv)(A, nx, ny, nz, x, r, b);
    memcpy(r0, r, sizeof(REAL) * (size_t)N);
    REAL r0_sq = SFX(dot)(r0, r0, N);
    const REAL rhs_sq = SFX(dot)(b, b, N);
    if (rhs_sq == (REAL)0) {
        for (int64_t k = 0; k < N; k++) x[k] = (REAL)0;
        *iters_out = 0; *err_out = (REAL)0;
        status = (variant == ORACLE_DEVICE) ? ORACLE_NO_CONVERGENCE : ORACLE_OK;
        goto done;
    }
    REAL rho = 1, alpha = 1, w = 1;
    const REAL tol2 = tol * tol * rhs_sq;
    const REAL eps2 = ORACLE_REAL_EPS * ORACLE_REAL_EPS;
    uint64_t i = 0, restarts = 0;
    REAL rsq = SFX(dot)(r, r, N);
    while (rsq > tol2 && i < max_iter) {
        const REAL rho_old = rho;
        rho = SFX(dot)(r0, r, N);
        if ((REAL)fabs((double)rho) < eps2 * r0_sq) {
            SFX(spmv)(A, nx, ny, nz, x, r, b);
            memcpy(r0, r, sizeof(REAL) * (size_t)N);
            rho = r0_sq = SFX(dot)(r, r, N);
            if (variant == ORACLE_EIGEN) {
                if (restarts++ == 0) i = 0;
            } else {
                restarts++;
            }
        }
        const REAL beta = (rho / rho_old) * (alpha / w);
        if (variant == ORACLE_DEVICE) {
            /* __aPlusBetaBGammaPlusCKernel(p, v, r, -w, beta): p = beta*(p + (-w)*v) + r */
            const REAL nw = -w;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) p[k] = beta * (p[k] + nw * v[k]) + r[k];
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) y[k] = p[k] * (REAL)1.0 / diag[k];
        } else {
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) p[k] = r[k] + beta * (p[k] - w * v[k]);
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) y[k] = ((REAL)1 / diag[k]) * p[k];
        }
        SFX(spmv)(A, nx, ny, nz, y, v, NULL);
        alpha = rho / SFX(dot)(r0, v, N);
        const REAL nalpha = -alpha;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < N; k++) s[k] = (variant == ORACLE_DEVICE) ? r[k] + nalpha * v[k]
                                                                           : r[k] - alpha * v[k];
        if (variant == ORACLE_DEVICE) {
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) zz[k] = s[k] * (REAL)1.0 / diag[k];
        } else {
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < N; k++) zz[k] = ((REAL)1 / diag[k]) * s[k];
        }
        SFX(spmv)(A, nx, ny, nz, zz, t, NULL);
        const REAL tmp = SFX(dot)(t, t, N);
        if (tmp > (REAL)0)
            w = SFX(dot)(t, s, N) / tmp;
        else
            w = (REAL)0;
        const REAL nw2 = -w;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < N; k++) {
            x[k] += alpha * y[k] + w * zz[k];
            r[k] = (variant == ORACLE_DEVICE) ? s[k] + nw2 * t[k] : s[k] - w * t[k];
        }
        rsq = SFX(dot)(r, r, N);
        if (variant == ORACLE_DEVICE && rsq > (REAL)10e+10) break; /* BICGSTAB.cu:206-209 */
        ++i;
    }
    (void)restarts;
    *iters_out = i;
    *err_out = (REAL)sqrt((double)(SFX(dot)(r, r, N) / rhs_sq));
    if (variant == ORACLE_DEVICE)
        status = (rsq <= tol2) ? ORACLE_OK : ORACLE_NO_CONVERGENCE;
    else
        status = (*err_out <= tol) ? ORACLE_OK : ORACLE_NO_CONVERGENCE;
done:
    free(r0); free(r); free(p); free(v); free(s); free(t); free(y); free(zz);
    return status;
}

/* ------------------------------------------------------------------------ */
/* tau: the plane-flux reduction of fastlib/src/volume/VolumeMeasures.cpp:   */
/* 188-275, in T precision, single-threaded, in the same loop order.         */
/* ------------------------------------------------------------------------ */
static REAL SFX(tau_from_conc)(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir,
                               float c0, float c1, const REAL *conc, REAL porosity)
{
    const int64_t dim[3] = {nx, ny, nz};
    const int primary = dir_index(dir);
    const int sec0 = (primary + 1) % 3, sec1 = (primary + 2) % 3;
    const int n = (int)(dim[sec0] * dim[sec1]);
    int64_t dpos[3] = {0, 0, 0};
    dpos[primary] = dir_sgn(dir);
    REAL dc_sum = (REAL)0;
    for (int64_t k = 0; k < dim[primary]; k++) {
        REAL sum = (REAL)0;
        for (int64_t j = 0; j < dim[sec1]; j++) {
            for (int64_t i = 0; i < dim[sec0]; i++) {
                int64_t pos[3];
                pos[primary] = k; pos[sec0] = i; pos[sec1] = j;
                const int64_t vi = pos[0] + nx * (pos[1] + ny * pos[2]);
                const REAL coeff_here = (REAL)((mask[vi] == 0) ? c0 : c1);
                const REAL here = conc[vi];
                REAL prev = (REAL)0.0;
                REAL dx = (REAL)0.5;
                const int64_t q[3] = {pos[0] + dpos[0], pos[1] + dpos[1], pos[2] + dpos[2]};
                if (q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] < nx && q[1] < ny && q[2] < nz) {
                    prev = conc[q[0] + nx * (q[1] + ny * q[2])];
                    dx = (REAL)1.0;
                }
                sum += coeff_here * (here - prev) / dx;
            }
        }
        const REAL dc_plane = sum / (REAL)n;
        dc_sum += dc_plane;
    }
    const REAL dc = dc_sum / (REAL)dim[primary];
    return porosity / (dc * (REAL)dim[primary]);
}

/* ------------------------------------------------------------------------ */
/* Public entry points (extern, suffixed).                                   */
/* ------------------------------------------------------------------------ */

int SFX(oracle_assemble)(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir,
                         double d0, double d1, float cell, REAL *A, REAL *b, REAL *x0)
{
    if (nx <= 0 || ny <= 0 || nz <= 0 || dir < 0 || dir > 5) return ORACLE_BAD_ARG;
    SFX(assemble)(mask, nx, ny, nz, dir, d0, d1, cell, A, b, x0);
    return ORACLE_OK;
}

void SFX(oracle_spmv)(const REAL *A, int64_t nx, int64_t ny, int64_t nz, const REAL *x, REAL *y)
{
    SFX(spmv)(A, nx, ny, nz, x, y, NULL);
}

void SFX(oracle_residual)(const REAL *A, int64_t nx, int64_t ny, int64_t nz, const REAL *x,
                          const REAL *b, REAL *r)
{
    SFX(spmv)(A, nx, ny, nz, x, r, b);
}

int SFX(oracle_solve)(const REAL *A, int64_t nx, int64_t ny, int64_t nz, const REAL *b, REAL *x,
                      int solver, double tol, uint64_t max_iter, int variant, uint64_t *iters,
                      double *err)
{
    REAL e = 0;
    int st;
    if (solver == ORACLE_SOLVER_CG)
        st = SFX(cg)(A, nx, ny, nz, b, x, (REAL)tol, max_iter, variant, iters, &e);
    else
        st = SFX(bicgstab)(A, nx, ny, nz, b, x, (REAL)tol, max_iter, variant, iters, &e);
    *err = (double)e;
    return st;
}

double SFX(oracle_tau)(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir, float c0,
                       float c1, const REAL *conc, double porosity)
{
    return (double)SFX(tau_from_conc)(mask, nx, ny, nz, dir, c0, c1, conc, (REAL)porosity);
}

/*
 * The whole getTortuosity<T> pipeline (VolumeMeasures.cpp:42-285):
 * assembly -> solve -> status check -> porosity -> tau.  Returns tau, or 0 on
 * a non-success status (VolumeMeasures.cpp:157-159).  porosity < 0 means
 * "compute it", as getPorosity<T> does (VolumeMeasures.cpp:289-292).
 */
double SFX(oracle_get_tortuosity)(const uint8_t *mask, int64_t nx, int64_t ny, int64_t nz, int dir,
                                  int solver, double tol, uint64_t max_iter, float c0, float c1,
                                  double porosity, int variant, REAL *x_out, uint64_t *iters,
                                  double *err, int *status)
{
    const int64_t N = nx * ny * nz;
    *iters = 0; *err = 0; *status = ORACLE_BAD_ARG;
    if (nx <= 0 || ny <= 0 || nz <= 0 || dir < 0 || dir > 5) return 0.0;
    int64_t max_dim = nx;
    if (ny > max_dim) max_dim = ny;
    if (nz > max_dim) max_dim = nz;
    const float cell = 1.0f / (float)max_dim;
    REAL *A = (REAL *)malloc(sizeof(REAL) * (size_t)(7 * N));
    REAL *b = (REAL *)malloc(sizeof(REAL) * (size_t)N);
    REAL *x = x_out ? x_out : (REAL *)malloc(sizeof(REAL) * (size_t)N);
    if (!A || !b || !x) { *status = ORACLE_NOMEM; free(A); free(b); if (!x_out) free(x); return 0.0; }
    SFX(assemble)(mask, nx, ny, nz, dir, (double)c0, (double)c1, cell, A, b, x);
    *status = SFX(oracle_solve)(A, nx, ny, nz, b, x, solver, tol, max_iter, variant, iters, err);
    double tau = 0.0;
    if (*status == ORACLE_OK) {
        REAL phi;
        if (porosity >= 0.0)
            phi = (REAL)porosity;
        else
            phi = (REAL)oracle_count_pores(mask, N) / (REAL)N;
        tau = (double)SFX(tau_from_conc)(mask, nx, ny, nz, dir, c0, c1, x, phi);
    }
    free(A); free(b);
    if (!x_out) free(x);
    return tau;
}
