/*
 * C restatement of crossbarHspice V1 array2D::nodeBasedGS, the lexicographic
 * node-based Gauss-Seidel/SOR ("Au") solve.  TEST INFRASTRUCTURE ONLY: it is the
 * timed CPU baseline ("port") and a cross-check of the reference's sweep
 * order; the GPU library never links it.
 *
 * Followed line by line in behaviour (not copied):
 *   set-up, g = 1/R, u = vin, d = vout        crossbarHspice/2dArray.cc:1391-1413
 *   per sweep, rows i = 0..n-1, cols j = 0..m-1: update u[i][j] from the NEW
 *   left node, the OLD right node and the OLD bitline node, then d[i][j] from
 *   the NEW upper node, the OLD lower node and the NEW wordline node
 *                                             crossbarHspice/2dArray.cc:1551-1590
 *   break when max |new - old| < tol           crossbarHspice/2dArray.cc:1592-1608
 *   output buffer selection                    crossbarHspice/2dArray.cc:1614-1619
 *   bitline currents                           crossbarHspice/2dArray.cc:1670-1674
 * Wire resistance is uniform (one value), as the reference's GS assumes
 * (2dArray.cc:1380 reads only RDLine[0][0] for g_wire).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Returns the number of sweeps executed (the break sweep index + 1 when the
 * break fired, else iters).  g, vup, vdown: n*m row-major; vin: n; vout: m;
 * iout: m.  Any of vup/vdown/iout may be NULL. */
int au_gs_solve(int n, int m, const double *g, const double *vin, const double *vout, double r_wire,
                int iters, double w, int enable_break, double tol, double *vup_out, double *vdown_out,
                double *iout)
{
    if (n < 2 || m < 2) return -1;
    size_t nm = (size_t)n * m;
    double *U = (double *)malloc(sizeof(double) * nm * 2);
    double *D = (double *)malloc(sizeof(double) * nm * 2);
    if (!U || !D) { free(U); free(D); return -2; }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < m; ++j) {
            U[i * m + j] = U[nm + i * m + j] = vin[i];
            D[i * m + j] = D[nm + i * m + j] = vout[j];
        }
    const double R = r_wire;
    int record = -1;
    for (int it = 0; it < iters; ++it) {
        double *un = U + (size_t)(it & 1) * nm, *uo = U + (size_t)(1 - (it & 1)) * nm;
        double *dn = D + (size_t)(it & 1) * nm, *dold = D + (size_t)(1 - (it & 1)) * nm;
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j < m; ++j) {
                const double gij = g[i * m + j];
                double l = (j == 0) ? vin[i] : un[i * m + j - 1];
                double o = dold[i * m + j], sumg, r;
                if (j == m - 1) {
                    sumg = 1.0 / R + gij;
                    un[i * m + j] = w * (l / R + gij * o) / sumg + (1 - w) * uo[i * m + j];
                } else {
                    r = uo[i * m + j + 1];
                    sumg = 1.0 / R + 1.0 / R + gij;
                    un[i * m + j] = w * (l / R + r / R + gij * o) / sumg + (1 - w) * uo[i * m + j];
                }
                r = (i == n - 1) ? vout[j] : dold[(i + 1) * m + j];
                o = un[i * m + j];
                if (i == 0) {
                    sumg = 1.0 / R + gij;
                    dn[i * m + j] = w * (r / R + gij * o) / sumg + (1 - w) * dold[i * m + j];
                } else {
                    l = dn[(i - 1) * m + j];
                    sumg = 1.0 / R + 1.0 / R + gij;
                    dn[i * m + j] = w * (l / R + r / R + gij * o) / sumg + (1 - w) * dold[i * m + j];
                }
            }
        }
        if (enable_break) {
            double mx = 0;
            for (size_t k = 0; k < nm; ++k) {
                double a = fabs(dn[k] - dold[k]), b = fabs(un[k] - uo[k]);
                if (a > mx) mx = a;
                if (b > mx) mx = b;
            }
            if (mx < tol) { record = it; break; }
        }
    }
    /* the newest buffer: (iters-1)&1 after a full run, record&1 after a break */
    int fin = (record != -1) ? (record & 1) : (1 - (iters & 1));
    const double *uf = U + (size_t)fin * nm, *df = D + (size_t)fin * nm;
    if (vup_out) memcpy(vup_out, uf, sizeof(double) * nm);
    if (vdown_out) memcpy(vdown_out, df, sizeof(double) * nm);
    if (iout) {
        for (int j = 0; j < m; ++j) iout[j] = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < m; ++j) iout[j] += (uf[i * m + j] - df[i * m + j]) * g[i * m + j];
    }
    free(U);
    free(D);
    return record != -1 ? record + 1 : iters;
}

/* count independent solves (one tile and one input vector each) spread over
 * OpenMP threads; g: count*n*m, vin: count*n, iout: count*m, sweeps: count. */
int au_gs_solve_many(int count, int n, int m, const double *g, const double *vin, double r_wire, int iters,
                     double w, int enable_break, double tol, double *iout, int *sweeps)
{
    int bad = 0;
    double *vout = (double *)calloc((size_t)m, sizeof(double));
    if (!vout) return -2;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : bad)
    for (int k = 0; k < count; ++k) {
        int s = au_gs_solve(n, m, g + (size_t)k * n * m, vin + (size_t)k * n, vout, r_wire, iters, w,
                            enable_break, tol, NULL, NULL, iout + (size_t)k * m);
        if (s < 0) bad += 1;
        if (sweeps) sweeps[k] = s;
    }
    free(vout);
    return bad ? -1 : 0;
}

int au_gs_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
