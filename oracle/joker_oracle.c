/*
 * CPU oracle (test infrastructure only; never linked into the product).
 *
 * A plain-C FP64 restatement of the reference's per-sample marginal likelihood:
 *   CJokerHelper.batch_marginal_ln_likelihood   thejoker/src/fast_likelihood.pyx:428-469
 *   CJokerHelper.likelihood_worker              thejoker/src/fast_likelihood.pyx:359-425
 *   CJokerHelper.make_AAinv                     thejoker/src/fast_likelihood.pyx:255-297
 *   CJokerHelper.make_bBBinv                    thejoker/src/fast_likelihood.pyx:299-357
 * It follows the same steps: the N x N matrix B = C + M^T Lambda M, its inverse
 * by the Woodbury identity through A = (Lambda^-1 + M C^-1 M^T)^-1, the log
 * determinant from an LU factorisation of B with partial pivoting, and
 * lnL = -(chi2 + sum_i log(2 pi |U_ii|)) / 2.  Failure returns mirror the
 * reference: a singular Lambda^-1 + M C^-1 M^T gives +INF (:283-284, :381-382),
 * a singular B gives -INF through an infinite log-determinant (:347-348).
 *
 * jitter_mode 0 reproduces the reference Cython, which computes the jittered
 * inverse variance (:458) but never reads it; jitter_mode 1 applies
 * ivar / (1 + s^2 ivar) as the reference's NumPy test oracle does
 * (thejoker/src/tests/py_likelihood.py:17-29, :168-170).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "kepler.h"

static const double PI_D = 3.1415926535897932384626433832795;

/* In-place LU with partial pivoting (row-major n x n).  Returns 0, or i+1 when
 * the pivot of column i is exactly zero (the dgetrf "info > 0" case). */
static int lu_factor(double *a, int n, int *piv)
{
    int info = 0;
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(a[k * n + k]);
        for (int i = k + 1; i < n; ++i) {
            double v = fabs(a[i * n + k]);
            if (v > best) { best = v; p = i; }
        }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < n; ++j) {
                double tmp = a[k * n + j]; a[k * n + j] = a[p * n + j]; a[p * n + j] = tmp;
            }
        double d = a[k * n + k];
        if (d == 0.0) { if (!info) info = k + 1; continue; }
        for (int i = k + 1; i < n; ++i) {
            double l = a[i * n + k] / d;
            a[i * n + k] = l;
            for (int j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
        }
    }
    return info;
}

/* Inverse from an LU factorisation (row-major), column by column. */
static void lu_inverse(const double *lu, const int *piv, int n, double *inv, double *col)
{
    for (int c = 0; c < n; ++c) {
        for (int i = 0; i < n; ++i) col[i] = (i == c) ? 1.0 : 0.0;
        for (int k = 0; k < n; ++k)
            if (piv[k] != k) { double t = col[k]; col[k] = col[piv[k]]; col[piv[k]] = t; }
        for (int i = 0; i < n; ++i) {            /* L y = P e_c */
            double s = col[i];
            for (int j = 0; j < i; ++j) s -= lu[i * n + j] * col[j];
            col[i] = s;
        }
        for (int i = n - 1; i >= 0; --i) {       /* U x = y */
            double s = col[i];
            for (int j = i + 1; j < n; ++j) s -= lu[i * n + j] * col[j];
            col[i] = s / lu[i * n + i];
        }
        for (int i = 0; i < n; ++i) inv[i * n + c] = col[i];
    }
}

/*
 * trend_M: n_times x (n_linear-1), row-major, the same array CJokerHelper takes
 * (fast_likelihood.pyx:174-184).  mu, Lambda: n_linear entries in the
 * CJokerHelper index order (K, v0, offsets..., v1, ...).
 * k_prior_scaled: 1 when the K prior is FixedCompanionMass (the reference stores
 * this as fixed_K_prior == 0, :225-228); then per sample
 * Lambda[0] = min(max_K^2, sigma_K0^2 / (1 - e^2) * (P / P0)^(-2/3)) (:461-464).
 * chunk: n_samples x 5 row-major, columns P, e, omega, M0, s (:41, :448-451).
 */
int oracle_batch_marginal_ln_likelihood(
    int n_times, int n_linear, double t0,
    const double *t, const double *rv, const double *ivar_in,
    const double *trend_M, const double *mu, const double *Lambda_in,
    int k_prior_scaled, double sigma_K0, double P0, double max_K,
    int jitter_mode, const double *chunk, long n_samples, double *ll)
{
    const int N = n_times, L = n_linear;
    double *M_T = (double *)calloc((size_t)L * N, sizeof(double));
    double *ivar = (double *)malloc(sizeof(double) * N);
    double *Lam = (double *)malloc(sizeof(double) * L);
    double *Ainv = (double *)malloc(sizeof(double) * L * L);
    double *Atmp = (double *)malloc(sizeof(double) * L * L);
    double *A = (double *)malloc(sizeof(double) * L * L);
    double *b = (double *)malloc(sizeof(double) * N);
    double *B = (double *)malloc(sizeof(double) * N * N);
    double *Binv = (double *)malloc(sizeof(double) * N * N);
    double *colL = (double *)malloc(sizeof(double) * L);
    int *pivL = (int *)malloc(sizeof(int) * L);
    int *pivN = (int *)malloc(sizeof(int) * N);
    if (!M_T || !ivar || !Lam || !Ainv || !Atmp || !A || !b || !B || !Binv || !colL || !pivL || !pivN) {
        free(M_T); free(ivar); free(Lam); free(Ainv); free(Atmp); free(A); free(b);
        free(B); free(Binv); free(colL); free(pivL); free(pivN);
        return -1;
    }
    for (int n = 0; n < N; ++n)
        for (int i = 1; i < L; ++i) M_T[i * N + n] = trend_M[n * (L - 1) + (i - 1)];
    memcpy(Lam, Lambda_in, sizeof(double) * L);
    double *tt = (double *)t;

    for (long s = 0; s < n_samples; ++s) {
        const double P = chunk[s * 5 + 0], e = chunk[s * 5 + 1];
        const double om = chunk[s * 5 + 2], M0 = chunk[s * 5 + 3], jit = chunk[s * 5 + 4];
        c_rv_from_elements(tt, M_T, N, P, 1.0, e, om, M0, t0, 1e-10, 128);
        for (int n = 0; n < N; ++n)
            ivar[n] = jitter_mode ? ivar_in[n] / (1.0 + jit * jit * ivar_in[n]) : ivar_in[n];
        if (k_prior_scaled) {
            double v = sigma_K0 * sigma_K0 / (1.0 - e * e) * pow(P / P0, -2.0 / 3.0);
            Lam[0] = (max_K * max_K < v) ? max_K * max_K : v;
        }

        /* make_AAinv: Ainv = Lambda^-1 + M C^-1 M^T, A = Ainv^-1 */
        int failed = 0;
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) Ainv[i * L + j] = 0.0;
        for (int i = 0; i < L; ++i) {
            Ainv[i * L + i] = 1.0 / Lam[i];
            for (int j = 0; j < L; ++j) {
                for (int n = 0; n < N; ++n)
                    Ainv[i * L + j] += M_T[j * N + n] * ivar[n] * M_T[i * N + n];
                Atmp[i * L + j] = Ainv[i * L + j];
            }
        }
        if (lu_factor(Atmp, L, pivL) != 0) failed = 1;
        if (failed) { ll[s] = INFINITY; continue; }
        lu_inverse(Atmp, pivL, L, A, colL);

        /* make_bBBinv */
        for (int n = 0; n < N; ++n) {
            b[n] = 0.0;
            for (int i = 0; i < L; ++i) b[n] += M_T[i * N + n] * mu[i];
        }
        for (int n = 0; n < N; ++n)
            for (int m = 0; m < N; ++m) {
                double v = (n == m) ? 1.0 / ivar[n] : 0.0;
                for (int i = 0; i < L; ++i) v += M_T[i * N + n] * Lam[i] * M_T[i * N + m];
                B[n * N + m] = v;
            }
        for (int n = 0; n < N; ++n)
            for (int m = 0; m < N; ++m) {
                double v = (n == m) ? ivar[n] : 0.0;
                for (int i = 0; i < L; ++i)
                    for (int j = 0; j < L; ++j)
                        v -= ivar[n] * M_T[i * N + n] * A[i * L + j] * M_T[j * N + m] * ivar[m];
                Binv[n * N + m] = v;
            }
        double logdet;
        if (lu_factor(B, N, pivN) != 0) {
            logdet = INFINITY;
        } else {
            logdet = 0.0;
            for (int i = 0; i < N; ++i) logdet += log(2.0 * PI_D * fabs(B[i * N + i]));
        }
        double chi2 = 0.0;
        for (int n = 0; n < N; ++n)
            for (int m = 0; m < N; ++m)
                chi2 += (b[m] - rv[m]) * Binv[n * N + m] * (b[n] - rv[n]);
        ll[s] = -0.5 * (chi2 + logdet);
    }
    free(M_T); free(ivar); free(Lam); free(Ainv); free(Atmp); free(A); free(b);
    free(B); free(Binv); free(colL); free(pivL); free(pivN);
    return 0;
}

/* Unit-K RV column for a batch of samples (n_samples x n_times, row-major). */
void oracle_rv_unit_batch(int n_times, double t0, const double *t,
                          const double *chunk, long n_samples, double *out)
{
    for (long s = 0; s < n_samples; ++s)
        c_rv_from_elements((double *)t, out + s * n_times, n_times, chunk[s * 5 + 0], 1.0,
                           chunk[s * 5 + 1], chunk[s * 5 + 2], chunk[s * 5 + 3], t0, 1e-10, 128);
}
