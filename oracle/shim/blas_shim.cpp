/*
 * Plain-loop BLAS level-1/3 routines with the reference BLAS's semantics
 * and summation order, for the oracle's pinning build of the reference
 * (test infrastructure only).  Routines that the hot path never reaches
 * abort if called.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

extern "C" {
static void oracle_blas_unused(const char* n)
{
    fprintf(stderr, "oracle blas shim: %s not provided\n", n);
    abort();
}

void oracle_daxpy(const int* n, const double* a, const double* x, const int* ix, double* y, const int* iy)
{ for (int i = 0; i < *n; i++) y[i * *iy] += *a * x[i * *ix]; }
void oracle_saxpy(const int* n, const float* a, const float* x, const int* ix, float* y, const int* iy)
{ for (int i = 0; i < *n; i++) y[i * *iy] += *a * x[i * *ix]; }
void oracle_dscal(const int* n, const double* a, double* x, const int* ix)
{ for (int i = 0; i < *n; i++) x[i * *ix] *= *a; }
void oracle_sscal(const int* n, const float* a, float* x, const int* ix)
{ for (int i = 0; i < *n; i++) x[i * *ix] *= *a; }
void oracle_dcopy(const int* n, const double* x, const int* ix, double* y, const int* iy)
{ for (int i = 0; i < *n; i++) y[i * *iy] = x[i * *ix]; }
void oracle_scopy(const int* n, const float* x, const int* ix, float* y, const int* iy)
{ for (int i = 0; i < *n; i++) y[i * *iy] = x[i * *ix]; }
double oracle_ddot(const int* n, const double* x, const int* ix, const double* y, const int* iy)
{ double s = 0.; for (int i = 0; i < *n; i++) s += x[i * *ix] * y[i * *iy]; return s; }
float oracle_sdot(const int* n, const float* x, const int* ix, const float* y, const int* iy)
{ float s = 0.f; for (int i = 0; i < *n; i++) s += x[i * *ix] * y[i * *iy]; return s; }
double oracle_dnrm2(const int* n, const double* x, const int* ix)
{ double s = 0.; for (int i = 0; i < *n; i++) s += x[i * *ix] * x[i * *ix]; return sqrt(s); }
float oracle_snrm2(const int* n, const float* x, const int* ix)
{ float s = 0.f; for (int i = 0; i < *n; i++) s += x[i * *ix] * x[i * *ix]; return sqrtf(s); }
int oracle_idamax(const int* n, const double* x, const int* ix)
{ int k = 0; double m = -1.; for (int i = 0; i < *n; i++) if (fabs(x[i * *ix]) > m) { m = fabs(x[i * *ix]); k = i; } return k + 1; }
int oracle_isamax(const int* n, const float* x, const int* ix)
{ int k = 0; float m = -1.f; for (int i = 0; i < *n; i++) if (fabsf(x[i * *ix]) > m) { m = fabsf(x[i * *ix]); k = i; } return k + 1; }

/* C := alpha A^T A + beta C (trans 't', lower or upper), or alpha A A^T + beta C */
void oracle_dsyrk(const char* uplo, const char* trans, const int* n, const int* k, const double* alpha,
    const double* a, const int* lda, const double* beta, double* c, const int* ldc)
{
    const bool lower = (*uplo == 'l' || *uplo == 'L');
    const bool tr = (*trans == 't' || *trans == 'T' || *trans == 'c' || *trans == 'C');
    for (int j = 0; j < *n; j++)
        for (int i = lower ? j : 0; i < (lower ? *n : j + 1); i++)
        {
            double t = 0.;
            for (int l = 0; l < *k; l++)
                t += tr ? a[l + i * *lda] * a[l + j * *lda] : a[i + l * *lda] * a[j + l * *lda];
            c[i + j * *ldc] = (*beta == 0. ? 0. : *beta * c[i + j * *ldc]) + *alpha * t;
        }
}
void oracle_dgemm(const char* ta, const char* tb, const int* m, const int* n, const int* k,
    const double* alpha, const double* a, const int* lda, const double* b, const int* ldb,
    const double* beta, double* c, const int* ldc)
{
    const bool at = (*ta == 't' || *ta == 'T'), bt = (*tb == 't' || *tb == 'T');
    for (int j = 0; j < *n; j++)
        for (int i = 0; i < *m; i++)
        {
            double t = 0.;
            for (int l = 0; l < *k; l++)
                t += (at ? a[l + i * *lda] : a[i + l * *lda]) * (bt ? b[j + l * *ldb] : b[l + j * *ldb]);
            c[i + j * *ldc] = (*beta == 0. ? 0. : *beta * c[i + j * *ldc]) + *alpha * t;
        }
}
void oracle_ssyrk() { oracle_blas_unused("ssyrk"); }
void oracle_sgemm() { oracle_blas_unused("sgemm"); }
void oracle_dgemv() { oracle_blas_unused("dgemv"); }
void oracle_sgemv() { oracle_blas_unused("sgemv"); }
void oracle_dtrsm() { oracle_blas_unused("dtrsm"); }
void oracle_strsm() { oracle_blas_unused("strsm"); }
void oracle_dtrmm() { oracle_blas_unused("dtrmm"); }
void oracle_dsymv() { oracle_blas_unused("dsymv"); }
void oracle_dsymm() { oracle_blas_unused("dsymm"); }
void oracle_drot() { oracle_blas_unused("drot"); }
void oracle_srot() { oracle_blas_unused("srot"); }
void oracle_dpotri() { oracle_blas_unused("dpotri"); }

/* LAPACK stand-ins for the small Anderson system (AndersonMix.cc calls
 * DSYEV, DPOTRF, DPOTRS with uplo 'l'; only 'l' is implemented).
 * DPOTRF: the unblocked left-looking Cholesky of LAPACK's DPOTF2, info = j
 * (1-based) at the first non-positive pivot. */
void oracle_dpotrf(const char* uplo, const int* n, double* a, const int* lda, int* info)
{
    *info = 0;
    if (!(*uplo == 'l' || *uplo == 'L')) { oracle_blas_unused("dpotrf upper"); return; }
    const int N = *n, ld = *lda;
    for (int j = 0; j < N; j++)
    {
        double ajj = a[j + j * ld];
        for (int k = 0; k < j; k++)
            ajj -= a[j + k * ld] * a[j + k * ld];
        if (!(ajj > 0.))
        {
            a[j + j * ld] = ajj;
            *info = j + 1;
            return;
        }
        ajj = std::sqrt(ajj);
        a[j + j * ld] = ajj;
        for (int i = j + 1; i < N; i++)
        {
            double t = a[i + j * ld];
            for (int k = 0; k < j; k++)
                t -= a[i + k * ld] * a[j + k * ld];
            a[i + j * ld] = t / ajj;
        }
    }
}

/* DPOTRS, lower: L y = b, then L^T x = y, for nrhs columns of b */
void oracle_dpotrs(const char* uplo, const int* n, const int* nrhs, const double* a,
    const int* lda, double* b, const int* ldb, int* info)
{
    *info = 0;
    if (!(*uplo == 'l' || *uplo == 'L')) { oracle_blas_unused("dpotrs upper"); return; }
    const int N = *n, ld = *lda;
    for (int r = 0; r < *nrhs; r++)
    {
        double* x = b + (size_t)r * *ldb;
        for (int i = 0; i < N; i++)
        {
            double t = x[i];
            for (int k = 0; k < i; k++)
                t -= a[i + k * ld] * x[k];
            x[i] = t / a[i + i * ld];
        }
        for (int i = N - 1; i >= 0; i--)
        {
            double t = x[i];
            for (int k = i + 1; k < N; k++)
                t -= a[k + i * ld] * x[k];
            x[i] = t / a[i + i * ld];
        }
    }
}

/* DSYEV with jobz 'N': eigenvalues (ascending) of the symmetric matrix in
 * the lower triangle of a, by cyclic Jacobi rotations (LAPACK reduces to
 * tridiagonal form and iterates; the eigenvalues agree to rounding) */
void oracle_dsyev(const char* jobz, const char* uplo, const int* n, double* a, const int* lda,
    double* w, double* work, const int* lwork, int* info)
{
    (void)work;
    (void)lwork;
    *info = 0;
    if (!(*jobz == 'n' || *jobz == 'N') || !(*uplo == 'l' || *uplo == 'L'))
    {
        oracle_blas_unused("dsyev with vectors or upper");
        return;
    }
    const int N = *n, ld = *lda;
    std::vector<double> A((size_t)N * N);
    for (int j = 0; j < N; j++)
        for (int i = j; i < N; i++)
            A[i + (size_t)j * N] = A[j + (size_t)i * N] = a[i + j * ld];
    for (int sweep = 0; sweep < 100; sweep++)
    {
        double off = 0., tot = 0.;
        for (size_t t = 0; t < A.size(); t++)
        {
            tot += A[t] * A[t];
            if (t % N != t / N) off += A[t] * A[t];
        }
        if (off == 0. || off <= 1e-30 * tot) break;
        for (int p = 0; p < N - 1; p++)
            for (int q = p + 1; q < N; q++)
            {
                const double apq = A[p + (size_t)q * N];
                if (apq == 0.) continue;
                const double tau = (A[q + (size_t)q * N] - A[p + (size_t)p * N]) / (2. * apq);
                const double t = (tau >= 0. ? 1. : -1.) / (std::fabs(tau) + std::sqrt(1. + tau * tau));
                const double c = 1. / std::sqrt(1. + t * t), sn = t * c;
                for (int r = 0; r < N; r++)
                {
                    const double arp = A[r + (size_t)p * N], arq = A[r + (size_t)q * N];
                    A[r + (size_t)p * N] = c * arp - sn * arq;
                    A[r + (size_t)q * N] = sn * arp + c * arq;
                }
                for (int r = 0; r < N; r++)
                {
                    const double apr = A[p + (size_t)r * N], aqr = A[q + (size_t)r * N];
                    A[p + (size_t)r * N] = c * apr - sn * aqr;
                    A[q + (size_t)r * N] = sn * apr + c * aqr;
                }
            }
    }
    for (int i = 0; i < N; i++)
        w[i] = A[i + (size_t)i * N];
    std::sort(w, w + N);
}
}
