/*
 * Plain-loop BLAS level-1/3 routines with the reference BLAS's semantics
 * and summation order, for the oracle's pinning build of the reference
 * (test infrastructure only).  Routines that the hot path never reaches
 * abort if called.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>

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
void oracle_dpotrf() { oracle_blas_unused("dpotrf"); }
void oracle_dpotrs() { oracle_blas_unused("dpotrs"); }
void oracle_dpotri() { oracle_blas_unused("dpotri"); }
void oracle_dsyev() { oracle_blas_unused("dsyev"); }
}
