/* Build-time shim: standard CBLAS prototypes routed to scipy's OpenBLAS names.
 * Used only by oracle/build_ref.sh. */
#pragma once
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
extern "C" {
void scipy_cblas_dgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int m, int n, int k,
                       double alpha, const double *a, int lda, const double *b, int ldb,
                       double beta, double *c, int ldc);
void scipy_cblas_zgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int m, int n, int k,
                       const void *alpha, const void *a, int lda, const void *b, int ldb,
                       const void *beta, void *c, int ldc);
}
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_zgemm scipy_cblas_zgemm
