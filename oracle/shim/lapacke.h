/* Build-time shim for compiling the reference's headers as the oracle.
 * Declares the standard LAPACKE entry points the reference calls and routes
 * them to the symbol names exported by scipy's bundled OpenBLAS (LP64).
 * Used only by oracle/build_ref.sh; never linked into the product. */
#pragma once
#include <complex>
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
typedef int lapack_int;
extern "C" {
lapack_int scipy_LAPACKE_dsyevd(int layout, char jobz, char uplo, lapack_int n,
                                double *a, lapack_int lda, double *w);
lapack_int scipy_LAPACKE_zheevd(int layout, char jobz, char uplo, lapack_int n,
                                std::complex<double> *a, lapack_int lda, double *w);
lapack_int scipy_LAPACKE_zgeev(int layout, char jobvl, char jobvr, lapack_int n,
                               std::complex<double> *a, lapack_int lda,
                               std::complex<double> *w, std::complex<double> *vl,
                               lapack_int ldvl, std::complex<double> *vr, lapack_int ldvr);
lapack_int scipy_LAPACKE_dgeev(int layout, char jobvl, char jobvr, lapack_int n,
                               double *a, lapack_int lda, double *wr, double *wi,
                               double *vl, lapack_int ldvl, double *vr, lapack_int ldvr);
}
#define LAPACKE_dsyevd scipy_LAPACKE_dsyevd
#define LAPACKE_zheevd scipy_LAPACKE_zheevd
#define LAPACKE_zgeev scipy_LAPACKE_zgeev
#define LAPACKE_dgeev scipy_LAPACKE_dgeev
