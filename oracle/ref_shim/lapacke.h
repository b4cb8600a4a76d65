/* Test-infrastructure header: LAPACKE_dsyev for the reference oracle, mapped
 * onto scipy's bundled OpenBLAS export (see cblas.h in this folder). */
#ifndef CORR_ORACLE_LAPACKE_SHIM_H
#define CORR_ORACLE_LAPACKE_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

int scipy_LAPACKE_dsyev(int matrix_layout, char jobz, char uplo, int n, double* a, int lda,
                        double* w);
#define LAPACKE_dsyev scipy_LAPACKE_dsyev

#ifdef __cplusplus
}
#endif
#endif
