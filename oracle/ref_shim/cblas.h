/* Test-infrastructure header: maps the CBLAS names the reference calls onto
 * the prefixed exports of the OpenBLAS build that ships inside scipy
 * (scipy.libs/libscipy_openblas-*.so, LP64).  Only the reference oracle
 * (oracle/_ref) is compiled against it. */
#ifndef CORR_ORACLE_CBLAS_SHIM_H
#define CORR_ORACLE_CBLAS_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;

void scipy_cblas_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, int, int, int,
                       double, const double*, int, const double*, int, double, double*, int);
void scipy_cblas_dsbmv(enum CBLAS_ORDER, enum CBLAS_UPLO, int, int, double, const double*, int,
                       const double*, int, double, double*, int);
double scipy_cblas_ddot(int, const double*, int, const double*, int);
void scipy_cblas_dscal(int, double, double*, int);
void scipy_cblas_daxpy(int, double, const double*, int, double*, int);

#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dsbmv scipy_cblas_dsbmv
#define cblas_ddot scipy_cblas_ddot
#define cblas_dscal scipy_cblas_dscal
#define cblas_daxpy scipy_cblas_daxpy

#ifdef __cplusplus
}
#endif
#endif
