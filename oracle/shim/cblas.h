/* Minimal CBLAS declarations for building the reference solver against the
 * "scipy_"-prefixed CBLAS symbols of scipy's bundled OpenBLAS.  Test infrastructure. */
#ifndef ORACLE_SHIM_CBLAS_H
#define ORACLE_SHIM_CBLAS_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void scipy_cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                       int m, int n, int k, double alpha, const double* a, int lda,
                       const double* b, int ldb, double beta, double* c, int ldc);
#ifdef __cplusplus
}
#endif
#define cblas_dgemm scipy_cblas_dgemm
#endif
