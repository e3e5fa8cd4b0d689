/* Minimal LAPACKE declarations for building the reference solver against the
 * LAPACKE symbols exported (with a "scipy_" prefix) by scipy's bundled OpenBLAS.
 * Only the routines the reference calls are declared.  Test infrastructure. */
#ifndef ORACLE_SHIM_LAPACKE_H
#define ORACLE_SHIM_LAPACKE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int scipy_LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv);
lapack_int scipy_LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda, const lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int scipy_LAPACKE_dgecon(int layout, char norm, lapack_int n, const double* a, lapack_int lda, double anorm, double* rcond);
lapack_int scipy_LAPACKE_dgeqp3(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* jpvt, double* tau);
lapack_int scipy_LAPACKE_dtrtrs(int layout, char uplo, char trans, char diag, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda, double* b, lapack_int ldb);
lapack_int scipy_LAPACKE_dgeev(int layout, char jobvl, char jobvr, lapack_int n, double* a, lapack_int lda, double* wr, double* wi, double* vl, lapack_int ldvl, double* vr, lapack_int ldvr);
lapack_int scipy_LAPACKE_dgesvd(int layout, char jobu, char jobvt, lapack_int m, lapack_int n, double* a, lapack_int lda, double* s, double* u, lapack_int ldu, double* vt, lapack_int ldvt, double* superb);
void scipy_openblas_set_num_threads(int n);
#ifdef __cplusplus
}
#endif
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_dgetrs scipy_LAPACKE_dgetrs
#define LAPACKE_dgecon scipy_LAPACKE_dgecon
#define LAPACKE_dgeqp3 scipy_LAPACKE_dgeqp3
#define LAPACKE_dtrtrs scipy_LAPACKE_dtrtrs
#define LAPACKE_dgeev scipy_LAPACKE_dgeev
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#endif
