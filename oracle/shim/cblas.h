/* CBLAS declarations for the oracle build of the reference optimizer.
 *
 * Test infrastructure only. The reference headers call cblas_zgemm /
 * cblas_zgemv (pngf-opt/pngfopt.hpp:324-358, pngf-opt/linalg.hpp:23-31).
 * No system CBLAS is installed, so these names are bound to the LP64
 * OpenBLAS that scipy bundles, whose exported symbols carry a "scipy_"
 * prefix. The enum values are the standard CBLAS ones.
 */
#ifndef PNGF_ORACLE_CBLAS_SHIM_H
#define PNGF_ORACLE_CBLAS_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

void scipy_cblas_zgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                       int m, int n, int k, const void *alpha, const void *a, int lda,
                       const void *b, int ldb, const void *beta, void *c, int ldc);
void scipy_cblas_zgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, int m, int n,
                       const void *alpha, const void *a, int lda, const void *x, int incx,
                       const void *beta, void *y, int incy);
void scipy_zgetrf_(int *m, int *n, void *a, int *lda, int *ipiv, int *info);
void scipy_zgetri_(int *n, void *a, int *lda, int *ipiv, void *work, int *lwork, int *info);
void scipy_zgetrs_(char *trans, int *n, int *nrhs, void *a, int *lda, int *ipiv, void *b,
                   int *ldb, int *info);
void scipy_openblas_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#define cblas_zgemm scipy_cblas_zgemm
#define cblas_zgemv scipy_cblas_zgemv
#define zgetrf_ scipy_zgetrf_
#define zgetri_ scipy_zgetri_
#define zgetrs_ scipy_zgetrs_

#endif
