/* Minimal CBLAS declarations for building the reference's k-means (which
 * includes <cblas.h>) in an image that has no OpenBLAS headers. Only the two
 * routines the reference calls are declared; cblas_shim.c implements them.
 * Test infrastructure: used only to build the oracle's copy of the reference. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void cblas_sgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                 int m, int n, int k, float alpha, const float *a, int lda,
                 const float *b, int ldb, float beta, float *c, int ldc);
float cblas_sdot(int n, const float *x, int incx, const float *y, int incy);
#ifdef __cplusplus
}
#endif
