/* CBLAS shim for the oracle's build of the reference (test infrastructure).
 * With OPENBLAS64 defined it forwards to an ILP64 OpenBLAS that exports
 * scipy_cblas_* symbols (the copy bundled with numpy); otherwise it runs plain
 * loops, which are fine for the small indexes the fixtures use. k-means only
 * shapes the partition; search parity is defined over the written index files,
 * so the BLAS used here does not affect any parity claim. */
#include "cblas.h"
#include <stdint.h>

#ifdef OPENBLAS64
void scipy_cblas_sgemm64_(int order, int ta, int tb, int64_t m, int64_t n, int64_t k,
                          float alpha, const float *a, int64_t lda, const float *b,
                          int64_t ldb, float beta, float *c, int64_t ldc);
float scipy_cblas_sdot64_(int64_t n, const float *x, int64_t incx, const float *y,
                          int64_t incy);

void cblas_sgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                 int m, int n, int k, float alpha, const float *a, int lda,
                 const float *b, int ldb, float beta, float *c, int ldc) {
  scipy_cblas_sgemm64_(order, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
float cblas_sdot(int n, const float *x, int incx, const float *y, int incy) {
  return scipy_cblas_sdot64_(n, x, incx, y, incy);
}
#else
/* Row-major only, which is all the reference uses. */
void cblas_sgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                 int m, int n, int k, float alpha, const float *a, int lda,
                 const float *b, int ldb, float beta, float *c, int ldc) {
  (void)order;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      float s = 0.0f;
      for (int t = 0; t < k; ++t) {
        const float av = ta == CblasNoTrans ? a[(int64_t)i * lda + t] : a[(int64_t)t * lda + i];
        const float bv = tb == CblasNoTrans ? b[(int64_t)t * ldb + j] : b[(int64_t)j * ldb + t];
        s += av * bv;
      }
      c[(int64_t)i * ldc + j] = alpha * s + (beta == 0.0f ? 0.0f : beta * c[(int64_t)i * ldc + j]);
    }
}
float cblas_sdot(int n, const float *x, int incx, const float *y, int incy) {
  float s = 0.0f;
  for (int i = 0; i < n; ++i) s += x[(int64_t)i * incx] * y[(int64_t)i * incy];
  return s;
}
#endif
