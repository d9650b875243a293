/* Oracle shim (test infrastructure only): the four CBLAS routines the
 * reference's user kernels call (src/euler_rhs.h:240-243,285;
 * src/init_grid.h:20-65), as plain sequential loops.
 *
 * The reference links OpenBLAS (unpinned version, CMakeLists.txt:9-34),
 * which is absent here.  This shim fixes the summation order of dgemv to
 * ascending column index; the oracle restatement uses the same order, so
 * the two agree bit for bit when given the same operator tables.  OpenBLAS's
 * own blocking may change results at the rounding level only. */
#ifndef ORACLE_SHIM_CBLAS_H
#define ORACLE_SHIM_CBLAS_H

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112 };

static inline void cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, int m, int n,
                               double alpha, const double *a, int lda, const double *x, int incx,
                               double beta, double *y, int incy) {
  (void)order; (void)trans; /* only RowMajor/NoTrans is used by the reference */
  for (int i = 0; i < m; i++) {
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += a[i * lda + j] * x[j * incx];
    if (beta == 0.0) y[i * incy] = alpha * acc;
    else y[i * incy] = alpha * acc + beta * y[i * incy];
  }
}

static inline void cblas_dcopy(int n, const double *x, int incx, double *y, int incy) {
  for (int i = 0; i < n; i++) y[i * incy] = x[i * incx];
}

static inline void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy) {
  for (int i = 0; i < n; i++) y[i * incy] = y[i * incy] + alpha * x[i * incx];
}

static inline void cblas_dscal(int n, double alpha, double *x, int incx) {
  for (int i = 0; i < n; i++) x[i * incx] = alpha * x[i * incx];
}

#endif
