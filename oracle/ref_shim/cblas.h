/* CBLAS declarations for building the reference C++ sources against the
 * OpenBLAS that ships inside the SciPy wheel (its exported names carry a
 * `scipy_` prefix).  Test infrastructure only: used to compile the oracle
 * module under oracle/_ref, never linked into the product. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };

void scipy_cblas_dsyrk(enum CBLAS_ORDER, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE,
                       int n, int k, double alpha, const double *a, int lda,
                       double beta, double *c, int ldc);
void scipy_cblas_dsymv(enum CBLAS_ORDER, enum CBLAS_UPLO, int n, double alpha,
                       const double *a, int lda, const double *x, int incx,
                       double beta, double *y, int incy);
void scipy_cblas_dgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, int m, int n,
                       double alpha, const double *a, int lda, const double *x,
                       int incx, double beta, double *y, int incy);
void scipy_cblas_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                       int m, int n, int k, double alpha, const double *a, int lda,
                       const double *b, int ldb, double beta, double *c, int ldc);
void scipy_cblas_dsymm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO, int m,
                       int n, double alpha, const double *a, int lda,
                       const double *b, int ldb, double beta, double *c, int ldc);
void scipy_openblas_set_num_threads(int);
#ifdef __cplusplus
}
#endif
#define cblas_dsyrk scipy_cblas_dsyrk
#define cblas_dsymv scipy_cblas_dsymv
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dsymm scipy_cblas_dsymm
