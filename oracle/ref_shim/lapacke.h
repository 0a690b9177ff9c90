/* LAPACKE declarations mapped onto the SciPy-bundled OpenBLAS exports
 * (see cblas.h in this folder).  Test infrastructure only. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
int scipy_LAPACKE_dsyev(int layout, char jobz, char uplo, int n, double *a,
                        int lda, double *w);
int scipy_LAPACKE_dgeqrf(int layout, int m, int n, double *a, int lda, double *tau);
int scipy_LAPACKE_dorgqr(int layout, int m, int n, int k, double *a, int lda,
                         const double *tau);
#ifdef __cplusplus
}
#endif
#define LAPACKE_dsyev scipy_LAPACKE_dsyev
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
