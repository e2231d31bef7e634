/* ORACLE build support — test infrastructure only.
 *
 * SQUANDER's C++ sources call a handful of CBLAS/LAPACKE routines (32-bit integer
 * interface).  The reference's CI links the distribution's OpenBLAS; this file forwards
 * the same calls to the OpenBLAS build that ships inside numpy (64-bit integer
 * interface, symbols prefixed "scipy_" and suffixed "64_"), so that the reference's
 * zgemm-based derivative path runs on OpenBLAS as it does upstream.
 */
#include <cstdint>

typedef int64_t ilp64;

extern "C" {
void scipy_cblas_zgemm64_(int order, int ta, int tb, ilp64 m, ilp64 n, ilp64 k, const void* alpha,
                          const void* a, ilp64 lda, const void* b, ilp64 ldb, const void* beta, void* c,
                          ilp64 ldc);
void scipy_cblas_cgemm64_(int order, int ta, int tb, ilp64 m, ilp64 n, ilp64 k, const void* alpha,
                          const void* a, ilp64 lda, const void* b, ilp64 ldb, const void* beta, void* c,
                          ilp64 ldc);
double scipy_cblas_dznrm264_(ilp64 n, const void* x, ilp64 incx);
ilp64 scipy_LAPACKE_zgesdd64_(int layout, char jobz, ilp64 m, ilp64 n, void* a, ilp64 lda, double* s, void* u,
                              ilp64 ldu, void* vt, ilp64 ldvt);
ilp64 scipy_LAPACKE_cgesdd64_(int layout, char jobz, ilp64 m, ilp64 n, void* a, ilp64 lda, float* s, void* u,
                              ilp64 ldu, void* vt, ilp64 ldvt);
void scipy_openblas_set_num_threads64_(int n);

void cblas_zgemm(int order, int ta, int tb, int m, int n, int k, const void* alpha, const void* a, int lda,
                 const void* b, int ldb, const void* beta, void* c, int ldc) {
    scipy_cblas_zgemm64_(order, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void cblas_cgemm(int order, int ta, int tb, int m, int n, int k, const void* alpha, const void* a, int lda,
                 const void* b, int ldb, const void* beta, void* c, int ldc) {
    scipy_cblas_cgemm64_(order, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

double cblas_dznrm2(long n, const void* x, long incx) { return scipy_cblas_dznrm264_(n, x, incx); }

int LAPACKE_zgesdd(int layout, char jobz, int m, int n, void* a, int lda, double* s, void* u, int ldu, void* vt,
                   int ldvt) {
    return (int)scipy_LAPACKE_zgesdd64_(layout, jobz, m, n, a, lda, s, u, ldu, vt, ldvt);
}

int LAPACKE_cgesdd(int layout, char jobz, int m, int n, void* a, int lda, float* s, void* u, int ldu, void* vt,
                   int ldvt) {
    return (int)scipy_LAPACKE_cgesdd64_(layout, jobz, m, n, a, lda, s, u, ldu, vt, ldvt);
}

/* exposed to the driver: OpenBLAS's own thread count (1 keeps runs reproducible) */
void sqgr_blas_threads(int n) { scipy_openblas_set_num_threads64_(n); }
}
