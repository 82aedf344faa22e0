/* dgemm_ for the reference's Fortran-BLAS path (localcontract.cc, -DHOPPER),
 * forwarded to the ILP64 OpenBLAS that numpy bundles (symbol scipy_dgemm_64_).
 * Test infrastructure for oracle/_ref only. */
#include <cstdint>
extern "C" void scipy_dgemm_64_(const char*, const char*, const int64_t*, const int64_t*, const int64_t*,
                                const double*, const double*, const int64_t*, const double*, const int64_t*,
                                const double*, double*, const int64_t*, int, int);
extern "C" void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* alpha, double* a, int* lda,
                       double* b, int* ldb, double* beta, double* c, int* ldc) {
  int64_t M = *m, N = *n, K = *k, LDA = *lda, LDB = *ldb, LDC = *ldc;
  scipy_dgemm_64_(ta, tb, &M, &N, &K, alpha, a, &LDA, b, &LDB, beta, c, &LDC, 1, 1);
}
