/* Forwarders from the LAPACK/CBLAS names the reference calls to the
 * prefixed entry points of the OpenBLAS bundled with scipy (oracle build
 * only).  The library path is given at link time. */
#include <stddef.h>
extern void scipy_dspev_(const char*, const char*, const int*, double*, double*, double*, const int*, double*, int*, size_t, size_t);
extern void scipy_dsyev_(const char*, const char*, const int*, double*, const int*, double*, double*, const int*, int*, size_t, size_t);
extern void scipy_zhpev_(const char*, const char*, const int*, void*, double*, void*, const int*, void*, double*, int*, size_t, size_t);
extern void scipy_zheev_(const char*, const char*, const int*, void*, const int*, double*, void*, const int*, double*, int*, size_t, size_t);
extern void scipy_dgesv_(const int*, const int*, double*, const int*, int*, double*, const int*, int*);
extern void scipy_cblas_dgemm(int, int, int, int, int, int, double, const double*, int, const double*, int, double, double*, int);
extern void scipy_cblas_zgemm(int, int, int, int, int, int, const void*, const void*, int, const void*, int, const void*, void*, int);

void dspev_(const char* jobz, const char* uplo, const int* n, double* ap, double* w, double* z,
            const int* ldz, double* work, int* info) {
  scipy_dspev_(jobz, uplo, n, ap, w, z, ldz, work, info, 1, 1);
}
void dsyev_(const char* jobz, const char* uplo, const int* n, double* a, const int* lda, double* w,
            double* work, const int* lwork, int* info) {
  scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info, 1, 1);
}
void zhpev_(const char* jobz, const char* uplo, const int* n, void* ap, double* w, void* z,
            const int* ldz, void* work, double* rwork, int* info) {
  scipy_zhpev_(jobz, uplo, n, ap, w, z, ldz, work, rwork, info, 1, 1);
}
void zheev_(const char* jobz, const char* uplo, const int* n, void* a, const int* lda, double* w,
            void* work, const int* lwork, double* rwork, int* info) {
  scipy_zheev_(jobz, uplo, n, a, lda, w, work, lwork, rwork, info, 1, 1);
}
void dgesv_(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv, double* b,
            const int* ldb, int* info) {
  scipy_dgesv_(n, nrhs, a, lda, ipiv, b, ldb, info);
}
void cblas_dgemm(int o, int ta, int tb, int m, int n, int k, double alpha, const double* a, int lda,
                 const double* b, int ldb, double beta, double* c, int ldc) {
  scipy_cblas_dgemm(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
void cblas_zgemm(int o, int ta, int tb, int m, int n, int k, const void* alpha, const void* a, int lda,
                 const void* b, int ldb, const void* beta, void* c, int ldc) {
  scipy_cblas_zgemm(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
