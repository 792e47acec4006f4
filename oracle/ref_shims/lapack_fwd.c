/* Fortran-ABI LAPACK/BLAS entry points the reference sources call
 * (zheev_, zgeev_, dgeev_, zgemm_, zaxpy_), forwarded to the scipy_-prefixed
 * exports of the OpenBLAS that ships inside scipy (32-bit integers).
 * Written for this project; used only to link the reference as an oracle. */
#include <complex.h>


extern void scipy_zheev_(const char*, const char*, const int*, double complex*, const int*, double*,
                         double complex*, const int*, double*, int*);
extern void scipy_zgeev_(const char*, const char*, const int*, double complex*, const int*, double complex*,
                         double complex*, const int*, double complex*, const int*, double complex*, const int*,
                         double*, int*);
extern void scipy_dgeev_(const char*, const char*, const int*, double*, const int*, double*, double*, double*,
                         const int*, double*, const int*, double*, const int*, int*);
extern void scipy_zgemm_(const char*, const char*, const int*, const int*, const int*, const double complex*,
                         const double complex*, const int*, const double complex*, const int*,
                         const double complex*, double complex*, const int*);
extern void scipy_zaxpy_(const int*, const double complex*, const double complex*, const int*, double complex*,
                         const int*);

void zheev_(const char* jobz, const char* uplo, const int* n, double complex* a, const int* lda, double* w,
            double complex* work, const int* lwork, double* rwork, int* info) {
  scipy_zheev_(jobz, uplo, n, a, lda, w, work, lwork, rwork, info);
}
void zgeev_(const char* jobvl, const char* jobvr, const int* n, double complex* a, const int* lda,
            double complex* w, double complex* vl, const int* ldvl, double complex* vr, const int* ldvr,
            double complex* work, const int* lwork, double* rwork, int* info) {
  scipy_zgeev_(jobvl, jobvr, n, a, lda, w, vl, ldvl, vr, ldvr, work, lwork, rwork, info);
}
void dgeev_(const char* jobvl, const char* jobvr, const int* n, double* a, const int* lda, double* wr, double* wi,
            double* vl, const int* ldvl, double* vr, const int* ldvr, double* work, const int* lwork, int* info) {
  scipy_dgeev_(jobvl, jobvr, n, a, lda, wr, wi, vl, ldvl, vr, ldvr, work, lwork, info);
}
void zgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const double complex* alpha,
            const double complex* a, const int* lda, const double complex* b, const int* ldb,
            const double complex* beta, double complex* c, const int* ldc) {
  scipy_zgemm_(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
void zaxpy_(const int* n, const double complex* a, const double complex* x, const int* incx, double complex* y,
            const int* incy) {
  scipy_zaxpy_(n, a, x, incx, y, incy);
}
