/* zheevr_ -> scipy_zheevr_ (LAPACK zheevr as exported by scipy's bundled
 * OpenBLAS).  TEST INFRASTRUCTURE ONLY: lets the reference's litho.cpp link
 * its eigensolver call (litho.cpp:572-577) without a system LAPACK.  The
 * character arguments are passed by address as the Fortran ABI expects. */
typedef struct { double re, im; } zc;
extern void scipy_zheevr_(const char* jobz, const char* range, const char* uplo, int* n, zc* a, int* lda,
                          double* vl, double* vu, int* il, int* iu, double* abstol, int* m, double* w, zc* z,
                          int* ldz, int* isuppz, zc* work, int* lwork, double* rwork, int* lrwork, int* iwork,
                          int* liwork, int* info, unsigned long l1, unsigned long l2, unsigned long l3);
void zheevr_(const char* jobz, const char* range, const char* uplo, int* n, zc* a, int* lda, double* vl,
             double* vu, int* il, int* iu, double* abstol, int* m, double* w, zc* z, int* ldz, int* isuppz,
             zc* work, int* lwork, double* rwork, int* lrwork, int* iwork, int* liwork, int* info) {
  scipy_zheevr_(jobz, range, uplo, n, a, lda, vl, vu, il, iu, abstol, m, w, z, ldz, isuppz, work, lwork, rwork,
                lrwork, iwork, liwork, info, 1, 1, 1);
}
