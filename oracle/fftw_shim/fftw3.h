/* fftw3.h -- a minimal FFTW-3 API for building the reference's litho.cpp here.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle's build of the reference program).
 * Declares the subset of the FFTW-3 double-precision API that
 * validation/golden/src/litho.cpp and litho_thread.cpp call; fftw_shim.c
 * implements it with a project-written FP64 FFT.  Contract kept from FFTW:
 * unnormalised transforms, FFTW_FORWARD = e^{-i}, FFTW_BACKWARD = e^{+i},
 * r2c output of size n0 x (n1/2+1), c2r reading that half spectrum as the
 * non-redundant half of a Hermitian array. */
#ifndef LITHO_ORACLE_FFTW_SHIM_H
#define LITHO_ORACLE_FFTW_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct litho_fftw_plan_s* fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
#ifdef __cplusplus
}
#endif
#endif
