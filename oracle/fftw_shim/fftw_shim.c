/* FP64 FFT implementing the FFTW-3 subset declared in fftw3.h.
 *
 * TEST INFRASTRUCTURE ONLY.  Written from the DFT definition
 * X[k] = sum_n x[n] exp(sign * 2 pi i k n / N): iterative radix-2
 * Cooley-Tukey (bit-reversal permutation, then log2 N butterfly passes) for
 * power-of-two N, the direct O(N^2) sum otherwise.  2-D transforms run the 1-D
 * transform over rows then columns.  Thread-safe: plans own their scratch. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

enum { K_C2C = 0, K_R2C = 1, K_C2R = 2 };

struct litho_fftw_plan_s {
  int kind, n0, n1, sign;
  void* in;
  void* out;
  double* work; /* n0*n1 complex */
  double* line; /* max(n0,n1) complex */
};

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static void fft1d(double* v, int n, int sign, double* tmp) {
  if (n <= 1) return;
  if (!is_pow2(n)) {
    for (int k = 0; k < n; ++k) {
      double re = 0.0, im = 0.0;
      for (int j = 0; j < n; ++j) {
        const double a = sign * 2.0 * M_PI * (double)((long long)k * j % n) / (double)n;
        const double c = cos(a), s = sin(a);
        re += v[2 * j] * c - v[2 * j + 1] * s;
        im += v[2 * j] * s + v[2 * j + 1] * c;
      }
      tmp[2 * k] = re;
      tmp[2 * k + 1] = im;
    }
    memcpy(v, tmp, sizeof(double) * 2 * n);
    return;
  }
  for (int i = 1, j = 0; i < n; ++i) { /* bit reversal */
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t0 = v[2 * i], t1 = v[2 * i + 1];
      v[2 * i] = v[2 * j];
      v[2 * i + 1] = v[2 * j + 1];
      v[2 * j] = t0;
      v[2 * j + 1] = t1;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int h = len / 2;
    for (int k = 0; k < h; ++k) {
      const double a = sign * 2.0 * M_PI * (double)k / (double)len;
      const double wr = cos(a), wi = sin(a);
      for (int s = 0; s < n; s += len) {
        double* p = v + 2 * (s + k);
        double* q = v + 2 * (s + k + h);
        const double tr = q[0] * wr - q[1] * wi, ti = q[0] * wi + q[1] * wr;
        q[0] = p[0] - tr;
        q[1] = p[1] - ti;
        p[0] += tr;
        p[1] += ti;
      }
    }
  }
}

static void fft2d(double* a, int n0, int n1, int sign, double* line) {
  double* tmp = line + 2 * (n0 > n1 ? n0 : n1);
  for (int r = 0; r < n0; ++r) fft1d(a + 2 * (size_t)r * n1, n1, sign, tmp);
  for (int c = 0; c < n1; ++c) {
    for (int r = 0; r < n0; ++r) {
      line[2 * r] = a[2 * ((size_t)r * n1 + c)];
      line[2 * r + 1] = a[2 * ((size_t)r * n1 + c) + 1];
    }
    fft1d(line, n0, sign, tmp);
    for (int r = 0; r < n0; ++r) {
      a[2 * ((size_t)r * n1 + c)] = line[2 * r];
      a[2 * ((size_t)r * n1 + c) + 1] = line[2 * r + 1];
    }
  }
}

static fftw_plan mk(int kind, int n0, int n1, int sign, void* in, void* out) {
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  p->kind = kind;
  p->n0 = n0;
  p->n1 = n1;
  p->sign = sign;
  p->in = in;
  p->out = out;
  p->work = (double*)malloc(sizeof(double) * 2 * (size_t)n0 * n1);
  const int m = n0 > n1 ? n0 : n1;
  p->line = (double*)malloc(sizeof(double) * 4 * (size_t)m);
  return p;
}

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags) {
  (void)flags;
  return mk(K_C2C, n0, n1, sign, in, out);
}
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags) {
  (void)flags;
  return mk(K_R2C, n0, n1, FFTW_FORWARD, in, out);
}
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags) {
  (void)flags;
  return mk(K_C2R, n0, n1, FFTW_BACKWARD, in, out);
}

static void run(const fftw_plan p, void* in, void* out) {
  const int n0 = p->n0, n1 = p->n1, wt = n1 / 2 + 1;
  double* w = p->work;
  const size_t nn = (size_t)n0 * n1;
  if (p->kind == K_C2C) {
    memcpy(w, in, sizeof(double) * 2 * nn);
    fft2d(w, n0, n1, p->sign, p->line);
    memcpy(out, w, sizeof(double) * 2 * nn);
  } else if (p->kind == K_R2C) {
    const double* r = (const double*)in;
    for (size_t i = 0; i < nn; ++i) {
      w[2 * i] = r[i];
      w[2 * i + 1] = 0.0;
    }
    fft2d(w, n0, n1, FFTW_FORWARD, p->line);
    double* o = (double*)out;
    for (int a = 0; a < n0; ++a)
      for (int b = 0; b < wt; ++b) {
        o[2 * ((size_t)a * wt + b)] = w[2 * ((size_t)a * n1 + b)];
        o[2 * ((size_t)a * wt + b) + 1] = w[2 * ((size_t)a * n1 + b) + 1];
      }
  } else {
    /* Hermitian completion of the half spectrum, complex inverse, real part */
    const double* h = (const double*)in;
    for (int a = 0; a < n0; ++a)
      for (int b = 0; b < n1; ++b) {
        double re, im;
        if (b < wt) {
          re = h[2 * ((size_t)a * wt + b)];
          im = h[2 * ((size_t)a * wt + b) + 1];
        } else {
          const int a2 = (n0 - a) % n0, b2 = n1 - b;
          re = h[2 * ((size_t)a2 * wt + b2)];
          im = -h[2 * ((size_t)a2 * wt + b2) + 1];
        }
        w[2 * ((size_t)a * n1 + b)] = re;
        w[2 * ((size_t)a * n1 + b) + 1] = im;
      }
    fft2d(w, n0, n1, FFTW_BACKWARD, p->line);
    double* o = (double*)out;
    for (size_t i = 0; i < nn; ++i) o[i] = w[2 * i];
  }
}

void fftw_execute(const fftw_plan p) { run(p, p->in, p->out); }
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) { run(p, in, out); }
void fftw_destroy_plan(fftw_plan p) {
  if (!p) return;
  free(p->work);
  free(p->line);
  free(p);
}
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftw_cleanup_threads(void) {}
