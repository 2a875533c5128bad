/*
 * or_fft.c -- ORACLE (test infrastructure only; never part of the product
 * path).  FP64 3-D real transforms with FFTW's unnormalised conventions,
 * standing in for fftw_plan_dft_c2r_3d / fftw_plan_dft_r2c_3d
 * (fourier.c:81-125):
 *   c2r: x[n] = sum_k X[k] e^{+2 pi i k.n/N}, complex transforms along z and
 *        y, then a length-N real inverse along x that ignores the imaginary
 *        parts of the DC and Nyquist terms (FFTW's c2r semantics);
 *   r2c: X[k] = sum_n x[n] e^{-2 pi i k.n/N} for kx in [0, N/2].
 * Half spectra are [kz][ky][kx] with kx in [0, N/2] fastest; real grids
 * are unpadded [z][y][x].  Line lengths are 2^a 3^b (Stockham autosort,
 * radices 4, 2, 3, twiddles from libm in double).
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
  int n, nrad, rad[64];
  double complex *tw; /* e^{+2 pi i j/n} */
} plan1d;

static int plan_make(plan1d *p, int n)
{
  p->n = n;
  p->nrad = 0;
  int m = n;
  while (m % 4 == 0) p->rad[p->nrad++] = 4, m /= 4;
  while (m % 2 == 0) p->rad[p->nrad++] = 2, m /= 2;
  while (m % 3 == 0) p->rad[p->nrad++] = 3, m /= 3;
  if (m != 1) return -1;
  p->tw = malloc(n * sizeof(double complex));
  for (int j = 0; j < n; j++) p->tw[j] = cos(2 * M_PI * j / n) + I * sin(2 * M_PI * j / n);
  return 0;
}

static void plan_free(plan1d *p) { free(p->tw); }

/* In-place 1-D transform of x (length n, work w), sign +1 or -1. */
static void fft1d(const plan1d *p, double complex *x, double complex *w, int sign)
{
  const int L = p->n;
  int Ns = 1;
  double complex *a = x, *b = w;
  for (int s = 0; s < p->nrad; s++) {
    const int r = p->rad[s];
    for (int bI = 0; bI < L / r; bI++) {
      int k = bI % Ns;
      double complex v[4];
      for (int q = 0; q < r; q++) {
        double complex t = a[bI + q * (L / r)];
        int j = (q * k) * (L / (Ns * r));
        double complex tw = p->tw[j % L];
        v[q] = t * (sign > 0 ? tw : conj(tw));
      }
      double complex o[4];
      if (r == 2) {
        o[0] = v[0] + v[1];
        o[1] = v[0] - v[1];
      } else if (r == 4) {
        double complex s0 = v[0] + v[2], s1 = v[0] - v[2], s2 = v[1] + v[3];
        double complex s3 = (v[1] - v[3]) * (sign > 0 ? I : -I);
        o[0] = s0 + s2;
        o[2] = s0 - s2;
        o[1] = s1 + s3;
        o[3] = s1 - s3;
      } else {
        double complex w1 = cos(2 * M_PI / 3) + sign * I * sin(2 * M_PI / 3);
        o[0] = v[0] + v[1] + v[2];
        o[1] = v[0] + w1 * v[1] + w1 * w1 * v[2];
        o[2] = v[0] + w1 * w1 * v[1] + w1 * v[2];
      }
      int base = (bI / Ns) * Ns * r + k;
      for (int q = 0; q < r; q++) b[base + q * Ns] = o[q];
    }
    double complex *t = a;
    a = b;
    b = t;
    Ns *= r;
  }
  if (a != x) memcpy(x, a, L * sizeof(double complex));
}

int or_c2r_3d(int N, const double complex *in, double *out)
{
  const int NH = N / 2 + 1;
  plan1d p;
  if (plan_make(&p, N)) return -1;
  double complex *c = malloc((size_t)N * N * NH * sizeof(double complex));
  if (!c) return -2;
  memcpy(c, in, (size_t)N * N * NH * sizeof(double complex));
  /* z lines */
#pragma omp parallel
  {
    double complex *line = malloc(N * sizeof(double complex)), *wk = malloc(N * sizeof(double complex));
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * NH; q++) {
      for (int z = 0; z < N; z++) line[z] = c[(size_t)z * N * NH + q];
      fft1d(&p, line, wk, +1);
      for (int z = 0; z < N; z++) c[(size_t)z * N * NH + q] = line[z];
    }
    /* y lines */
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * NH; q++) {
      long z = q / NH, kx = q % NH;
      double complex *base = c + (size_t)z * N * NH + kx;
      for (int y = 0; y < N; y++) line[y] = base[(size_t)y * NH];
      fft1d(&p, line, wk, +1);
      for (int y = 0; y < N; y++) base[(size_t)y * NH] = line[y];
    }
    /* x rows: Hermitian extension, imaginary parts of DC and Nyquist dropped */
#pragma omp for schedule(static)
    for (long row = 0; row < (long)N * N; row++) {
      const double complex *X = c + (size_t)row * NH;
      line[0] = creal(X[0]);
      line[N / 2] = creal(X[N / 2]);
      for (int k = 1; k < N / 2; k++) {
        line[k] = X[k];
        line[N - k] = conj(X[k]);
      }
      fft1d(&p, line, wk, +1);
      for (int x = 0; x < N; x++) out[(size_t)row * N + x] = creal(line[x]);
    }
    free(line);
    free(wk);
  }
  free(c);
  plan_free(&p);
  return 0;
}

int or_r2c_3d(int N, const double *in, double complex *out)
{
  const int NH = N / 2 + 1;
  plan1d p;
  if (plan_make(&p, N)) return -1;
#pragma omp parallel
  {
    double complex *line = malloc(N * sizeof(double complex)), *wk = malloc(N * sizeof(double complex));
#pragma omp for schedule(static)
    for (long row = 0; row < (long)N * N; row++) {
      for (int x = 0; x < N; x++) line[x] = in[(size_t)row * N + x];
      fft1d(&p, line, wk, -1);
      for (int k = 0; k < NH; k++) out[(size_t)row * NH + k] = line[k];
    }
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * NH; q++) {
      long z = q / NH, kx = q % NH;
      double complex *base = out + (size_t)z * N * NH + kx;
      for (int y = 0; y < N; y++) line[y] = base[(size_t)y * NH];
      fft1d(&p, line, wk, -1);
      for (int y = 0; y < N; y++) base[(size_t)y * NH] = line[y];
    }
#pragma omp for schedule(static)
    for (long q = 0; q < (long)N * NH; q++) {
      for (int z = 0; z < N; z++) line[z] = out[(size_t)z * N * NH + q];
      fft1d(&p, line, wk, -1);
      for (int z = 0; z < N; z++) out[(size_t)z * N * NH + q] = line[z];
    }
    free(line);
    free(wk);
  }
  plan_free(&p);
  return 0;
}
