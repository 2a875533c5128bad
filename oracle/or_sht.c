/*
 * or_sht.c -- ORACLE (test infrastructure only): the Legendre part of the
 * FP64 spherical-harmonic analysis behind the maps' C_ell check
 * (he_map2alm / sht_wrapper, healpix_extra.c:399-435, on the HEALPix ring
 * geometry with pixel-area weights).
 *
 * Input: per m and per northern ring (the equator ring included) the
 * symmetric and antisymmetric combinations of the ring Fourier sums of the
 * ring and its southern mirror, S = F_north + F_south and
 * A = F_north - F_south, for K maps.  Since
 * lambda_lm(-z) = (-1)^(l+m) lambda_lm(z),
 *   a_lm = omega sum_{north rings} lambda_lm(z) (S if l+m even, else A).
 * lambda_lm are the orthonormal associated Legendre functions with the
 * Condon-Shortley phase: lambda_mm from its closed form in logarithms (the
 * polar rings underflow to zero, where they are negligible), then the
 * three-term recursion in l.  Parallel over m.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* F layout: [m][ring][k][2] (re, im), m = 0..lmax; alm: [k][l][m][2]. */
int or_sht_legendre(int lmax, int nring, int K, const double *z, const double *S, const double *A, double omega,
                    double *alm)
{
  const int L = lmax + 1;
  memset(alm, 0, sizeof(double) * 2 * (size_t)K * L * L);
  double *logc = malloc(sizeof(double) * L);
  if (!logc) return 1;
  logc[0] = 0.0;
  for (int m = 1; m < L; m++) logc[m] = logc[m - 1] + log((2.0 * m - 1.0) / (2.0 * m));
  int bad = 0;
#pragma omp parallel
  {
    double *acc = malloc(sizeof(double) * 2 * (size_t)K * L);
    double *al = malloc(sizeof(double) * L);
    if (!acc || !al) {
#pragma omp atomic write
      bad = 1;
    }
#pragma omp for schedule(dynamic, 1)
    for (int m = 0; m < L; m++) {
      if (!acc || !al) continue;
      memset(acc, 0, sizeof(double) * 2 * (size_t)K * L);
      for (int l = m + 2; l < L; l++) al[l] = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
      const double a1 = sqrt(2.0 * m + 3.0);
      const double c0 = 0.5 * (log((2.0 * m + 1.0) / (4.0 * M_PI)) + logc[m]);
      for (int r = 0; r < nring; r++) {
        const double zz = z[r];
        const double s2 = 1.0 - zz * zz;
        double lam = s2 > 0.0 ? exp(c0 + 0.5 * m * log(s2)) : (m == 0 ? exp(c0) : 0.0);
        if (m & 1) lam = -lam;
        if (lam == 0.0) continue;
        const double *fs = S + ((size_t)m * nring + r) * 2 * K;
        const double *fa = A + ((size_t)m * nring + r) * 2 * K;
        double p2 = 0.0, p1 = lam, ap = a1;
        for (int l = m; l < L; l++) {
          double p;
          if (l == m) p = lam;
          else if (l == m + 1) p = a1 * zz * lam;
          else {
            p = al[l] * (zz * p1 - p2 / ap);
            ap = al[l];
          }
          if (l > m) {
            p2 = p1;
            p1 = p;
          }
          const double *f = ((l + m) & 1) ? fa : fs;
          double *o = acc + 2 * (size_t)K * l;
          for (int k = 0; k < K; k++) {
            o[2 * k] += p * f[2 * k];
            o[2 * k + 1] += p * f[2 * k + 1];
          }
        }
      }
      for (int l = m; l < L; l++)
        for (int k = 0; k < K; k++) {
          double *o = alm + 2 * (((size_t)k * L + l) * L + m);
          o[0] = omega * acc[2 * ((size_t)K * l + k)];
          o[1] = omega * acc[2 * ((size_t)K * l + k) + 1];
        }
    }
    free(acc);
    free(al);
  }
  free(logc);
  return bad;
}
