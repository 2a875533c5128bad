/*
 * host_pred.c -- theory predictions of write_predictions
 * (predictions.c:26-173): for redshifts 0, dz, 2 dz, ... up to z_max, the
 * linear P(k) grown to z, the lognormal tracer spectra and correlation
 * functions of every source population, intensity species and custom map,
 * through the logarithmic Hankel transform FFTLog (Hamilton 2000, MNRAS
 * 312, 257; the calls of fftlog.c:93-157).
 *
 * Everything is FP64 host code: one 10^4-point transform per spectrum.
 * The complex FFT is a mixed-radix decimation in time written here, the
 * complex log-gamma the Stirling series after a recurrence shift.
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "colore_host.h"

/* ---- complex FFT of any length (recursive mixed radix, e^{sign 2 pi i jk/n}) ---- */
static int smallest_factor(int n)
{
  if (n % 4 == 0) return 4;
  for (int p = 2; p * p <= n; p++)
    if (n % p == 0) return p;
  return n;
}

/* out[k] = sum_j in[j s] w^{jk}, w = e^{sign 2 pi i / n}; tw[j] = e^{sign 2 pi i j / n0} of the top length n0 */
static void fft_rec(int n, int s, const double complex *in, double complex *out, const double complex *tw, int n0)
{
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  const int p = smallest_factor(n), m = n / p;
  for (int r = 0; r < p; r++) fft_rec(m, s * p, in + (size_t)r * s, out + (size_t)r * m, tw, n0);
  /* butterflies: out[k + q m] = sum_r w_n^{r (k + q m)} out_r[k] */
  double complex buf[64];
  double complex *t = p <= 64 ? buf : malloc((size_t)p * sizeof(double complex));
  const int step = n0 / n;
  for (int k = 0; k < m; k++) {
    for (int r = 0; r < p; r++) t[r] = out[(size_t)r * m + k];
    for (int q = 0; q < p; q++) {
      double complex acc = 0;
      for (int r = 0; r < p; r++) acc += t[r] * tw[((long long)r * (k + q * m) * step) % n0];
      out[(size_t)k + (size_t)q * m] = acc;
    }
  }
  if (t != buf) free(t);
}

static void fft(int n, double complex *a, int sign)
{
  double complex *tw = malloc((size_t)n * sizeof(double complex)), *out = malloc((size_t)n * sizeof(double complex));
  for (int j = 0; j < n; j++) tw[j] = cexp(sign * 2 * M_PI * I * (double)j / n);
  fft_rec(n, 1, a, out, tw, n);
  memcpy(a, out, (size_t)n * sizeof(double complex));
  free(tw);
  free(out);
}

/* ---- complex log-gamma: Stirling series for Re z >= 12 after lnG(z) = lnG(z+n) - sum ln(z+j) ---- */
static double complex lngamma_c(double complex z)
{
  double complex shift = 0;
  while (creal(z) < 12) {
    shift += clog(z);
    z += 1;
  }
  /* Bernoulli numbers B2k / (2k (2k-1)), k = 1..8 */
  static const double c[8] = {1.0 / 12, -1.0 / 360, 1.0 / 1260, -1.0 / 1680, 1.0 / 1188, -691.0 / 360360,
                              1.0 / 156, -3617.0 / 122400};
  const double complex iz = 1 / z, iz2 = iz * iz;
  double complex ser = 0, pw = iz;
  for (int k = 0; k < 8; k++) {
    ser += c[k] * pw;
    pw *= iz2;
  }
  return (z - 0.5) * clog(z) - z + 0.5 * log(2 * M_PI) + ser - shift;
}

/* low-ringing k_c r_c for the given (mu, q) (Hamilton 2000, eq. 174) */
static double goodkr(int n, double mu, double q, double L, double kr)
{
  const double xp = (mu + 1 + q) / 2, xm = (mu + 1 - q) / 2, y = M_PI * n / (2 * L);
  const double arg = log(2 / kr) * n / L + (cimag(lngamma_c(xp + I * y)) + cimag(lngamma_c(xm + I * y))) / M_PI;
  const double iarg = round(arg);
  if (arg != iarg) kr *= exp((arg - iarg) * L / n);
  return kr;
}

/* Fast Hankel transform of order mu with bias q on n log-spaced r: b(k)
 * at k_j = (k_c r_c) e^{-L} / r_0 e^{j L / n}. */
static void fht(int n, const double *r, const double complex *a, double *k, double complex *b, double mu, double q,
                double kcrc, int noring)
{
  const double L = log(r[n - 1] / r[0]) * n / (n - 1.0);
  if (noring) kcrc = goodkr(n, mu, q, L, kcrc);
  double complex *u = malloc((size_t)n * sizeof(double complex));
  const double y = M_PI / L, k0r0 = kcrc * exp(-L), t = -2 * y * log(k0r0 / 2);
  const double xp = (mu + 1 + q) / 2, xm = (mu + 1 - q) / 2;
  /* u_m = (k0 r0 / 2)^{-i 2 pi m / L} 2^q Gamma(xp + i m y) / Gamma(xm - i m y), and
   * lnGamma(conj w) = conj lnGamma(w) */
  for (int m = 0; m <= n / 2; m++) {
    const double complex gp = lngamma_c(xp + I * m * y), gm = lngamma_c(xm + I * m * y);
    u[m] = cexp(q * log(2) + creal(gp) - creal(gm) + I * (m * t + cimag(gp) + cimag(gm)));
  }
  for (int m = n / 2 + 1; m < n; m++) u[m] = conj(u[n - m]);
  if (n % 2 == 0) u[n / 2] = creal(u[n / 2]);
  memcpy(b, a, (size_t)n * sizeof(double complex));
  fft(n, b, -1);
  for (int m = 0; m < n; m++) b[m] *= u[m] / n;
  fft(n, b, +1);
  for (int j = 0; j < n / 2; j++) {
    const double complex tmp = b[j];
    b[j] = b[n - 1 - j];
    b[n - 1 - j] = tmp;
  }
  k[0] = k0r0 / r[0];
  for (int j = 1; j < n; j++) k[j] = k[0] * exp(j * L / n);
  free(u);
}

/* xi_l^m(r) = (2 pi r)^{-3/2} FHT_{l+1/2}[k^{m - 1/2} P(k)] (fftlog.c:134-145) */
static void xilm(int l, int m, int n, const double *k, const double *pk, double *r, double *xi)
{
  double complex *a = malloc((size_t)n * sizeof(double complex)), *b = malloc((size_t)n * sizeof(double complex));
  for (int j = 0; j < n; j++) a[j] = pow(k[j], m - 0.5) * pk[j];
  fht(n, k, a, r, b, l + 0.5, 0, 1, 1);
  for (int j = 0; j < n; j++) xi[j] = creal(pow(2 * M_PI * r[j], -1.5) * b[j]);
  free(a);
  free(b);
}

void cg_pk2xi(int n, const double *k, const double *pk, double *r, double *xi) { xilm(0, 2, n, k, pk, r, xi); }

void cg_xi2pk(int n, const double *r, const double *xi, double *k, double *pk)
{
  xilm(0, 2, n, r, xi, k, pk);
  for (int j = 0; j < n; j++) pk[j] *= 8 * M_PI * M_PI * M_PI;
}

/* ---- background on the host tables ---- */
static double bg_lin(const cg_params *p, const double *f, double f0, double ff, double r) /* cosmo.c:30-38 */
{
  if (r <= 0) return f0;
  if (r >= p->r_arr_r2z[CG_NA - 1]) return ff;
  const int ir = (int)(r * p->glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - p->r_arr_r2z[ir]) * p->glob_idr;
}

static double r_of_z_host(const cg_params *p, double z) /* cosmo.c:101-112 */
{
  const double a = 1. / (1 + z);
  if (a >= 1) return 0;
  if (a <= 0) return p->r_arr_a2r[0];
  const int ia = (int)(a * (CG_NA - 1));
  return p->r_arr_a2r[ia] + (p->r_arr_a2r[ia + 1] - p->r_arr_a2r[ia]) * (a - p->a_arr_a2r[ia]) * (CG_NA - 1.);
}

/* one tracer's files: lognormal P(k) and xi(r) at redshift z
 * (predictions.c:82-108).  As there, the transforms write their output
 * grids into ra and ka, which later rows and redshifts reuse. */
static int tracer_files(const cg_params *p, const char *kind, int ipop, double z, double bias, double rsm2_auto,
                        double rsm2_gm, double rsm2_mm, int nk, double *ka, const double *pklin, double *ra,
                        const double *xilin, double *pk, double *xi)
{
  for (int i = 0; i < nk; i++) pk[i] = pklin[i] * bias * bias * exp(-rsm2_auto * ka[i] * ka[i]);
  cg_pk2xi(nk, ka, pk, ra, xi);
  for (int i = 0; i < nk; i++) xi[i] = exp(xi[i]) - 1;
  cg_xi2pk(nk, ra, xi, ka, pk);
  char fpk[1200], fxi[1200];
  snprintf(fpk, sizeof(fpk), "%s_pk_%s_pop%i_z%.3lf.txt", p->prefix_out, kind, ipop, z);
  snprintf(fxi, sizeof(fxi), "%s_xi_%s_pop%i_z%.3lf.txt", p->prefix_out, kind, ipop, z);
  FILE *a = fopen(fpk, "w"), *b = fopen(fxi, "w");
  if (!a || !b) {
    if (a) fclose(a);
    if (b) fclose(b);
    return CG_EINVAL;
  }
  fprintf(a, "# k[h/Mpc] P_tt P_tl P_ll\n");
  /* the reference labels the first column of the non-source xi files k[Mpc/h] */
  fprintf(b, strcmp(kind, "srcs") ? "# k[Mpc/h] xi_tt xi_ll*b^2 xi_ll\n" : "# r[Mpc/h] xi_tt xi_ll*b^2 xi_ll\n");
  for (int i = 0; i < nk; i++) {
    if (ka[i] >= 1e-4 && ka[i] <= 100)
      fprintf(a, "%g %g %g %g\n", ka[i], pk[i], pklin[i] * bias * exp(-rsm2_gm * ka[i] * ka[i]),
              pklin[i] * exp(-rsm2_mm * ka[i] * ka[i]));
    if (ra[i] >= 0.5 && ra[i] <= 300.) fprintf(b, "%g %g %g %g\n", ra[i], xi[i], xilin[i] * bias, xilin[i]);
  }
  fclose(a);
  fclose(b);
  return CG_OK;
}

int cg_write_predictions(const cg_params *p)
{
  if (!p) return CG_EINVAL;
  if (p->n_srcs == 0 && p->n_imap == 0 && p->n_cstm == 0) return CG_OK; /* predictions.c:28 */
  if (!(p->pred_dz > 0)) return CG_EINVAL;
  const int nk = 10000;
  const double kmin = 1e-4, kmax = 100;
  double *ka = malloc(nk * sizeof(double)), *pk = malloc(nk * sizeof(double)), *pklin = malloc(nk * sizeof(double)),
         *ra = malloc(nk * sizeof(double)), *xi = malloc(nk * sizeof(double)), *xilin = malloc(nk * sizeof(double));
  if (!ka || !pk || !pklin || !ra || !xi || !xilin) return CG_ENOMEM;
  for (int i = 0; i < nk; i++) ka[i] = kmin * pow((kmax / kmin), i * 1.0 / (nk - 1));
  const double dx = p->l_box / p->n_grid;
  const double rsm2_gg = p->r2_smooth + 0.9 * pow(dx, 2) / 12.;
  const double rsm2_gm = p->r2_smooth + 2.0 * pow(dx, 2) / 6.;
  const double rsm2_mm = p->r2_smooth + 1.88 * pow(dx, 2) / 6.;
  char fname[1200];
  snprintf(fname, sizeof(fname), "%s_gbias.txt", p->prefix_out);
  FILE *fg = fopen(fname, "w");
  int rc = fg ? CG_OK : CG_EINVAL;
  if (fg) {
    fprintf(fg, "#1-z 2-r(z) 3-g(z) ");
    for (int i = 0; i < p->n_srcs; i++) fprintf(fg, "%d-bg_%d(z) ", i + 4, i + 1);
    for (int i = 0; i < p->n_imap; i++) fprintf(fg, "%d-bi_%d(z) ", i + 4 + p->n_srcs, i + 1);
    for (int i = 0; i < p->n_cstm; i++) fprintf(fg, "%d-bc_%d(z) ", i + 4 + p->n_srcs + p->n_imap, i + 1);
    fprintf(fg, "\n");
  }
  for (double z = 0; !rc && z <= p->z_max; z += p->pred_dz) { /* predictions.c:63 */
    const double r = r_of_z_host(p, z);
    const double g = bg_lin(p, p->growth_d_arr, 1, p->growth_d_arr[CG_NA - 1], r);
    fprintf(fg, "%g %g %g ", z, r, g);
    for (int i = 0; i < nk; i++) pklin[i] = cg_pk_linear0(p, log10(ka[i])) * g * g;
    cg_pk2xi(nk, ka, pklin, ra, xilin);
    for (int ip = 0; !rc && ip < p->n_srcs; ip++) {
      const double b = bg_lin(p, p->srcs_bz_arr[ip], p->srcs_bz_arr[ip][0], 1, r);
      fprintf(fg, "%g ", b);
      rc = tracer_files(p, "srcs", ip, z, b, rsm2_gg, rsm2_gm, rsm2_mm, nk, ka, pklin, ra, xilin, pk, xi);
    }
    for (int ip = 0; !rc && ip < p->n_imap; ip++) {
      const double b = bg_lin(p, p->imap_bz_arr[ip], p->imap_bz_arr[ip][0], 1, r);
      fprintf(fg, "%g ", b);
      rc = tracer_files(p, "imap", ip, z, b, rsm2_gg, rsm2_gm, rsm2_mm, nk, ka, pklin, ra, xilin, pk, xi);
    }
    for (int ip = 0; !rc && ip < p->n_cstm; ip++) {
      const double b = bg_lin(p, p->cstm_bz_arr[ip], p->cstm_bz_arr[ip][0], 1, r);
      fprintf(fg, "%g ", b);
      rc = tracer_files(p, "custom", ip, z, b, rsm2_mm, rsm2_gm, rsm2_mm, nk, ka, pklin, ra, xilin, pk, xi);
    }
    fprintf(fg, "\n");
  }
  if (fg) fclose(fg);
  free(ka);
  free(pk);
  free(pklin);
  free(ra);
  free(xi);
  free(xilin);
  return rc;
}
