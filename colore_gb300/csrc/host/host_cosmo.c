/*
 * host_cosmo.c -- FP64 host tables of the GPU path.
 *
 * Restates the background cosmology of cosmo_mad.c (csm_hubble,
 * csm_radial_comoving_distance, csm_growth_factor, csm_f_growth,
 * csm_omega_m: cosmo_mad.c:160-520), the table construction of cosmo_set
 * (cosmo.c:516-717), the P(k) reading/re-splining/sigma_8 normalisation of
 * pk_linear_set (cosmo.c:444-495) and compute_tracer_cosmo
 * (cosmo.c:818-849).  GSL is replaced by an adaptive Gauss-Legendre
 * quadrature (nodes from Newton iteration on P_n) and a natural cubic spline
 * (the gsl_interp_cspline boundary conditions), both written here.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "colore_host.h"

#define HMPC 2997.92458                 /* c/H0 in Mpc/h, cosmo_mad.h:35 */
#define RTOD_REF 57.2957795             /* RTOD of common.h:124          */
#define TWOPIPIINVLOGTEN 0.1166503235296796 /* ln(10)/(2 pi^2), common.h:130 */

/* ------------------------------------------------------------------ */
/* quadrature                                                          */
/* ------------------------------------------------------------------ */
#define GL_N 20
static double gl_x[GL_N], gl_w[GL_N];
static int gl_ready = 0;

static void gl_init(void)
{
  if (gl_ready) return;
  for (int i = 0; i < GL_N; i++) {
    double x = cos(M_PI * (i + 0.75) / (GL_N + 0.5));
    double dp = 0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= GL_N; k++) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = GL_N * (x * p1 - p0) / (x * x - 1);
      double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) break;
    }
    gl_x[i] = x;
    gl_w[i] = 2 / ((1 - x * x) * dp * dp);
  }
  gl_ready = 1;
}

static double gl_panel(double (*f)(double, void *), void *par, double a, double b)
{
  double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0;
  for (int i = 0; i < GL_N; i++) s += gl_w[i] * f(c + h * gl_x[i], par);
  return s * h;
}

static double gl_adapt(double (*f)(double, void *), void *par, double a, double b, double whole, double rtol,
                       int depth)
{
  double m = 0.5 * (a + b);
  double l = gl_panel(f, par, a, m), r = gl_panel(f, par, m, b);
  double s = l + r;
  if (depth > 40 || fabs(s - whole) <= rtol * fabs(s) || fabs(s - whole) < 1e-300) return s;
  return gl_adapt(f, par, a, m, l, rtol, depth + 1) + gl_adapt(f, par, m, b, r, rtol, depth + 1);
}

double cg_integrate(double (*f)(double, void *), void *par, double a, double b, double rtol)
{
  gl_init();
  if (a == b) return 0;
  return gl_adapt(f, par, a, b, gl_panel(f, par, a, b), rtol, 0);
}

/* ------------------------------------------------------------------ */
/* natural cubic spline                                                */
/* ------------------------------------------------------------------ */
int cg_spline_init(cg_spline *s, const double *x, const double *y, int n)
{
  if (n < 3) return CG_EINVAL;
  for (int i = 1; i < n; i++)
    if (!(x[i] > x[i - 1])) return CG_EINVAL;
  s->n = n;
  s->x = malloc(n * sizeof(double));
  s->y = malloc(n * sizeof(double));
  s->m = calloc(n, sizeof(double));
  double *cp = malloc(n * sizeof(double)), *dp = malloc(n * sizeof(double));
  if (!s->x || !s->y || !s->m || !cp || !dp) return CG_ENOMEM;
  memcpy(s->x, x, n * sizeof(double));
  memcpy(s->y, y, n * sizeof(double));
  /* tridiagonal system for the interior second derivatives, m_0 = m_{n-1} = 0 */
  cp[0] = 0;
  dp[0] = 0;
  for (int i = 1; i < n - 1; i++) {
    double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
    double a = h0, b = 2 * (h0 + h1), c = h1;
    double r = 6 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
    double den = b - a * cp[i - 1];
    cp[i] = c / den;
    dp[i] = (r - a * dp[i - 1]) / den;
  }
  s->m[n - 1] = 0;
  for (int i = n - 2; i >= 1; i--) s->m[i] = dp[i] - cp[i] * s->m[i + 1];
  s->m[0] = 0;
  free(cp);
  free(dp);
  return CG_OK;
}

double cg_spline_eval(const cg_spline *s, double x)
{
  const int n = s->n;
  if (x < s->x[0] || x > s->x[n - 1]) return NAN;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) / 2;
    if (s->x[mid] > x) hi = mid;
    else lo = mid;
  }
  double h = s->x[hi] - s->x[lo];
  double a = (s->x[hi] - x) / h, b = (x - s->x[lo]) / h;
  return a * s->y[lo] + b * s->y[hi] + ((a * a * a - a) * s->m[lo] + (b * b * b - b) * s->m[hi]) * h * h / 6;
}

void cg_spline_free(cg_spline *s)
{
  free(s->x);
  free(s->y);
  free(s->m);
  s->x = s->y = s->m = NULL;
}

/* ------------------------------------------------------------------ */
/* background cosmology                                                */
/* ------------------------------------------------------------------ */
static double apow(const cg_cosmo *c, double a) { return c->normal_de ? a * a * a : pow(a, -3 * c->w0); }
static double xfun(const cg_cosmo *c, double a) { return c->om + c->ol * apow(c, a) + c->ok * a; }
static double na2hm1(double a, void *p) { const cg_cosmo *c = p; return 1 / sqrt(a * xfun(c, a)); }
static double nahm1(const cg_cosmo *c, double a) { return sqrt(a / xfun(c, a)); }
static double nahm3(double a, void *p)
{
  double v = nahm1((const cg_cosmo *)p, a);
  return v * v * v;
}

static double parthor(const cg_cosmo *c, double a)
{
  double alim = 0.01 * c->a_eq;
  if (a <= alim) return 2 * sqrt(a / c->om) * HMPC;
  return (2 * sqrt(alim / c->om) + cg_integrate(na2hm1, (void *)c, alim, a, 1e-11)) * HMPC;
}

static double gfac(const cg_cosmo *c, double a)
{
  double alim = 0.01 * c->a_eq;
  if (a <= alim) return a;
  double int0 = 0.4 * sqrt(alim * alim * alim * alim * alim / (c->om * c->om * c->om));
  return (int0 + cg_integrate(nahm3, (void *)c, alim, a, 1e-11)) * 2.5 * c->om / (a * nahm1(c, a));
}

int cg_cosmo_init(cg_cosmo *c, double om, double ol, double ob, double w, double h)
{
  memset(c, 0, sizeof(*c));
  c->om = om;
  c->ol = ol;
  c->ob = ob;
  c->ok = 1 - om - ol;
  c->h = h;
  c->w0 = w;
  c->normal_de = fabs(w + 1) < 1e-6;                     /* cosmo_mad.c:446-459 */
  c->ksign = fabs(c->ok) < 1e-6 ? 0 : (c->ok > 0 ? -1 : 1);
  if (om <= 0 || om < ob || w > -0.333333) return CG_EINVAL; /* cosmo_mad.c:468-481 */
  double aeqk = c->ksign != 0 ? om / fabs(c->ok) : 1;      /* aeqmin, cosmo_mad.c:160-179 */
  double aeql = 1;
  if (ol != 0) aeql = c->normal_de ? pow(om / ol, 0.333) : pow(om / ol, -1 / (3 * w));
  c->a_eq = aeqk < aeql ? aeqk : aeql;
  c->phorizon = parthor(c, 1);
  c->growth0 = gfac(c, 1);
  return CG_OK;
}

double cg_cosmo_hubble(const cg_cosmo *c, double a) { return sqrt(xfun(c, a) / (a * a * a)) / HMPC; }
double cg_cosmo_chi(const cg_cosmo *c, double a) { return c->phorizon - parthor(c, a); }
double cg_cosmo_growth(const cg_cosmo *c, double a) { return gfac(c, a); }
double cg_cosmo_omega_m(const cg_cosmo *c, double a) { return c->om / xfun(c, a); }
double cg_cosmo_fgrowth(const cg_cosmo *c, double a)
{
  double d = gfac(c, a), ap = apow(c, a), coeff = c->normal_de ? 0 : (1 + c->w0);
  return 0.5 * (5 * c->om * a / d - (3 * c->om + 3 * coeff * c->ol * ap + 2 * c->ok * a)) / xfun(c, a);
}

/* ------------------------------------------------------------------ */
/* P(k)                                                                */
/* ------------------------------------------------------------------ */
static double pk_lin0(const cg_params *p, double lgk) /* pk_linear0, cosmo.c:291-308 */
{
  int ik = (int)((lgk - p->logkmin) * p->idlogk);
  if (ik < 0) return p->pkarr[0] * pow(10, p->ns * (lgk - p->logkmin));
  if (ik < p->numk - 1)
    return p->pkarr[ik] + (lgk - p->logkarr[ik]) * (p->pkarr[ik + 1] - p->pkarr[ik]) * p->idlogk;
  return p->pkarr[p->numk - 1] * pow(10, -3 * (lgk - p->logkmax));
}

double cg_pk_linear0(const cg_params *p, double lgk) { return pk_lin0(p, lgk); }

static double wind(double x, int setwf) /* cosmo.c:265-289 */
{
  if (setwf == 1) return exp(-0.5 * x * x);
  if (x < 0.1)
    return 1. - 0.1 * x * x + 0.003571429 * x * x * x * x - 6.61376E-5 * x * x * x * x * x * x +
           7.51563E-7 * x * x * x * x * x * x * x * x;
  return 3 * (sin(x) - x * cos(x)) / (x * x * x);
}

typedef struct {
  const cg_params *p;
  double R;
  int wf;
} sig_par;

static double sig_integrand(double lk, void *vp) /* integxiL_NO at r = 0, cosmo.c:350-368 */
{
  const sig_par *s = vp;
  double k = pow(10, lk);
  double w = wind(k * s->R, s->wf);
  return TWOPIPIINVLOGTEN * pk_lin0(s->p, lk) * k * k * k * w * w;
}

/* sigL2(R,R,wf,wf), cosmo.c:435-442: the integral over log10 k below logkmax */
static double sigL2(const cg_params *p, double R, int wf)
{
  sig_par s = {p, R, wf};
  double lo = p->logkmin - 12;
  /* split at the table edge and at the decades so every panel is smooth */
  double tot = 0, a = lo;
  while (a < p->logkmax) {
    double b = floor(a) + 1;
    if (b > p->logkmax) b = p->logkmax;
    if (a < p->logkmin && b > p->logkmin) b = p->logkmin;
    tot += cg_integrate(sig_integrand, &s, a, b, 1e-10);
    a = b;
  }
  return tot;
}

static int count_lines(FILE *f)
{
  int n = 0;
  char buf[1000];
  while (fgets(buf, sizeof(buf), f)) n++;
  rewind(f);
  return n;
}

static int read_two_columns(const char *fname, double **x, double **y, int *n, char *err, size_t el)
{
  FILE *f = fopen(fname, "r");
  if (!f) return snprintf(err, el, "Couldn't open file %s", fname), CG_EINVAL;
  int m = count_lines(f);
  *x = malloc((m > 0 ? m : 1) * sizeof(double));
  *y = malloc((m > 0 ? m : 1) * sizeof(double));
  for (int i = 0; i < m; i++) {
    if (fscanf(f, "%lf %lf", &(*x)[i], &(*y)[i]) != 2) {
      fclose(f);
      return snprintf(err, el, "Error reading file %s, line %d", fname, i + 1), CG_EINVAL;
    }
  }
  fclose(f);
  *n = m;
  return CG_OK;
}

/* pk_linear_set, cosmo.c:444-495 */
static int pk_set(cg_params *p, char *err, size_t el)
{
  double *k = NULL, *pk = NULL;
  int n, rc;
  if ((rc = read_two_columns(p->pk_filename, &k, &pk, &n, err, el))) return rc;
  if (n < 3) return snprintf(err, el, "P(k) file %s too short", p->pk_filename), CG_EINVAL;
  p->numk = n;
  p->logkarr = malloc(n * sizeof(double));
  p->pkarr = pk;
  for (int i = 0; i < n; i++) p->logkarr[i] = log10(k[i]);
  free(k);
  p->logkmin = p->logkarr[0];
  p->logkmax = p->logkarr[n - 1];
  p->idlogk = (n - 1) / (p->logkmax - p->logkmin);
  cg_spline s;
  if (cg_spline_init(&s, p->logkarr, p->pkarr, n))
    return snprintf(err, el, "P(k) file must be increasing in k"), CG_EINVAL;
  for (int i = 0; i < n - 1; i++) {
    double lk = p->logkmin + i / p->idlogk;
    p->pkarr[i] = cg_spline_eval(&s, lk);
    p->logkarr[i] = lk;
  }
  cg_spline_free(&s);
  double s8 = sigL2(p, 8, 0);
  p->sigma8_input = sqrt(s8);
  double norm = p->sigma8 * p->sigma8 / s8;
  for (int i = 0; i < n; i++) p->pkarr[i] *= norm;
  double reff = sqrt(p->r2_smooth + pow(0.45 * p->l_box / p->n_grid, 2));
  p->sigma2_gauss_theory = sigL2(p, reff, 1);
  return CG_OK;
}

/* read one tracer input file into a natural cubic spline over z */
static int tracer_spline(const char *fname, const cg_cosmo *c, int is_nz, double zmin, double zmax, cg_spline *s,
                         const char *what, char *err, size_t el)
{
  double *z, *f;
  int n, rc;
  if ((rc = read_two_columns(fname, &z, &f, &n, err, el))) return rc;
  if (is_nz) { /* cosmo.c:571-582: deg^-2 per dz -> per volume */
    for (int i = 0; i < n; i++) {
      double a = 1. / (1 + z[i]);
      double hz = cg_cosmo_hubble(c, a), rz = cg_cosmo_chi(c, a);
      f[i] *= RTOD_REF * RTOD_REF * hz / (rz * rz);
    }
    if (n > 1 && z[0] == 0) f[0] = f[1];
  }
  if (n < 3 || z[0] > zmin || z[n - 1] < zmax) {
    free(z);
    free(f);
    return snprintf(err, el, "%s z-range is too small (%s)", what, fname), CG_EINVAL;
  }
  rc = cg_spline_init(s, z, f, n);
  free(z);
  free(f);
  if (rc) return snprintf(err, el, "%s: z must increase (%s)", what, fname), CG_EINVAL;
  return CG_OK;
}

/* cosmo_set (cosmo.c:516-717) and compute_tracer_cosmo (cosmo.c:818-849). */
int cg_host_cosmo_set(cg_params *p, char *err, size_t el)
{
  cg_cosmo c;
  if (cg_cosmo_init(&c, p->omega_m, p->omega_l, p->omega_b, p->w, p->h))
    return snprintf(err, el, "invalid cosmological parameters"), CG_EINVAL;
  p->fgrowth_0 = cg_cosmo_fgrowth(&c, 1);
  p->hubble_0 = cg_cosmo_hubble(&c, 1);
  p->r_min = cg_cosmo_chi(&c, 1 / (1 + p->z_min));
  p->r_max = cg_cosmo_chi(&c, 1 / (1 + p->z_max));
  p->prefac_lensing = 1.5 * p->hubble_0 * p->hubble_0 * p->omega_m;
  /* cosmo.c:544-547; l_box is a flouble, a float in the single-precision
   * build (common.h:277) that this path reproduces, so the box side is the
   * float nearest the double expression and the observer sits at its half */
  p->l_box = (double)(float)(2 * p->r_max * (1 + 2. / p->n_grid));
  p->pos_obs[0] = p->pos_obs[1] = p->pos_obs[2] = 0.5 * p->l_box;
  int rc;
  cg_spline snz[CG_NPOP_MAX], sbz[CG_NPOP_MAX], stz[CG_NPOP_MAX], sbi[CG_NPOP_MAX], skc[CG_NPOP_MAX],
      sbc[CG_NPOP_MAX];
  for (int i = 0; i < p->n_srcs; i++) {
    if ((rc = tracer_spline(p->fname_bz_srcs[i], &c, 0, p->z_min, p->z_max, &sbz[i], "Bias", err, el))) return rc;
    if ((rc = tracer_spline(p->fname_nz_srcs[i], &c, 1, p->z_min, p->z_max, &snz[i], "N(z)", err, el))) return rc;
    p->srcs_nz_arr[i] = malloc(CG_NA * sizeof(double));
    p->srcs_bz_arr[i] = malloc(CG_NA * sizeof(double));
  }
  for (int i = 0; i < p->n_imap; i++) {
    if ((rc = tracer_spline(p->fname_bz_imap[i], &c, 0, p->z_min, p->z_max, &sbi[i], "Bias", err, el))) return rc;
    if ((rc = tracer_spline(p->fname_tz_imap[i], &c, 0, p->z_min, p->z_max, &stz[i], "T(z)", err, el))) return rc;
    p->imap_tz_arr[i] = malloc(CG_NA * sizeof(double));
    p->imap_bz_arr[i] = malloc(CG_NA * sizeof(double));
  }
  for (int i = 0; i < p->n_cstm; i++) { /* cosmo.c:631-662 */
    if ((rc = tracer_spline(p->fname_bz_cstm[i], &c, 0, p->z_min, p->z_max, &sbc[i], "Bias", err, el))) return rc;
    if ((rc = tracer_spline(p->fname_kz_cstm[i], &c, 0, p->z_min, p->z_max, &skc[i], "K(z)", err, el))) return rc;
    p->cstm_kz_arr[i] = malloc(CG_NA * sizeof(double));
    p->cstm_bz_arr[i] = malloc(CG_NA * sizeof(double));
  }
  for (int i = 0; i < CG_NA; i++) {
    double a = ((double)i) / (CG_NA - 1);
    p->a_arr_a2r[i] = a;
    p->r_arr_a2r[i] = cg_cosmo_chi(&c, a);
  }
  double growth0 = cg_cosmo_growth(&c, 1);
  p->glob_idr = (CG_NA - 1) / p->r_arr_a2r[0];
  int ia = 0;
  for (int i = 0; i < CG_NA; i++) {
    double r = i / p->glob_idr;
    double a; /* a_of_r_provisional, cosmo.c:88-99 (the search restarts at 0 there) */
    if (r <= 0) a = 1;
    else if (r >= p->r_arr_a2r[0]) a = 1E-6;
    else {
      ia = 0;
      while (r <= p->r_arr_a2r[ia]) ia++;
      a = p->a_arr_a2r[ia - 1] + (p->a_arr_a2r[ia] - p->a_arr_a2r[ia - 1]) * (r - p->r_arr_a2r[ia - 1]) /
                                     (p->r_arr_a2r[ia] - p->r_arr_a2r[ia - 1]);
    }
    double z = 1. / a - 1;
    double gz = cg_cosmo_growth(&c, a) / growth0;
    double om = cg_cosmo_omega_m(&c, a);
    double fz = cg_cosmo_fgrowth(&c, a);
    double hhz = cg_cosmo_hubble(&c, a);
    p->z_arr_r2z[i] = z;
    p->r_arr_r2z[i] = r;
    p->growth_d_arr[i] = gz;
    p->growth_d2_arr[i] = -0.42857142857 * gz * gz * pow(om, -0.00699300699);
    p->growth_v_arr[i] = (gz * hhz * fz) / (p->fgrowth_0 * p->hubble_0);
    p->growth_pd_arr[i] = gz * hhz * (fz - 1);
    p->ihub_arr[i] = 1. / hhz;
    for (int k = 0; k < p->n_srcs; k++) {
      p->srcs_nz_arr[k][i] = cg_spline_eval(&snz[k], z);
      p->srcs_bz_arr[k][i] = cg_spline_eval(&sbz[k], z);
    }
    for (int k = 0; k < p->n_imap; k++) {
      p->imap_tz_arr[k][i] = cg_spline_eval(&stz[k], z);
      p->imap_bz_arr[k][i] = cg_spline_eval(&sbi[k], z);
    }
    for (int k = 0; k < p->n_cstm; k++) {
      p->cstm_kz_arr[k][i] = cg_spline_eval(&skc[k], z);
      p->cstm_bz_arr[k][i] = cg_spline_eval(&sbc[k], z);
    }
  }
  for (int k = 0; k < p->n_cstm; k++) {
    cg_spline_free(&skc[k]);
    cg_spline_free(&sbc[k]);
  }
  for (int k = 0; k < p->n_srcs; k++) {
    cg_spline_free(&snz[k]);
    cg_spline_free(&sbz[k]);
  }
  for (int k = 0; k < p->n_imap; k++) {
    cg_spline_free(&stz[k]);
    cg_spline_free(&sbi[k]);
  }
  if ((rc = pk_set(p, err, el))) return rc;
  /* compute_tracer_cosmo: shell and source-plane distances */
  for (int k = 0; k < p->n_imap; k++) {
    double *nu0, *nuf;
    int n;
    if ((rc = read_two_columns(p->fname_nu_imap[k], &nu0, &nuf, &n, err, el))) return rc;
    if (n < 1) return snprintf(err, el, "empty frequency table %s", p->fname_nu_imap[k]), CG_EINVAL;
    p->imap_nr[k] = n;
    p->imap_r0[k] = malloc(n * sizeof(double));
    p->imap_rf[k] = malloc(n * sizeof(double));
    for (int i = 0; i < n; i++) {
      p->imap_r0[k][i] = cg_cosmo_chi(&c, nuf[i] / p->nu0_imap[k]);
      p->imap_rf[k][i] = cg_cosmo_chi(&c, nu0[i] / p->nu0_imap[k]);
    }
    free(nu0);
    free(nuf);
  }
  for (int i = 0; i < p->n_kappa; i++) {
    if (p->z_kappa_out[i] > p->z_max)
      return snprintf(err, el, "Source plane %d outside redshift range", i + 1), CG_EINVAL;
    p->kappa_r[i] = cg_cosmo_chi(&c, 1. / (1 + p->z_kappa_out[i]));
  }
  for (int i = 0; i < p->n_isw; i++) {
    if (p->z_isw_out[i] > p->z_max)
      return snprintf(err, el, "Source plane %d outside redshift range", i + 1), CG_EINVAL;
    p->isw_r[i] = cg_cosmo_chi(&c, 1. / (1 + p->z_isw_out[i]));
  }
  return CG_OK;
}
