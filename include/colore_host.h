/*
 * colore_host.h -- host side of the GPU path, in C: the run parameters of
 * CoLoRe (ParamCoLoRe, src/common.h:220-381, hot-path fields only), the
 * param-file reader (read_run_params, src/io.c:246-563) and the FP64 tables
 * it builds (cosmo_set, src/cosmo.c:516-816; compute_tracer_cosmo,
 * src/cosmo.c:818-849), plus their translation into a cg_config.
 *
 * GSL, libconfig and FFTW are not needed: the quadratures, the natural cubic
 * spline and the libconfig-grammar parser are implemented in
 * colore_gb300/csrc/host/.
 */
#ifndef COLORE_HOST_H
#define COLORE_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "colore_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  /* global */
  char prefix_out[256], pk_filename[256], output_format[16];
  double z_min, z_max;
  int output_density;
  unsigned long long seed;
  int write_pred, just_write_pred; /* write_pred, just_write_pred (io.c:272-276) */
  double pred_dz;
  /* field_par */
  double r_smooth;          /* as read; r2_smooth = r_smooth^2 (io.c:453-458) */
  double r2_smooth;
  int do_smoothing, smooth_potential, n_grid, dens_type, lpt_interp_type, output_lpt;
  double lpt_buffer_fraction;
  /* cosmo_par */
  double omega_m, omega_l, omega_b, h, w, ns, sigma8;
  /* derived cosmology */
  double fgrowth_0, hubble_0, prefac_lensing, r_min, r_max, l_box, pos_obs[3];
  double sigma2_gauss_theory, sigma8_input;
  /* P(k) */
  int numk;
  double logkmin, logkmax, idlogk;
  double *logkarr, *pkarr;
  /* background tables */
  double glob_idr;
  double a_arr_a2r[CG_NA], r_arr_a2r[CG_NA], z_arr_r2z[CG_NA], r_arr_r2z[CG_NA];
  double growth_d_arr[CG_NA], growth_d2_arr[CG_NA], growth_v_arr[CG_NA], growth_pd_arr[CG_NA], ihub_arr[CG_NA];
  /* sources */
  int n_srcs;
  char fname_nz_srcs[CG_NPOP_MAX][256], fname_bz_srcs[CG_NPOP_MAX][256];
  int lensing_srcs[CG_NPOP_MAX], skw_srcs[CG_NPOP_MAX], skw_gauss[CG_NPOP_MAX], nside_count[CG_NPOP_MAX];
  double *srcs_nz_arr[CG_NPOP_MAX], *srcs_bz_arr[CG_NPOP_MAX];
  /* intensity maps */
  int n_imap;
  char fname_tz_imap[CG_NPOP_MAX][256], fname_bz_imap[CG_NPOP_MAX][256], fname_nu_imap[CG_NPOP_MAX][256];
  double nu0_imap[CG_NPOP_MAX];
  int nside_imap[CG_NPOP_MAX], imap_nr[CG_NPOP_MAX];
  double *imap_tz_arr[CG_NPOP_MAX], *imap_bz_arr[CG_NPOP_MAX], *imap_r0[CG_NPOP_MAX], *imap_rf[CG_NPOP_MAX];
  /* kappa */
  int do_kappa, n_kappa, nside_kappa;
  double z_kappa_out[CG_NPLANES_MAX], kappa_r[CG_NPLANES_MAX];
  /* isw (io.c:421-426) */
  int do_isw, n_isw, nside_isw;
  double z_isw_out[CG_NPLANES_MAX], isw_r[CG_NPLANES_MAX];
  /* custom maps custom1, custom2, ... (io.c:344-364) */
  int n_cstm;
  char fname_kz_cstm[CG_NPOP_MAX][256], fname_bz_cstm[CG_NPOP_MAX][256];
  int nside_cstm[CG_NPOP_MAX];
  double *cstm_kz_arr[CG_NPOP_MAX], *cstm_bz_arr[CG_NPOP_MAX];
  /* out-of-scope sections seen in the file (reported, not run) */
  int do_skewers, do_srcs_lensing;
  int need_beaming, nside_base, bias_model;
} cg_params;

/* read_run_params: parse the file, read the input tables and build every
 * FP64 table.  Returns 0 or a CG_E* code with a message in err. */
int cg_read_run_params(const char *fname, cg_params **out, char *err, size_t errlen);
void cg_params_free(cg_params *p);
/* Point cfg at p's tables (p must outlive cfg). */
int cg_params_to_config(const cg_params *p, cg_config *cfg);

/* Background cosmology of cosmo_mad.c (flat or curved, constant w). */
typedef struct {
  double om, ol, ob, ok, h, w0;
  int ksign, normal_de;
  double a_eq, phorizon, growth0;
} cg_cosmo;
int cg_cosmo_init(cg_cosmo *c, double om, double ol, double ob, double w, double h);
double cg_cosmo_hubble(const cg_cosmo *c, double a);            /* h/Mpc           */
double cg_cosmo_chi(const cg_cosmo *c, double a);               /* Mpc/h           */
double cg_cosmo_growth(const cg_cosmo *c, double a);            /* unnormalised D  */
double cg_cosmo_fgrowth(const cg_cosmo *c, double a);
double cg_cosmo_omega_m(const cg_cosmo *c, double a);

/* Natural cubic spline (the gsl_interp_cspline of the reference). */
typedef struct {
  int n;
  double *x, *y, *m; /* m = second derivatives */
} cg_spline;
int cg_spline_init(cg_spline *s, const double *x, const double *y, int n);
double cg_spline_eval(const cg_spline *s, double x); /* NaN outside [x0, x_{n-1}] */
void cg_spline_free(cg_spline *s);

/* Adaptive Gauss-Legendre quadrature of f on [a, b] to relative tolerance. */
double cg_integrate(double (*f)(double, void *), void *par, double a, double b, double rtol);

/* Output writers of io.c (no cfitsio needed) ------------------------------ */
#define CG_OUT_ASCII 0
#define CG_OUT_FITS 1
/* One HEALPix map (RING, 12 nside^2 floats) as a FITS binary table with the
 * keywords of he_write_healpix_map (src/healpix_extra.c:4-57). */
int cg_write_healpix_map(const char *fname, const float *map, long nside);
/* Skewers appended to a FITS catalogue (write_catalog, src/io.c:1140-1189):
 * dens and vel hold nsrc x nr values; r, z, d1, v1 the background at the nr
 * step centres; sigma_g the standard deviation of the Gaussian field. */
typedef struct {
  int nr, gauss;
  const float *dens, *vel;
  const float *r, *z, *d1, *v1;
  float sigma_g;
} cg_skewer_set;
/* Catalogue of population ipop from Src records (9 floats per source) as
 * <prefix>_srcs_s<ipop+1>_0.fits (columns TYPE, RA, DEC, Z_COSMO, DZ_RSD,
 * and E1, E2, KAPPA, DRA, DDEC with has_lensing) or .txt, as write_catalog
 * (src/io.c:1069-1236).  skw (FITS only, may be NULL) appends the skewer
 * images and the background table. */
int cg_write_catalog(const char *prefix, int ipop, int format, const float *src9, long long n, int has_lensing,
                     const cg_skewer_set *skw);
/* Background at the skewer step centres r_i = (i + 0.5) r_max / nr: z, the
 * growth factor and the velocity growth (get_bg, src/cosmo.c:40-86), as
 * write_catalog tabulates them (src/io.c:1166-1176). */
int cg_skewer_background(const cg_params *p, int nr, float *r, float *z, float *d1, float *v1);
/* <prefix>_dens_<tag>_0.dat from a padded [N][N][2(N/2+1)] float grid, the
 * layout of write_density_grid (src/io.c:565-595) on one node. */
int cg_write_density_grid(const char *prefix, const char *tag, const float *grid, int n_grid, double l_box);

/* Theory predictions (write_predictions, src/predictions.c:26-173): for z =
 * 0, pred_dz, ... <= z_max, <prefix>_gbias.txt and, per source population,
 * intensity species and custom map, <prefix>_{pk,xi}_{srcs,imap,custom}_pop<i>_z<z>.txt
 * with the linear and lognormal spectra and correlation functions. */
int cg_write_predictions(const cg_params *p);
/* linear P(k) at log10 k (pk_linear0, src/cosmo.c:291-308) */
double cg_pk_linear0(const cg_params *p, double lgk);
/* FFTLog transforms of pk2xi / xi2pk (src/fftlog.c:147-157) on n log-spaced
 * points: the output grid is written to r (resp. k). */
void cg_pk2xi(int n, const double *k, const double *pk, double *r, double *xi);
void cg_xi2pk(int n, const double *r, const double *xi, double *k, double *pk);

#ifdef __cplusplus
}
#endif

#endif /* COLORE_HOST_H */
