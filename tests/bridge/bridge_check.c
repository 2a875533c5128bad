/*
 * bridge_check.c -- test driver of include/gpu_bridge.c: reads a param file
 * with the host side (cg_read_run_params), lays its tables out in a
 * ParamCoLoRe as CoLoRe's read_run_params and cosmo_set leave them (float
 * box side and shell edges in the single-precision build), runs gpu_init
 * with cg_create replaced by a recorder, and compares the cg_config the
 * binding built with the host side's, field by field.  Exit status 0 when
 * every field agrees.
 */
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "colore_cuda.h"
#include "colore_host.h"

void gpu_init(ParamCoLoRe *par);

static cg_config seen;
int cg_create(cg_ctx **out, const cg_config *cfg, int device)
{
  (void)device;
  seen = *cfg;
  *out = (cg_ctx *)&seen;
  return 0;
}
const char *cg_last_error(const cg_ctx *c) { (void)c; return "recorder"; }
int cg_download_grid(cg_ctx *c, int which, void *dst) { (void)c; (void)which; (void)dst; return 0; }
void cg_destroy(cg_ctx *c) { (void)c; }
void report_error(int level, char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  if (level) exit(2);
}

static int bad = 0;
#define EQ(f)                                                        \
  do {                                                               \
    if (memcmp(&seen.f, &ref.f, sizeof(ref.f))) {                    \
      fprintf(stderr, "field %s differs\n", #f);                    \
      bad++;                                                         \
    }                                                                \
  } while (0)
/* the NA-entry tables: ParamCoLoRe holds its own copies */
#define EQT(f)                                                       \
  do {                                                               \
    if (memcmp(seen.f, ref.f, NA * sizeof(double))) {               \
      fprintf(stderr, "table %s differs\n", #f);                   \
      bad++;                                                         \
    }                                                                \
  } while (0)
#define EQF(a, b, what)                                              \
  do {                                                               \
    if ((float)(a) != (float)(b)) {                                  \
      fprintf(stderr, "%s differs: %g %g\n", what, (double)(a), (double)(b)); \
      bad++;                                                         \
    }                                                                \
  } while (0)

_Static_assert(NA == CG_NA, "table length");
_Static_assert(NPOP_MAX == CG_NPOP_MAX && NPLANES_MAX == CG_NPLANES_MAX, "population limits");

int main(int argc, char **argv)
{
  if (argc < 2) return 3;
  char err[512];
  cg_params *p = NULL;
  if (cg_read_run_params(argv[1], &p, err, sizeof(err))) {
    fprintf(stderr, "%s\n", err);
    return 3;
  }
  cg_config ref;
  cg_params_to_config(p, &ref);
  static ParamCoLoRe par;
  memset(&par, 0, sizeof(par));
  par.OmegaM = ref.omega_m;
  par.fgrowth_0 = ref.fgrowth_0;
  par.hubble_0 = ref.hubble_0;
  par.prefac_lensing = ref.prefac_lensing;
  par.r_max = ref.r_max;
  par.n_scal = ref.n_scal;
  memcpy(par.a_arr_a2r, ref.a_arr_a2r, sizeof(par.a_arr_a2r));
  memcpy(par.r_arr_a2r, ref.r_arr_a2r, sizeof(par.r_arr_a2r));
  memcpy(par.z_arr_r2z, ref.z_arr_r2z, sizeof(par.z_arr_r2z));
  memcpy(par.r_arr_r2z, ref.r_arr_r2z, sizeof(par.r_arr_r2z));
  memcpy(par.growth_d_arr, ref.growth_d_arr, sizeof(par.growth_d_arr));
  memcpy(par.growth_d2_arr, ref.growth_d2_arr, sizeof(par.growth_d2_arr));
  memcpy(par.growth_v_arr, ref.growth_v_arr, sizeof(par.growth_v_arr));
  memcpy(par.growth_pd_arr, ref.growth_pd_arr, sizeof(par.growth_pd_arr));
  memcpy(par.ihub_arr, ref.ihub_arr, sizeof(par.ihub_arr));
  par.glob_idr = ref.glob_idr;
  par.numk = ref.numk;
  par.logkmin = ref.logkmin;
  par.logkmax = ref.logkmax;
  par.idlogk = ref.idlogk;
  par.pkarr = (double *)ref.pkarr;
  par.r2_smooth = ref.r2_smooth;
  par.do_smoothing = ref.do_smoothing;
  par.smooth_potential = ref.smooth_potential;
  par.dens_type = ref.dens_type;
  par.lpt_interp_type = ref.lpt_interp_type;
  par.seed_rng = (unsigned int)ref.seed;
  par.n_grid = ref.n_grid;
  par.l_box = (flouble)ref.l_box;
  for (int i = 0; i < 3; i++) par.pos_obs[i] = 0.5 * par.l_box; /* cosmo.c:545-547 */
  par.do_cstm = ref.n_cstm > 0;
  par.n_cstm = ref.n_cstm;
  for (int i = 0; i < ref.n_cstm; i++) {
    par.cstm_kz_arr[i] = (double *)ref.cstm_kz_arr[i];
    par.cstm_bz_arr[i] = (double *)ref.cstm_bz_arr[i];
    par.nside_cstm[i] = ref.nside_cstm[i];
  }
  par.n_srcs = ref.n_srcs;
  for (int i = 0; i < ref.n_srcs; i++) {
    par.srcs_nz_arr[i] = (double *)ref.srcs_nz_arr[i];
    par.srcs_bz_arr[i] = (double *)ref.srcs_bz_arr[i];
    par.lensing_srcs[i] = ref.lensing_srcs[i];
    par.skw_srcs[i] = ref.skw_srcs[i];
    par.skw_gauss[i] = ref.skw_gauss[i];
  }
  par.n_imap = ref.n_imap;
  HealpixShells *shells = calloc(CG_NPOP_MAX, sizeof(HealpixShells));
  HealpixShells *ptrs[CG_NPOP_MAX];
  for (int i = 0; i < ref.n_imap; i++) {
    shells[i].nr = ref.imap_nr[i];
    shells[i].r0 = malloc(ref.imap_nr[i] * sizeof(flouble));
    shells[i].rf = malloc(ref.imap_nr[i] * sizeof(flouble));
    for (int k = 0; k < ref.imap_nr[i]; k++) {
      shells[i].r0[k] = (flouble)ref.imap_r0[i][k];
      shells[i].rf[k] = (flouble)ref.imap_rf[i][k];
    }
    ptrs[i] = &shells[i];
    par.imap_tz_arr[i] = (double *)ref.imap_tz_arr[i];
    par.imap_bz_arr[i] = (double *)ref.imap_bz_arr[i];
    par.nside_imap[i] = ref.nside_imap[i];
  }
  par.imap = ptrs;
  HealpixShells km = {0, NULL, NULL}, pm = {0, NULL, NULL};
  par.do_kappa = ref.do_kappa;
  if (ref.do_kappa) {
    par.n_kappa = ref.n_kappa;
    par.nside_kappa = ref.nside_kappa;
    km.nr = ref.n_kappa;
    km.r0 = malloc(ref.n_kappa * sizeof(flouble));
    for (int i = 0; i < ref.n_kappa; i++) km.r0[i] = (flouble)ref.kappa_r[i];
  }
  par.kmap = &km;
  par.do_isw = ref.do_isw;
  if (ref.do_isw) {
    par.n_isw = ref.n_isw;
    par.nside_isw = ref.nside_isw;
    pm.nr = ref.n_isw;
    pm.r0 = malloc(ref.n_isw * sizeof(flouble));
    for (int i = 0; i < ref.n_isw; i++) pm.r0[i] = (flouble)ref.isw_r[i];
  }
  par.pd_map = &pm;
  par.nside_base = ref.nside_base;
  par.need_beaming = ref.need_beaming;

  gpu_init(&par);

  EQ(precision); EQ(n_grid); EQ(l_box); EQ(pos_obs); EQ(seed); EQ(omega_m); EQ(hubble_0); EQ(fgrowth_0);
  EQ(prefac_lensing); EQ(r_max); EQ(r2_smooth); EQ(do_smoothing); EQ(smooth_potential); EQ(dens_type);
  EQ(bias_model); EQ(numk); EQ(logkmin); EQ(logkmax); EQ(idlogk); EQ(n_scal); EQ(pkarr); EQ(glob_idr);
  EQT(r_arr_r2z); EQT(z_arr_r2z); EQT(growth_d_arr); EQT(growth_d2_arr); EQT(growth_v_arr); EQT(growth_pd_arr);
  EQT(ihub_arr); EQT(a_arr_a2r); EQT(r_arr_a2r); EQ(n_srcs); EQ(nside_base); EQ(n_imap); EQ(nside_imap);
  EQ(imap_nr); EQ(do_kappa); EQ(n_kappa); EQ(nside_kappa); EQ(need_beaming); EQ(do_isw); EQ(n_isw);
  EQ(nside_isw); EQ(lpt_interp_type); EQ(n_cstm); EQ(nside_cstm); EQ(lensing_srcs); EQ(skw_srcs); EQ(skw_gauss);
  for (int i = 0; i < ref.n_srcs; i++) {
    if (seen.srcs_nz_arr[i] != ref.srcs_nz_arr[i] || seen.srcs_bz_arr[i] != ref.srcs_bz_arr[i]) bad++;
  }
  for (int i = 0; i < ref.n_imap; i++) {
    if (seen.imap_tz_arr[i] != ref.imap_tz_arr[i] || seen.imap_bz_arr[i] != ref.imap_bz_arr[i]) bad++;
    for (int k = 0; k < ref.imap_nr[i]; k++) {
      EQF(seen.imap_r0[i][k], ref.imap_r0[i][k], "imap r0");
      EQF(seen.imap_rf[i][k], ref.imap_rf[i][k], "imap rf");
    }
  }
  for (int i = 0; i < ref.n_cstm; i++)
    if (seen.cstm_kz_arr[i] != ref.cstm_kz_arr[i] || seen.cstm_bz_arr[i] != ref.cstm_bz_arr[i]) bad++;
  for (int i = 0; i < ref.n_kappa; i++) EQF(seen.kappa_r[i], ref.kappa_r[i], "kappa_r");
  for (int i = 0; i < ref.n_isw; i++) EQF(seen.isw_r[i], ref.isw_r[i], "isw_r");
  /* the count maps have no counterpart in the reference: the binding leaves them off */
  for (int i = 0; i < ref.n_srcs; i++)
    if (seen.nside_count[i] != 0) bad++;
  printf("fields differing: %d\n", bad);
  cg_params_free(p);
  return bad ? 1 : 0;
}
