/*
 * gpu_bridge.c -- the reference-side binding of the GB300 path: the file a
 * maintainer adds to CoLoRe's src/ (next to main.c) to run its hot path on
 * one GB300 through the C ABI of colore_cuda.h.
 *
 * It needs one field in ParamCoLoRe (src/common.h:220-381):
 *     cg_ctx *gpu;   GB300 context, NULL when running on the CPU
 * and the calls listed in INTEGRATION.md in place of the bodies of the
 * hot-path functions.  Everything is read from ParamCoLoRe after
 * read_run_params and cosmo_set / compute_tracer_cosmo have run.
 *
 * The GPU path holds float grids, as CoLoRe's single-precision build
 * (USE_SINGLE_PRECISION, _SPREC) does; a double build receives its grids
 * through gpu_download_grid, which widens them.
 */
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "colore_cuda.h"

#define GPU_TRY(par, x)                                                              \
  do {                                                                               \
    int rc_ = (x);                                                                   \
    if (rc_) report_error(1, "GPU: %s\n", cg_last_error((par)->gpu));               \
  } while (0)

/* Shell edges of the intensity maps, kept in double for cg_config. */
static double gpu_shell_r0[CG_NPOP_MAX][CG_NPLANES_MAX * 64], gpu_shell_rf[CG_NPOP_MAX][CG_NPLANES_MAX * 64];

/* cg_config from ParamCoLoRe: scalars copied, table pointers shared. */
void gpu_fill_config(ParamCoLoRe *par, cg_config *c)
{
  memset(c, 0, sizeof(*c));
  c->precision = CG_PREC_F32;
  c->n_grid = par->n_grid;
  c->l_box = par->l_box;
  for (int i = 0; i < 3; i++) c->pos_obs[i] = par->pos_obs[i];
  c->seed = par->seed_rng;
  c->omega_m = par->OmegaM;
  c->hubble_0 = par->hubble_0;
  c->fgrowth_0 = par->fgrowth_0;
  c->prefac_lensing = par->prefac_lensing;
  c->r_max = par->r_max;
  c->r2_smooth = par->r2_smooth;
  c->do_smoothing = par->do_smoothing;
  c->smooth_potential = par->smooth_potential;
  c->dens_type = par->dens_type;
  c->lpt_interp_type = par->lpt_interp_type; /* CIC unless the param file says otherwise (io.c:66) */
#if defined(_BIAS_MODEL_2)
  c->bias_model = CG_BIAS_MODEL_EXPLIN;
#elif defined(_BIAS_MODEL_3)
  c->bias_model = CG_BIAS_MODEL_LIN;
#else
  c->bias_model = CG_BIAS_MODEL_POW;
#endif
  c->numk = par->numk;
  c->logkmin = par->logkmin;
  c->logkmax = par->logkmax;
  c->idlogk = par->idlogk;
  c->n_scal = par->n_scal;
  c->pkarr = par->pkarr;
  c->glob_idr = par->glob_idr;
  c->r_arr_r2z = par->r_arr_r2z;
  c->z_arr_r2z = par->z_arr_r2z;
  c->growth_d_arr = par->growth_d_arr;
  c->growth_d2_arr = par->growth_d2_arr;
  c->growth_v_arr = par->growth_v_arr;
  c->growth_pd_arr = par->growth_pd_arr;
  c->ihub_arr = par->ihub_arr;
  c->a_arr_a2r = par->a_arr_a2r;
  c->r_arr_a2r = par->r_arr_a2r;
  c->n_srcs = par->n_srcs;
  c->nside_base = par->nside_base;
  for (int i = 0; i < par->n_srcs; i++) {
    c->srcs_nz_arr[i] = par->srcs_nz_arr[i];
    c->srcs_bz_arr[i] = par->srcs_bz_arr[i];
    c->lensing_srcs[i] = par->lensing_srcs[i];
    c->skw_srcs[i] = par->skw_srcs[i];
    c->skw_gauss[i] = par->skw_gauss[i];
    c->nside_count[i] = 0; /* the count maps have no counterpart in the reference */
  }
  c->n_imap = par->n_imap;
  for (int i = 0; i < par->n_imap; i++) {
    const HealpixShells *sh = par->imap[i];
    if (sh->nr > CG_NPLANES_MAX * 64) report_error(1, "GPU: %d intensity shells\n", sh->nr);
    for (int k = 0; k < sh->nr; k++) {
      gpu_shell_r0[i][k] = sh->r0[k];
      gpu_shell_rf[i][k] = sh->rf[k];
    }
    c->imap_tz_arr[i] = par->imap_tz_arr[i];
    c->imap_bz_arr[i] = par->imap_bz_arr[i];
    c->nside_imap[i] = par->nside_imap[i];
    c->imap_nr[i] = sh->nr;
    c->imap_r0[i] = gpu_shell_r0[i];
    c->imap_rf[i] = gpu_shell_rf[i];
  }
  c->do_kappa = par->do_kappa;
  if (par->do_kappa) {
    c->n_kappa = par->n_kappa;
    c->nside_kappa = par->nside_kappa;
    for (int i = 0; i < par->n_kappa; i++) c->kappa_r[i] = par->kmap->r0[i];
  }
  c->do_isw = par->do_isw;
  if (par->do_isw) {
    c->n_isw = par->n_isw;
    c->nside_isw = par->nside_isw;
    for (int i = 0; i < par->n_isw; i++) c->isw_r[i] = par->pd_map->r0[i];
  }
  c->n_cstm = par->do_cstm ? par->n_cstm : 0;
  for (int i = 0; i < c->n_cstm; i++) {
    c->cstm_kz_arr[i] = par->cstm_kz_arr[i];
    c->cstm_bz_arr[i] = par->cstm_bz_arr[i];
    c->nside_cstm[i] = par->nside_cstm[i];
  }
  c->need_beaming = par->need_beaming;
}

/* At the end of read_run_params (io.c:558), after compute_tracer_cosmo. */
void gpu_init(ParamCoLoRe *par)
{
  cg_config c;
  gpu_fill_config(par, &c);
  if (cg_create(&par->gpu, &c, 0)) report_error(1, "GPU: cg_create failed\n");
}

/* A grid into par's flouble array (write_density_grid, io.c:565-595): the
 * device holds floats; a double build widens them here. */
void gpu_download_grid(ParamCoLoRe *par, int which, flouble *dst)
{
  if (sizeof(flouble) == sizeof(float)) {
    GPU_TRY(par, cg_download_grid(par->gpu, which, dst));
    return;
  }
  const size_t n = (size_t)par->n_grid * par->n_grid * 2 * (par->n_grid / 2 + 1);
  float *tmp = malloc(n * sizeof(float));
  if (!tmp) report_error(1, "GPU: out of host memory\n");
  GPU_TRY(par, cg_download_grid(par->gpu, which, tmp));
  for (size_t i = 0; i < n; i++) dst[i] = tmp[i];
  free(tmp);
}

/* In param_colore_free (io.c:1247). */
void gpu_free(ParamCoLoRe *par)
{
  if (par->gpu) cg_destroy(par->gpu);
  par->gpu = NULL;
}
