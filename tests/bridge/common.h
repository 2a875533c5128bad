/*
 * common.h (test stand-in) -- the parts of CoLoRe's src/common.h that
 * include/gpu_bridge.c reads, restated for the binding's compile-and-fill
 * test: the ParamCoLoRe fields (src/common.h:220-381) and HealpixShells
 * (src/common.h:208-218) under their own names and types, flouble a float
 * as in the single-precision build, report_error (src/common.c:290-306).
 */
#ifndef STUB_COMMON_H
#define STUB_COMMON_H

#include <stdio.h>

#define NA 5001
#define NPOP_MAX 10
#define NPLANES_MAX 100

typedef float flouble;

typedef struct {
  int nr;
  flouble *r0, *rf;
} HealpixShells;

typedef struct cg_ctx cg_ctx;

typedef struct {
  double OmegaM, fgrowth_0, hubble_0, prefac_lensing, r_max, n_scal;
  double a_arr_a2r[NA], r_arr_a2r[NA], z_arr_r2z[NA], r_arr_r2z[NA];
  double growth_d_arr[NA], growth_d2_arr[NA], growth_v_arr[NA], growth_pd_arr[NA], ihub_arr[NA];
  double glob_idr;
  int numk;
  double logkmax, logkmin, idlogk;
  double *pkarr;
  double r2_smooth;
  int do_smoothing, smooth_potential, dens_type, lpt_interp_type;
  unsigned int seed_rng;
  int n_grid;
  flouble l_box;
  double pos_obs[3];
  int do_cstm, n_cstm;
  double *cstm_kz_arr[NPOP_MAX], *cstm_bz_arr[NPOP_MAX];
  int nside_cstm[NPOP_MAX];
  int n_srcs;
  double *srcs_nz_arr[NPOP_MAX], *srcs_bz_arr[NPOP_MAX];
  int lensing_srcs[NPOP_MAX], skw_srcs[NPOP_MAX], skw_gauss[NPOP_MAX];
  int n_imap;
  double *imap_tz_arr[NPOP_MAX], *imap_bz_arr[NPOP_MAX];
  int nside_imap[NPOP_MAX];
  HealpixShells **imap;
  int do_kappa, n_kappa, nside_kappa;
  HealpixShells *kmap;
  int do_isw, n_isw, nside_isw;
  HealpixShells *pd_map;
  int nside_base, need_beaming;
  cg_ctx *gpu; /* the field the binding adds */
} ParamCoLoRe;

void report_error(int level, char *fmt, ...);

#endif
