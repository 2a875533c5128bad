/*
 * srcs_api.h -- launch interface of srcs.cu.
 */
#ifndef CG_SRCS_API_H
#define CG_SRCS_API_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "cg_exact.h"

struct cg_srcs_params {
  cg::Box box;
  cg::Grid1 g;
  cg::Tab zt, v1, nz, bz, norm;
  const float *a_a2r, *r_a2r; /* r_of_z table */
  int na;
  int bias_model;
  uint32_t kp0, kp1; /* Poisson stream key  */
  uint32_t kq0, kq1; /* position stream key */
  float rlim;        /* L/2 + 20, srcs.c:169 */
  float cell_vol;
  float factor_vel;  /* -f0/(1.5 H0 Om), srcs.c:233 */
  int need_beaming;
  int64_t nside_base, nside_count;
  const int *base_r2n;       /* RING -> NEST ids at nside_base, or NULL (computed per source) */
  int *cmap;                 /* count map or NULL */
  unsigned short *counts;    /* N^3; CG_COUNT_ESC marks a cell in the overflow list */
  long long *ovf_cell;       /* cells holding CG_COUNT_ESC or more sources ...     */
  int *ovf_cnt;              /* ... and their counts                             */
  int *ovf_n;                /* entries used (zeroed by cg_srcs_count)           */
  long long *block_sums;     /* per block, then the scan's tile sums; exclusive offsets after the scan */
  long long capacity;
  float4 *pos;
  int *ipix;
  float *src;                /* 9 floats per source (Src) */
  unsigned int *err;
  /* the count and pixel decisions of the reference's double arithmetic
   * (cg_exact.h): float and double tables, corners; the double corners of
   * the emitted positions; every decision in double when force_double;
   * xstats[0] cells and xstats[1] pixels decided in double */
  cg_pois_args pa;
  double dx64, p64[3];
  const float *cl[3];  /* low parts of the float corners (pa.xc..: c + l = the double corner) */
  float dxh, dxl;      /* dx as a float pair */
  int force_double;
  unsigned long long *xstats;
};

/* Per-cell counts are stored as uint16; the few cells at or above the escape
 * value (in practice the cells touching the observer, where n(z) ~ 1/r^2)
 * go to an overflow list of CG_OVF_CAP entries. */
#define CG_COUNT_ESC 65535
#define CG_OVF_CAP 4096

/* Line-of-sight quantities at the sources of one population
 * (srcs_get_beam_properties_single and srcs_beams_postproc_single,
 * srcs.c:452-733): lensing (shear, convergence, deflection) integrated with
 * the nearest-cell tidal tensor, and skewers sampled with trilinear
 * interpolation, on nr = N/2 radial steps of dr up to each source. */
struct cg_los_params {
  cg::Box box;
  cg::Grid1 g;
  cg::Tab d1;            /* growth factor, for Gaussian skewers */
  const float4 *pos;     /* catalogue positions */
  float *src;            /* 9 floats per source; lensing writes e1 e2 kappa dra ddec */
  long long nsrc;        /* sources, or their upper bound when nsrc_dev is set */
  const long long *nsrc_dev; /* NULL, or the device total (min with nsrc) */
  int nr;
  float dr, idr;
  const float *lfac;     /* 2 nr: 2 pg dr, then rm pg dr, pg = D(rm) (1 + z(rm)) */
  const float *vfac;     /* nr: V1(rm) factor_vel */
  float *skw_d, *skw_v;  /* nsrc x nr each */
  int skw_gauss;
  const float *sigma2;   /* device sigma^2 of the Gaussian field */
};

long long cg_srcs_nblocks(int N);
/* Scan scratch that block_sums needs past its nb entries (the tile sums). */
long long cg_srcs_scan_room(long long nb);
cudaError_t cg_srcs_count(cudaStream_t s, const float *grid, const cg_srcs_params *p, long long *total);
cudaError_t cg_srcs_emit(cudaStream_t s, const float *phi, const cg_srcs_params *p);
/* nsrc sources, or with nsrc_dev non-NULL min(*nsrc_dev, nsrc) read on the
 * device (a graph-captured sequence, whose totals stay on the device). */
cudaError_t cg_srcs_beam_rsd(cudaStream_t s, const float *phi, const cg_srcs_params *p, long long nsrc,
                             const long long *nsrc_dev, int nsm);
cudaError_t cg_srcs_lensing(cudaStream_t s, const float *phi, const cg_los_params *p, int nsm);
cudaError_t cg_srcs_skewers(cudaStream_t s, const float *dens, const float *phi, const cg_los_params *p, int nsm);
#endif
