/*
 * srcs_api.h -- launch interface of srcs.cu.
 */
#ifndef CG_SRCS_API_H
#define CG_SRCS_API_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"

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
  int *cmap;                 /* count map or NULL */
  unsigned short *counts;    /* N^3; CG_COUNT_ESC marks a cell in the overflow list */
  long long *ovf_cell;       /* cells holding CG_COUNT_ESC or more sources ...     */
  int *ovf_cnt;              /* ... and their counts                             */
  int *ovf_n;                /* entries used (zeroed by cg_srcs_count)           */
  long long *block_sums;     /* per block; exclusive offsets after the scan */
  long long capacity;
  float4 *pos;
  int *ipix;
  float *src;                /* 9 floats per source (Src) */
  unsigned int *err;
};

/* Per-cell counts are stored as uint16; the few cells at or above the escape
 * value (in practice the cells touching the observer, where n(z) ~ 1/r^2)
 * go to an overflow list of CG_OVF_CAP entries. */
#define CG_COUNT_ESC 65535
#define CG_OVF_CAP 4096

long long cg_srcs_nblocks(int N);
cudaError_t cg_srcs_count(cudaStream_t s, const float *grid, const cg_srcs_params *p, long long *total);
cudaError_t cg_srcs_emit(cudaStream_t s, const float *phi, const cg_srcs_params *p);
cudaError_t cg_srcs_beam_rsd(cudaStream_t s, const float *phi, const cg_srcs_params *p, long long nsrc, int nsm);

#endif
