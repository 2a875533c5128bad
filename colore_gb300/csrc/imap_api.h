/*
 * imap_api.h -- launch interface of imap.cu.
 */
#ifndef CG_IMAP_API_H
#define CG_IMAP_API_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"

struct cg_imap_params {
  cg::Box box;
  cg::Grid1 g;
  cg::Tab tz, bz, norm, v1, ih;
  int bias_model;
  float factor_vel;
  int nr;             /* shells, sorted by r0 (imap_preproc, imap.c:105-133) */
  const float *r0, *rf;
  const int *nsub;    /* per shell (imap.c:158-172) */
  int nsub_lo, nsub_hi;
  float rmin_here, rmax_here;
  int64_t nside, npix;
  float *data;        /* nr * npix, RING */
  int *nadd;          /* nr * npix       */
  unsigned int *err;
};

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm);

#endif
