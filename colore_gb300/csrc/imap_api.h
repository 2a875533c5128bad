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
  /* Cells with at least nsub_heavy sub-samples per side are listed by the
   * first kernel and painted by the second with their samples split evenly
   * over all warps.  ctr[0] packs (heavy records << 40) | heavy samples,
   * ctr[1] counts heavy chunks taken, ctr[2] rows taken, ctr[3] and ctr[4]
   * the samples painted by each kernel (all zeroed per launch). */
  int nsub_heavy;
  long long heavy_cap;
  unsigned long long *ctr;
  long long *heavy_off;            /* first sample of each record          */
  struct cg_heavy_cell *heavy;     /* heavy_cap records                    */
};

struct __align__(16) cg_heavy_cell {
  float x0, y0, z0, temp, drr, dxs;
  int nsub, irad0;
};

/* Sub-samples per side from which a cell is painted by the heavy pass, and
 * the largest heavy list (records of 40 bytes). */
#define CG_NSUB_HEAVY 8
#define CG_HEAVY_MAX (1LL << 23)

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm);

#endif
