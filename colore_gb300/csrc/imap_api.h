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
  /* per shell index + 1 (index -1 below the shells, nr beyond them):
   * nsub (imap.c:158-174, as int bits), dx / nsub, 1 / nsub */
  const float4 *shp;
  float rmin_here, rmax_here;
  int64_t nside, npix;
  float *data;        /* nr * npix, RING */
  int *nadd;          /* nr * npix       */
  unsigned int *err;
  /* The first kernel lists every cell it computes (while the list has room)
   * and the second paints the listed cells' samples, split evenly over all
   * warps.  ctr[0] counts records, ctr[1] sample chunks taken, ctr[2] rows
   * taken, ctr[3] and ctr[4] the samples painted by each kernel (all zeroed
   * per launch). */
  long long list_cap;
  unsigned long long *ctr;
  struct cg_imap_cell *cells;     /* list_cap records                       */
  unsigned int *cell_n;           /* samples of each record (nsub^3)        */
  long long *cell_off;            /* first sample of each record (scanned)  */
  long long *scan_tmp;            /* cg_imap_scan_blocks(list_cap) entries  */
};

/* One listed cell: corner, brightness, radial shift, sub-cell size, 1/nsub,
 * and nsub | (shell index + 1) << 11. */
struct __align__(16) cg_imap_cell {
  float x0, y0, z0, temp, drr, dxs, inv_ns;
  int packed;
};

/* Bytes per listed cell (record, sample count, offset). */
#define CG_IMAP_CELL_BYTES (sizeof(struct cg_imap_cell) + sizeof(unsigned int) + sizeof(long long))

long long cg_imap_scan_blocks(long long cap);
cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm);

#endif
