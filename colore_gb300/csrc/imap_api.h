/*
 * imap_api.h -- launch interface of imap.cu.
 */
#ifndef CG_IMAP_API_H
#define CG_IMAP_API_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "cg_exact.h"

/* One listed cell (16 bytes): ix | iy << 16; iz | flags << 11 | half(edrr)
 * << 16 with the flags the shell mode (2 bits, CG_SH_*), delta + 1 (2 bits)
 * and double (16: every sample decided in double); brightness; radial
 * shift.  Grids up to 2048 cells a side. */
struct __align__(16) cg_imap_rec {
  unsigned int ixy, izf;
  float temp, drr;
};

#define CG_IMAP_REC_BYTES 16
#define CG_IMAP_BUCKETS_MAX 4100 /* shells -1 .. nr: nr <= 4096 */

struct cg_imap_params {
  cg::Box box;
  cg_imap_args a;    /* tables, corners, shells (device pointers) */
  int nr, nbk;       /* shells; buckets nbk = nr + 2, bucket j + 1 for shell j */
  long long npix;
  float *data;       /* nr * npix, RING */
  int *nadd;         /* nr * npix       */
  unsigned int *err;
  unsigned long long *xstats; /* [2] cells, [3] samples decided in double */
  int force_double;
  /* cells are listed per bucket (the shell of their corner, which fixes
   * nsub), in the slots [base[b], base[b] + cap[b]); cnt[b] counts them
   * (may exceed cap: those cells are painted by the listing kernel) */
  cg_imap_rec *recs;
  const long long *base, *cap;
  unsigned long long *cnt;
  /* chunks of the painting pass: chunk_off[b] the first chunk of bucket b
   * (nbk + 1 entries, set on the device) */
  unsigned long long *chunk_off;
  /* ctr: [0] chunks taken, [1] rows taken, [2] samples drawn, [3] samples
   * painted by the listing kernel, [4] double-queue entries */
  unsigned long long *ctr;
  unsigned long long *queue; /* record << 30 | sample, for the double pass */
  long long queue_cap;
};

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm);
/* RING pixels of n float directions (device arrays) at nside by the
 * margin-checked decision the painting uses, with coordinate error ein
 * relative to r; -1 where only double can decide. */
cudaError_t cg_pix_checked_dev(cudaStream_t s, int nside, const float *xyz, long long n, float ein, long long *pix,
                               int nsm);
/* Shared memory of the painting kernel for nr shells and nbk buckets. */
size_t cg_imap_shell_smem(int nr, int nbk);

#endif
