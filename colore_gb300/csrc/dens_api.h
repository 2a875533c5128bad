/*
 * dens_api.h -- launch interface of dens.cu.
 */
#ifndef CG_DENS_API_H
#define CG_DENS_API_H

#include <cuda_runtime.h>
#include <stddef.h>

#include "cg_dev.cuh"

struct cg_bins_params {
  cg::Box box;
  cg::Grid1 g;
  cg::Tab zt, d1;
  int mode;
  const float *sigma2f;   /* device scalar, lognormal only */
  int nz;
  float idz;
  int nt, bias_model;
  cg::Tab bz[8];          /* bias tables of the tracers of this launch */
  unsigned long long *ncount; /* [nz], zeroed by the caller */
  unsigned long long *acc;    /* [1 + nt][nz][2] fixed-point sums, zeroed by the caller */
  double *zsum;               /* [nz], written from acc */
  double *bsum;               /* [nt][nz], written from acc */
  unsigned int *err;          /* device error bits (mode CG_DMODE_RHO) */
};

struct cg_lpt_params {
  cg::Box box;
  cg::Grid1 g;
  cg::Tab d1;
  int interp; /* 0 NGP, 1 CIC, 2 TSC (pos_2_dens, density.c:178-187) */
  /* 2LPT: second-order displacements and the D2 growth (density.c:890), or NULL */
  const float *d2x, *d2y, *d2z;
  cg::Tab d2;
};
/* Second-order source of 2LPT (density.c:739-759), in place into zz:
 * xx yy + xx zz + yy zz - xy^2 - xz^2 - yz^2 over the N^3 cells of the
 * padded grids. */
cudaError_t cg_lpt2_source(cudaStream_t s, const float *xx, const float *xy, const float *xz, const float *yy,
                           const float *yz, float *zz, int N, int nsm);

cudaError_t cg_moments_final(cudaStream_t s, const double2 *part, size_t n, double inv_ncell, double *stats,
                             float *s2f);
cudaError_t cg_dens_bins(cudaStream_t s, float *grid, const cg_bins_params *p, int nsm);
int cg_dens_bins_max_tracers(void);
/* Normalisation tables from the bin sums, on the device (the host part of
 * compute_density_normalization, density.c:1272-1355, in the same double
 * operations): per tracer t, out[t (CG_NA + 2) + i] = norm(z(r_i)) for the
 * CG_NA table radii, then the two edge values, and the same in double into
 * out64 (or NULL).  zr: z(r_i) (CG_NA doubles); zlast: z(L/2).
 * nz <= CG_NORM_NZ_MAX. */
#define CG_NORM_NZ_MAX 3072
#define CG_MAX_DEVICES 64
cudaError_t cg_norm_tables(cudaStream_t s, const unsigned long long *ncount, const double *zsum, const double *bsum,
                           int nz, int nt, double zlast, const double *zr, float *out, double *out64);

/* Largest number of redshift bins of the allocation-free bins entry, whose
 * scratch (per bin: cell count, redshift sum and one bias sum per tracer,
 * for up to cg_dens_bins_max_tracers() = 8 tracers, and a 16-byte
 * accumulator for each sum) is a fixed device array of
 * CG_BINS_STATIC_NZ * 28 * 8 bytes = 224 KiB. */
#define CG_BINS_STATIC_NZ 1024
#define CG_BINS_STATIC_BYTES ((size_t)CG_BINS_STATIC_NZ * 28 * 8)
/* Device address and size of that array in the current device's context. */
cudaError_t cg_dens_bins_static_scratch(void **ptr, size_t *bytes);
cudaError_t cg_lpt_cic(cudaStream_t s, float *grid, const float *dx, const float *dy, const float *dz,
                       const cg_lpt_params *p, int nsm);

#endif
