/*
 * kappa_api.h -- launch interface of kappa.cu.
 */
#ifndef CG_KAPPA_API_H
#define CG_KAPPA_API_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"

struct cg_kappa_params {
  cg::Box box;
  int64_t nside, npix;
  int nplanes;            /* sorted by distance (kappa_beams_preproc, kappa.c:39-76) */
  const int *ir_min, *ir_max;
  const float *inv_r_max;
  int nr;                 /* radial steps N/2 (get_radial_params, common.c:333-337) */
  float dr;
  const float *fac1, *fac2; /* r D (1+z) dr and r^2 D (1+z) dr, kappa.c:109-116 */
  float *map;             /* nplanes * npix, RING order */
};

cudaError_t cg_kappa_integrate(cudaStream_t s, const float *phi, const cg_kappa_params *p);
/* Custom map (cstm_get_beam_properties, cstm.c:68-145): per pixel,
 * dr * sum over ir_min..ir_max of kz (bias_model(d, bz) norm - 1), with d the
 * CIC-interpolated density at the step (interpolate_from_grid, beaming.c:183-265). */
struct cg_cstm_params {
  cg::Box box;
  cg::Grid1 g;
  cg::Tab norm; /* normalisation table of this map, evaluated at each step centre */
  int64_t nside, npix;
  int ir_min, ir_max, bias_model;
  float dr;
  const float *kz, *bz; /* K(z)/H(z) and b(z) at the step centres, from the FP64 tables */
  float *map;           /* npix, NEST order */
};
cudaError_t cg_cstm_integrate(cudaStream_t s, const float *dens, const cg_cstm_params *p);

/* ISW: fac1 = 2 PD(r) dr (isw.c:105-111); fac2 and inv_r_max unused. */
cudaError_t cg_isw_integrate(cudaStream_t s, const float *phi, const cg_kappa_params *p);

#endif
