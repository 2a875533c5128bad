/*
 * field_api.h -- launch interface between capi.cu and the per-grid-size
 * instantiations of field_impl.cu.
 */
#ifndef CG_FIELD_API_H
#define CG_FIELD_API_H

#include <cuda_runtime.h>
#include <stddef.h>

#include "cg_dev.cuh"

struct cg_field_launch {
  cudaStream_t stream;
  float2 *f[3];         /* grids (half spectrum in, padded real out) */
  cg::FillParams fill;  /* Fourier-space fill                       */
  float norm;           /* real-space scale applied in the x pass    */
  double2 *partials;    /* per-block (sum d, sum d^2) of grid 0       */
  const float2 *twN;    /* exp(+2 pi i j/N), j < N                   */
  const float2 *twH;    /* exp(+2 pi i j/(N/2)), j < N/2             */
  float2 *src;          /* 2LPT: the source grid (padded real in, destroyed) */
  unsigned int *err;    /* device error word (bulk-copy timeouts) */
  cudaEvent_t *ev;      /* NULL, or events recorded after each pass (fill+z, y, x) */
  int var[4];           /* tile variant of each pass (CG_PASS_*): 0 the plan's, 1 half, 2 twice */
};

/* Passes whose tile width the autotuner picks. */
#define CG_PASS_FILL2 0 /* fill + z of the Gaussian field and potential */
#define CG_PASS_FILL3 1 /* fill + z of the 1LPT displacements          */
#define CG_PASS_Y 2     /* column transforms along y                   */
#define CG_PASS_X 3     /* row c2r along x (without the moment sums)   */

#define CG_FIELD_SIZES(X) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(1024) X(2048)

#define CG_FIELD_DECL(n)                                                 \
  extern "C" cudaError_t cg_field_gauss_##n(const cg_field_launch *L); \
  extern "C" cudaError_t cg_field_lpt_##n(const cg_field_launch *L);   \
  extern "C" cudaError_t cg_field_lpt2_##n(const cg_field_launch *L);  \
  extern "C" size_t cg_field_npartials_##n(void);                      \
  extern "C" int cg_field_tile_##n(int pass, int v);                    \
  extern "C" cudaError_t cg_field_pass_##n(const cg_field_launch *L, int pass, int v, int nf);
CG_FIELD_SIZES(CG_FIELD_DECL)
#undef CG_FIELD_DECL

#endif /* CG_FIELD_API_H */
