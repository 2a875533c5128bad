/*
 * oracle.h -- ORACLE: CPU restatement of CoLoRe's mock-generation path.
 *
 * Test infrastructure only.  Nothing in the product (colore_gb300/,
 * include/) links, imports or calls this code; only tests/, the smoke check
 * of __graft_entry__.py and the CPU-baseline leg of bench.py do, as the
 * checker and as the timed CPU reference.
 *
 * Two restatements live here:
 *   ref64 (or_ref64.c): the reference's arithmetic in double precision with
 *         libm, loop by loop (file:line cited per function).  It is the
 *         tolerance oracle for floating-point outputs and the CPU baseline.
 *   dev32 (or_dev32.c): the same loops evaluated with the single-precision
 *         per-cell arithmetic that the GPU kernels define (cg_cell.h), so
 *         that integer outputs -- Poisson counts, catalogue order, HEALPix
 *         pixel ids, hit counts -- can be compared bit for bit.
 * Real grids passed to dev32 functions use the padded in-place layout of
 * the GPU (index ix + 2(N/2+1)(iy + N iz)); ref64 grids are unpadded N^3.
 *
 * Parity against the reference binary itself is unpinned: the reference
 * cannot be built here (GSL, FFTW, libconfig, cfitsio, chealpix absent) and
 * ships no tests or fixtures; see the tests for the known-answer values it
 * does pin (cosmology from the notebook log, Philox vectors).
 */
#ifndef CG_ORACLE_H
#define CG_ORACLE_H

#include <complex.h>
#include <stdint.h>

#include "../include/colore_cuda.h"

/* ---- FFT (or_fft.c) ---- */
int or_c2r_3d(int N, const double complex *in, double *out);
int or_r2c_3d(int N, const double *in, double complex *out);

/* ---- ref64 (or_ref64.c) ---- */
int or_fill64(const cg_config *cfg, double complex *dk, double complex *pk);
int or_field64(const cg_config *cfg, double *dens, double *npot, double stats[4]);
int or_density64(const cg_config *cfg, double *dens, double sigma2);
int or_lpt64(const cg_config *cfg, const double *dens_gauss, double *dens_out, double *disp);
int or_lpt2_64(const cg_config *cfg, const double *dens_gauss, double *dens_out, double *disp, double *disp2);
int or_bins64(const cg_config *cfg, const double *dens, int nz, double idz, unsigned long long *narr, double *zarr,
              double *bsum);
int or_norm_tables64(const cg_config *cfg, double *tabs, double *e0f, int *nz_out, unsigned long long *narr,
                     double *zarr, double *bsum, const double *dens);
int or_lambda64(const cg_config *cfg, int ipop, const double *dens, const double *normtab, double n0, double nf,
                double *lambda);
int or_kappa64(const cg_config *cfg, const double *npot, double *map);
int or_isw64(const cg_config *cfg, const double *npot, double *map);
int or_cstm_steps(const cg_config *cfg, int ipop, double *kz, double *bz, int *ir_min, int *ir_max);
int or_cstm64(const cg_config *cfg, int ipop, const double *dens, const double *normtab, double n0, double nf,
              double *map);
int or_lens64(const cg_config *cfg, const double *npot, long long n, const float *pos4, double *out);
int or_skw64(const cg_config *cfg, const double *dens, const double *npot, int gauss, double sigma2, long long n,
             const float *pos4, double *dout, double *vout);
/* sprec: the reference built with _SPREC (float grids and shells, float
 * potential differences), the build the FP32 path matches; 0: the double
 * build, which the FP64 baseline path matches. */
int or_imap64(const cg_config *cfg, int ipop, const double *dens, const double *npot, const double *normtab,
              double n0, double nf, double *data, int *nadd, int sprec);
int or_imap64_part(const cg_config *cfg, int ipop, const double *dens, const double *npot, const double *normtab,
                   double n0, double nf, int iz_stride, double *data, int *nadd, long long *nsamp, int sprec);
long long or_imap_samples(const cg_config *cfg, int ipop);
int or_kappa64_part(const cg_config *cfg, const double *npot, int pix_stride, double *map);
long long or_poisson_total64(const cg_config *cfg, int ipop, const double *lam);
/* Counts and catalogue in double (srcs.c:156-283, 386-416) from the float
 * density as doubles (unpadded) and the double normalisation table (CG_NA
 * values, then the two edges); or_emit64 takes the counts and the potential
 * (unpadded doubles of the float grid). */
int or_counts64(const cg_config *cfg, int ipop, const double *dens, const double *normtab, int *counts,
                long long *total);
int or_emit64(const cg_config *cfg, int ipop, const double *npot, const int *counts, long long cap, float *pos4,
              int *ipix, float *src9, int *cmap, long long *nsrc);
int or_run_mock64(const cg_config *cfg, int nthreads_hint, long long *nsrc_total, double *checksum);

/* ---- dev32 (or_dev32.c) ---- */
int or_density32(const cg_config *cfg, float *dens, float sigma2f, int mode);
int or_bins32(const cg_config *cfg, const float *dens, int nz, double idz, unsigned long long *narr, double *zarr,
              double *bsum);
/* Source counts and catalogue as the GPU computes them: float margins with
 * double decisions where they do not hold (cg_exact.h).  norm32 / norm64:
 * the normalisation table (CG_NA values, then the two edges) in float and
 * double; *fallbacks: cells (counts) or pixels (emit) decided in double. */
int or_counts32(const cg_config *cfg, int ipop, const float *dens, const float *norm32, const double *norm64,
                int *counts, long long *total, long long *fallbacks);
int or_emit32(const cg_config *cfg, int ipop, const float *dens, const float *npot, const float *norm32,
              const double *norm64, long long cap, float *pos4, int *ipix, float *src9, int *cmap, long long *nsrc,
              long long *fallbacks);
int or_beam_rsd32(const cg_config *cfg, const float *npot, long long n, const float *pos4, float *src9);
/* The intensity map as the GPU paints it (float margins, double where they
 * do not hold); stats: cells and samples decided in double, samples drawn. */
int or_imap32(const cg_config *cfg, int ipop, const float *dens, const float *npot, const float *norm32,
              const double *norm64, float *data, int *nadd, long long *stats);
int or_kappa32(const cg_config *cfg, const float *npot, float *map);
int or_isw32(const cg_config *cfg, const float *npot, float *map);
int or_cstm32(const cg_config *cfg, int ipop, const float *dens, const float *normtab, float n0, float nf,
              float *map);
int or_lens32(const cg_config *cfg, const float *npot, long long n, const float *pos4, float *src9);
int or_skw32(const cg_config *cfg, const float *dens, const float *npot, int gauss, float sigma2f, long long n,
             const float *pos4, float *dout, float *vout);

/* or_sht.c: Legendre part of the FP64 map -> a_lm analysis (per m and
 * northern ring, symmetric / antisymmetric ring Fourier sums of K maps). */
int or_sht_legendre(int lmax, int nring, int K, const double *z, const double *S, const double *A, double omega,
                    double *alm);

void or_src_offset_checked(long n, const double *x0, double dx, const uint32_t *bits, float *out, int *ok, float *ref);

void or_ptrs_checked(long n, const float *lam, const float *elam, const double *lam64, const long long *cid, uint32_t k0,
                     uint32_t k1, int *got, int *ref);

#endif
