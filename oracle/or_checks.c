/*
 * or_checks.c -- ORACLE (test infrastructure only).  Array wrappers around
 * the shared scalar functions of cg_math.h / cg_cell.h so that tests can
 * check them against libm, numpy and HEALPix identities on the CPU.
 */
#include <stdint.h>

#include "../colore_gb300/csrc/cg_exact.h"

void or_vec_expf(const float *x, float *y, long n) { for (long i = 0; i < n; i++) y[i] = cg_expf(x[i]); }
void or_vec_logf(const float *x, float *y, long n) { for (long i = 0; i < n; i++) y[i] = cg_logf(x[i]); }
void or_vec_log1pf(const float *x, float *y, long n) { for (long i = 0; i < n; i++) y[i] = cg_log1pf(x[i]); }
void or_vec_acosf(const float *x, float *y, long n) { for (long i = 0; i < n; i++) y[i] = cg_acosf(x[i]); }
void or_vec_atan2f(const float *y, const float *x, float *o, long n)
{
  for (long i = 0; i < n; i++) o[i] = cg_atan2f(y[i], x[i]);
}
void or_vec_sincosf(const float *x, float *s, float *c, long n)
{
  for (long i = 0; i < n; i++) cg_sincosf(x[i], &s[i], &c[i]);
}
/* Largest |cg_atan01_q(t) - atan(t) / (pi/2)| over every float t in [0, 1]
 * (libm's double atan as the reference). */
double or_atan_q_maxerr(void)
{
  const uint32_t top = 0x3f800000u; /* 1.0f */
  double mx = 0;
#pragma omp parallel for reduction(max : mx) schedule(static, 65536)
  for (long long b = 0; b <= (long long)top; b++) {
    const float t = cg_u2f((uint32_t)b);
    const double e = fabs((double)cg_atan01_q(t) - atan((double)t) * 0.63661977236758134308);
    if (e > mx) mx = e;
  }
  return mx;
}

void or_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out)
{
  cg_u32x4 r = cg_philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  for (int i = 0; i < 4; i++) out[i] = r.v[i];
}
void or_poisson(const float *lam, int *k, long n, uint32_t k0, uint32_t k1)
{
  for (long i = 0; i < n; i++) k[i] = cg_poisson(lam[i], k0, k1, (uint32_t)i, (uint32_t)(i >> 32));
}
void or_ang2pix(long nside, const float *cth, const float *phi, long long *pix, long n)
{
  for (long i = 0; i < n; i++) pix[i] = cg_ang2pix_ring(nside, cth[i], phi[i]);
}
void or_nest2ring(long nside, const long long *in, long long *out, long n)
{
  for (long i = 0; i < n; i++) out[i] = cg_nest2ring(nside, in[i]);
}
void or_ring2nest(long nside, const long long *in, long long *out, long n)
{
  for (long i = 0; i < n; i++) out[i] = cg_ring2nest(nside, in[i]);
}
void or_pix2vec_nest(long nside, const long long *in, float *v, long n)
{
  for (long i = 0; i < n; i++) cg_pix2vec_nest(nside, in[i], v + 3 * i);
}
void or_shell_index(const float *r0, const float *rf, int nr, const float *r, int *walk, int *bisect, long n)
{
  float rfm[4096];
  for (int i = 0; i < nr && i < 4096; i++) rfm[i] = i == 0 ? rf[0] : (rf[i] > rfm[i - 1] ? rf[i] : rfm[i - 1]);
  for (long i = 0; i < n; i++) {
    walk[i] = cg_shell_index(r0, rf, nr, r[i], 0);
    bisect[i] = cg_shell_index0(r0, rfm, nr, r[i]);
  }
}

/* RING pixels of float directions by the margin-checked single-precision
 * path (cg_pix_checked; -1 where it defers to double), with coordinate
 * error ein relative to r. */
void or_pix_checked(long nside, const float *xyz, long n, float ein, long long *pix)
{
  for (long i = 0; i < n; i++) {
    const cg_dir d = cg_dir_of(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], ein);
    pix[i] = cg_pix_checked(&d, (int)nside, ein);
  }
}

/* The float-float operations of cg_ff.h on n operand pairs: op 0 sum,
 * 1 product, 2 quotient, 3 square root of x, 4 product by the float y.h;
 * x and y as (h, l) pairs in xh/xl, yh/yl, the result in oh/ol. */
void or_ff_ops(int op, const float *xh, const float *xl, const float *yh, const float *yl, long n, float *oh,
               float *ol)
{
  for (long i = 0; i < n; i++) {
    const cg_ff x = cg_ff_make(xh[i], xl[i]), y = cg_ff_make(yh[i], yl[i]);
    cg_ff r;
    if (op == 0) r = cg_ff_add(x, y);
    else if (op == 1) r = cg_ff_mul(x, y);
    else if (op == 2) r = cg_ff_div(x, y);
    else if (op == 3) r = cg_ff_sqrt(x);
    else r = cg_ff_mulf(x, y.h);
    oh[i] = r.h;
    ol[i] = r.l;
  }
}

/* RING pixels of float-float positions (6 floats each: x, its rest, y, ...)
 * by the float-float tier (cg_pix_ff; -1 where it defers to double), each
 * within eP[i] of the double position. */
void or_pix_ff(long nside, const float *p, const float *eP, long n, long long *pix)
{
  float att[2 * (CG_ATT_N + 1)];
  cg_att_table(att);
  for (long i = 0; i < n; i++) {
    const float *q = p + 6 * i;
    pix[i] = cg_pix_ff(cg_ff_make(q[0], q[1]), cg_ff_make(q[2], q[3]), cg_ff_make(q[4], q[5]), eP[i], (int)nside,
                       att);
  }
}

/* The same decision by the double restatement shared with the kernels
 * (cgx_cart2sph + cgx_ang2pix). */
void or_pix_cgx(long nside, const double *xyz, long n, long long *pix)
{
  for (long i = 0; i < n; i++) {
    double r, cth, ph;
    cgx_cart2sph(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], &r, &cth, &ph);
    pix[i] = cgx_ang2pix(nside, cth, ph);
  }
}

/* cg_src_offset_checked on n (corner, uniform) pairs with one dx: out[i] the
 * float coordinate (0 when not certain), ok[i] 1 when certain; ref[i] the
 * double expression rounded to float (cgx_src_offset). */
void or_src_offset_checked(long n, const double *x0, double dx, const uint32_t *bits, float *out, int *ok, float *ref)
{
  const float dh = (float)dx, dl = (float)(dx - (double)(float)dx);
  for (long i = 0; i < n; i++) {
    const float c = (float)x0[i], l = (float)(x0[i] - (double)(float)x0[i]);
    float f = 0.0f;
    ok[i] = cg_src_offset_checked(c, l, dh, dl, bits[i], &f);
    out[i] = f;
    ref[i] = cgx_src_offset(x0[i], dx, bits[i]);
  }
}

/* cg_poisson_ptrs_checked against cgx_poisson_ptrs on n means: got[i] the
 * single-precision count (-1: left to double), ref[i] the double one, for
 * float means lam[i] known within elam[i] of the double mean lam64[i]. */
void or_ptrs_checked(long n, const float *lam, const float *elam, const double *lam64, const long long *cid, uint32_t k0,
                     uint32_t k1, int *got, int *ref)
{
  for (long i = 0; i < n; i++) {
    got[i] = cg_poisson_ptrs_checked(lam[i], elam[i], cid[i], k0, k1);
    ref[i] = cgx_poisson_ptrs(lam64[i], cid[i], k0, k1);
  }
}
