/*
 * cg_exact.h -- integer outputs equal to the reference's double-precision
 * arithmetic.
 *
 * Poisson counts, HEALPix pixel ids, intensity-map shells and hit counts are
 * decisions: a comparison or a truncation of a value that the reference
 * computes in double precision (srcs.c:156-183, healpix_extra.c:141-172,
 * imap.c:179-231).  The kernels compute those values in single precision
 * together with a bound on their distance to the reference's double value,
 * and keep the single-precision decision only when the value is farther from
 * the decision boundary than the bound; otherwise they decide again with the
 * double-precision restatement below.  The result is the reference
 * arithmetic's decision in every case, at the cost of single precision for
 * all but a small fraction of the decisions.
 *
 * Part 1 restates the reference's double arithmetic (expression order
 * included: products and sums associate as in the C source, never
 * contracted into fused multiply-adds).  On the device the elementary
 * functions are CUDA's double exp, log, pow, atan2 and fmod; on the host
 * libm's.  Those two may differ in the last bit, which moves a decision only
 * when a value falls within ~1e-16 relative of its boundary.
 *
 * Part 2 holds the single-precision evaluations and their error bounds.
 * Bounds are stated for the device's documented accuracies (rsqrt.approx
 * and rcp.approx: relative error below 2^-22; expf: 2 ulp), which also cover
 * the host's correctly rounded operations.
 */
#ifndef CG_EXACT_H
#define CG_EXACT_H

#include "cg_cell.h"
#include "cg_ff.h"
#include "colore_cuda.h"

#if defined(__CUDA_ARCH__)
#define X_ADD(a, b) __dadd_rn((a), (b))
#define X_SUB(a, b) __dsub_rn((a), (b))
#define X_MUL(a, b) __dmul_rn((a), (b))
#define X_DIV(a, b) __ddiv_rn((a), (b))
#define X_SQRT(a) __dsqrt_rn((a))
#else
#define X_ADD(a, b) ((double)(a) + (double)(b))
#define X_SUB(a, b) ((double)(a) - (double)(b))
#define X_MUL(a, b) ((double)(a) * (double)(b))
#define X_DIV(a, b) ((double)(a) / (double)(b))
#define X_SQRT(a) sqrt((double)(a))
#endif

#define CGX_TWOPI 6.283185307179586476925286766559005768394  /* healpix_extra.c:137 */
#define CGX_INV_HALFPI 0.6366197723675813430755350534900574   /* healpix_extra.c:139 */
#define CGX_2PI_M (2 * 3.14159265358979323846)                /* 2*M_PI, srcs.c:82 */

/* ======================================================================= */
/* Part 1: the reference's double-precision arithmetic                     */
/* ======================================================================= */

/* f_of_r_linear, cosmo.c:30-38. */
CG_HD double cgx_bg(const double *f, const double *r_arr, double idr, double r_last, double f0, double ff, double r)
{
  if (r <= 0) return f0;
  if (r >= r_last) return ff;
  const int ir = (int)X_MUL(r, idr);
  return X_ADD(f[ir], X_MUL(X_MUL(X_SUB(f[ir + 1], f[ir]), X_SUB(r, r_arr[ir])), idr));
}

/* bias_model, common.h:414-431. */
CG_HD double cgx_bias(double d, double b, int model)
{
  if (d <= -1) return 0;
  if (model == CG_BIAS_EXPLIN) {
    if (d < 0) return exp(X_DIV(X_MUL(b, d), X_ADD(1.0, d)));
    return X_ADD(1.0, X_MUL(b, d));
  }
  if (model == CG_BIAS_LIN) {
    const double v = X_ADD(1.0, X_MUL(b, d));
    return v > 0 ? v : 0;
  }
  return pow(X_ADD(1.0, d), b);
}

/* Cell corner i*dx - p (srcs.c:159-167, imap.c:184-192). */
CG_HD double cgx_coord(int i, double dx, double p) { return X_SUB(X_MUL((double)i, dx), p); }

/* sqrt(x*x+y*y+z*z) (srcs.c:168, imap.c:195, cart2sph srcs.c:70). */
CG_HD double cgx_norm3(double x, double y, double z)
{
  return X_SQRT(X_ADD(X_ADD(X_MUL(x, x), X_MUL(y, y)), X_MUL(z, z)));
}

/* Tables of one source population in double: the background radii, n(r),
 * b(r) and the normalisation (CG_NA values, then its two edge values). */
typedef struct {
  const double *r, *nz, *bz, *norm;
  double idr, r_last, bz0;
  double dx, cell_vol, rlim, p[3];
  int bias_model;
} cgx_srcs_tabs;

/* lambda = ndens*cell_vol*bias_model(d,b)*dnorm of a cell (srcs.c:163-178);
 * 0 where the reference draws no deviate (r >= L/2+20 or ndens <= 0). */
CG_HD double cgx_lambda(const cgx_srcs_tabs *t, int ix, int iy, int iz, float d)
{
  const double x0 = cgx_coord(ix, t->dx, t->p[0]), y0 = cgx_coord(iy, t->dx, t->p[1]);
  const double z0 = cgx_coord(iz, t->dx, t->p[2]);
  const double r = cgx_norm3(x0, y0, z0);
  if (!(r < t->rlim)) return 0;
  const double nd = cgx_bg(t->nz, t->r, t->idr, t->r_last, 0, 0, r);
  if (!(nd > 0)) return 0;
  const double b = cgx_bg(t->bz, t->r, t->idr, t->r_last, t->bz0, 1, r);
  const double dn = cgx_bg(t->norm, t->r, t->idr, t->r_last, t->norm[CG_NA], t->norm[CG_NA + 1], r);
  return X_MUL(X_MUL(X_MUL(nd, t->cell_vol), cgx_bias((double)d, b, t->bias_model)), dn);
}

/* The Poisson stream (replacing gsl_ran_poisson, common.c:185-189, whose
 * MT19937 stream follows the OpenMP thread count): cells 4m..4m+3 take the
 * four words of one Philox4x32-10 block with counter (m, 0, 0, 0); a cell's
 * uniform is its word's top 24 bits times 2^-24, exact in float and double.
 * The PTRS branch draws its pairs from counter (cell, iteration, 1, 0). */
CG_HD uint32_t cg_pois_word(long long cid, uint32_t k0, uint32_t k1)
{
  const unsigned long long m = (unsigned long long)cid >> 2;
  const cg_u32x4 w = cg_philox4x32_10((uint32_t)m, (uint32_t)(m >> 32), 0u, 0u, k0, k1);
  return w.v[cid & 3];
}

/* Poisson deviate with mean lam in double: inversion by sequential search
 * for lam < 10 with the cell's uniform u; PTRS transformed rejection
 * (W. Hormann, "The transformed rejection method for generating Poisson
 * random variables", Insurance: Mathematics and Economics 12 (1993) 39-45)
 * for lam >= 10, with log k! from lgamma.  Iterations are bounded. */
CG_HD_COLD int cgx_poisson_ptrs(double lam, long long cid, uint32_t k0, uint32_t k1)
{
  const double slam = X_SQRT(lam);
  const double loglam = log(lam);
  const double b = X_ADD(X_MUL(2.53, slam), 0.931);
  const double a = X_ADD(X_MUL(0.02483, b), -0.059);
  const double invalpha = X_ADD(1.1239, X_DIV(1.1328, X_SUB(b, 3.4)));
  const double vr = X_SUB(0.9277, X_DIV(3.6224, X_SUB(b, 2.0)));
  for (uint32_t it = 0; it < 64u; it++) {
    const cg_u32x4 w = cg_philox4x32_10((uint32_t)cid, (uint32_t)((unsigned long long)cid >> 32), it, 1u, k0, k1);
    const double U = X_SUB((double)cg_u01f(w.v[0]), 0.5);
    const double V = (double)cg_u01f(w.v[1]);
    const double us = X_SUB(0.5, fabs(U));
    const double kd = floor(X_ADD(X_ADD(X_MUL(X_ADD(X_DIV(X_MUL(2.0, a), us), b), U), lam), 0.43));
    if (us >= 0.07 && V <= vr) return (int)kd;
    if (kd < 0 || (us < 0.013 && V > us)) continue;
    const double lhs = X_ADD(log(V), X_SUB(log(invalpha), log(X_ADD(X_DIV(a, X_MUL(us, us)), b))));
    const double rhs = X_SUB(X_SUB(X_MUL(kd, loglam), lam), lgamma(X_ADD(kd, 1.0)));
    if (lhs <= rhs) return (int)kd;
  }
  return (int)floor(lam);
}

CG_HD int cgx_poisson(double lam, double u, long long cid, uint32_t k0, uint32_t k1)
{
  if (!(lam > 0)) return 0;
  if (lam < 10) {
    double p = exp(-lam), F = p;
    int k = 0;
    while (u >= F && k < 200) {
      k++;
      p = X_MUL(p, X_DIV(lam, (double)k));
      F = X_ADD(F, p);
    }
    return k;
  }
  return cgx_poisson_ptrs(lam, cid, k0, k1);
}

/* cart2sph, srcs.c:68-85 and imap.c:24-41: the direction normalised by r
 * before atan2, phi shifted into [0, 2 pi]. */
CG_HD void cgx_cart2sph(double x, double y, double z, double *r, double *cth, double *phi)
{
  *r = cgx_norm3(x, y, z);
  if (*r == 0) {
    *cth = 1;
    *phi = 0;
    return;
  }
  const double xn = X_DIV(x, *r), yn = X_DIV(y, *r);
  *cth = X_DIV(z, *r);
  *phi = atan2(yn, xn);
  if (*phi < 0) *phi = X_ADD(*phi, CGX_2PI_M);
}

/* he_ang2pix (RING), healpix_extra.c:118-172. */
CG_HD double cgx_fmodulo(double v1, double v2)
{
  if (v1 >= 0) return (v1 < v2) ? v1 : fmod(v1, v2);
  const double tmp = X_ADD(fmod(v1, v2), v2);
  return (tmp == v2) ? 0. : tmp;
}

CG_HD long long cgx_ang2pix(long long nside, double cth, double phi)
{
  const double ctha = fabs(cth);
  const double tt = X_MUL(cgx_fmodulo(phi, CGX_TWOPI), CGX_INV_HALFPI);
  const double ns = (double)nside;
  if (ctha <= 2.0 / 3.0) {
    const double temp1 = X_MUL(ns, X_ADD(0.5, tt));
    const double temp2 = X_MUL(X_MUL(ns, cth), 0.75);
    const int jp = (int)X_SUB(temp1, temp2), jm = (int)X_ADD(temp1, temp2);
    const int ir = (int)nside + 1 + jp - jm;
    const int kshift = 1 - (ir & 1);
    int ip = (jp + jm - (int)nside + kshift + 1) / 2;
    ip %= 4 * (int)nside;
    if (ip < 0) ip += 4 * (int)nside;
    return nside * (nside - 1) * 2 + (long long)(ir - 1) * 4 * nside + ip;
  }
  const double tp = X_SUB(tt, (double)(int)tt);
  const double tmp = X_MUL(ns, X_SQRT(X_MUL(3.0, X_SUB(1.0, ctha))));
  const int jp = (int)X_MUL(tp, tmp), jm = (int)X_MUL(X_SUB(1.0, tp), tmp);
  const int ir = jp + jm + 1;
  int ip = (int)X_MUL(tt, (double)ir);
  ip %= 4 * ir;
  if (ip < 0) ip += 4 * ir;
  if (cth > 0) return 2LL * ir * (ir - 1) + ip;
  return 12 * nside * nside - 2LL * ir * (ir + 1) + ip;
}

/* vec2pix_ring (chealpix, srcs.c:268) for the base pixels: z = v_z/|v| and
 * phi = atan2(v_y, v_x) into the same RING pixelisation. */
CG_HD long long cgx_vec2pix_ring(long long nside, double x, double y, double z)
{
  const double vlen = cgx_norm3(x, y, z);
  return cgx_ang2pix(nside, X_DIV(z, vlen), atan2(y, x));
}

/* Source position component x0 + dx (u - 1/2) in double, stored as float
 * (srcs.c:261-263). */
CG_HD float cgx_src_offset(double x0, double dx, uint32_t bits)
{
  return (float)X_ADD(x0, X_MUL(dx, X_SUB((double)cg_u01f(bits), 0.5)));
}

/* The same float coordinate from single-precision arithmetic: 1 with *out
 * when it is certainly the double expression rounded to float, 0 otherwise.
 * The corner x0 and dx come as float pairs (c + l, dh + dl; each pair
 * within 2^-48 of the double value); u - 1/2 is exact in float.  The sum
 * x0 + dx (u - 1/2) is carried as s + lo (dh t split exactly by an FMA,
 * c + dh t by TwoSum), within 2^-44 (|c| + |s| + dh) of the reference's
 * double value including its two roundings; f = fl(s + lo) is then the
 * double value's float rounding unless s + lo lies that close to the
 * midpoint between f and its neighbour on the side of s + lo. */
CG_HD int cg_src_offset_checked(float c, float l, float dh, float dl, uint32_t bits, float *out)
{
  const float t = CG_SUB(cg_u01f(bits), 0.5f); /* exact: 24-bit uniform */
  const float ph = CG_MUL(dh, t);
  const float pe = CG_FMA(dh, t, -ph); /* dh t = ph + pe exactly */
  const float q = CG_MUL(dl, t);
  const float s = CG_ADD(c, ph); /* TwoSum: c + ph = s + e */
  const float bv = CG_SUB(s, c);
  const float e = CG_ADD(CG_SUB(c, CG_SUB(s, bv)), CG_SUB(ph, bv));
  const float lo = CG_ADD(CG_ADD(e, l), CG_ADD(pe, q));
  const float f = CG_ADD(s, lo);
  const float r = CG_ADD(CG_SUB(s, f), lo); /* s - f exact: f is within an ulp of s */
  const float nb = nextafterf(f, r >= 0.0f ? 3.0e38f : -3.0e38f);
  const float h = CG_MUL(0.5f, cg_fabsf(CG_SUB(nb, f)));
  const float E = CG_FMA(cg_fabsf(r), 1.2e-7f, CG_MUL(5.7e-14f, CG_ADD(CG_ADD(cg_fabsf(c), cg_fabsf(s)), dh)));
  if (!(CG_SUB(h, cg_fabsf(r)) > E)) return 0;
  *out = f;
  return 1;
}

/* Shell of radius r among contiguous sorted shells (edges b[0..nr], shell i
 * between b[i] and b[i+1]): the walk of get_r_index_imap (imap.c:76-103)
 * gives this from any start; -1 below the shells, nr at or beyond them. */
CG_HD int cgx_shell(const float *b, int nr, double r)
{
  if (r < (double)b[0]) return -1;
  if (r >= (double)b[nr]) return nr;
  int lo = 0, hi = nr - 1; /* last i with b[i] <= r */
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((double)b[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

/* ======================================================================= */
/* Part 2: single precision with error bounds                              */
/* ======================================================================= */

#define CG_E24 5.9604644775390625e-08f /* 2^-24 */
#define CG_E22 2.384185791015625e-07f  /* 2^-22 */

/* Fast reciprocal square root and reciprocal: the device's approximate
 * instructions (relative error below 2^-22), correctly rounded on the host. */
CG_HD float cg_rsqrt_fast(float x)
{
#if defined(__CUDA_ARCH__)
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
#else
  return 1.0f / sqrtf(x);
#endif
}

CG_HD float cg_rcp_fast(float x)
{
#if defined(__CUDA_ARCH__)
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
#else
  return 1.0f / x;
#endif
}

CG_HD float cg_fmaxf(float a, float b) { return a > b ? a : b; }
CG_HD float cg_fminf(float a, float b) { return a < b ? a : b; }
/* min / max of values that are never NaN (magnitudes of finite coordinates,
 * distances to integers): fminf / fmaxf, one instruction on the device,
 * where the selects above (which keep a NaN bound NaN) take two. */
CG_HD float cg_min_nn(float a, float b) { return fminf(a, b); }
CG_HD float cg_max_nn(float a, float b) { return fmaxf(a, b); }

/* Distance of x >= 0 to the nearest integer, and floor(x). */
CG_HD float cg_int_dist(float x, int *fl)
{
  const float f = floorf(x);
  *fl = (int)f;
  const float d = CG_SUB(x, f); /* exact: x and f share the exponent range */
  return d < 0.5f ? d : CG_SUB(1.0f, d);
}

/* Table lookup f_of_r_linear in single precision with a bound on its
 * distance to the double lookup of the double table at the double radius.
 * tf: float table (the double table rounded); ir, t from the float radius;
 * dt bounds |t - t_double| in units of one table step.  Near a node the
 * double radius may fall in the neighbouring segment: the slope bound then
 * takes the larger of the adjacent segments. */
typedef struct {
  float v, e;
} cg_ve;

CG_HD cg_ve cg_tab_ve(const float *tf, int na, int ir, float t, float dt)
{
  const float fi = tf[ir], fj = tf[ir + 1];
  const float df = CG_SUB(fj, fi);
  cg_ve o;
  o.v = CG_FMA(df, t, fi);
  float sl = cg_fabsf(df);
  if (t < dt && ir > 0) sl = cg_fmaxf(sl, cg_fabsf(CG_SUB(fi, tf[ir - 1])));
  if (t > 1.0f - dt && ir + 2 < na) sl = cg_fmaxf(sl, cg_fabsf(CG_SUB(tf[ir + 2], fj)));
  const float mag = cg_fmaxf(cg_fabsf(fi), cg_fabsf(fj));
  /* table roundings (2 x 2^-24 of the nodes), the slope times the radius
   * error, the subtraction and the fused multiply-add (2 x 2^-24), with a
   * factor 2 to spare */
  o.e = CG_MUL(2.0f, CG_FMA(sl, CG_ADD(dt, CG_E24), CG_MUL(4.0f * CG_E24, CG_ADD(mag, cg_fabsf(o.v)))));
  return o;
}

/* bias_model in single precision, value and absolute error bound given an
 * absolute error eb on b (d is exact: the same float on both sides). */
CG_HD cg_ve cg_bias_ve(float d, float b, float eb, int model)
{
  cg_ve o;
  o.v = 0.0f;
  o.e = 0.0f;
  if (d <= -1.0f) return o;
  if (model == CG_BIAS_EXPLIN && d < 0.0f) {
    const float q = CG_DIV(d, CG_ADD(1.0f, d)); /* d/(1+d), relative error 2^-23 */
    const float e = CG_MUL(b, q);
    o.v = expf(e);
    /* exponent error |q| eb + |e| 2^-22; expf 2 ulp; then e^x scaling */
    const float ee = CG_FMA(cg_fabsf(q), eb, CG_MUL(cg_fabsf(e), CG_E22));
    o.e = CG_MUL(o.v, CG_ADD(CG_MUL(2.0f, ee), 8.0f * CG_E24));
    return o;
  }
  if (model == CG_BIAS_EXPLIN || model == CG_BIAS_LIN) {
    float v = CG_FMA(b, d, 1.0f);
    const float ev = CG_FMA(cg_fabsf(d), eb, CG_MUL(2.0f * CG_E24, cg_fabsf(v) + 1.0f));
    if (model == CG_BIAS_LIN && v <= 0.0f) v = 0.0f;
    o.v = v;
    o.e = CG_MUL(2.0f, ev);
    return o;
  }
  /* (1+d)^b = exp(b log1p(d)) */
  const float l = cg_log1pf(d); /* within 4 ulp */
  const float e = CG_MUL(b, l);
  o.v = expf(e);
  const float ee = CG_FMA(cg_fabsf(l), eb, CG_MUL(cg_fabsf(e), 6.0f * CG_E24));
  o.e = CG_MUL(o.v, CG_ADD(CG_MUL(2.0f, ee), 8.0f * CG_E24));
  return o;
}

/* Poisson inversion in single precision for lam < 10 with a proof that the
 * double inversion at a mean within elam of lam gives the same count:
 * returns the count, or -1 when u lies too close to a cumulative value.
 * dF_j/dlam = -p_j(lam), and p_j <= 1/sqrt(2 pi j) for j >= 1 (Stirling),
 * p_0 <= 1.  The recursion p_j = p_{j-1} (lam r_j), r_j the approximate
 * reciprocal of j (2^-22), has relative error (6j + 2) 2^-24 with expf's two
 * ulp; with the additions, F_j is within (7j + 3) 2^-24 of F_j(lam). */
CG_HD int cg_poisson_inv_checked(float lam, float elam, float u)
{
  /* most cells: u < 1 - lam_d <= exp(-lam_d) = F_0, so the count is 0
   * (lam_d <= lam + elam; 2^-23 covers the two float roundings) */
  if (u < CG_SUB(CG_SUB(1.0f, lam), CG_ADD(elam, 2.0f * CG_E24))) return 0;
  float p = expf(-lam), F = p;
  float Fp = 0.0f;
  int k = 0;
  while (u >= F && k < 64) {
    k++;
    p = CG_MUL(p, CG_MUL(lam, cg_rcp_fast((float)k)));
    Fp = F;
    F = CG_ADD(F, p);
  }
  if (k >= 64) return -1;
  /* margins of the two cumulative values that bracket u */
  const float pk = k == 0 ? 1.0f : CG_MUL(0.4f, cg_rsqrt_fast((float)k));
  const float mk = CG_MUL(1.25f, CG_FMA(elam, pk, (float)(7 * k + 6) * CG_E24));
  if (!(CG_SUB(F, u) > mk)) return -1;
  if (k > 0) {
    const float pj = k == 1 ? 1.0f : CG_MUL(0.4f, cg_rsqrt_fast((float)(k - 1)));
    const float mj = CG_MUL(1.25f, CG_FMA(elam, pj, (float)(7 * k + 3) * CG_E24));
    if (!(CG_SUB(u, Fp) > mj)) return -1;
  }
  return k;
}

/* PTRS (cgx_poisson_ptrs) in single precision for lam - elam >= 10: the
 * same uniforms, and each decision -- the floor that gives the candidate k
 * and the quick acceptance V <= v_r -- taken in float where a bound on its
 * distance to the double value proves it (the uniforms' own comparisons,
 * us >= 0.07, us < 0.013, V > us, are exact: us and V are multiples of
 * 2^-24), then the logarithmic acceptance test with its own bound.  Returns
 * the count, or -1 when a margin fails (the cell then goes to double). */
CG_HD int cg_poisson_ptrs_checked(float lam, float elam, long long cid, uint32_t k0, uint32_t k1)
{
  /* us >= 0.07 and us < 0.013 for multiples of 2^-24: ceil(0.07 2^24) = 1174406,
   * ceil(0.013 2^24) = 218104 */
  const float T07 = 1174406.0f * CG_E24, T013 = 218104.0f * CG_E24;
  const float slam = CG_SQRT(lam);
  const float es = CG_FMA(slam, CG_E24, CG_DIV(elam, CG_MUL(2.0f, CG_SQRT(CG_SUB(lam, elam)))));
  const float b = CG_FMA(2.53f, slam, 0.931f);
  const float eb = CG_FMA(2.53f, es, CG_FMA(2.5e-7f, CG_ADD(slam, 1.0f), CG_MUL(CG_E24, b)));
  const float a = CG_FMA(0.02483f, b, -0.059f);
  const float ea = CG_FMA(0.025f, eb, CG_FMA(1e-8f, CG_ADD(b, 1.0f), CG_MUL(CG_E24, cg_fabsf(a))));
  const float g = CG_SUB(b, 2.0f);
  const float h = CG_DIV(3.6224f, g);
  const float vr = CG_SUB(0.9277f, h);
  const float evr = CG_ADD(CG_DIV(CG_MUL(3.63f, CG_FMA(CG_E24, g, eb)), CG_MUL(g, g)),
                           CG_FMA(2.0f * CG_E24, h, CG_FMA(CG_E24, cg_fabsf(vr), 1e-7f)));
  for (uint32_t it = 0; it < 64u; it++) {
    const cg_u32x4 w = cg_philox4x32_10((uint32_t)cid, (uint32_t)((unsigned long long)cid >> 32), it, 1u, k0, k1);
    const float U = CG_SUB(cg_u01f(w.v[0]), 0.5f); /* exact */
    const float V = cg_u01f(w.v[1]);
    const float us = CG_SUB(0.5f, cg_fabsf(U)); /* exact */
    const float t1 = CG_DIV(CG_MUL(2.0f, a), us);
    const float t2 = CG_ADD(t1, b);
    const float t3 = CG_MUL(t2, U);
    const float x1 = CG_ADD(t3, lam);
    const float X = CG_ADD(x1, 0.43f);
    float eX = CG_MUL(cg_fabsf(U), CG_ADD(CG_ADD(CG_DIV(CG_MUL(2.0f, ea), us), eb),
                                          CG_MUL(CG_E24, CG_ADD(cg_fabsf(t1), cg_fabsf(t2)))));
    eX = CG_ADD(eX, CG_ADD(elam, CG_MUL(CG_E24, CG_ADD(CG_ADD(cg_fabsf(t3), cg_fabsf(x1)), cg_fabsf(X)))));
    eX = CG_FMA(1.5f, eX, 2e-8f); /* and 0.43's representation */
    const float fx = cg_floorf(X);
    const float dX = CG_SUB(X, fx);
    if (!(cg_fminf(dX, CG_SUB(1.0f, dX)) > eX)) return -1;
    const int kd = (int)fx;
    if (us >= T07) {
      if (V < CG_SUB(vr, evr)) return kd;
      if (!(V > CG_ADD(vr, evr))) return -1;
    }
    if (kd < 0 || (us < T013 && V > us)) continue;
    /* the logarithmic test, log(V invalpha / (a / us^2 + b)) <= k log(lam) -
     * lam - log k!, with the logarithms of cg_logf (within 12 2^-24 of the
     * result, 2e-8 absolute) and log k! exact below 10, else Stirling's
     * series to 1/(360 n^3) (truncation below 1e-8 for n >= 11) */
    if (!(V > 0.0f)) return kd; /* log 0: accepted in double too */
    const float lV = cg_logf(V);
    const float ia = CG_ADD(1.1239f, CG_DIV(1.1328f, CG_SUB(b, 3.4f)));
    const float eia = CG_FMA(1.1328f, CG_DIV(eb, CG_MUL(CG_SUB(b, 3.4f), CG_SUB(b, 3.4f))), CG_MUL(4.0f * CG_E24, ia));
    const float us2 = CG_MUL(us, us);
    const float qd = CG_ADD(CG_DIV(a, us2), b);
    const float eqd = CG_ADD(CG_ADD(CG_DIV(ea, us2), eb), CG_MUL(4.0f * CG_E24, CG_ADD(CG_DIV(cg_fabsf(a), us2), qd)));
    const float lia = cg_logf(ia), lq = cg_logf(qd);
    const float lhs = CG_ADD(lV, CG_SUB(lia, lq));
    float el = CG_FMA(12.0f * CG_E24, CG_ADD(CG_ADD(cg_fabsf(lV), cg_fabsf(lia)), cg_fabsf(lq)), 6e-8f);
    el = CG_ADD(el, CG_ADD(CG_DIV(eia, ia), CG_DIV(eqd, qd)));
    el = CG_FMA(2.0f * CG_E24, CG_ADD(cg_fabsf(lhs), CG_ADD(cg_fabsf(lia), cg_fabsf(lq))), el);
    const float ll = cg_logf(lam);
    const float ell = CG_ADD(CG_FMA(12.0f * CG_E24, cg_fabsf(ll), 2e-8f), CG_DIV(elam, lam));
    const float kf = (float)kd;
    float lg, elg;
    if (kd < 10) {
      lg = cg_logfact_small(kd);
      elg = CG_MUL(CG_E24, lg);
    } else {
      const float nn = CG_ADD(kf, 1.0f);
      const float ln = cg_logf(nn);
      const float t = CG_MUL(CG_SUB(nn, 0.5f), ln);
      const float inn = CG_DIV(1.0f, nn);
      const float corr = CG_MUL(inn, CG_SUB(0.0833333358f, CG_MUL(CG_MUL(inn, inn), 0.00277777785f)));
      lg = CG_ADD(CG_ADD(CG_SUB(t, nn), 0.918938533f), corr);
      elg = CG_FMA(CG_SUB(nn, 0.5f), CG_FMA(12.0f * CG_E24, ln, 2e-8f),
                   CG_FMA(2.0f * CG_E24, CG_ADD(CG_ADD(cg_fabsf(t), nn), cg_fabsf(lg)), 6e-8f));
    }
    const float kl = CG_MUL(kf, ll);
    const float rhs = CG_SUB(CG_SUB(kl, lam), lg);
    float er = CG_FMA(kf, ell, CG_ADD(elam, elg));
    er = CG_FMA(2.0f * CG_E24, CG_ADD(CG_ADD(cg_fabsf(kl), cg_fabsf(CG_SUB(kl, lam))), cg_fabsf(rhs)), er);
    const float m = CG_MUL(1.5f, CG_ADD(el, er));
    const float dlr = CG_SUB(lhs, rhs);
    if (dlr < -m) return kd;
    if (!(dlr > m)) return -1;
  }
  return -1;
}

/* ---- RING pixel with a margin ----------------------------------------- */

/* Direction of (x, y, z) in the form the pixel decisions need: cos(theta),
 * the quadrant q and fraction f of tt = phi / (pi/2) = q + f, rho^2 =
 * x^2 + y^2 and 1/r, with error bounds ecth and ef given a relative error
 * ein of the coordinates (0 when the float position is the reference's).
 * f is formed from the octant-reduced atan of min/max, so that it carries
 * absolute, not relative-to-2pi, rounding. */
typedef struct {
  float cth, f, rho2, r2, rinv, ecth, ef;
  int q;
} cg_dir;

CG_HD cg_dir cg_dir_of(float x, float y, float z, float ein)
{
  cg_dir o;
  o.rho2 = CG_FMA(x, x, CG_MUL(y, y));
  const float r2 = CG_FMA(z, z, o.rho2);
  o.r2 = r2;
  o.rinv = cg_rsqrt_fast(r2);
  o.cth = CG_MUL(z, o.rinv);
  const float ax = cg_fabsf(x), ay = cg_fabsf(y);
  const float mx = cg_max_nn(ax, ay), mn = cg_min_nn(ax, ay);
  const float t = CG_MUL(mn, cg_rcp_fast(cg_max_nn(mx, 1e-30f))); /* atan2(0, 0) = 0 */
  const float g = cg_atan01_q(t); /* atan(min/max) / (pi/2) */
  /* tt = phi / (pi/2) in [0, 4) is base + g' or base - g' with
   * g' = atan(ay/ax) / (pi/2) (g, or 1 - g when ay > ax) and, by quadrant,
   * (base, sign) = (0, +) x >= 0 y >= 0, (2, -) x < 0 y >= 0, (2, +) x < 0 y < 0,
   * (4, -) x >= 0 y < 0; q and f = tt - q follow without forming tt, so f
   * keeps absolute rounding */
  const int neg = (x < 0.0f) != (y < 0.0f);
  const int swap = ay > ax;
  int q = ((x < 0.0f) ? 2 : ((y < 0.0f) ? 4 : 0)) - neg;
  float f = (swap != neg) ? CG_SUB(1.0f, g) : g;
  if (f >= 1.0f) { /* g' = 0 on the negative side: tt is the next integer */
    f = 0.0f;
    q = q + 1;
  }
  q &= 3;
  o.q = q;
  o.f = f;
  /* cos(theta): r^2 (2 roundings), rsqrt (2^-22), product (2^-24); the
   * inputs' error ein (relative to r) moves cos(theta) by at most 2 ein */
  o.ecth = CG_FMA(cg_fabsf(o.cth), 8.0f * CG_E24, CG_MUL(2.0f, ein));
  /* f: cg_atan01_q within 8.2e-8 of atan / (pi/2) on [0,1]; the ratio's
   * relative error 2^-22 moves atan by at most that times t/(1+t^2) <= 1/2
   * (6e-8 rad, 3.8e-8 in quarter turns); the rounding of 1 - g (3e-8):
   * 1.5e-7 in all, taken as 2.5e-7.  The inputs' share, which depends on
   * 1/sin(theta), is added by cg_pix_checked. */
  o.ef = 2.5e-7f;
  return o;
}

/* An integer-valued float x with |x| < 2^22 as int: x + 1.5 2^23 holds x in
 * its low mantissa bits (exact), read without a conversion instruction. */
CG_HD int cg_fint(float x) { return (int)(cg_f2u(CG_ADD(x, 12582912.0f)) - 0x4B400000u); }

/* RING pixel of a direction at nside (a power of two), or -1 when a decision
 * lies within its error bound of the boundary.  ein bounds the distance of
 * the float coordinates to the reference's double ones relative to r (0 when
 * they are the same floats); cg_dir_of was given the same ein. */
CG_HD long long cg_pix_checked(const cg_dir *d, int nside, float ein)
{
  const float ns = (float)nside;
  const float ctha = cg_fabsf(d->cth);
  const float c23 = 0.666666686534881592f; /* float(2/3) = 2/3 + 1.99e-8 */
  /* region: ctha <= 2/3 in double; the float constant is 2e-8 above 2/3 */
  const int region_ok = cg_fabsf(CG_SUB(ctha, c23)) > CG_ADD(d->ecth, 4.0e-8f);
  if (ctha < c23) {
    /* phi error from the inputs: sqrt(2) ein / sin(theta) with
     * sin(theta) >= sqrt(5)/3 here, times 2/pi */
    /* temp1 -+ temp2 = ns (q + 0.5 + f -+ 0.75 cth): the integer ns q is
     * split off and ns v is exact (ns a power of two) */
    const float hf = CG_ADD(0.5f, d->f);
    const float A = CG_MUL(ns, CG_FMA(-0.75f, d->cth, hf));
    const float B = CG_MUL(ns, CG_FMA(0.75f, d->cth, hf));
    /* v's bound: 0.75 ecth, f's bound d->ef plus the inputs' share
     * 1.21 ein, and the roundings of 0.5 + f (<= 1.5) and of the fused
     * multiply-add (<= 2.25): 1.8e-7, taken as 2.5e-7 */
    const float ev = CG_FMA(ns, CG_FMA(0.75f, d->ecth, CG_FMA(1.21f, ein, CG_ADD(d->ef, 2.5e-7f))), 1e-9f);
    const float fa = floorf(A), fb = floorf(B);
    const float da = CG_SUB(A, fa), db = CG_SUB(B, fb);
    const float dm = cg_min_nn(cg_min_nn(da, CG_SUB(1.0f, da)), cg_min_nn(db, CG_SUB(1.0f, db)));
    if (!(region_ok && dm > ev)) return -1;
    /* jp = nside q + floor(A), jm = nside q + floor(B): the floors read from
     * the bits of fa + 1.5 2^23 (cg_fint), whose offsets cancel in jp - jm
     * and are removed once from jp + jm (in unsigned arithmetic, which wraps) */
    const unsigned ua = cg_f2u(CG_ADD(fa, 12582912.0f)), ub = cg_f2u(CG_ADD(fb, 12582912.0f));
    const int ir = nside + 1 + (int)(ua - ub);
    const int kshift = 1 - (ir & 1);
    /* ip mod 4 nside: with q in 0..3 and 0 <= A/ns, B/ns < 2.25, jp + jm is
     * in [nside - 1, 2 (3 + 2.25) nside) (each floor loses less than 1), so
     * ip is in [0, 5 nside) and one subtraction is the modulo */
    int ip = (int)((unsigned)(2 * nside * d->q - nside + kshift + 1) + ua + ub - 2u * 0x4B400000u) >> 1;
    const int m = 4 * nside;
    if (ip >= m) ip -= m;
    return (long long)(nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip);
  }
  /* polar caps: tmp = ns sqrt(3 (1 - |cth|)) with 1 - |cth| = sin^2(theta) /
   * (1 + |cth|), free of the cancellation near the poles */
  if (!region_ok || !(d->rho2 > 0.0f)) return -1; /* or on the polar axis */
  const float rho = CG_MUL(d->rho2, cg_rsqrt_fast(d->rho2));
  const float sth = CG_MUL(rho, d->rinv); /* sin(theta), relative error 2^-21 */
  if (!(sth > 1e-20f)) return -1;
  const float s = CG_MUL(sth, CG_MUL(1.7320508075688772f, cg_rsqrt_fast(CG_ADD(1.0f, ctha))));
  const float tmp = CG_MUL(ns, s);
  /* relative error of s: rho (2^-22 + 2^-24), rinv 2^-22, |cth| through
   * 1/sqrt(1+|cth|) by ecth/2, rsqrt 2^-22, three products; the inputs move
   * sin(theta) by at most 2 ein, relatively 2 ein / sin(theta) */
  const float isth = cg_rcp_fast(sth);
  const float es = CG_MUL(tmp, CG_FMA(0.5f, d->ecth, CG_FMA(2.0f * ein, isth, 20.0f * CG_E24)));
  /* phi: the inputs move it by at most sqrt(2) ein / sin(theta) */
  const float ef = CG_FMA(0.91f * ein, isth, d->ef);
  const float tp = d->f;
  const float p1 = CG_MUL(tp, tmp), p2 = CG_MUL(CG_SUB(1.0f, tp), tmp);
  /* p1 = tp tmp: tmp ef + tp es and its rounding; p2 = (1 - tp) tmp: one
   * more rounding in 1 - tp; with p1, p2 <= tmp and tp, 1 - tp <= 1, one
   * bound covers both */
  const float e12 = CG_FMA(tmp, CG_ADD(ef, 3.0f * CG_E24), CG_ADD(es, 2.0f * CG_E24 + 1e-9f));
  const float f1 = floorf(p1), f2 = floorf(p2);
  const float d1 = CG_SUB(p1, f1), d2 = CG_SUB(p2, f2);
  const int jp = cg_fint(f1), jm = cg_fint(f2);
  const int ir = jp + jm + 1;
  const float fir = CG_ADD(CG_ADD(f1, f2), 1.0f); /* ir, exact */
  const float p3 = CG_MUL(d->f, fir);
  const float f3 = floorf(p3), d3 = CG_SUB(p3, f3);
  const float e3 = CG_FMA(fir, ef, CG_FMA(2.0f * CG_E24, p3, 2.0f * CG_E24 + 1e-9f));
  if (!(cg_min_nn(cg_min_nn(d1, CG_SUB(1.0f, d1)), cg_min_nn(d2, CG_SUB(1.0f, d2))) > e12 &&
        cg_min_nn(d3, CG_SUB(1.0f, d3)) > e3))
    return -1;
  int ip = d->q * ir + cg_fint(f3);
  const int m = 4 * ir;
  if (ip >= m) ip -= m;
  if (d->cth > 0.0f) return (long long)(2 * ir * (ir - 1) + ip);
  return (long long)(12 * nside * nside - 2 * ir * (ir + 1) + ip);
}

/* ---- Poisson counts (srcs.c:156-183) ------------------------------------ */

/* Everything a cell's count needs: the float tables with the float corners
 * (each the double corner i*dx - p rounded once), and the double tables. */
typedef struct {
  const float *r, *nz, *bz, *norm; /* norm: CG_NA values, then the two edges */
  const float *xc, *yc, *zc;       /* cell corners per axis */
  float idr, r_last, bz0, cell_vol, rlim;
  int na, bias_model;
  cgx_srcs_tabs x;
} cg_pois_args;

/* lambda of cell (ix, iy, iz) in single precision with a bound *elam on its
 * distance to cgx_lambda: returns 0 when the double lambda is 0, 1 when
 * (*lam, *elam) hold and lambda < 10 (inversion), 3 when they hold and
 * lambda >= 10 (PTRS), 2 when only the double computation can decide. */
CG_HD int cg_lambda_checked(const cg_pois_args *a, int ix, int iy, int iz, float d, float *lam, float *elam)
{
  *lam = 0.0f;
  *elam = 0.0f;
  const float x = a->xc[ix], y = a->yc[iy], z = a->zc[iz];
  const float r2 = CG_FMA(z, z, CG_FMA(y, y, CG_MUL(x, x)));
  const float r = r2 > 0.0f ? CG_MUL(r2, cg_rsqrt_fast(r2)) : 0.0f;
  /* corners rounded once (2^-24 each), r^2 (3 roundings), rsqrt, product */
  const float er = CG_MUL(r, 8.0f * CG_E24);
  if (cg_fabsf(CG_SUB(r, a->rlim)) <= CG_FMA(a->rlim, CG_E24, er)) return 2;
  if (!(r < a->rlim)) return 0;
  cg_ve nd, b, dn;
  if (r > 0.0f) {
    if (!(r < a->r_last) || cg_fabsf(CG_SUB(r, a->r_last)) <= er) return 2;
    const int ir = (int)CG_MUL(r, a->idr);
    const float t = CG_MUL(CG_SUB(r, a->r[ir]), a->idr);
    /* t against the double t: the radius, the float node radius, the
     * subtraction and the product */
    const float dt = CG_FMA(CG_FMA(r, CG_E24, er), a->idr, 4.0f * CG_E24);
    nd = cg_tab_ve(a->nz, a->na, ir, t, dt);
    b = cg_tab_ve(a->bz, a->na, ir, t, dt);
    dn = cg_tab_ve(a->norm, a->na, ir, t, dt);
  } else { /* the observer's cell: the edge values below r = 0 */
    nd.v = 0.0f;
    nd.e = 0.0f;
    b.v = a->bz0;
    b.e = CG_MUL(cg_fabsf(a->bz0), 2.0f * CG_E24);
    dn.v = a->norm[a->na];
    dn.e = CG_MUL(cg_fabsf(dn.v), 2.0f * CG_E24);
  }
  const cg_ve bm = cg_bias_ve(d, b.v, b.e, a->bias_model);
  if (!(nd.v > nd.e)) { /* ndens > 0 (srcs.c:171) not certain */
    if (nd.e == 0.0f) return 0;
    /* the double lambda is 0 (ndens <= 0: no source) or lies in
     * (0, (nd + e_nd) cv (bm + e_bm) (dn + e_dn)]: inversion with lambda 0
     * and that upper end as its bound (six roundings, taken as 2^-20) */
    const float lhi = CG_MUL(CG_MUL(CG_MUL(CG_MUL(CG_ADD(nd.v, nd.e), a->cell_vol), CG_ADD(bm.v, bm.e)),
                                    CG_ADD(dn.v, dn.e)), 1.000001f);
    *elam = lhi;
    return lhi < 10.0f ? 1 : 2;
  }
  const float nc = CG_MUL(nd.v, a->cell_vol);
  const float l = CG_MUL(CG_MUL(nc, bm.v), dn.v);
  const float bmh = CG_ADD(bm.v, bm.e), dnh = CG_ADD(dn.v, dn.e);
  /* |d lambda| <= cv (e_nd bm dn + nd e_bm dn + nd bm e_dn) to first order
   * (the hatted factors keep the second order), plus the cell volume's and
   * the three products' roundings */
  float e = CG_MUL(CG_MUL(nd.e, bmh), dnh);
  e = CG_FMA(CG_MUL(nd.v, bm.e), dnh, e);
  e = CG_FMA(CG_MUL(nd.v, bm.v), dn.e, e);
  e = CG_FMA(CG_MUL(1.01f, a->cell_vol), e, CG_MUL(l, 8.0f * CG_E24));
  *lam = l;
  *elam = e;
  if (!(l > 0.0f)) return e == 0.0f ? 0 : (e < 10.0f ? 1 : 2); /* lambda in [0, e]: inversion with lambda 0 */
  if (!(CG_ADD(l, e) < 10.0f)) return CG_SUB(l, e) >= 10.0f ? 3 : 2; /* PTRS, or too close to the switch */
  return 1;
}

/* The count of one cell given its Poisson word w: single precision when its
 * margins hold, the double restatement otherwise (*fb set to 1). */
CG_HD int cg_count_cell(const cg_pois_args *a, int ix, int iy, int iz, float d, long long cid, uint32_t w,
                        uint32_t k0, uint32_t k1, int *fb)
{
  float lam, elam;
  int st = cg_lambda_checked(a, ix, iy, iz, d, &lam, &elam);
  *fb = 0;
  if (st == 0) return 0;
  if (st == 1) {
    const int n = cg_poisson_inv_checked(lam, elam, cg_u01f(w));
    if (n >= 0) return n;
  } else if (st == 3) {
    const int n = cg_poisson_ptrs_checked(lam, elam, cid, k0, k1);
    if (n >= 0) return n;
  }
  *fb = 1;
  return cgx_poisson(cgx_lambda(&a->x, ix, iy, iz, d), (double)cg_u01f(w), cid, k0, k1);
}

/* ---- source pixels (srcs.c:268-270 and the count map) ---------------------
 * The base pixel is vec2pix_ring of the source's float position, the count
 * map's pixel he_ang2pix of that position's (cos theta, phi) from cart2sph:
 * both the reference's double arithmetic, decided in single precision where
 * the margins allow (*fb counts the double decisions). */
CG_HD void cg_src_pixels(float px, float py, float pz, int nside_base, int nside_count, long long *pix_base,
                         long long *pix_count, int *fb)
{
  const cg_dir dr = cg_dir_of(px, py, pz, 0.0f);
  long long pb = cg_pix_checked(&dr, nside_base, 0.0f);
  if (pb < 0) {
    pb = cgx_vec2pix_ring(nside_base, (double)px, (double)py, (double)pz);
    (*fb)++;
  }
  *pix_base = pb;
  if (nside_count > 0) {
    long long pc = cg_pix_checked(&dr, nside_count, 0.0f);
    if (pc < 0) {
      double r, cth, ph;
      cgx_cart2sph((double)px, (double)py, (double)pz, &r, &cth, &ph);
      pc = cgx_ang2pix(nside_count, cth, ph);
      (*fb)++;
    }
    *pix_count = pc;
  }
}

/* ---- intensity maps (imap.c:135-245) ------------------------------------ */

/* Shells as intervals between their sorted distinct edges b[0..nb-1] (the
 * float r0 and rf of imap_preproc, imap.c:105-133): interval k is
 * [b[k], b[k+1]) (k = -1 below b[0], nb-1 at or above b[nb-1]) and
 * shell_of[k+1] its shell (-1 below the shells, nr beyond).  For contiguous
 * shells (each rf the next r0) this is get_r_index_imap's answer from any
 * start (imap.c:76-103); otherwise it is the walk's answer from shell 0. */
typedef struct {
  const float *b;
  const int *shell_of; /* nb + 1 */
  int nb, nr;
  int contig; /* shell k is interval k (each rf the next r0) */
} cg_shells;

CG_HD int cg_interval(const cg_shells *sh, float r)
{
  int lo = -1, hi = sh->nb - 1; /* last k with b[k] <= r, -1 if none */
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sh->b[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

CG_HD int cgx_interval(const cg_shells *sh, double r)
{
  int lo = -1, hi = sh->nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((double)sh->b[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

/* Interval of r found from interval k0 by walking (a few steps when r is
 * near the edges of k0). */
CG_HD int cg_interval_from(const cg_shells *sh, int k0, float r)
{
  int k = k0 < -1 ? -1 : (k0 >= sh->nb ? sh->nb - 1 : k0);
  for (int it = 0; it < 8; it++) {
    if (k >= 0 && r < sh->b[k]) k--;
    else if (k + 1 < sh->nb && r >= sh->b[k + 1]) k++;
    else return k;
  }
  return cg_interval(sh, r);
}

/* Distance of r to the edges of its interval k. */
CG_HD float cg_interval_margin(const cg_shells *sh, int k, float r)
{
  const float below = k >= 0 ? CG_SUB(r, sh->b[k]) : 3.0e38f;
  const float above = k + 1 < sh->nb ? CG_SUB(sh->b[k + 1], r) : 3.0e38f;
  return cg_min_nn(below, above);
}

/* Everything a species' cells and samples need, in float and in double. */
typedef struct {
  const float *r, *tz, *bz, *norm, *v1, *ih; /* norm: CG_NA values then the two edges */
  const float *xc, *yc, *zc;                 /* corners i*dx - p rounded once */
  const float *xl, *yl, *zl;                 /* the rest: corner - rounded corner */
  float idr, r_last, bz0, v10, v1f, ih0, ihf;
  float rmin, rmax;                          /* r0[0] - 20, rf[nr-1] + 20 (imap.c:151-152) */
  float fvh;                                 /* factor_vel * 0.5 * idx */
  float dx;
  int na, bias_model, nside;
  cg_shells sh;
  const int *nsub;                           /* nsub of shell s + 1, s = -1 .. nr (imap.c:153-174) */
  const float *dxs;                          /* dx / nsub, the same index, rounded once */
  const float *dxsl;                         /* the rest: dx / nsub - dxs */
  const float *att;                          /* cg_att_table: atan in quarter turns */
  /* double */
  const double *r64, *tz64, *bz64, *norm64, *v164, *ih64;
  double idr64, r_last64, dx64, p64[3], idx64, fv64, rmin64, rmax64;
} cg_imap_args;

/* One listed cell.  mode says how its samples find their shell:
 * CG_SH_SINGLE every sample's shifted radius is certainly in shell j + delta;
 * CG_SH_EDGE the shifted radii certainly lie in intervals kl = j + delta and
 * kl + 1, so one comparison with the edge b[kl + 1] decides; CG_SH_WALK the
 * interval is searched per sample. */
#define CG_SH_WALK 0
#define CG_SH_SINGLE 1
#define CG_SH_EDGE 2
typedef struct {
  float temp, drr, edrr;
  int j;     /* shell of the cell's corner radius: its nsub */
  int mode;
  int delta;
} cg_imap_cell;

/* Float lookup with its bound at radius r (0 < r < r_last) whose own bound
 * is er. */
CG_HD cg_ve cg_tab_at(const float *tf, int na, float idr, const float *rt, float r, float er)
{
  const int ir = (int)CG_MUL(r, idr);
  const float t = CG_MUL(CG_SUB(r, rt[ir]), idr);
  const float dt = CG_FMA(CG_FMA(r, CG_E24, er), idr, 4.0f * CG_E24);
  return cg_tab_ve(tf, na, ir, t, dt);
}

/* A cell in single precision (imap.c:184-208): returns 0 when the double
 * arithmetic certainly leaves it out (outside [rmin, rmax] or T(r) <= 0), 1
 * with *o filled when it certainly lists it, 2 when only double can decide.
 * d: the cell's density; v: the potential's centred differences
 * (float - float, as the reference forms them). */
CG_HD int cg_imap_cell_checked(const cg_imap_args *a, int ix, int iy, int iz, float d, const float v[3],
                               cg_imap_cell *o)
{
  const float x0 = a->xc[ix], y0 = a->yc[iy], z0 = a->zc[iz];
  const float r2 = CG_FMA(z0, z0, CG_FMA(y0, y0, CG_MUL(x0, x0)));
  if (!(r2 > 0.0f)) return 0; /* the observer's corner: T = 0 below r = 0 */
  const float rinv = cg_rsqrt_fast(r2);
  const float rc = CG_MUL(r2, rinv);
  const float erc = CG_MUL(rc, 8.0f * CG_E24);
  if (cg_fabsf(CG_SUB(rc, a->rmax)) <= CG_FMA(cg_fabsf(a->rmax), CG_E24, erc)) return 2;
  if (cg_fabsf(CG_SUB(rc, a->rmin)) <= CG_FMA(cg_fabsf(a->rmin), CG_E24, erc)) return 2;
  if (!(rc <= a->rmax && rc >= a->rmin)) return 0;
  if (!(rc < a->r_last) || cg_fabsf(CG_SUB(rc, a->r_last)) <= erc) return 2;
  /* one table position for the five lookups at rc */
  const int ir = (int)CG_MUL(rc, a->idr);
  const float tt = CG_MUL(CG_SUB(rc, a->r[ir]), a->idr);
  const float dt = CG_FMA(CG_FMA(rc, CG_E24, erc), a->idr, 4.0f * CG_E24);
  const cg_ve tm = cg_tab_ve(a->tz, a->na, ir, tt, dt);
  if (!(tm.v > tm.e)) return (tm.v == 0.0f && tm.e == 0.0f) ? 0 : 2;
  /* the shell of the corner radius fixes nsub; near an edge it is decided
   * on the double radius (the listing is certain, only j was open) */
  int k = cg_interval(&a->sh, rc);
  if (!(cg_interval_margin(&a->sh, k, rc) > erc)) {
    const double r64 = cgx_norm3(cgx_coord(ix, a->dx64, a->p64[0]), cgx_coord(iy, a->dx64, a->p64[1]),
                                 cgx_coord(iz, a->dx64, a->p64[2]));
    k = cgx_interval(&a->sh, r64);
  }
  const int j = a->sh.shell_of[k + 1];
  o->j = j;
  /* brightness (imap.c:199, 201) and radial shift (imap.c:196-198) */
  const cg_ve b = cg_tab_ve(a->bz, a->na, ir, tt, dt);
  const cg_ve dn = cg_tab_ve(a->norm, a->na, ir, tt, dt);
  o->temp = CG_MUL(CG_MUL(tm.v, cg_bias_model(d, b.v, a->bias_model)), dn.v);
  const float u0 = CG_MUL(x0, rinv), u1 = CG_MUL(y0, rinv), u2 = CG_MUL(z0, rinv);
  const float t0 = CG_MUL(v[0], u0), t1 = CG_MUL(v[1], u1), t2 = CG_MUL(v[2], u2);
  const float dot = CG_ADD(CG_ADD(t0, t1), t2);
  const cg_ve v1 = cg_tab_ve(a->v1, a->na, ir, tt, dt);
  const cg_ve ih = cg_tab_ve(a->ih, a->na, ir, tt, dt);
  const float g = CG_MUL(CG_MUL(a->fvh, v1.v), ih.v);
  o->drr = CG_MUL(dot, g);
  /* the dot product against the double one (unit vector 2^-22 per
   * component, products and sums), the tables and the constants */
  const float sabs = CG_ADD(CG_ADD(cg_fabsf(t0), cg_fabsf(t1)), cg_fabsf(t2));
  const float erel_t = CG_ADD(CG_DIV(v1.e, cg_fmaxf(cg_fabsf(v1.v), 1e-30f)),
                              CG_DIV(ih.e, cg_fmaxf(cg_fabsf(ih.v), 1e-30f)));
  o->edrr = CG_MUL(2.0f, CG_FMA(CG_MUL(cg_fabsf(g), sabs), 12.0f * CG_E24,
                                CG_MUL(cg_fabsf(o->drr), CG_ADD(erel_t, 8.0f * CG_E24))));
  /* every sample in one shell?  Sample centres span [c + dxs/2, c + dx -
   * dxs/2] per axis: the nearest and farthest points of that box */
  const float hs = CG_MUL(0.5f, a->dxs[j + 1]);
  const float lo[3] = {CG_ADD(x0, hs), CG_ADD(y0, hs), CG_ADD(z0, hs)};
  const float hi[3] = {CG_SUB(CG_ADD(x0, a->dx), hs), CG_SUB(CG_ADD(y0, a->dx), hs), CG_SUB(CG_ADD(z0, a->dx), hs)};
  float n2 = 0.0f, f2 = 0.0f;
  for (int q = 0; q < 3; q++) {
    const float nq = lo[q] > 0.0f ? lo[q] : (hi[q] < 0.0f ? hi[q] : 0.0f);
    const float fq = cg_fmaxf(cg_fabsf(lo[q]), cg_fabsf(hi[q]));
    n2 = CG_FMA(nq, nq, n2);
    f2 = CG_FMA(fq, fq, f2);
  }
  const float rlo = n2 > 0.0f ? CG_MUL(n2, cg_rsqrt_fast(n2)) : 0.0f;
  const float rhi = CG_MUL(f2, cg_rsqrt_fast(f2));
  /* the samples' radii against the double ones: positions within
   * 2^-24 (|x| + 2 dx) per axis, the radius arithmetic 8 2^-24 */
  const float er = CG_FMA(rhi, 16.0f * CG_E24, CG_MUL(a->dx, 8.0f * CG_E24));
  const float e = CG_ADD(CG_ADD(er, o->edrr), CG_MUL(1e-6f, a->dx));
  const float slo = CG_SUB(CG_ADD(rlo, o->drr), e), shi = CG_ADD(CG_ADD(rhi, o->drr), e);
  const int kl = a->sh.contig ? cg_interval_from(&a->sh, k, slo) : cg_interval(&a->sh, slo);
  const int kh = a->sh.contig ? cg_interval_from(&a->sh, k, shi) : cg_interval(&a->sh, shi);
  o->mode = CG_SH_WALK;
  o->delta = 0;
  if (kl == kh) {
    const int sh = a->sh.shell_of[kl + 1];
    if (sh - j >= -1 && sh - j <= 1) {
      o->mode = CG_SH_SINGLE;
      o->delta = sh - j;
    }
  } else if (kh == kl + 1 && kl - j >= -1 && kl - j <= 1) {
    o->mode = CG_SH_EDGE;
    o->delta = kl - j;
  }
  return 1;
}

/* The cell in double (imap.c:184-208): 0 when not painted, 1 with the shell
 * of its corner radius (*j) and the radial shift (*drr). */
CG_HD int cgx_imap_cell(const cg_imap_args *a, int ix, int iy, int iz, const float v[3], int *j, double *drr)
{
  const double x0 = cgx_coord(ix, a->dx64, a->p64[0]), y0 = cgx_coord(iy, a->dx64, a->p64[1]);
  const double z0 = cgx_coord(iz, a->dx64, a->p64[2]);
  const double r0 = cgx_norm3(x0, y0, z0);
  const double tmean = cgx_bg(a->tz64, a->r64, a->idr64, a->r_last64, 0, 0, r0);
  if (!(r0 <= a->rmax64 && r0 >= a->rmin64)) return 0;
  if (!(tmean > 0)) return 0;
  *j = a->sh.shell_of[cgx_interval(&a->sh, r0) + 1];
  const double u0 = X_DIV(x0, r0), u1 = X_DIV(y0, r0), u2 = X_DIV(z0, r0);
  const double dot = X_ADD(X_ADD(X_MUL((double)v[0], u0), X_MUL((double)v[1], u1)), X_MUL((double)v[2], u2));
  const double rvel = X_MUL(a->fv64, X_MUL(X_MUL(0.5, a->idx64), dot));
  const double v1 = cgx_bg(a->v164, a->r64, a->idr64, a->r_last64, a->v164[0], a->v164[CG_NA - 1], r0);
  const double ih = cgx_bg(a->ih64, a->r64, a->idr64, a->r_last64, a->ih64[0], a->ih64[CG_NA - 1], r0);
  *drr = X_MUL(X_MUL(rvel, v1), ih);
  return 1;
}

/* Coordinate of sub-cell centre s of cell i along one axis: the corner as
 * a double-float pair (c, l) plus (s + 1/2) dxs, within 2^-24 (|x| + 2 dx) of
 * the double centre (imap.c:212-218). */
CG_HD float cg_imap_coord(const float *c, const float *l, int i, int s, float dxs)
{
  return CG_ADD(c[i], CG_FMA(CG_ADD((float)s, 0.5f), dxs, l[i]));
}

/* The shell of a sample at float radius r (relative position error ein) of
 * cell c: 1 with *s when the double arithmetic certainly agrees, 0 when
 * only double can decide. */
CG_HD int cg_imap_shell_checked(const cg_imap_args *a, const cg_imap_cell *c, float r, float ein, int *s)
{
  if (c->mode == CG_SH_SINGLE) {
    *s = c->j + c->delta;
    return 1;
  }
  const float rs = CG_ADD(r, c->drr);
  const float e = CG_ADD(CG_FMA(r, CG_ADD(8.0f * CG_E24, ein), c->edrr), CG_MUL(2.0f * CG_E24, cg_fabsf(rs)));
  if (c->mode == CG_SH_EDGE) {
    const int kl = c->j + c->delta;
    const float B = a->sh.b[kl + 1];
    if (!(cg_fabsf(CG_SUB(rs, B)) > e)) return 0;
    *s = a->sh.shell_of[(rs >= B ? kl + 1 : kl) + 1];
    return 1;
  }
  const int k = a->sh.contig ? cg_interval_from(&a->sh, c->j, rs) : cg_interval(&a->sh, rs);
  if (!(cg_interval_margin(&a->sh, k, rs) > e)) return 0;
  *s = a->sh.shell_of[k + 1];
  return 1;
}

/* Shell and RING pixel of the sample at float position (x, y, z) of cell c
 * (imap.c:210-231): 1 with *s (maybe -1 or nr: not painted) and *pix when the
 * double arithmetic certainly agrees, 0 when only double can decide. */
CG_HD int cg_imap_decide(const cg_imap_args *a, const cg_imap_cell *c, float x, float y, float z, int *s,
                         long long *pix)
{
  cg_dir dr = cg_dir_of(x, y, z, 0.0f);
  /* coordinates within 2^-24 (|x| + 2 dx) of the double ones: relative to
   * r, 1.8 2^-24 (1 + 2 dx / r) */
  const float ein = CG_FMA(CG_MUL(3.6f * CG_E24, a->dx), dr.rinv, 1.8f * CG_E24);
  if (!cg_imap_shell_checked(a, c, CG_MUL(dr.r2, dr.rinv), ein, s)) return 0;
  if (*s < 0 || *s >= a->sh.nr) return 1;
  dr.ecth = CG_FMA(2.0f, ein, dr.ecth);
  const long long p = cg_pix_checked(&dr, a->nside, ein);
  if (p < 0) return 0;
  *pix = p;
  return 1;
}

/* A sample in single precision: sub-cell (sx, sy, sz) of the listed cell c
 * at (ix, iy, iz). */
CG_HD int cg_imap_sample_checked(const cg_imap_args *a, int ix, int iy, int iz, const cg_imap_cell *c, int ns,
                                 int sx, int sy, int sz, int *s, long long *pix)
{
  const float dxs = a->dxs[c->j + 1];
  (void)ns;
  const float x = cg_imap_coord(a->xc, a->xl, ix, sx, dxs);
  const float y = cg_imap_coord(a->yc, a->yl, iy, sy, dxs);
  const float z = cg_imap_coord(a->zc, a->zl, iz, sz, dxs);
  return cg_imap_decide(a, c, x, y, z, s, pix);
}

/* The sample in double (imap.c:210-231). */
CG_HD void cgx_imap_sample(const cg_imap_args *a, int ix, int iy, int iz, int ns, double drr, int sx, int sy, int sz,
                           int *s, long long *pix)
{
  const double dxs = X_DIV(a->dx64, (double)ns);
  const double x = X_ADD(cgx_coord(ix, a->dx64, a->p64[0]), X_MUL(X_ADD((double)sx, 0.5), dxs));
  const double y = X_ADD(cgx_coord(iy, a->dx64, a->p64[1]), X_MUL(X_ADD((double)sy, 0.5), dxs));
  const double z = X_ADD(cgx_coord(iz, a->dx64, a->p64[2]), X_MUL(X_ADD((double)sz, 0.5), dxs));
  double r, cth, phi;
  cgx_cart2sph(x, y, z, &r, &cth, &phi);
  *s = a->sh.shell_of[cgx_interval(&a->sh, X_ADD(r, drr)) + 1];
  if (*s >= 0 && *s < a->sh.nr) *pix = cgx_ang2pix(a->nside, cth, phi);
}

/* ---- The float-float tier ---------------------------------------------- */

/* Samples whose single-precision margins fail are decided again in
 * float-float arithmetic (cg_ff.h, about 48 bits) before any double
 * arithmetic: the same decision structure as cg_pix_checked with bounds of a
 * few hundred u^2 instead of a few u, so that all but ~1e-9 of them are
 * settled on the FP32 pipes.  The bounds below are sums of the double-word
 * operations' relative error bounds (cg_ff.h) along each expression, plus
 * the reference's own double roundings (2^-53 = u^2 / 32 per operation), each
 * term rounded up; the margins take them 1.25 times. */

#define CG_ATT_N 256 /* atan table nodes t = i / CG_ATT_N, i = 0 .. CG_ATT_N */

/* atan(i / CG_ATT_N) in quarter turns (times 2/pi) as float pairs, t[2 i] +
 * t[2 i + 1] within 0.6 u^2 of the value (libm's double atan, one ulp);
 * host code. */
#if defined(__CUDACC__)
static inline __host__ void cg_att_table(float *t)
#else
static inline void cg_att_table(float *t)
#endif
{
  for (int i = 0; i <= CG_ATT_N; i++) {
    const double v = atan((double)i / CG_ATT_N) * 0.63661977236758134308;
    t[2 * i] = (float)v;
    t[2 * i + 1] = (float)(v - (double)t[2 * i]);
  }
}

/* phi / (pi/2) of (x, y) as the quadrant q and f = tt - q in [0, 1), with the
 * octant reduction of cg_dir_of: |f - f_exact| <= 17 u^2 (atan of the
 * nearest table node plus atan((t - t_i) / (1 + t t_i)) by its series to
 * the fifth power, whose truncation is below 1e-20 for |t - t_i| <= 1/512). */
CG_HD void cg_ff_quarter(cg_ff x, cg_ff y, const float *att, int *q, cg_ff *f)
{
  const cg_ff ax = cg_ff_abs(x), ay = cg_ff_abs(y);
  const int swap = cg_ff_cmp(ay, ax) > 0;
  const cg_ff mx = swap ? ay : ax, mn = swap ? ax : ay;
  cg_ff g = cg_ff_make(0.0f, 0.0f);
  if (mx.h > 0.0f) {
    const cg_ff t = cg_ff_div(mn, mx);
    int i = (int)CG_ADD(CG_MUL(t.h, (float)CG_ATT_N), 0.5f);
    i = i < 0 ? 0 : (i > CG_ATT_N ? CG_ATT_N : i);
    const float ti = CG_MUL((float)i, 1.0f / CG_ATT_N); /* exact */
    const cg_ff num = cg_ff_add(t, cg_ff_make(-ti, 0.0f));
    const cg_ff den = cg_ff_add(cg_ff_make(1.0f, 0.0f), cg_ff_mulf(t, ti));
    const cg_ff d = cg_ff_div(num, den);
    const float d2 = CG_MUL(d.h, d.h);
    const float corr = CG_MUL(CG_MUL(d.h, d2), CG_FMA(d2, 0.2f, -0.333333343f)); /* -d^3/3 + d^5/5 */
    const cg_ff at = cg_ff_add(d, cg_ff_make(corr, 0.0f));
    g = cg_ff_add(cg_ff_make(att[2 * i], att[2 * i + 1]), cg_ff_mul(at, cg_ff_make(0.636619746685028076f, 2.56825530e-08f)));
  }
  const int xneg = x.h < 0.0f, yneg = y.h < 0.0f;
  const int neg = xneg != yneg;
  int qq = (xneg ? 2 : (yneg ? 4 : 0)) - neg;
  cg_ff ff = (swap != neg) ? cg_ff_add(cg_ff_make(1.0f, 0.0f), cg_ff_neg(g)) : g;
  if (cg_ff_cmp(ff, cg_ff_make(1.0f, 0.0f)) >= 0) { /* g' = 0 on the negative side */
    ff = cg_ff_add(ff, cg_ff_make(-1.0f, 0.0f));
    qq++;
  }
  *q = qq & 3;
  *f = ff;
}

CG_HD cg_ff cg_ff_scale(cg_ff x, float p2) { return cg_ff_make(CG_MUL(x.h, p2), CG_MUL(x.l, p2)); } /* p2 a power of 2 */

/* RING pixel at nside (a power of two) of the float-float position
 * (X, Y, Z), which lies within eP (Euclidean) of the reference's double
 * position, or -1 when a decision lies within its bound of the boundary:
 * cg_pix_checked's decisions with float-float values. */
CG_HD long long cg_pix_ff(cg_ff X, cg_ff Y, cg_ff Z, float eP, int nside, const float *att)
{
  const float U = CG_U2;
  const cg_ff rho2 = cg_ff_add(cg_ff_mul(X, X), cg_ff_mul(Y, Y));
  const cg_ff r2 = cg_ff_add(rho2, cg_ff_mul(Z, Z));
  if (!(r2.h > 0.0f)) return -1;
  const cg_ff R = cg_ff_sqrt(r2);
  const cg_ff cth = cg_ff_div(Z, R);
  /* the position's error relative to r moves cos(theta) by at most ein and
   * phi by at most ein / sin(theta) */
  const float ein = CG_MUL(1.01f, CG_DIV(eP, R.h));
  const float sth = CG_DIV(CG_SQRT(rho2.h), R.h);
  /* cos(theta): rho^2 9u^2, r^2 13, R 10.5, quotient 16 + 10.5; the
   * reference's cart2sph 0.125 */
  const float ecth = CG_FMA(1.01f, ein, 28.0f * U);
  int q;
  cg_ff f;
  cg_ff_quarter(X, Y, att, &q, &f);
  /* f: 17u^2, the reference's atan2, shift and product 0.52 */
  const float ef = CG_ADD(18.0f * U, CG_DIV(CG_MUL(0.65f, ein), sth));
  const float ns = (float)nside;
  const cg_ff ctha = cg_ff_abs(cth);
  const cg_ff c23 = cg_ff_make(0.666666686534881592f, -1.98682155e-08f); /* the double 2/3 within u^2 */
  const cg_ff dreg = cg_ff_sub(ctha, c23);
  const int region_ok = cg_fabsf(dreg.h) > CG_FMA(1.25f, ecth, 3.0f * U);
  if (dreg.h < 0.0f) {
    /* 0.5 + f (6u^2), 0.75 cth (1), the sums (9), the reference's temp1 and
     * temp2 (0.34) */
    const cg_ff hf = cg_ff_add(cg_ff_make(0.5f, 0.0f), f);
    const cg_ff c75 = cg_ff_mulf(cth, 0.75f);
    const cg_ff A = cg_ff_scale(cg_ff_sub(hf, c75), ns), B = cg_ff_scale(cg_ff_add(hf, c75), ns);
    const float ev = CG_MUL(1.25f, CG_MUL(ns, CG_ADD(CG_FMA(0.75f, ecth, ef), 17.0f * U)));
    float fa, fb;
    const float da = cg_ff_floor_dist(A, &fa), db = cg_ff_floor_dist(B, &fb);
    if (!(region_ok && da > ev && db > ev)) return -1;
    const int jp = nside * q + cg_fint(fa), jm = nside * q + cg_fint(fb);
    const int ir = nside + 1 + jp - jm;
    const int kshift = 1 - (ir & 1);
    int ip = (jp + jm - nside + kshift + 1) >> 1;
    const int m = 4 * nside;
    if (ip >= m) ip -= m;
    return (long long)(nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip);
  }
  if (!region_ok || !(sth > 1e-20f)) return -1;
  /* 1 - |cth| = rho^2 / (R (R + |Z|)): 56u^2 relative; the reference's
   * 1 - |cth| is within 0.125 u^2 of the exact value; the position moves it
   * by at most sin(theta) ein */
  const cg_ff u1 = cg_ff_div(rho2, cg_ff_mul(R, cg_ff_add(R, cg_ff_abs(Z))));
  if (!(u1.h > 0.0f)) return -1;
  const float eu1 = CG_FMA(60.0f * U, u1.h, CG_FMA(1.01f, CG_MUL(sth, ein), 0.125f * U));
  const cg_ff tmp = cg_ff_scale(cg_ff_sqrt(cg_ff_mulf(u1, 3.0f)), ns);
  /* 3 (1 - |cth|) and its root: 6u^2, the reference's 0.06, and half the
   * relative error of 1 - |cth| */
  const float etmp = CG_MUL(tmp.h, CG_ADD(7.0f * U, CG_DIV(eu1, CG_MUL(2.0f, u1.h))));
  const cg_ff omf = cg_ff_add(cg_ff_make(1.0f, 0.0f), cg_ff_neg(f));
  const cg_ff p1 = cg_ff_mul(f, tmp), p2 = cg_ff_mul(omf, tmp);
  const float e1 = CG_MUL(1.25f, CG_FMA(tmp.h, ef, CG_FMA(f.h, etmp, CG_MUL(6.0f * U, p1.h))));
  const float e2 = CG_MUL(1.25f, CG_FMA(tmp.h, CG_ADD(ef, 4.0f * U), CG_FMA(omf.h, etmp, CG_MUL(6.0f * U, p2.h))));
  float f1, f2;
  const float d1 = cg_ff_floor_dist(p1, &f1), d2 = cg_ff_floor_dist(p2, &f2);
  if (!(d1 > e1 && d2 > e2)) return -1;
  const int jp = cg_fint(f1), jm = cg_fint(f2);
  const int ir = jp + jm + 1;
  /* f ir (2u^2) and the reference's tt ir (0.125 u^2 ir) */
  const cg_ff p3 = cg_ff_mulf(f, (float)ir);
  const float e3 = CG_MUL(1.25f, CG_FMA((float)ir, CG_ADD(ef, 0.2f * U), CG_MUL(3.0f * U, p3.h)));
  float f3;
  const float d3 = cg_ff_floor_dist(p3, &f3);
  if (!(d3 > e3)) return -1;
  int ip = q * ir + cg_fint(f3);
  const int m = 4 * ir;
  if (ip >= m) ip -= m;
  if (cth.h > 0.0f) return (long long)(2 * ir * (ir - 1) + ip);
  return (long long)(12 * nside * nside - 2 * ir * (ir + 1) + ip);
}

/* A sample of cell c whose single-precision decision was left open, again:
 * the shell as cg_imap_decide takes it, then the RING pixel in float-float
 * from the double-float corner and sub-cell step.  1 with *s (maybe -1 or
 * nr: not painted) and *pix when the double arithmetic certainly agrees, 0
 * when only double can decide. */
CG_HD int cg_imap_decide_ff(const cg_imap_args *a, const cg_imap_cell *c, int ix, int iy, int iz, int sx, int sy,
                            int sz, int *s, long long *pix)
{
  const int k = c->j + 1;
  const float dxs = a->dxs[k];
  const float x = cg_imap_coord(a->xc, a->xl, ix, sx, dxs);
  const float y = cg_imap_coord(a->yc, a->yl, iy, sy, dxs);
  const float z = cg_imap_coord(a->zc, a->zl, iz, sz, dxs);
  const float r2 = CG_FMA(z, z, CG_FMA(x, x, CG_MUL(y, y)));
  const float rinv = cg_rsqrt_fast(r2);
  const float ein = CG_MUL(1.8f * CG_E24, CG_FMA(2.0f * a->dx, rinv, 1.0f));
  if (!cg_imap_shell_checked(a, c, CG_MUL(r2, rinv), ein, s)) return 0;
  if (*s < 0 || *s >= a->sh.nr) return 1;
  /* corner pairs within u^2 of the double corners, the step within u^2 of
   * dx / nsub; times (s + 1/2) 2u^2, the sum 4u^2 of the result, the
   * reference's two roundings: per axis u^2 (5.1 |x| + 5.1 dx), taken
   * Euclidean as 6 u^2 (r + 2 dx) and doubled */
  const cg_ff dd = cg_ff_make(dxs, a->dxsl[k]);
  const cg_ff X = cg_ff_add(cg_ff_make(a->xc[ix], a->xl[ix]), cg_ff_mulf(dd, CG_ADD((float)sx, 0.5f)));
  const cg_ff Y = cg_ff_add(cg_ff_make(a->yc[iy], a->yl[iy]), cg_ff_mulf(dd, CG_ADD((float)sy, 0.5f)));
  const cg_ff Z = cg_ff_add(cg_ff_make(a->zc[iz], a->zl[iz]), cg_ff_mulf(dd, CG_ADD((float)sz, 0.5f)));
  const float eP = CG_MUL(12.0f * CG_U2, CG_FMA(r2, rinv, 2.0f * a->dx));
  const long long p = cg_pix_ff(X, Y, Z, eP, a->nside, a->att);
  if (p < 0) return 0;
  *pix = p;
  return 1;
}

/* Host set-up of a species' shells (imap_preproc, imap.c:105-133, and the
 * sub-sampling factors, imap.c:153-174): the float edges sorted by r0
 * (stable), the distinct edge values b (nb of them), the shell of each
 * interval, nsub and dx/nsub of shells -1 .. nr.  Arrays: r0f, rff, nr
 * floats; b, 2 nr floats; shell_of, 2 nr + 1 ints; nsub and dxs, nr + 2.
 * Returns nb. */
static inline int cg_imap_shells(const double *r0d, const double *rfd, int nr, double dx, long long npix,
                                 float *r0f, float *rff, float *b, int *shell_of, int *nsub, float *dxs)
{
  for (int i = 0; i < nr; i++) {
    r0f[i] = (float)r0d[i];
    rff[i] = (float)rfd[i];
  }
  for (int i = 1; i < nr; i++) /* stable insertion sort by r0 */
    for (int k = i; k > 0 && r0f[k] < r0f[k - 1]; k--) {
      float t = r0f[k];
      r0f[k] = r0f[k - 1];
      r0f[k - 1] = t;
      t = rff[k];
      rff[k] = rff[k - 1];
      rff[k - 1] = t;
    }
  int nb = 0;
  for (int i = 0; i < nr; i++) {
    b[nb++] = r0f[i];
    b[nb++] = rff[i];
  }
  for (int i = 1; i < nb; i++)
    for (int k = i; k > 0 && b[k] < b[k - 1]; k--) {
      const float t = b[k];
      b[k] = b[k - 1];
      b[k - 1] = t;
    }
  int m = 0;
  for (int i = 0; i < nb; i++)
    if (m == 0 || b[i] != b[m - 1]) b[m++] = b[i];
  nb = m;

  /* the walk from shell 0 at each interval's lower edge */
  float rfm[4096];
  for (int i = 0; i < nr && i < 4096; i++) rfm[i] = i == 0 ? rff[0] : (rff[i] > rfm[i - 1] ? rff[i] : rfm[i - 1]);
  for (int k = -1; k < nb; k++) {
    const float r = k < 0 ? b[0] - 1.0f : b[k];
    shell_of[k + 1] = cg_shell_index0(r0f, rfm, nr, r);
  }
  const double ps = sqrt(4 * 3.14159265358979323846 / (double)npix);
  for (int i = -1; i <= nr; i++) {
    const int q = i < 0 ? 0 : (i >= nr ? nr - 1 : i);
    const double a0 = r0f[q], a1 = rff[q];
    const double vol = (a1 * a1 * a1 - a0 * a0 * a0) * ps * ps / 3;
    const double sc0 = fmin(pow(vol, 0.333333), fmin(a0 * ps, a1 - a0));
    nsub[i + 1] = (int)(dx / sc0 + 0.5) + 1;
    dxs[i + 1] = (float)(dx / nsub[i + 1]);
  }
  return nb;
}

/* Whether the sorted shells are contiguous (each rf the next r0): then
 * interval k is shell k. */
static inline int cg_imap_contig(const float *r0f, const float *rff, int nr, int nb)
{
  if (nb != nr + 1) return 0;
  for (int i = 0; i + 1 < nr; i++)
    if (rff[i] != r0f[i + 1]) return 0;
  return 1;
}

#endif /* CG_EXACT_H */
