/*
 * cg_ff.h -- float-float ("double-word") arithmetic, shared by the sm_103a
 * kernels and host C code, for the decisions that single precision leaves
 * open.
 *
 * A value is the unevaluated sum h + l of two floats, |l| <= ulp(h) / 2,
 * about 48 significant bits carried on the FP32 pipes.  The building blocks
 * are the error-free transforms TwoSum (Knuth, The Art of Computer
 * Programming vol. 2, 4.2.2), Fast2Sum (Dekker 1971) and TwoProd by a fused
 * multiply-add, and the double-word algorithms of Joldes, Muller and
 * Popescu, "Tight and rigorous error bounds for basic building blocks of
 * double-word arithmetic" (ACM TOMS 44(2), 2017): AccurateDWPlusDW,
 * DWTimesFP3, DWTimesDW3 and DWDivDW2; the square root is the double-word
 * root of Lefevre, Louvet, Muller, Picot and Rideau ("Accurate calculation of
 * Euclidean norms using double-word arithmetic", ACM TOMS 49(1), 2023).  With
 * u = 2^-24 their relative errors are below 3u^2 (sum), 2u^2 (times a
 * float), 5u^2 (product), 15u^2 + 56u^3 (quotient) and 25/8 u^2 (root), in
 * the absence of underflow and overflow; the callers' bounds use 4, 2, 5, 16
 * and 4 u^2.  Every operation is spelled out through the CG_* macros, so
 * host and device give the same bits.
 */
#ifndef CG_FF_H
#define CG_FF_H

#include "cg_math.h"

typedef struct {
  float h, l;
} cg_ff;

#define CG_U2 3.5527136788005009e-15f /* u^2 = 2^-48 */

CG_HD cg_ff cg_ff_make(float h, float l)
{
  cg_ff r;
  r.h = h;
  r.l = l;
  return r;
}

/* Fast2Sum: s + t = a + b exactly when |a| >= |b| (or a = 0). */
CG_HD cg_ff cg_fast2sum(float a, float b)
{
  const float s = CG_ADD(a, b);
  const float z = CG_SUB(s, a);
  return cg_ff_make(s, CG_SUB(b, z));
}

/* TwoSum: s + t = a + b exactly, any order. */
CG_HD cg_ff cg_2sum(float a, float b)
{
  const float s = CG_ADD(a, b);
  const float ap = CG_SUB(s, b);
  const float bp = CG_SUB(s, ap);
  const float da = CG_SUB(a, ap);
  const float db = CG_SUB(b, bp);
  return cg_ff_make(s, CG_ADD(da, db));
}

/* TwoProd: p + e = a b exactly. */
CG_HD cg_ff cg_2prod(float a, float b)
{
  const float p = CG_MUL(a, b);
  return cg_ff_make(p, CG_FMA(a, b, -p));
}

/* AccurateDWPlusDW. */
CG_HD cg_ff cg_ff_add(cg_ff x, cg_ff y)
{
  const cg_ff s = cg_2sum(x.h, y.h);
  const cg_ff t = cg_2sum(x.l, y.l);
  const cg_ff v = cg_fast2sum(s.h, CG_ADD(s.l, t.h));
  return cg_fast2sum(v.h, CG_ADD(t.l, v.l));
}

CG_HD cg_ff cg_ff_neg(cg_ff x) { return cg_ff_make(-x.h, -x.l); }
CG_HD cg_ff cg_ff_sub(cg_ff x, cg_ff y) { return cg_ff_add(x, cg_ff_neg(y)); }
CG_HD cg_ff cg_ff_abs(cg_ff x) { return x.h < 0.0f ? cg_ff_neg(x) : x; }

/* DWTimesFP3: x times the float y. */
CG_HD cg_ff cg_ff_mulf(cg_ff x, float y)
{
  const cg_ff c = cg_2prod(x.h, y);
  return cg_fast2sum(c.h, CG_FMA(x.l, y, c.l));
}

/* DWTimesDW3. */
CG_HD cg_ff cg_ff_mul(cg_ff x, cg_ff y)
{
  const cg_ff c = cg_2prod(x.h, y.h);
  const float t0 = CG_MUL(x.l, y.l);
  const float t1 = CG_FMA(x.h, y.l, t0);
  const float c2 = CG_FMA(x.l, y.h, t1);
  return cg_fast2sum(c.h, CG_ADD(c.l, c2));
}

/* DWDivDW2 (y nonzero). */
CG_HD cg_ff cg_ff_div(cg_ff x, cg_ff y)
{
  const float th = CG_DIV(x.h, y.h);
  const cg_ff r = cg_ff_mulf(y, th);
  const float ph = CG_SUB(x.h, r.h);
  const float dl = CG_SUB(x.l, r.l);
  const float tl = CG_DIV(CG_ADD(ph, dl), y.h);
  return cg_fast2sum(th, tl);
}

/* Double-word square root (x > 0). */
CG_HD cg_ff cg_ff_sqrt(cg_ff x)
{
  const float sh = CG_SQRT(x.h);
  const cg_ff p = cg_2prod(sh, sh);
  const float d = CG_ADD(CG_SUB(CG_SUB(x.h, p.h), p.l), x.l);
  return cg_fast2sum(sh, CG_DIV(d, CG_MUL(2.0f, sh)));
}

/* Sign of x - y: -1, 0 or 1 (a normalised pair is zero only when h is). */
CG_HD int cg_ff_cmp(cg_ff x, cg_ff y)
{
  const cg_ff d = cg_ff_sub(x, y);
  return d.h > 0.0f ? 1 : (d.h < 0.0f ? -1 : 0);
}

/* floor of x as a float pair, and the distance of x to the nearest integer
 * (for |x| < 2^22). */
CG_HD float cg_ff_floor_dist(cg_ff x, float *fl)
{
  float f = floorf(x.h);
  cg_ff d = cg_ff_add(x, cg_ff_make(-f, 0.0f)); /* x - floor(x.h), in (-1, 1) */
  if (d.h < 0.0f || (d.h == 0.0f && d.l < 0.0f)) {
    f = CG_SUB(f, 1.0f);
    d = cg_ff_add(d, cg_ff_make(1.0f, 0.0f));
  }
  *fl = f;
  const cg_ff u = cg_ff_add(cg_ff_make(1.0f, 0.0f), cg_ff_neg(d)); /* 1 - frac, without cancellation */
  const float fr = CG_ADD(d.h, d.l), up = CG_ADD(u.h, u.l);
  return fr < up ? fr : up;
}

#endif
