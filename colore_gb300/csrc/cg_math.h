/*
 * cg_math.h -- deterministic single-precision arithmetic shared by the
 * sm_103a kernels and by host C code.
 *
 * Every function here compiles to the same sequence of IEEE-754 operations
 * on the GPU (nvcc) and on the host (gcc with -ffp-contract=off): additions,
 * multiplications, divisions and square roots are spelled out through the
 * CG_* macros, which map to the non-contractible __f*_rn intrinsics on the
 * device, and fused multiply-adds are always explicit (fmaf / __fmaf_rn,
 * both correctly rounded).  With identical inputs the results are therefore
 * bit-identical on both sides, which is what makes Poisson counts and
 * HEALPix pixel indices reproducible between the GPU and a CPU run.
 *
 * The elementary functions (exp, log, log1p, atan2, acos) are written from
 * their textbook definitions: Cody-Waite range reduction plus the Taylor
 * series of e^r for exp; the atanh series log(1+f) = 2 atanh(f/(2+f)) for
 * log; a minimax polynomial for atan(t)/t on [0, 1] (the coefficients were
 * fitted for this file by Remez exchange) after the octant reduction of
 * atan2.  Accuracy is within 2 ulp of the correctly rounded result over the
 * ranges used.
 *
 * The counter-based generator is Philox4x32-10 (Salmon, Moraes, Dror and
 * Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11).
 */
#ifndef CG_MATH_H
#define CG_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define CG_HD __host__ __device__ __forceinline__
/* rarely taken paths: one out-of-line copy instead of one per call site */
#define CG_HD_COLD static __host__ __device__ __noinline__
#else
#define CG_HD static inline
#define CG_HD_COLD static
#include <math.h>
#include <string.h>
#endif

#if defined(__CUDA_ARCH__)
#define CG_ADD(a, b) __fadd_rn((a), (b))
#define CG_SUB(a, b) __fsub_rn((a), (b))
#define CG_MUL(a, b) __fmul_rn((a), (b))
#define CG_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define CG_DIV(a, b) __fdiv_rn((a), (b))
#define CG_SQRT(a) __fsqrt_rn((a))
#define CG_DADD(a, b) __dadd_rn((a), (b))
#define CG_DMUL(a, b) __dmul_rn((a), (b))
#else
#define CG_ADD(a, b) ((float)(a) + (float)(b))
#define CG_SUB(a, b) ((float)(a) - (float)(b))
#define CG_MUL(a, b) ((float)(a) * (float)(b))
#define CG_FMA(a, b, c) fmaf((a), (b), (c))
#define CG_DIV(a, b) ((float)(a) / (float)(b))
#define CG_SQRT(a) sqrtf((a))
#define CG_DADD(a, b) ((double)(a) + (double)(b))
#define CG_DMUL(a, b) ((double)(a) * (double)(b))
#endif

#define CG_PI_F 3.14159265358979323846f
#define CG_TWOPI_F 6.28318530717958647692f
#define CG_HALFPI_F 1.57079632679489661923f
#define CG_QUARTERPI_F 0.78539816339744830962f

CG_HD uint32_t cg_f2u(float x)
{
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

CG_HD float cg_u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

/* |x|: the sign bit cleared (fabsf, which the device folds into the
 * operands of the instructions that use it). */
CG_HD float cg_fabsf(float x) { return fabsf(x); }

/* floor for |x| < 2^31, exact on both sides (truncation then correction). */
CG_HD float cg_floorf(float x)
{
  float t = (float)(int)x;
  return (t > x) ? CG_SUB(t, 1.0f) : t;
}

/* 2^k as a float for -126 <= k <= 127. */
CG_HD float cg_pow2i(int k) { return cg_u2f((uint32_t)(k + 127) << 23); }

/* e^x, |error| <= 2 ulp, flushes to 0 below -103.9 and to +inf above 88.72. */
CG_HD float cg_expf(float x)
{
  if (x > 88.7228317f) return cg_u2f(0x7f800000u);
  if (x < -103.972084f) return 0.0f;
  /* j = round-to-nearest(x * log2(e)) through the 1.5*2^23 shifter */
  const float shifter = 12582912.0f;
  float j = CG_SUB(CG_FMA(x, 1.44269504088896341f, shifter), shifter);
  int k = (int)j;
  /* r = x - j*ln2 with a two-part ln2 (Cody-Waite) */
  float r = CG_FMA(j, -0.693145751953125f, x);
  r = CG_FMA(j, -1.42860682030941723e-06f, r);
  /* Taylor series of e^r to degree 7, Horner form */
  float p = 1.98412698412698413e-04f;            /* 1/7! */
  p = CG_FMA(p, r, 1.38888888888888889e-03f);    /* 1/6! */
  p = CG_FMA(p, r, 8.33333333333333333e-03f);    /* 1/5! */
  p = CG_FMA(p, r, 4.16666666666666667e-02f);    /* 1/4! */
  p = CG_FMA(p, r, 1.66666666666666667e-01f);    /* 1/3! */
  p = CG_FMA(p, r, 0.5f);
  p = CG_FMA(p, r, 1.0f);
  p = CG_FMA(p, r, 1.0f);
  /* scale by 2^k in two steps so that subnormal results are formed once */
  if (k > 126) return CG_MUL(CG_MUL(p, 2.0f), cg_pow2i(k - 1));
  if (k < -125) return CG_MUL(CG_MUL(p, cg_pow2i(k + 64)), 5.42101086242752217e-20f);
  return CG_MUL(p, cg_pow2i(k));
}

/* log(1+f) for f in [sqrt(2)/2-1, sqrt(2)-1] via 2*atanh(f/(2+f)). */
CG_HD float cg_log1p_reduced(float f)
{
  float s = CG_DIV(f, CG_ADD(2.0f, f));
  float w = CG_MUL(s, s);
  float R = 1.11111111111111111e-01f;            /* 1/9 */
  R = CG_FMA(R, w, 1.42857142857142857e-01f);    /* 1/7 */
  R = CG_FMA(R, w, 2.0e-01f);                    /* 1/5 */
  R = CG_FMA(R, w, 3.33333333333333333e-01f);    /* 1/3 */
  R = CG_MUL(R, w);
  float s2 = CG_MUL(2.0f, s);
  return CG_FMA(s2, R, s2);
}

/* Natural logarithm, |error| <= 2 ulp for finite x > 0; -inf at 0, NaN below. */
CG_HD float cg_logf(float x)
{
  if (!(x > 0.0f)) return (x == 0.0f) ? cg_u2f(0xff800000u) : cg_u2f(0x7fc00000u);
  if (x == cg_u2f(0x7f800000u)) return x;
  int e = 0;
  if (x < 1.17549435e-38f) { /* subnormal input */
    x = CG_MUL(x, 16777216.0f);
    e = -24;
  }
  uint32_t u = cg_f2u(x);
  e += (int)((u >> 23) & 0xff) - 127;
  float m = cg_u2f((u & 0x007fffffu) | 0x3f800000u); /* [1,2) */
  if (m > 1.41421356237309505f) {
    m = CG_MUL(m, 0.5f);
    e += 1;
  }
  float f = CG_SUB(m, 1.0f);
  float lp = cg_log1p_reduced(f);
  float ef = (float)e;
  /* e*ln2 split in a part exact in e*hi and a small correction */
  return CG_FMA(ef, 0.693145751953125f, CG_FMA(ef, 1.42860682030941723e-06f, lp));
}

/* log(1+x) for x > -1 keeping relative accuracy for small |x|. */
CG_HD float cg_log1pf(float x)
{
  float u = CG_ADD(1.0f, x);
  if (u == 1.0f) return x;
  float d = CG_SUB(u, 1.0f);
  /* log(u) * x/(u-1) corrects the rounding of 1+x */
  return CG_MUL(cg_logf(u), CG_DIV(x, d));
}

/* atan(a) for a in [0, 1]: a * P(a^2) with P of degree 9, a minimax fit of
 * atan(a)/a on [0, 1] (Remez exchange on the relative error, fitted for this
 * code); within 1.3 ulp of atan in FP32 with FMA Horner evaluation, and
 * branch-free so that the lanes of a warp do not diverge. */
CG_HD float cg_atan01(float a)
{
  const float w = CG_MUL(a, a);
  float p = -0.00175393012f;
  p = CG_FMA(p, w, 0.0107269445f);
  p = CG_FMA(p, w, -0.0308045968f);
  p = CG_FMA(p, w, 0.057552103f);
  p = CG_FMA(p, w, -0.0837731585f);
  p = CG_FMA(p, w, 0.109420307f);
  p = CG_FMA(p, w, -0.142619327f);
  p = CG_FMA(p, w, 0.199982658f);
  p = CG_FMA(p, w, -0.333332837f);
  p = CG_FMA(p, w, 1.0f);
  return CG_MUL(a, p);
}

/* atan(a) / (pi/2) on [0, 1]: cg_atan01's coefficients times 2/pi, each
 * rounded to float, so that the quarter-turn angle costs no extra product;
 * within 8.2e-8 of the value over every float of [0, 1] (checked
 * exhaustively against libm's double atan). */
CG_HD float cg_atan01_q(float a)
{
  const float w = CG_MUL(a, a);
  float p = -0.00111658662f;
  p = CG_FMA(p, w, 0.00682898518f);
  p = CG_FMA(p, w, -0.0196108148f);
  p = CG_FMA(p, w, 0.0366388075f);
  p = CG_FMA(p, w, -0.0533316508f);
  p = CG_FMA(p, w, 0.0696591288f);
  p = CG_FMA(p, w, -0.0907942802f);
  p = CG_FMA(p, w, 0.127312914f);
  p = CG_FMA(p, w, -0.212206274f);
  p = CG_FMA(p, w, 0.636619747f);
  return CG_MUL(a, p);
}

/* atan2(y, x) in (-pi, pi]; atan2(0, 0) = 0. */
CG_HD float cg_atan2f(float y, float x)
{
  float ax = cg_fabsf(x), ay = cg_fabsf(y);
  if (ax == 0.0f && ay == 0.0f) return 0.0f;
  float mx = ax > ay ? ax : ay;
  float mn = ax > ay ? ay : ax;
  float th = cg_atan01(CG_DIV(mn, mx));
  if (ay > ax) th = CG_SUB(CG_HALFPI_F, th);
  if (x < 0.0f) th = CG_SUB(CG_PI_F, th);
  if (y < 0.0f) th = -th;
  return th;
}

/* acos(c) for c in [-1, 1] as atan2(sqrt((1-c)(1+c)), c). */
CG_HD float cg_acosf(float c)
{
  if (c > 1.0f) c = 1.0f;
  if (c < -1.0f) c = -1.0f;
  float s = CG_SQRT(CG_MUL(CG_SUB(1.0f, c), CG_ADD(1.0f, c)));
  return cg_atan2f(s, c);
}

/* ---------------------------------------------------------------------- */
/* Philox4x32-10                                                          */
/* ---------------------------------------------------------------------- */
typedef struct {
  uint32_t v[4];
} cg_u32x4;

CG_HD void cg_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo)
{
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

CG_HD cg_u32x4 cg_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                uint32_t k0, uint32_t k1)
{
  for (int round = 0; round < 10; round++) {
    uint32_t hi0, lo0, hi1, lo1;
    cg_mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    cg_mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  cg_u32x4 r;
  r.v[0] = c0;
  r.v[1] = c1;
  r.v[2] = c2;
  r.v[3] = c3;
  return r;
}

/* Uniform in [0,1) with 24 random bits: exactly representable as a float. */
CG_HD float cg_u01f(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }

/* Uniform in [0,1) with 53 random bits. */
CG_HD double cg_u01d(uint32_t hi, uint32_t lo)
{
  uint64_t m = ((uint64_t)hi << 21) ^ (uint64_t)(lo >> 11);
  return (double)m * 1.1102230246251565404e-16;
}

/* Stream identifiers: the high key word is seed_hi ^ stream tag. */
#define CG_STREAM_FIELD 0x46494c44u   /* Gaussian field modes   */
#define CG_STREAM_POIS 0x504f4953u    /* Poisson counts (+ipop) */
#define CG_STREAM_POS 0x504f5350u     /* source offsets (+ipop) */

#endif /* CG_MATH_H */
