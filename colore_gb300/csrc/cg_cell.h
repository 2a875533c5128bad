/*
 * cg_cell.h -- per-cell and per-sample scalar functions of the mock
 * generation path, written once for the sm_103a kernels and for the CPU
 * build that reproduces their arithmetic (oracle "dev32" mode).
 *
 * Each function restates one function of CoLoRe (file:line given in its
 * comment) in single precision with a fixed operation order, using only
 * the deterministic primitives of cg_math.h.
 */
#ifndef CG_CELL_H
#define CG_CELL_H

#include "cg_math.h"

#define CG_BIAS_POW 1   /* (1+d)^b           common.h:429 (no flag)        */
#define CG_BIAS_EXPLIN 2 /* _BIAS_MODEL_2    common.h:418-422               */
#define CG_BIAS_LIN 3   /* _BIAS_MODEL_3     common.h:423-427               */

/* Linear interpolation on the r-uniform background grid, cosmo.c:30-38.
 * f: table of na values at r_i = i/idr; below r<=0 returns f0, at or beyond
 * r_last = r_{na-1} returns ff. */
CG_HD float cg_bg_eval(const float *f, const float *r_arr, float f0, float ff,
                       float r, float r_last, float idr)
{
  if (r <= 0.0f) return f0;
  if (r >= r_last) return ff;
  int ir = (int)CG_MUL(r, idr);
  float fi = f[ir];
  float df = CG_SUB(f[ir + 1], fi);
  return CG_FMA(df, CG_MUL(CG_SUB(r, r_arr[ir]), idr), fi);
}

/* bias_model, common.h:414-431. */
CG_HD float cg_bias_model(float d, float b, int model)
{
  if (d <= -1.0f) return 0.0f;
  if (model == CG_BIAS_EXPLIN) {
    if (d < 0.0f) return cg_expf(CG_DIV(CG_MUL(b, d), CG_ADD(1.0f, d)));
    return CG_FMA(b, d, 1.0f);
  }
  if (model == CG_BIAS_LIN) {
    float v = CG_FMA(b, d, 1.0f);
    return v > 0.0f ? v : 0.0f;
  }
  return cg_expf(CG_MUL(b, cg_log1pf(d)));
}

/* Comoving cell-corner coordinate i*dx - p (density.c:1087-1094). */
CG_HD float cg_cell_coord(int i, float dx, float p) { return CG_SUB(CG_MUL((float)i, dx), p); }

CG_HD float cg_norm3(float x, float y, float z)
{
  return CG_SQRT(CG_ADD(CG_ADD(CG_MUL(x, x), CG_MUL(y, y)), CG_MUL(z, z)));
}

/* log(k!) for k < 10 (exact values rounded once). */
CG_HD float cg_logfact_small(int k)
{
  return k <= 1 ? 0.0f
       : k == 2 ? 0.693147180559945f
       : k == 3 ? 1.79175946922805f
       : k == 4 ? 3.17805383034795f
       : k == 5 ? 4.78749174278205f
       : k == 6 ? 6.57925121201010f
       : k == 7 ? 8.52516136106541f
       : k == 8 ? 10.6046029027453f
                : 12.8018274800815f;
}

/* Poisson deviate with mean lam from the Philox stream (key k0,k1; counter
 * c0,c1 identifies the cell).  This stands in for gsl_ran_poisson
 * (common.c:185-189), whose stream cannot be reproduced here.
 *   lam < 10 : inversion by sequential search (one uniform);
 *   lam >= 10: PTRS transformed rejection, W. Hormann, "The transformed
 *              rejection method for generating Poisson random variables",
 *              Insurance: Mathematics and Economics 12 (1993) 39-45,
 *              with the log-factorial written through Stirling's series
 *              and log1p so that single precision keeps ~1e-6 absolute
 *              accuracy in the acceptance test.
 * Iterations are bounded; the bound is never reached for finite lam. */
/* PTRS branch of cg_poisson (lam >= 10), out of line: the per-cell loops
 * that sample counts stay small enough for the instruction cache. */
CG_HD_COLD int cg_poisson_ptrs(float lam, uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1)
{
  float slam = CG_SQRT(lam);
  float b = CG_FMA(2.53f, slam, 0.931f);
  float a = CG_FMA(0.02483f, b, -0.059f);
  float invalpha = CG_ADD(1.1239f, CG_DIV(1.1328f, CG_SUB(b, 3.4f)));
  float vr = CG_SUB(0.9277f, CG_DIV(3.6224f, CG_SUB(b, 2.0f)));
  float loginvalpha = cg_logf(invalpha);
  for (uint32_t it = 0; it < 64u; it++) {
    cg_u32x4 w = cg_philox4x32_10(c0, c1, it, 0u, k0, k1);
    float U = CG_SUB(cg_u01f(w.v[0]), 0.5f);
    float V = cg_u01f(w.v[1]);
    float us = CG_SUB(0.5f, cg_fabsf(U));
    float kf = cg_floorf(CG_ADD(CG_FMA(CG_ADD(CG_DIV(CG_MUL(2.0f, a), us), b), U, lam), 0.43f));
    if (us >= 0.07f && V <= vr) return (int)kf;
    if (kf < 0.0f || (us < 0.013f && V > us)) continue;
    int k = (int)kf;
    /* lhs = log(V*invalpha/(a/us^2+b)) */
    float lhs = CG_SUB(CG_ADD(cg_logf(V), loginvalpha),
                       cg_logf(CG_ADD(CG_DIV(a, CG_MUL(us, us)), b)));
    /* rhs = -lam + k*log(lam) - log(k!) */
    float rhs;
    if (k < 10) {
      rhs = CG_SUB(CG_FMA(kf, cg_logf(lam), -lam), cg_logfact_small(k));
    } else {
      /* Stirling: log k! = k log k - k + 0.5 log(2 pi k) + 1/(12k) - 1/(360k^3)
       * rhs = (k-lam) - k*log1p((k-lam)/lam) - 0.5 log(2 pi k) - corr(k) */
      float dk = CG_SUB(kf, lam);
      float ik = CG_DIV(1.0f, kf);
      float corr = CG_MUL(ik, CG_FMA(CG_MUL(ik, ik), -2.77777777777777778e-03f,
                                     8.33333333333333333e-02f));
      rhs = CG_SUB(dk, CG_MUL(kf, cg_log1pf(CG_DIV(dk, lam))));
      rhs = CG_SUB(rhs, CG_MUL(0.5f, cg_logf(CG_MUL(CG_TWOPI_F, kf))));
      rhs = CG_SUB(rhs, corr);
    }
    if (lhs <= rhs) return k;
  }
  return (int)cg_floorf(lam);
}


CG_HD int cg_poisson(float lam, uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1)
{
  if (!(lam > 0.0f)) return 0;
  if (lam < 10.0f) {
    cg_u32x4 w = cg_philox4x32_10(c0, c1, 0u, 0u, k0, k1);
    float u = cg_u01f(w.v[0]);
    float p = cg_expf(-lam);
    float F = p;
    int k = 0;
    while (u >= F && k < 200) {
      k++;
      p = CG_MUL(p, CG_DIV(lam, (float)k));
      F = CG_ADD(F, p);
    }
    return k;
  }
  return cg_poisson_ptrs(lam, k0, k1, c0, c1);
}

/* cart2sph, srcs.c:68-85 / imap.c:24-41.  phi = atan2(y, x): the reference
 * normalises x and y by r first, which leaves the angle unchanged and costs
 * two divisions. */
CG_HD void cg_cart2sph(float x, float y, float z, float *r, float *cth, float *phi)
{
  float rr = cg_norm3(x, y, z);
  *r = rr;
  if (rr == 0.0f) {
    *cth = 1.0f;
    *phi = 0.0f;
    return;
  }
  *cth = CG_DIV(z, rr);
  float ph = cg_atan2f(y, x);
  if (ph < 0.0f) ph = CG_ADD(ph, CG_TWOPI_F);
  *phi = ph;
}

/* he_ang2pix (RING), healpix_extra.c:118-172, for phi already in
 * [0, 2 pi).  Integer work is 32-bit: every intermediate fits for
 * nside <= 8192 (NSIDE_MAX_HPX, common.h:94). */
CG_HD int64_t cg_ang2pix_ring_02pi(int64_t nside64, float cth, float ph)
{
  const int nside = (int)nside64;
  float ctha = cg_fabsf(cth);
  float tt = CG_MUL(ph, 0.636619772367581343f); /* in [0,4] */
  float ns = (float)nside;
  if (ctha <= 0.666666666666666667f) {
    float temp1 = CG_MUL(ns, CG_ADD(0.5f, tt));
    float temp2 = CG_MUL(CG_MUL(ns, cth), 0.75f);
    int jp = (int)CG_SUB(temp1, temp2);
    int jm = (int)CG_ADD(temp1, temp2);
    int ir = nside + 1 + jp - jm;
    int kshift = 1 - (ir & 1);
    int ip = (jp + jm - nside + kshift + 1) >> 1; /* the sum is >= kshift >= 0 (below) */
    /* ip mod 4 nside: phi in [0, 2 pi) puts tt in [0, 4] and temp1 in
     * [nside / 2, 4.5 nside], so jp + jm is in [nside - 1, 9 nside + 1]
     * (each truncation loses less than 1), ip in [0, 4 nside + 1], and one
     * subtraction gives the modulo */
    const int m = 4 * nside;
    if (ip >= m) ip -= m;
    return (int64_t)(nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip);
  } else {
    float tp = CG_SUB(tt, (float)(int)tt);
    float tmp = CG_MUL(ns, CG_SQRT(CG_MUL(3.0f, CG_SUB(1.0f, ctha))));
    int jp = (int)CG_MUL(tp, tmp);
    int jm = (int)CG_MUL(CG_SUB(1.0f, tp), tmp);
    int ir = jp + jm + 1;
    int ip = (int)CG_MUL(tt, (float)ir);
    /* ip mod 4 ir: tt in [0, 4] makes ip 4 ir at most (exactly when tt * ir
     * rounds up to it) */
    const int m = 4 * ir;
    if (ip >= m) ip -= m;
    if (cth > 0.0f) return (int64_t)(2 * ir * (ir - 1) + ip);
    return (int64_t)(12 * nside * nside - 2 * ir * (ir + 1) + ip);
  }
}

/* he_ang2pix (RING) for any phi: reduced to [0, 2 pi) first. */
CG_HD int64_t cg_ang2pix_ring(int64_t nside64, float cth, float phi)
{
  float ph = phi;
  if (ph >= 0.0f) {
    if (!(ph < CG_TWOPI_F)) ph = fmodf(ph, CG_TWOPI_F);
  } else {
    float tmp = CG_ADD(fmodf(ph, CG_TWOPI_F), CG_TWOPI_F);
    ph = (tmp == CG_TWOPI_F) ? 0.0f : tmp;
  }
  return cg_ang2pix_ring_02pi(nside64, cth, ph);
}

/* ---- NEST <-> RING (Gorski et al. 2005, ApJ 622, 759), integer only ---- */
CG_HD int cg_jrll(int f) { return (f < 4) ? 2 : ((f < 8) ? 3 : 4); }
CG_HD int cg_jpll(int f) { return f < 4 ? 2 * f + 1 : (f < 8 ? 2 * (f - 4) : 2 * (f - 8) + 1); }

CG_HD uint32_t cg_compact_bits(uint64_t v)
{
  v &= 0x5555555555555555ull;
  v = (v ^ (v >> 1)) & 0x3333333333333333ull;
  v = (v ^ (v >> 2)) & 0x0f0f0f0f0f0f0f0full;
  v = (v ^ (v >> 4)) & 0x00ff00ff00ff00ffull;
  v = (v ^ (v >> 8)) & 0x0000ffff0000ffffull;
  v = (v ^ (v >> 16)) & 0x00000000ffffffffull;
  return (uint32_t)v;
}

CG_HD uint64_t cg_spread_bits(uint32_t x)
{
  uint64_t v = x;
  v = (v | (v << 16)) & 0x0000ffff0000ffffull;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}

/* Ring index jr (1..4nside-1), position jp (1..4nr), ring length info for a
 * NEST pixel.  kshift and nr as in the HEALPix papers. */
CG_HD void cg_nest_ringpos(int64_t nside, int64_t ipix, int64_t *jr_o, int64_t *jp_o,
                           int64_t *nr_o, int64_t *kshift_o)
{
  int64_t npface = nside * nside;
  int face = (int)(ipix / npface);
  int64_t ipf = ipix % npface;
  int64_t ix = cg_compact_bits((uint64_t)ipf);
  int64_t iy = cg_compact_bits((uint64_t)ipf >> 1);
  int64_t jrt = ix + iy, jpt = ix - iy;
  int64_t jr = (int64_t)cg_jrll(face) * nside - jrt - 1;
  int64_t nr, kshift;
  if (jr < nside) {
    nr = jr;
    kshift = 0;
  } else if (jr > 3 * nside) {
    nr = 4 * nside - jr;
    kshift = 0;
  } else {
    nr = nside;
    kshift = (jr - nside) & 1;
  }
  int64_t jp = ((int64_t)cg_jpll(face) * nr + jpt + 1 + kshift) / 2;
  if (jp > 4 * nside) jp -= 4 * nside;
  if (jp < 1) jp += 4 * nside;
  *jr_o = jr;
  *jp_o = jp;
  *nr_o = nr;
  *kshift_o = kshift;
}

/* nest2ring, as used by he_nest2ring_inplace (healpix_extra.c:292-317). */
CG_HD int64_t cg_nest2ring(int64_t nside, int64_t ipix)
{
  int64_t jr, jp, nr, ks;
  cg_nest_ringpos(nside, ipix, &jr, &jp, &nr, &ks);
  int64_t ncap = 2 * nside * (nside - 1);
  int64_t npix = 12 * nside * nside;
  if (jr < nside) return 2 * jr * (jr - 1) + jp - 1;
  if (jr > 3 * nside) return npix - 2 * (nr + 1) * nr + jp - 1;
  return ncap + (jr - nside) * 4 * nside + jp - 1;
}

/* ring2nest (chealpix ring2nest, used at srcs.c:269). */
CG_HD int64_t cg_ring2nest(int64_t nside, int64_t ipring)
{
  int64_t ncap = 2 * nside * (nside - 1);
  int64_t npix = 12 * nside * nside;
  int64_t iring, iphi, kshift, nr;
  int face;
  if (ipring < ncap) { /* north cap */
    int64_t t = ipring + 1;
    /* iring = floor((1+sqrt(2t-1))/2) found exactly with integers */
    iring = 1;
    while (2 * (iring + 1) * iring < t) iring++;
    iphi = t - 2 * iring * (iring - 1);
    kshift = 0;
    nr = iring;
    face = (int)((iphi - 1) / nr);
  } else if (ipring < npix - ncap) { /* equatorial */
    int64_t ip = ipring - ncap;
    int64_t tmp = ip / (4 * nside);
    iring = tmp + nside;
    iphi = ip - tmp * 4 * nside + 1;
    kshift = (iring + nside) & 1;
    nr = nside;
    int64_t ire = tmp + 1, irm = 2 * nside + 2 - ire;
    int64_t ifm = (iphi - ire / 2 + nside - 1) / nside;
    int64_t ifp = (iphi - irm / 2 + nside - 1) / nside;
    if (ifp == ifm) face = (int)((ifp == 4) ? 4 : ifp + 4);
    else if (ifp < ifm) face = (int)ifp;
    else face = (int)(ifm + 8);
  } else { /* south cap */
    int64_t t = npix - ipring;
    int64_t irs = 1;
    while (2 * (irs + 1) * irs < t) irs++;
    iphi = 4 * irs + 1 - (t - 2 * irs * (irs - 1));
    kshift = 0;
    nr = irs;
    iring = 4 * nside - irs;
    face = (int)((iphi - 1) / nr) + 8;
  }
  int64_t irt = iring - (int64_t)cg_jrll(face) * nside + 1;
  int64_t ipt = 2 * iphi - (int64_t)cg_jpll(face) * nr - kshift - 1;
  if (ipt >= 2 * nside) ipt -= 8 * nside;
  int64_t ix = (ipt - irt) >> 1;
  int64_t iy = (-(ipt + irt)) >> 1;
  return (int64_t)face * nside * nside +
         (int64_t)(cg_spread_bits((uint32_t)ix) | (cg_spread_bits((uint32_t)iy) << 1));
}

/* sin and cos of x in [-2pi, 2pi]: quadrant reduction plus Taylor series. */
CG_HD void cg_sincosf(float x, float *s, float *c)
{
  const float shifter = 12582912.0f;
  float j = CG_SUB(CG_FMA(x, 0.636619772367581343f, shifter), shifter);
  int q = (int)j;
  float r = CG_FMA(j, -1.5707969665527344f, x);
  r = CG_FMA(j, 6.3975784811191261e-07f, r);
  r = CG_FMA(j, -5.3903029534742385e-15f, r);
  float w = CG_MUL(r, r);
  float ps = -2.50521083854417188e-08f;            /* -1/11! */
  ps = CG_FMA(ps, w, 2.75573192239858907e-06f);    /*  1/9!  */
  ps = CG_FMA(ps, w, -1.98412698412698413e-04f);   /* -1/7!  */
  ps = CG_FMA(ps, w, 8.33333333333333333e-03f);    /*  1/5!  */
  ps = CG_FMA(ps, w, -1.66666666666666667e-01f);   /* -1/3!  */
  float sr = CG_FMA(CG_MUL(ps, w), r, r);
  float pc = 2.08767569878680990e-09f;             /*  1/12! */
  pc = CG_FMA(pc, w, -2.75573192239858907e-07f);   /* -1/10! */
  pc = CG_FMA(pc, w, 2.48015873015873016e-05f);    /*  1/8!  */
  pc = CG_FMA(pc, w, -1.38888888888888889e-03f);   /* -1/6!  */
  pc = CG_FMA(pc, w, 4.16666666666666667e-02f);    /*  1/4!  */
  pc = CG_FMA(pc, w, -0.5f);
  float cr = CG_FMA(pc, w, 1.0f);
  switch (q & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

/* pix2vec_nest (chealpix, used by hp_shell_alloc common.c:536). */
CG_HD void cg_pix2vec_nest(int64_t nside, int64_t ipix, float v[3])
{
  int64_t jr, jp, nr, ks;
  cg_nest_ringpos(nside, ipix, &jr, &jp, &nr, &ks);
  float z, sth;
  float fact2 = CG_DIV(4.0f, (float)(12 * nside * nside));
  if (jr < nside) {
    float t = CG_MUL(CG_MUL((float)nr, (float)nr), fact2);
    z = CG_SUB(1.0f, t);
    sth = CG_SQRT(CG_MUL(t, CG_SUB(2.0f, t)));
  } else if (jr > 3 * nside) {
    float t = CG_MUL(CG_MUL((float)nr, (float)nr), fact2);
    z = CG_SUB(t, 1.0f);
    sth = CG_SQRT(CG_MUL(t, CG_SUB(2.0f, t)));
  } else {
    z = CG_DIV(CG_MUL((float)(2 * nside - jr), 2.0f), CG_MUL(3.0f, (float)nside));
    sth = CG_SQRT(CG_MUL(CG_SUB(1.0f, z), CG_ADD(1.0f, z)));
  }
  float phi = CG_DIV(CG_MUL(CG_SUB((float)jp, CG_MUL((float)(ks + 1), 0.5f)), CG_HALFPI_F),
                     (float)nr);
  float s, c;
  cg_sincosf(phi, &s, &c);
  v[0] = CG_MUL(sth, c);
  v[1] = CG_MUL(sth, s);
  v[2] = z;
}

/* Shell search of get_r_index_imap, imap.c:76-103, bounded so that a gap
 * between shells (where the reference walk would never stop) returns -1. */
CG_HD int cg_shell_index(const float *r0, const float *rf, int nr, float r, int start)
{
  int ir = start < 0 ? 0 : (start >= nr ? nr - 1 : start);
  for (int it = 0; it < 2 * nr + 4; it++) {
    if (ir == -1 || ir == nr) return ir;
    if (r < r0[ir]) ir--;
    else if (r >= rf[ir]) ir++;
    else return ir;
  }
  return -1;
}

/* cg_shell_index(r0, rf, nr, r, 0) in O(log nr) steps.  The walk from shell
 * 0 climbs while r >= r0[i] and r >= rf[i] and stops at the first shell j
 * where r < r0[j] (a gap or below the shells: the walk then oscillates and
 * gives -1) or r < rf[j] (r0[j] <= r: shell j); past the last shell it gives
 * nr.  With r0 sorted ascending and rfm the running maximum of rf
 * (rfm[i] = max(rf[0..i])), j is the first index with r < r0[j] or
 * r < rfm[j], both found by bisection. */
CG_HD int cg_shell_index0(const float *r0, const float *rfm, int nr, float r)
{
  int lo = 0, hi = nr; /* first i with r < r0[i] (nr if none) */
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (r < r0[mid]) hi = mid;
    else lo = mid + 1;
  }
  const int j0 = lo;
  lo = 0;
  hi = nr; /* first i with r < rfm[i] */
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (r < rfm[mid]) hi = mid;
    else lo = mid + 1;
  }
  const int jf = lo;
  if (jf < j0) return jf;
  return j0 == nr ? nr : -1;
}

/* Radial velocity from a centred potential difference (get_rvel,
 * srcs.c:87-118): 0.5*idx*(dphi . u) with u = x * (1/r). */
CG_HD float cg_rvel(float vx, float vy, float vz, float x0, float y0, float z0, float rr, float idx)
{
  const float ir = CG_DIV(1.0f, rr);
  float ux = CG_MUL(x0, ir), uy = CG_MUL(y0, ir), uz = CG_MUL(z0, ir);
  float dot = CG_ADD(CG_ADD(CG_MUL(vx, ux), CG_MUL(vy, uy)), CG_MUL(vz, uz));
  return CG_MUL(CG_MUL(0.5f, idx), dot);
}

/* ---- compound per-cell expressions shared by kernels and CPU checks ---- */

/* density transforms of compute_physical_density_field (density.c:1105-1119) */
#define CG_DMODE_NONE 0 /* field already physical                        */
#define CG_DMODE_LGNR 1 /* lognormalize, density.c:1070-1103              */
#define CG_DMODE_CLIP 2 /* densclip, density.c:1034-1067                  */
#define CG_DMODE_RHO 3  /* 1LPT normalisation d = rho - 1, density.c:610-624 */

CG_HD float cg_dens_transform(int mode, float d, float D, float s2)
{
  if (mode == CG_DMODE_LGNR) return CG_SUB(cg_expf(CG_MUL(D, CG_SUB(d, CG_MUL(CG_MUL(0.5f, D), s2)))), 1.0f);
  if (mode == CG_DMODE_CLIP) {
    float v = CG_FMA(D, d, 1.0f);
    return CG_SUB(v > 0.0f ? v : 0.0f, 1.0f);
  }
  if (mode == CG_DMODE_RHO) return CG_SUB(d, 1.0f);
  return d;
}

/* lambda = ndens*cell_vol*bias_model(d,b)*dnorm, srcs.c:174 */
CG_HD float cg_src_lambda(float nd, float cell_vol, float d, float b, float dn, int model)
{
  return CG_MUL(CG_MUL(CG_MUL(nd, cell_vol), cg_bias_model(d, b, model)), dn);
}

/* source coordinate x0 + dx (u - 1/2), srcs.c:261-263 */
CG_HD float cg_src_offset(float x0, float dx, uint32_t bits)
{
  return CG_ADD(x0, CG_MUL(dx, CG_SUB(cg_u01f(bits), 0.5f)));
}

/* ra, dec in degrees of the direction (x, y, z) with azimuth ph in
 * [0, 2 pi], srcs.c:408-409: ra = RTOD phi and dec = 90 - RTOD theta, with
 * theta = atan2(sqrt(x^2 + y^2), z) (acos of z/r loses half its digits near
 * the poles in single precision). */
CG_HD void cg_radec(float x, float y, float z, float ph, float *ra, float *dec)
{
  *ra = CG_MUL(57.2957795f, ph);
  const float rho = CG_SQRT(CG_FMA(x, x, CG_MUL(y, y)));
  *dec = CG_SUB(90.0f, CG_MUL(57.2957795f, cg_atan2f(rho, z)));
}

/* sub-cell centre c0 + (i + 1/2) dxs, imap.c:212-218 */
CG_HD float cg_sub_centre(float c0, int i, float dxs) { return CG_FMA(CG_ADD((float)i, 0.5f), dxs, c0); }

/* y^2 + z^2 of an x-line of sub-samples */
CG_HD float cg_yz2(float y, float z) { return CG_FMA(y, y, CG_MUL(z, z)); }

/* imap brightness and radial shift, imap.c:199-201 */
CG_HD float cg_imap_temp(float tmean, float d, float bias, float dnorm, int model)
{
  return CG_MUL(CG_MUL(tmean, cg_bias_model(d, bias, model)), dnorm);
}
CG_HD float cg_imap_drsd(float rvel, float v1, float ih) { return CG_MUL(CG_MUL(rvel, v1), ih); }

/* One intensity-map sub-sample of imap.c:210-231 at (x, y, z), with
 * yz2 = y^2 + z^2 shared by the samples of an x-line: returns the shell
 * index (or -1 / nr outside the shells) and the RING pixel.  The radius is
 * sqrt(x^2 + yz2) (one fused multiply-add); cos(theta) = z/r and
 * phi = atan2(y, x) as in cart2sph. */
CG_HD int cg_imap_sample(float x, float y, float z, float yz2, float drr, const float *r0, const float *rf, int nr,
                         int start, int64_t nside, int64_t *pix)
{
  const float r = CG_SQRT(CG_FMA(x, x, yz2));
  const float rs = CG_ADD(r, drr);
  /* most samples stay in the shell of their cell: the walk from there */
  const int ir = (start >= 0 && start < nr && rs >= r0[start] && rs < rf[start])
                     ? start
                     : cg_shell_index(r0, rf, nr, rs, start);
  if (ir < 0 || ir >= nr) return ir;
  float cth = 1.0f, ph = 0.0f;
  if (r != 0.0f) {
    cth = CG_DIV(z, r);
    ph = cg_atan2f(y, x);
    if (ph < 0.0f) ph = CG_ADD(ph, CG_TWOPI_F);
  }
  /* atan2 in (-pi, pi] shifted by 2 pi below 0 gives [0, 2 pi] in exact
   * arithmetic; the rounded sum can reach 2 pi itself, which the general
   * entry point maps to 0 */
  if (!(ph < CG_TWOPI_F)) ph = 0.0f;
  *pix = cg_ang2pix_ring_02pi(nside, cth, ph);
  return ir;
}

/* CIC cell and weights along a ray, interpolate_from_grid trilinear branch
 * (beaming.c:183-204): x = (rm u + po) idx, i0 = (int)x, h0 = x - i0. */
CG_HD void cg_cic_axis(float rm, float u, float po, float idx, int N, int *i0, int *i1, float *h0, float *h1)
{
  const float x = CG_MUL(CG_ADD(CG_MUL(rm, u), po), idx);
  int a = (int)x;
  *h0 = CG_SUB(x, (float)a);
  *h1 = CG_SUB(1.0f, *h0);
  int b = a + 1;
  a = a >= N ? a - N : (a < 0 ? a + N : a);
  b = b >= N ? b - N : (b < 0 ? b + N : b);
  *i0 = a;
  *i1 = b;
}

/* Trilinear combination of the eight corner values v[bx + 2 by + 4 bz]
 * (b = 0 for the i0 cell, 1 for the i1 cell of each axis): the four terms
 * of the i0[2] plane, then the four of the i1[2] plane, in the order of
 * interpolate_from_grid (beaming.c:205-262), chained with FMAs. */
CG_HD float cg_cic_combine(const float v[8], const float h0[3], const float h1[3])
{
  const float wa = h1[2], wb = h0[2];
  const float w00 = CG_MUL(h1[1], h1[0]), w01 = CG_MUL(h1[1], h0[0]);
  const float w10 = CG_MUL(h0[1], h1[0]), w11 = CG_MUL(h0[1], h0[0]);
  float d = CG_MUL(v[0], CG_MUL(wa, w00));
  d = CG_FMA(v[1], CG_MUL(wa, w01), d);
  d = CG_FMA(v[2], CG_MUL(wa, w10), d);
  d = CG_FMA(v[3], CG_MUL(wa, w11), d);
  d = CG_FMA(v[4], CG_MUL(wb, w00), d);
  d = CG_FMA(v[5], CG_MUL(wb, w01), d);
  d = CG_FMA(v[6], CG_MUL(wb, w10), d);
  d = CG_FMA(v[7], CG_MUL(wb, w11), d);
  return d;
}

/* Trilinear value of a padded grid (row stride 2(N/2+1)) */
CG_HD float cg_cic_value(const float *g, const int i0[3], const int i1[3], const float h0[3], const float h1[3], int N)
{
  const long long ngx = 2 * (N / 2 + 1);
  const float *pa = g + (long long)i0[2] * ngx * N, *pb = g + (long long)i1[2] * ngx * N;
  const long long ya = (long long)i0[1] * ngx, yb = (long long)i1[1] * ngx;
  const float v[8] = {pa[ya + i0[0]], pa[ya + i1[0]], pa[yb + i0[0]], pa[yb + i1[0]],
                      pb[ya + i0[0]], pb[ya + i1[0]], pb[yb + i0[0]], pb[yb + i1[0]]};
  return cg_cic_combine(v, h0, h1);
}

/* Gaussian field of a physical (lognormal) density cell, get_element
 * RETURN_GAUSS (beaming.c:54-66): log(1 + d) / D(r) + D(r) sigma^2 / 2 with
 * D the growth factor at the cell's own radius. */
CG_HD float cg_gauss_of_dens(float d, float dg, float sigma2)
{
  return CG_ADD(CG_DIV(cg_log1pf(d), dg), CG_MUL(CG_MUL(dg, sigma2), 0.5f));
}

/* NGP cell along a ray, interpolate_from_grid NGP branch (beaming.c:148-157) */
CG_HD int cg_ngp_cell(float rm, float u, float po, float idx, int N)
{
  float xn = CG_MUL(CG_ADD(CG_MUL(rm, u), po), idx);
  int i = (int)CG_ADD(xn, 0.5f);
  return i >= N ? i - N : (i < 0 ? i + N : i);
}

/* transverse projection coefficients of the tidal tensor, kappa.c:131-145 */
CG_HD void cg_kappa_rot(const float u[3], float prefac, float rot[6])
{
  float cth = u[2];
  if (cth >= 1.0f) cth = 1.0f;
  if (cth <= -1.0f) cth = -1.0f;
  const float sth = CG_SQRT(CG_MUL(CG_SUB(1.0f, cth), CG_ADD(1.0f, cth)));
  float cph = 1.0f, sph = 0.0f;
  if (sth != 0.0f) {
    cph = CG_DIV(u[0], sth);
    sph = CG_DIV(u[1], sth);
  }
  const float c2 = CG_MUL(cth, cth);
  rot[0] = CG_MUL(CG_ADD(CG_MUL(CG_MUL(c2, cph), cph), CG_MUL(sph, sph)), prefac);
  rot[1] = CG_MUL(CG_MUL(CG_MUL(CG_MUL(2.0f, cph), sph), CG_SUB(c2, 1.0f)), prefac);
  rot[2] = CG_MUL(CG_MUL(CG_MUL(CG_MUL(-2.0f, cth), sth), cph), prefac);
  rot[3] = CG_MUL(CG_ADD(CG_MUL(CG_MUL(c2, sph), sph), CG_MUL(cph, cph)), prefac);
  rot[4] = CG_MUL(CG_MUL(CG_MUL(CG_MUL(-2.0f, cth), sth), sph), prefac);
  rot[5] = CG_MUL(CG_MUL(sth, sth), prefac);
}

/* Projections of srcs_get_beam_properties_single (srcs.c:536-581) for one
 * source direction: ux, uy take the potential gradient to the deflection
 * (prefac_m = idx / (2 r)); rk, re1, re2 take the tidal tensor to the
 * convergence and the two shear components (prefac = idx^2 / r). */
CG_HD void cg_lens_rot(const float u[3], float prefac, float prefac_m, float ux[3], float uy[3], float rk[6],
                       float re1[6], float re2[6])
{
  float cth = u[2];
  if (cth >= 1.0f) cth = 1.0f;
  if (cth <= -1.0f) cth = -1.0f;
  const float sth = CG_SQRT(CG_MUL(CG_SUB(1.0f, cth), CG_ADD(1.0f, cth)));
  float cph = 1.0f, sph = 0.0f;
  if (sth != 0.0f) {
    cph = CG_DIV(u[0], sth);
    sph = CG_DIV(u[1], sth);
  }
  ux[0] = CG_MUL(CG_MUL(cth, cph), prefac_m);
  ux[1] = CG_MUL(CG_MUL(cth, sph), prefac_m);
  ux[2] = CG_MUL(-sth, prefac_m);
  uy[0] = CG_MUL(-sph, prefac_m);
  uy[1] = CG_MUL(cph, prefac_m);
  uy[2] = 0.0f;
  const float c2 = CG_MUL(cth, cth);
  const float cc = CG_MUL(cph, cph), ss = CG_MUL(sph, sph), cs = CG_MUL(cph, sph);
  rk[0] = CG_MUL(CG_ADD(CG_MUL(c2, cc), ss), prefac);
  rk[1] = CG_MUL(CG_MUL(CG_MUL(2.0f, cs), CG_SUB(c2, 1.0f)), prefac);
  rk[2] = CG_MUL(CG_MUL(CG_MUL(CG_MUL(-2.0f, cth), sth), cph), prefac);
  rk[3] = CG_MUL(CG_ADD(CG_MUL(c2, ss), cc), prefac);
  rk[4] = CG_MUL(CG_MUL(CG_MUL(CG_MUL(-2.0f, cth), sth), sph), prefac);
  rk[5] = CG_MUL(CG_MUL(sth, sth), prefac);
  re1[0] = CG_MUL(CG_SUB(CG_MUL(c2, cc), ss), prefac);
  re1[1] = CG_MUL(CG_MUL(CG_MUL(2.0f, cs), CG_ADD(c2, 1.0f)), prefac);
  re1[2] = rk[2];
  re1[3] = CG_MUL(CG_SUB(CG_MUL(c2, ss), cc), prefac);
  re1[4] = rk[4];
  re1[5] = rk[5];
  re2[0] = CG_MUL(CG_MUL(CG_MUL(-2.0f, cth), cs), prefac);
  re2[1] = CG_MUL(CG_MUL(CG_MUL(2.0f, cth), CG_SUB(cc, ss)), prefac);
  re2[2] = CG_MUL(CG_MUL(CG_MUL(2.0f, sth), sph), prefac);
  re2[3] = CG_MUL(CG_MUL(CG_MUL(2.0f, cth), cs), prefac);
  re2[4] = CG_MUL(CG_MUL(CG_MUL(-2.0f, sth), cph), prefac);
  re2[5] = 0.0f;
}

/* tidal tensor from the 19-point stencil, get_element (beaming.c:84-116);
 * order XX, XY, XZ, YY, YZ, ZZ.  f[] = {000, x+, x-, y+, y-, z+, z-,
 * x+y+, x-y-, x+y-, x-y+, x+z+, x-z-, x+z-, x-z+, y+z+, y-z-, y+z-, y-z+} */
CG_HD void cg_tidal(const float f[19], float t[6])
{
  const float two0 = CG_MUL(2.0f, f[0]);
  t[0] = CG_SUB(CG_ADD(f[1], f[2]), two0);
  t[3] = CG_SUB(CG_ADD(f[3], f[4]), two0);
  t[5] = CG_SUB(CG_ADD(f[5], f[6]), two0);
  t[1] = CG_MUL(0.25f, CG_SUB(CG_SUB(CG_ADD(f[7], f[8]), f[9]), f[10]));
  t[2] = CG_MUL(0.25f, CG_SUB(CG_SUB(CG_ADD(f[11], f[12]), f[13]), f[14]));
  t[4] = CG_MUL(0.25f, CG_SUB(CG_SUB(CG_ADD(f[15], f[16]), f[17]), f[18]));
}

CG_HD float cg_dot3(const float a[3], const float b[3])
{
  return CG_FMA(a[2], b[2], CG_FMA(a[1], b[1], CG_MUL(a[0], b[0])));
}

CG_HD float cg_dot6(const float a[6], const float b[6])
{
  float d = CG_MUL(a[0], b[0]);
  for (int i = 1; i < 6; i++) d = CG_FMA(a[i], b[i], d);
  return d;
}

CG_HD void cg_kahan_add(float *s, float *c, float x)
{
  float y = CG_SUB(x, *c);
  float t = CG_ADD(*s, y);
  *c = CG_SUB(CG_SUB(t, *s), y);
  *s = t;
}

#endif /* CG_CELL_H */
