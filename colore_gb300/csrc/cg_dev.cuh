/*
 * cg_dev.cuh -- device-side structures shared by the kernels of
 * libcolore_cuda.so: background/tracer tables, the error word and the
 * per-pass parameter blocks.
 */
#ifndef CG_DEV_CUH
#define CG_DEV_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_cell.h"
#include "colore_cuda.h"

namespace cg {

/* Error bits written by kernels (never trapping). */
enum : unsigned int {
  ERR_COUNT_OVERFLOW = 1u,  /* count overflow list full, lambda > 2^30,
                               or > 2^31-1 sources in 2048 cells      */
  ERR_CATALOG_OVERFLOW = 2u, /* emit wrote past the allocated catalog  */
  ERR_SHELL_WALK = 4u,       /* imap shell search did not terminate    */
  ERR_IMAP_NSUB = 8u,        /* sub-sampling factor out of range       */
  ERR_IMAP_QUEUE = 16u,      /* intensity-map double-decision queue full */
  ERR_DEPOSIT_OVERFLOW = 64u, /* a cell of the particle deposit holds 2^11 or more */
};

/* The particle deposit accumulates mass in fixed point, 2^20 units per
 * particle, with integer atomics: integer addition is associative, so the
 * density does not depend on the order in which threads add (float atomics
 * would make every run differ in the last bits).  A cell holds up to
 * 2^11 - 2^-20 particles. */
constexpr float DEPOSIT_ONE = 1048576.0f;          /* 2^20 */
constexpr float DEPOSIT_UNIT = 9.5367431640625e-7f; /* 2^-20 */

/* One background table with the edge values of get_bg (cosmo.c:40-86). */
struct Tab {
  const float *f;
  float f0, ff;
};

/* r-uniform grid shared by all background and tracer tables. */
struct Grid1 {
  const float *r; /* r_i = i / idr, NA entries */
  float r_last, idr;
};

__device__ __forceinline__ float bg(const Tab &t, const Grid1 &g, float r)
{
  return cg_bg_eval(t.f, g.r, t.f0, t.ff, r, g.r_last, g.idr);
}

/* One r shared by several table lookups: bg(t, g, r) == bgv(t, bg_at(g, r)). */
struct BgAt {
  int ir, where; /* where: 0 inside, -1 at or below r = 0, 1 at or beyond r_last */
  float t;       /* (r - r_ir) * idr */
};

__device__ __forceinline__ BgAt bg_at(const Grid1 &g, float r)
{
  BgAt a;
  a.where = r <= 0.0f ? -1 : (r >= g.r_last ? 1 : 0);
  a.ir = a.where ? 0 : (int)CG_MUL(r, g.idr);
  a.t = a.where ? 0.0f : CG_MUL(CG_SUB(r, g.r[a.ir]), g.idr);
  return a;
}

__device__ __forceinline__ float bgv(const Tab &t, const BgAt &a)
{
  if (a.where) return a.where < 0 ? t.f0 : t.ff;
  const float fi = t.f[a.ir];
  return CG_FMA(CG_SUB(t.f[a.ir + 1], fi), a.t, fi);
}

/* Normalisation tables hold CG_NA values followed by their two edge values
 * (below r = 0, then at or beyond r_last), so that a table built on the
 * device needs no host round trip: bgvn and bgn read the edges from it. */
__device__ __forceinline__ float bgvn(const Tab &t, const BgAt &a)
{
  if (a.where) return __ldg(t.f + (a.where < 0 ? CG_NA : CG_NA + 1));
  const float fi = t.f[a.ir];
  return CG_FMA(CG_SUB(t.f[a.ir + 1], fi), a.t, fi);
}

__device__ __forceinline__ float bgn(const Tab &t, const Grid1 &g, float r) { return bgvn(t, bg_at(g, r)); }

/* r_of_z, cosmo.c:101-112, on the a-uniform table of NA entries. */
__device__ __forceinline__ float r_of_z(const float *a_arr, const float *r_arr, int na, float z)
{
  float a = CG_DIV(1.0f, CG_ADD(1.0f, z));
  if (a >= 1.0f) return 0.0f;
  if (a <= 0.0f) return r_arr[0];
  float nm1 = (float)(na - 1);
  int ia = (int)CG_MUL(a, nm1);
  return CG_FMA(CG_SUB(r_arr[ia + 1], r_arr[ia]), CG_MUL(CG_SUB(a, a_arr[ia]), nm1), r_arr[ia]);
}

/* Padded real index of cell (ix, iy, iz), fourier.c:46-51. */
__device__ __forceinline__ long long pidx(int ix, int iy, int iz, int N)
{
  return (long long)ix + (long long)(2 * (N / 2 + 1)) * ((long long)iy + (long long)N * iz);
}

__device__ __forceinline__ int wrap(int i, int N) { return i >= N ? i - N : (i < 0 ? i + N : i); }

/* The 19 potential values of get_element's tidal stencil (beaming.c:84-116)
 * around cell (x0, y0, z0), in the order cg_tidal takes them. */
__device__ __forceinline__ void stencil19(const float *__restrict__ phi, int x0, int y0, int z0, int N, float f[19])
{
  const int ngx = 2 * (N / 2 + 1);
  const size_t plane = (size_t)ngx * N;
  if (x0 > 0 && x0 < N - 1 && y0 > 0 && y0 < N - 1 && z0 > 0 && z0 < N - 1) {
    /* away from the box faces: nine row pointers, the x neighbours at
     * constant offsets from them */
    const float *c = phi + (size_t)z0 * plane + (size_t)y0 * ngx + x0;
    const float *yp = c + ngx, *ym = c - ngx, *zp = c + plane, *zm = c - plane;
    f[0] = __ldg(c);
    f[1] = __ldg(c + 1);
    f[2] = __ldg(c - 1);
    f[3] = __ldg(yp);
    f[4] = __ldg(ym);
    f[5] = __ldg(zp);
    f[6] = __ldg(zm);
    f[7] = __ldg(yp + 1);
    f[8] = __ldg(ym - 1);
    f[9] = __ldg(ym + 1);
    f[10] = __ldg(yp - 1);
    f[11] = __ldg(zp + 1);
    f[12] = __ldg(zm - 1);
    f[13] = __ldg(zm + 1);
    f[14] = __ldg(zp - 1);
    f[15] = __ldg(zp + ngx);
    f[16] = __ldg(zm - ngx);
    f[17] = __ldg(zm + ngx);
    f[18] = __ldg(zp - ngx);
    return;
  }
  const int xh = wrap(x0 + 1, N), xl = wrap(x0 - 1, N);
  const int yh = wrap(y0 + 1, N), yl = wrap(y0 - 1, N);
  const int zh = wrap(z0 + 1, N), zl = wrap(z0 - 1, N);
  const float *P0 = phi + (size_t)z0 * plane, *Ph = phi + (size_t)zh * plane, *Pl = phi + (size_t)zl * plane;
  const int o0 = y0 * ngx, oh = yh * ngx, ol = yl * ngx;
#define CG_PHI(X, OY, PZ) __ldg((PZ) + (OY) + (X))
  f[0] = CG_PHI(x0, o0, P0);
  f[1] = CG_PHI(xh, o0, P0);
  f[2] = CG_PHI(xl, o0, P0);
  f[3] = CG_PHI(x0, oh, P0);
  f[4] = CG_PHI(x0, ol, P0);
  f[5] = CG_PHI(x0, o0, Ph);
  f[6] = CG_PHI(x0, o0, Pl);
  f[7] = CG_PHI(xh, oh, P0);
  f[8] = CG_PHI(xl, ol, P0);
  f[9] = CG_PHI(xh, ol, P0);
  f[10] = CG_PHI(xl, oh, P0);
  f[11] = CG_PHI(xh, o0, Ph);
  f[12] = CG_PHI(xl, o0, Pl);
  f[13] = CG_PHI(xh, o0, Pl);
  f[14] = CG_PHI(xl, o0, Ph);
  f[15] = CG_PHI(x0, oh, Ph);
  f[16] = CG_PHI(x0, ol, Pl);
  f[17] = CG_PHI(x0, oh, Pl);
  f[18] = CG_PHI(x0, ol, Ph);
#undef CG_PHI
}

/* Parameters of the Fourier-space fill (fourier.c:285-359). */
struct FillParams {
  int N, NH;
  float dk, idk3, prefac, r2s;
  int do_smooth, smooth_pot;
  const float *pk; /* numk values on logk_i = logkmin + i/idlogk */
  int numk;
  float logkmin, logkmax, idlogk, n_scal;
  uint32_t key0, key1;
  float lpt_norm; /* (sqrt(2 pi)/L)^3, used by the 1LPT displacement fill */
  int lpt_kind;   /* three-field fill: 0 Psi_x,y,z; 1 phi_xx,xy,xz; 2 phi_yy,yz,zz */
};

/* Geometry of the Cartesian box. */
struct Box {
  int N;
  float dx, idx, L, hL;
  float p0, p1, p2;   /* observer */
  unsigned long long mN; /* floor((2^64 - 1) / N) + 1, see divN */
};

/* floor(x / N) for 0 <= x < 2^40 (cell and row indices) and N <= 2^13:
 * x * mN / 2^64 = x / N + e with 0 <= e < x / 2^64 < 2^-24, and x / N is at
 * least 1/N >= 2^-13 below the next integer, so the high word is exact. */
__device__ __forceinline__ long long divN(long long x, const Box &b)
{
  return (long long)__umul64hi((unsigned long long)x, b.mN);
}

} /* namespace cg */

#endif /* CG_DEV_CUH */
