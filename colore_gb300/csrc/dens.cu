/*
 * dens.cu -- physical density field (density.c:1034-1126) and the
 * redshift-bin sums of the bias normalisation (density.c:1128-1211).
 *
 *  k_moments_final : fixed-order FP64 sum of the per-block (sum d, sum d^2)
 *                    partials of the x pass -> <d>, sigma^2 (fourier.c:24-79).
 *  k_dens_bins     : one streaming pass over the grid that applies the
 *                    lognormal (or clipped, or 1LPT "rho-1") transform in
 *                    place and accumulates, per redshift bin, the cell count,
 *                    the summed redshift and the summed bias_model of every
 *                    tracer.  A warp owns 32 consecutive cells of a row;
 *                    lanes sharing a bin are reduced with shuffles (one pass
 *                    when the 32 cells share a bin, the common case) and lane
 *                    0 adds the sums to the warp's private bins in shared
 *                    memory: integer counts and compensated (Kahan) FP32
 *                    sums, since FP64 arithmetic is scarce on this GPU.  Each
 *                    block combines its warps' bins in FP64 in a fixed order
 *                    and adds them to global 128-bit fixed-point
 *                    accumulators with integer atomics, whose sum does not
 *                    depend on the order the blocks arrive in.
 *  k_bins_finish   : the accumulators back to FP64 sums, the same bits on
 *                    every run.
 *  k_lpt_deposit   : 1LPT particle positions (density.c:473-501) and their
 *                    NGP, CIC or TSC deposit (density.c:37-187), staged per
 *                    tile of particles in shared memory.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "dens_api.h"

namespace {
using namespace cg;

__global__ void k_moments_final(const double2 *__restrict__ part, size_t n, double inv_ncell,
                                double *stats, float *s2f)
{
  __shared__ double sa[1024], sb[1024];
  double a = 0.0, b = 0.0;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
    double2 v = part[i];
    a += v.x;
    b += v.y;
  }
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double mean = sa[0] * inv_ncell;
    double s2 = sb[0] * inv_ncell - mean * mean;
    stats[0] = sa[0];
    stats[1] = sb[0];
    stats[2] = mean;
    stats[3] = s2;
    *s2f = (float)s2;
  }
}

constexpr int MAXT = 8;      /* tracers per bins launch */
constexpr int BINS_WARPS = 8; /* warps per block at most  */

/* Warp reduction of v over the lanes whose mask bit is set (others add 0). */
__device__ __forceinline__ float wsum(float v, bool mine)
{
  float x = mine ? v : 0.0f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

/* Compensated FP32 accumulation s += v (c holds the running correction). */
__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

/* 128-bit two's-complement fixed point with FIX_FRAC fraction bits, as a
 * (low, high) pair of u64: integer additions commute, so the total of the
 * blocks' FP64 partials is the same whatever order they arrive in.  A
 * partial x (|x| < 2^(127 - FIX_FRAC)) is rounded to the nearest multiple
 * of 2^-FIX_FRAC: |x| 2^(FIX_FRAC - 64) splits exactly into its integer part
 * (the high word) and its fraction, which scaled by 2^64 is the low word. */
constexpr int FIX_FRAC = 60;
constexpr double FIX_HI = 16.0;                                        /* 2^(64 - FIX_FRAC) */
constexpr double FIX_LO = 1.0 / 1152921504606846976.0;                 /* 2^-FIX_FRAC */
constexpr double FIX_TO_HI = 1.0 / 16.0;                               /* 2^(FIX_FRAC - 64) */
constexpr double TWO64 = 18446744073709551616.0;

__device__ __forceinline__ void fix_add(unsigned long long *a, double x)
{
  const bool neg = x < 0.0;
  const double y = __dmul_rn(fabs(x), FIX_TO_HI);
  const double h = floor(y);
  const double f = __dsub_rn(y, h); /* exact: y >= 0 */
  unsigned long long hi = __double2ull_rn(h), lo = __double2ull_rn(__dmul_rn(f, TWO64));
  if (neg) {
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  const unsigned long long old = atomicAdd(a, lo);
  const unsigned long long carry = (old + lo < old) ? 1ull : 0ull;
  if (hi + carry) atomicAdd(a + 1, hi + carry);
}

/* Shared-memory bytes of one warp's bins: u32 count, then (sum, correction)
 * for the redshift and every tracer. */
__host__ __device__ inline size_t bins_warp_bytes(int nz, int nt) { return (size_t)nz * (4 + 8 * (1 + nt)); }

/* Up to three tracers the kernel fits 32 registers, eight blocks per SM
 * (11.2 -> 10.8 ms at 1024^3 with two); more tracers keep two. */
template <int NT>
__global__ void __launch_bounds__(BINS_WARPS * 32, NT <= 3 ? 8 : 2) k_dens_bins(float *grid, cg_bins_params p)
{
  extern __shared__ unsigned char sbins[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  constexpr int nt = NT, MT = NT > 0 ? NT : 1;
  const int nz = p.nz, W = 1 + nt;
  unsigned int *cnt = reinterpret_cast<unsigned int *>(sbins + (size_t)wid * bins_warp_bytes(nz, nt));
  float *acc = reinterpret_cast<float *>(cnt + nz); /* [nz][W] sums, then [nz][W] corrections */
  float *cor = acc + (size_t)nz * W;
  for (int i = lane; i < nz; i += 32) cnt[i] = 0u;
  for (int i = lane; i < 2 * nz * W; i += 32) acc[i] = 0.0f;
  __syncwarp();
  const int N = p.box.N;
  const int nseg_row = (N + 31) / 32;
  const int nrow = N * N;
  const float s2 = p.sigma2f ? *p.sigma2f : 0.0f;
  const bool need_d1 = (p.mode == CG_DMODE_LGNR || p.mode == CG_DMODE_CLIP);
  const int gw = blockIdx.x * nwb + wid;
  const int nw = gridDim.x * nwb;
  /* a warp takes whole rows, 32 cells at a time */
  for (int row = gw; row < nrow; row += nw)
  for (int sr = 0; sr < nseg_row; sr++) {
    const int iz = row / N, iy = row - iz * N;
    const int ix = sr * 32 + lane;
    int bin = -1;
    float zz = 0.0f, bs[MT];
#pragma unroll
    for (int t = 0; t < MT; t++) bs[t] = 0.0f;
    if (ix < N) {
      float *ptr = grid + pidx(ix, iy, iz, N);
      float d = *ptr;
      const float x0 = cg_cell_coord(ix, p.box.dx, p.box.p0);
      const float y0 = cg_cell_coord(iy, p.box.dx, p.box.p1), z0 = cg_cell_coord(iz, p.box.dx, p.box.p2);
      const float r = cg_norm3(x0, y0, z0);
      const BgAt at = bg_at(p.g, r);
      if (p.mode != CG_DMODE_NONE) {
        if (p.mode == CG_DMODE_RHO) {
          /* the particle deposit's fixed-point mass (never negative unless
           * a cell overflowed) */
          const int m = __float_as_int(d);
          if (m < 0 && p.err) atomicOr(p.err, ERR_DEPOSIT_OVERFLOW);
          d = CG_MUL((float)m, DEPOSIT_UNIT);
        }
        d = cg_dens_transform(p.mode, d, need_d1 ? bgv(p.d1, at) : 0.0f, s2);
        *ptr = d;
      }
      if (nz > 0) {
        const float z = bgv(p.zt, at);
        const int b = (int)CG_MUL(z, p.idz) + 1;
        if (b >= 0 && b < nz) {
          bin = b;
          zz = z;
#pragma unroll
          for (int t = 0; t < nt; t++) bs[t] = cg_bias_model(d, bgv(p.bz[t], at), p.bias_model);
        }
      }
    }
    if (nz == 0) continue;
    /* segmented reduction by bin; one pass when the 32 cells share a bin */
    unsigned todo = __ballot_sync(0xffffffffu, bin >= 0);
    while (todo) {
      const int lb = __shfl_sync(0xffffffffu, bin, __ffs(todo) - 1);
      const bool mine = (bin == lb);
      const unsigned grp = __ballot_sync(0xffffffffu, mine);
      const float zsum = wsum(zz, mine);
      float bsum[MT];
#pragma unroll
      for (int t = 0; t < nt; t++) bsum[t] = wsum(bs[t], mine);
      if (lane == 0) {
        float *a = acc + (size_t)lb * W, *c = cor + (size_t)lb * W;
        cnt[lb] += (unsigned)__popc(grp);
        kahan_add(a[0], c[0], zsum);
#pragma unroll
        for (int t = 0; t < nt; t++) kahan_add(a[1 + t], c[1 + t], bsum[t]);
      }
      todo &= ~grp;
    }
    __syncwarp();
  }
  __syncthreads();
  /* combine the warps' bins in FP64 in fixed order, one global update each */
  const size_t wb = bins_warp_bytes(nz, nt);
  for (int i = threadIdx.x; i < nz * (1 + W); i += blockDim.x) {
    const int b = i / (1 + W), k = i - b * (1 + W);
    if (k == 0) {
      unsigned long long n = 0;
      for (int w = 0; w < nwb; w++) n += reinterpret_cast<const unsigned int *>(sbins + (size_t)w * wb)[b];
      if (n) atomicAdd(&p.ncount[b], n);
    } else {
      double sum = 0.0;
      for (int w = 0; w < nwb; w++) {
        const unsigned int *cw = reinterpret_cast<const unsigned int *>(sbins + (size_t)w * wb);
        const float *aw = reinterpret_cast<const float *>(cw + nz);
        sum += (double)aw[(size_t)b * W + k - 1] - (double)aw[(size_t)nz * W + (size_t)b * W + k - 1];
      }
      if (sum != 0.0) fix_add(p.acc + 2 * ((size_t)(k - 1) * nz + b), sum);
    }
  }
}

/* Accumulator value v -> FP64: redshift sums v = b, bias sums of tracer t at
 * v = (1 + t) nz + b.  One rounding from the exact 128-bit sum (the high
 * part holds at most 2^53 in magnitude for any realistic grid). */
__global__ void __launch_bounds__(256) k_bins_finish(const unsigned long long *__restrict__ acc, int nz, int nt,
                                                    double *__restrict__ zsum, double *__restrict__ bsum)
{
  const int nv = nz * (1 + nt);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    unsigned long long lo = acc[2 * (size_t)v], hi = acc[2 * (size_t)v + 1];
    const bool neg = (long long)hi < 0;
    if (neg) { /* two's complement of the 128-bit pair */
      lo = ~lo + 1ull;
      hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    /* value = hi 2^(64 - FIX_FRAC) + lo 2^-FIX_FRAC */
    double d = __dadd_rn(__dmul_rn(__ull2double_rn(hi), FIX_HI), __dmul_rn(__ull2double_rn(lo), FIX_LO));
    if (neg) d = -d;
    if (v < nz) zsum[v] = d;
    else bsum[v - nz] = d;
  }
}

/* 1LPT: x = q + D(r) Psi (wrapped into the box), then the mass assignment of
 * pos_2_dens (density.c:178-187): NGP (S = 0, density.c:37-62), CIC (S = 1,
 * density.c:64-105) or TSC (S = 2, density.c:107-176).  A block takes a tile
 * of CT_X x CT_Y x CT_Z particles (lattice cells) and deposits into a
 * shared-memory box that extends the tile by CT_H cells on every side; the
 * box is added to the grid at the end with one atomic per non-zero cell.
 * Deposits that fall outside the box (particles displaced by more than about
 * CT_H - 1 cells) go straight to the grid.  Masses are fixed point
 * (DEPOSIT_ONE per particle, integer atomics; the grid holds the int32 bits
 * until the density pass turns them into rho - 1), so the result does not
 * depend on the order of the atomic additions. */
constexpr int CT_X = 32, CT_Y = 8, CT_Z = 8, CT_H = 2;
constexpr int CB_X = CT_X + 2 * CT_H, CB_Y = CT_Y + 2 * CT_H, CB_Z = CT_Z + 2 * CT_H;

template <int S>
__global__ void __launch_bounds__(256) k_lpt_deposit(int *grid, const float *__restrict__ dx_,
                                                     const float *__restrict__ dy_, const float *__restrict__ dz_,
                                                     cg_lpt_params p)
{
  constexpr int K = S + 1; /* cells per axis of the stencil */
  __shared__ int box[CB_Z][CB_Y][CB_X];
  const int N = p.box.N;
  const int ntx = (N + CT_X - 1) / CT_X, nty = (N + CT_Y - 1) / CT_Y;
  const int t = blockIdx.x;
  const int tx0 = (t % ntx) * CT_X, ty0 = ((t / ntx) % nty) * CT_Y, tz0 = (t / (ntx * nty)) * CT_Z;
  for (int i = threadIdx.x; i < CB_X * CB_Y * CB_Z; i += blockDim.x) (&box[0][0][0])[i] = 0;
  __syncthreads();
  const float iag = CG_DIV((float)N, p.box.L);
  const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
  const int org[3] = {tx0 - CT_H, ty0 - CT_H, tz0 - CT_H};
  const int ext[3] = {CB_X, CB_Y, CB_Z};
  for (int k = threadIdx.x; k < CT_X * CT_Y * CT_Z; k += blockDim.x) {
    const int ix = tx0 + (k % CT_X), iy = ty0 + (k / CT_X) % CT_Y, iz = tz0 + k / (CT_X * CT_Y);
    if (ix >= N || iy >= N || iz >= N) continue;
    const long long id = pidx(ix, iy, iz, N);
    float xv[3] = {cg_cell_coord(ix, p.box.dx, p.box.p0), cg_cell_coord(iy, p.box.dx, p.box.p1),
                   cg_cell_coord(iz, p.box.dx, p.box.p2)};
    const float r = cg_norm3(xv[0], xv[1], xv[2]);
    const float dg = bg(p.d1, p.g, r);
    const float dsp[3] = {__ldg(&dx_[id]), __ldg(&dy_[id]), __ldg(&dz_[id])};
    /* 2LPT: x = q + D1 Psi1 + D2 Psi2 (density.c:890) */
    const bool two = p.d2x != nullptr;
    const float d2g = two ? bg(p.d2, p.g, r) : 0.0f;
    const float ds2[3] = {two ? __ldg(&p.d2x[id]) : 0.0f, two ? __ldg(&p.d2y[id]) : 0.0f,
                          two ? __ldg(&p.d2z[id]) : 0.0f};
    int ib[3], bb[3]; /* first stencil cell of each axis, in the grid and in the box */
    float w[3][K];
    bool inbox = true;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float q = CG_FMA(dg, dsp[a], xv[a]);
      if (two) q = CG_FMA(d2g, ds2[a], q);
      q = CG_ADD(q, po[a]);
      if (q < 0.0f) q = CG_ADD(q, p.box.L);
      if (q >= p.box.L) q = CG_SUB(q, p.box.L);
      const float u = CG_MUL(q, iag);
      int i0;
      if (S == 0) {
        i0 = (int)CG_ADD(u, 0.5f);
        w[a][0] = 1.0f;
      } else if (S == 1) {
        i0 = (int)u;
        const float a1 = CG_SUB(u, (float)i0);
        w[a][0] = CG_SUB(1.0f, a1);
        w[a][K - 1] = a1;
      } else {
        i0 = (int)floorf(CG_ADD(u, 0.5f));
        const float a0 = CG_SUB(u, (float)i0);
        const float hm = CG_SUB(0.5f, a0), hp = CG_ADD(0.5f, a0);
        w[a][0] = CG_MUL(0.5f, CG_MUL(hm, hm));
        w[a][1] = CG_SUB(0.75f, CG_MUL(a0, a0));
        w[a][K - 1] = CG_MUL(0.5f, CG_MUL(hp, hp));
        i0 -= 1; /* the stencil starts one cell below the nearest */
      }
      /* q is in [0, L) unless the displacement exceeds the box: then a full
       * modulo keeps the cell index inside the grid */
      if ((unsigned)i0 >= (unsigned)N) i0 = ((i0 % N) + N) % N;
      ib[a] = i0;
      /* position of the first stencil cell in the box, the shorter way round */
      int d = i0 - org[a];
      if (d < -N / 2) d += N;
      if (d >= N / 2) d -= N;
      bb[a] = d;
      inbox = inbox && d >= 0 && d + K - 1 < ext[a];
    }
#pragma unroll
    for (int cz = 0; cz < K; cz++)
#pragma unroll
      for (int cy = 0; cy < K; cy++)
#pragma unroll
        for (int cx = 0; cx < K; cx++) {
          /* the weight in units of 2^-20, rounded to nearest (the
           * scaling by a power of two is exact) */
          const int v = __float2int_rn(CG_MUL(CG_MUL(CG_MUL(w[0][cx], w[1][cy]), w[2][cz]), DEPOSIT_ONE));
          if (inbox) {
            atomicAdd(&box[bb[2] + cz][bb[1] + cy][bb[0] + cx], v);
          } else {
            const int gx = ib[0] + cx >= N ? ib[0] + cx - N : ib[0] + cx;
            const int gy = ib[1] + cy >= N ? ib[1] + cy - N : ib[1] + cy;
            const int gz = ib[2] + cz >= N ? ib[2] + cz - N : ib[2] + cz;
            atomicAdd(&grid[pidx(gx, gy, gz, N)], v);
          }
        }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < CB_X * CB_Y * CB_Z; i += blockDim.x) {
    const int v = (&box[0][0][0])[i];
    if (v == 0) continue;
    const int bx = i % CB_X, by = (i / CB_X) % CB_Y, bz = i / (CB_X * CB_Y);
    /* box cells lie within one period of the tile */
    int gx = org[0] + bx, gy = org[1] + by, gz = org[2] + bz;
    gx = gx < 0 ? gx + N : (gx >= N ? gx - N : gx);
    gy = gy < 0 ? gy + N : (gy >= N ? gy - N : gy);
    gz = gz < 0 ? gz + N : (gz >= N ? gz - N : gz);
    atomicAdd(&grid[pidx(gx, gy, gz, N)], v);
  }
}

/* compute_density_normalization after the bin sums (density.c:1272-1355):
 * mean redshift and count / sum(bias) per bin, the first and last bins
 * copied from their neighbours, then the linear spline in z evaluated at
 * z(r_i) with GSL's bracketing (largest bin centre <= z).  One block per
 * tracer; every double operation is an explicitly rounded one, in the order
 * of the host restatement, so the tables do not depend on contraction. */
__global__ void __launch_bounds__(256) k_norm_tables(const unsigned long long *__restrict__ ncount,
                                                     const double *__restrict__ zsum,
                                                     const double *__restrict__ bsum, int nz, double zlast,
                                                     const double *__restrict__ zr, float *out, double *out64)
{
  extern __shared__ double nsh[];
  double *zz = nsh, *y = nsh + nz;
  const int t = blockIdx.x;
  for (int iz = threadIdx.x; iz < nz; iz += blockDim.x) {
    const unsigned long long n = ncount[iz];
    const double b = bsum[(size_t)t * nz + iz];
    zz[iz] = n > 0 ? __ddiv_rn(zsum[iz], __ull2double_rn(n)) : zsum[iz];
    y[iz] = n > 0 ? __ddiv_rn(__ull2double_rn(n), b) : b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    zz[0] = 0;
    zz[nz - 1] = zlast;
    y[0] = y[1];
    y[nz - 1] = y[nz - 2];
  }
  __syncthreads();
  float *o = out + (size_t)t * (CG_NA + 2);
  double *o64 = out64 ? out64 + (size_t)t * (CG_NA + 2) : nullptr;
  for (int i = threadIdx.x; i < CG_NA; i += blockDim.x) {
    const double z = zr[i];
    double nm;
    if (z < zz[0]) {
      nm = y[0];
    } else if (z >= zz[nz - 1]) {
      nm = y[nz - 1];
    } else {
      int lo = 0, hi = nz - 1;
      while (hi > lo + 1) {
        const int mid = (lo + hi) / 2;
        if (zz[mid] > z) hi = mid;
        else lo = mid;
      }
      nm = __dadd_rn(y[lo], __ddiv_rn(__dmul_rn(__dsub_rn(z, zz[lo]), __dsub_rn(y[hi], y[lo])), __dsub_rn(zz[hi], zz[lo])));
    }
    o[i] = (float)nm;
    if (o64) o64[i] = nm;
  }
  if (threadIdx.x == 0) {
    o[CG_NA] = (float)y[0];
    o[CG_NA + 1] = (float)y[nz - 1];
    if (o64) {
      o64[CG_NA] = y[0];
      o64[CG_NA + 1] = y[nz - 1];
    }
  }
}

__global__ void __launch_bounds__(256) k_lpt2_source(const float *__restrict__ xx, const float *__restrict__ xy,
                                                     const float *__restrict__ xz, const float *__restrict__ yy,
                                                     const float *__restrict__ yz, float *zz, int N)
{
  const long long ncell = (long long)N * N * N;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const long long row = c / N;
    const int ix = (int)(c - row * N);
    const long long id = (long long)ix + (long long)(2 * (N / 2 + 1)) * row;
    const float a = xx[id], b = yy[id], d = zz[id], e = xy[id], f = xz[id], g = yz[id];
    float v = CG_ADD(CG_ADD(CG_MUL(a, b), CG_MUL(a, d)), CG_MUL(b, d));
    v = CG_SUB(CG_SUB(CG_SUB(v, CG_MUL(e, e)), CG_MUL(f, f)), CG_MUL(g, g));
    zz[id] = v;
  }
}

} /* namespace */

cudaError_t cg_lpt2_source(cudaStream_t s, const float *xx, const float *xy, const float *xz, const float *yy,
                           const float *yz, float *zz, int N, int nsm)
{
  const long long ncell = (long long)N * N * N;
  long long blocks = (ncell + 255) / 256;
  if (blocks > (long long)nsm * 16) blocks = (long long)nsm * 16;
  k_lpt2_source<<<(unsigned)blocks, 256, 0, s>>>(xx, xy, xz, yy, yz, zz, N);
  return cudaGetLastError();
}

cudaError_t cg_norm_tables(cudaStream_t s, const unsigned long long *ncount, const double *zsum, const double *bsum,
                           int nz, int nt, double zlast, const double *zr, float *out, double *out64)
{
  if (nz < 2 || nz > CG_NORM_NZ_MAX || nt < 1) return cudaErrorInvalidValue;
  const size_t smem = 2 * sizeof(double) * (size_t)nz;
  if (smem > 48 * 1024) {
    static bool set[CG_MAX_DEVICES]; /* opt-in above 48 KiB, once per device */
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= CG_MAX_DEVICES) return cudaErrorInvalidDevice;
    if (!set[dev]) {
      cudaError_t e = cudaFuncSetAttribute(k_norm_tables, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           2 * (int)sizeof(double) * CG_NORM_NZ_MAX);
      if (e != cudaSuccess) return e;
      set[dev] = true;
    }
  }
  k_norm_tables<<<nt, 256, smem, s>>>(ncount, zsum, bsum, nz, zlast, zr, out, out64);
  return cudaGetLastError();
}

cudaError_t cg_moments_final(cudaStream_t s, const double2 *part, size_t n, double inv_ncell, double *stats,
                             float *s2f)
{
  k_moments_final<<<1, 1024, 0, s>>>(part, n, inv_ncell, stats, s2f);
  return cudaGetLastError();
}

cudaError_t cg_dens_bins(cudaStream_t s, float *grid, const cg_bins_params *p, int nsm)
{
  if (p->nt < 0 || p->nt > MAXT || p->nz < 0) return cudaErrorInvalidValue;
  /* as many warps per block (up to 8) as the bins of each fit in 200 KiB */
  const size_t wb = bins_warp_bytes(p->nz, p->nt);
  int nwb = BINS_WARPS;
  while (nwb > 1 && (size_t)nwb * wb > 200u * 1024u) nwb--;
  if ((size_t)nwb * wb > 200u * 1024u) return cudaErrorInvalidValue;
  const size_t smem = (size_t)nwb * wb;
  if (smem > 48u * 1024u) {
    static bool set[CG_MAX_DEVICES]; /* raised once per device to the largest size a launch asks for */
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= CG_MAX_DEVICES) return cudaErrorInvalidDevice;
    if (!set[dev]) {
      cudaError_t e = cudaSuccess;
#define X(k) \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dens_bins<k>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8)
#undef X
      if (e != cudaSuccess) return e;
      set[dev] = true;
    }
  }
  long long nrow = (long long)p->box.N * p->box.N;
  long long blocks = (nrow + nwb - 1) / nwb;
  long long cap = (long long)nsm * 8;
  if (blocks > cap) blocks = cap;
  switch (p->nt) { /* one instantiation per tracer count: loops of exact length */
#define X(k)                                                           \
  case k:                                                              \
    k_dens_bins<k><<<(unsigned)blocks, nwb * 32, smem, s>>>(grid, *p); \
    break;
    X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8)
#undef X
  }
  if (p->nz > 0) {
    const int nv = p->nz * (1 + p->nt);
    k_bins_finish<<<(nv + 255) / 256, 256, 0, s>>>(p->acc, p->nz, p->nt, p->zsum, p->bsum);
  }
  return cudaGetLastError();
}

int cg_dens_bins_max_tracers(void) { return MAXT; }

/* Scratch of the allocation-free bins entry: u64 counts [CG_BINS_STATIC_NZ],
 * redshift sums [CG_BINS_STATIC_NZ], bias sums [MAXT][nz] (doubles), then
 * the 128-bit accumulators [1 + MAXT][nz][2] (u64).  A module-scope array
 * costs no allocation call at run time: it exists in every context that
 * loads this module. */
static_assert(CG_BINS_STATIC_BYTES == (size_t)CG_BINS_STATIC_NZ * ((2 + MAXT) + 2 * (1 + MAXT)) * 8,
              "static bins scratch layout");
static __device__ __align__(256) unsigned char g_bins_scratch[CG_BINS_STATIC_BYTES];

cudaError_t cg_dens_bins_static_scratch(void **ptr, size_t *bytes)
{
  *bytes = sizeof(g_bins_scratch);
  return cudaGetSymbolAddress(ptr, g_bins_scratch);
}

cudaError_t cg_lpt_cic(cudaStream_t s, float *grid, const float *dx, const float *dy, const float *dz,
                       const cg_lpt_params *p, int nsm)
{
  (void)nsm;
  const long long N = p->box.N;
  const long long tiles = ((N + CT_X - 1) / CT_X) * ((N + CT_Y - 1) / CT_Y) * ((N + CT_Z - 1) / CT_Z);
  /* the grid (zeroed by the caller) holds int32 fixed-point masses until
   * the density pass of mode CG_DMODE_RHO */
  int *mass = reinterpret_cast<int *>(grid);
  if (p->interp == 0) k_lpt_deposit<0><<<(unsigned)tiles, 256, 0, s>>>(mass, dx, dy, dz, *p);
  else if (p->interp == 2) k_lpt_deposit<2><<<(unsigned)tiles, 256, 0, s>>>(mass, dx, dy, dz, *p);
  else k_lpt_deposit<1><<<(unsigned)tiles, 256, 0, s>>>(mass, dx, dy, dz, *p);
  return cudaGetLastError();
}
