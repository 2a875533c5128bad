/*
 * srcs.cu -- biased Poisson sources (srcs.c:120-283), their local
 * properties (srcs.c:386-416), the source count map, and the line-of-sight
 * redshift-space distortion at each source (srcs.c:425-504, 634-662).
 *
 * Sampling is count -> scan -> emit:
 *   k_pois_count : one block per 2048 consecutive cells; per cell lambda and
 *                  a Poisson deviate keyed by (seed, population, cell), so the
 *                  result does not depend on the launch shape; counts are kept
 *                  as uint16 and the block totals written out.  A cell with
 *                  CG_COUNT_ESC or more sources stores the escape value and
 *                  appends (cell, count) to a short overflow list.
 *   k_scan_*     : exclusive scan of the block totals (three coalesced passes).
 *   k_emit       : re-reads the counts, scans them inside the block and writes
 *                  every source at its final catalog index, in cell order (the
 *                  order of the reference run with one thread); the block's
 *                  sources are spread evenly over its threads, each finding
 *                  its cell by binary search on the scanned offsets.  Positions,
 *                  the NGP velocity (get_rvel, srcs.c:87-118), ra/dec/z, the
 *                  base-pixel id and the count-map increment are fused.
 *
 * Along the line of sight to each source (one thread per source):
 *   k_beam_rsd    : trilinear RSD at the source.
 *   k_src_lensing : shear, convergence and deflection from the nearest-cell
 *                   tidal tensor and potential gradient at N/2 radial steps.
 *   k_src_skewers : trilinear density (or Gaussian field) and radial velocity
 *                   at every step up to the source.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "srcs_api.h"

namespace {
using namespace cg;

constexpr int CPT = 8;                 /* cells per thread */
constexpr int SB = 256;                /* threads per block */
constexpr int CPB = CPT * SB;          /* cells per block   */

__device__ __forceinline__ void cell_of(long long c, const Box &b, int &ix, int &iy, int &iz)
{
  const long long q = divN(c, b), z = divN(q, b);
  ix = (int)(c - q * b.N);
  iy = (int)(q - z * b.N);
  iz = (int)z;
}

/* True count of a cell whose stored count is the escape value. */
__device__ __forceinline__ int ovf_lookup(const cg_srcs_params &p, long long cid)
{
  int n = *p.ovf_n;
  if (n > CG_OVF_CAP) n = CG_OVF_CAP;
  for (int k = 0; k < n; k++)
    if (p.ovf_cell[k] == cid) return p.ovf_cnt[k];
  return CG_COUNT_ESC;
}

/* The count of a cell that the float margins leave open: the reference's
 * double arithmetic (out of line: rare, and long). */
__device__ __noinline__ int count_double(const cg_srcs_params &p, int ix, int iy, int iz, float d, long long cid,
                                         uint32_t w)
{
  const double lam = cgx_lambda(&p.pa.x, ix, iy, iz, d);
  if (lam > 1073741824.0) {
    atomicOr(p.err, ERR_COUNT_OVERFLOW);
    return 0;
  }
  return cgx_poisson(lam, (double)cg_u01f(w), cid, p.kp0, p.kp1);
}

/* PTRS in single precision (lambda >= 10: the cells next to the observer,
 * or dense coarse grids), out of line like the double path. */
__device__ __noinline__ int ptrs_float(float lam, float elam, long long cid, uint32_t k0, uint32_t k1)
{
  return cg_poisson_ptrs_checked(lam, elam, cid, k0, k1);
}

/* Counts of CPT consecutive cells of one row per thread.  Each cell's lambda
 * is formed in single precision with a bound on its distance to the
 * reference's double lambda, and the Poisson inversion keeps its float
 * count when the uniform lies farther from the bracketing cumulative values
 * than that bound carries them (cg_exact.h); the other cells -- and every
 * cell with lambda >= 10, for PTRS -- take the double arithmetic.  Cells
 * 4m..4m+3 share one Philox block, drawn only when one of them has a
 * positive lambda.  The cell loop is not unrolled (unrolled, the kernel ran
 * instruction-fetch bound); the counts are packed in two 64-bit registers.
 * Each warp adds its total to the block's entry (zeroed before the launch),
 * so warps that finish early do not wait for the block's slowest.  Six
 * blocks per SM (40 registers): the table lookups' latency wants the warps
 * more than the few spills cost (13.1 -> 12.0 ms at 1024^3 against four). */
__global__ void __launch_bounds__(SB, 6) k_pois_count(const float *__restrict__ grid, cg_srcs_params p)
{
  const int N = p.box.N;
  const long long ncell = (long long)N * N * N;
  const long long c0 = (long long)blockIdx.x * CPB + (long long)threadIdx.x * CPT;
  long long tot = 0;
  unsigned int nfb = 0;
  if (c0 < ncell) {
    int ix, iy, iz;
    cell_of(c0, p.box, ix, iy, iz);
    const float *row = grid + pidx(ix, iy, iz, N);
    unsigned long long lo = 0, hi = 0;
    long long wm = -1; /* the Philox block held in w */
    cg_u32x4 w;
    w.v[0] = w.v[1] = w.v[2] = w.v[3] = 0u;
#pragma unroll 1
    for (int h = 0; h < CPT; h++) {
      const long long cid = c0 + h;
      const float d = __ldg(row + h);
      float lam, elam;
      int st = cg_lambda_checked(&p.pa, ix + h, iy, iz, d, &lam, &elam);
      if (p.force_double && (st == 1 || st == 3)) st = 2;
      int n = 0;
      if (st != 0) {
        if ((cid >> 2) != wm) {
          wm = cid >> 2;
          w = cg_philox4x32_10((uint32_t)wm, (uint32_t)((unsigned long long)wm >> 32), 0u, 0u, p.kp0, p.kp1);
        }
        const int q = (int)(cid & 3);
        const uint32_t wq = q == 0 ? w.v[0] : (q == 1 ? w.v[1] : (q == 2 ? w.v[2] : w.v[3]));
        n = st == 1 ? cg_poisson_inv_checked(lam, elam, cg_u01f(wq))
                    : (st == 3 ? ptrs_float(lam, elam, cid, p.kp0, p.kp1) : -1);
        if (n < 0) {
          n = count_double(p, ix + h, iy, iz, d, cid, wq);
          nfb++;
        }
      }
      unsigned long long v = (unsigned long long)n;
      if (n >= CG_COUNT_ESC) {
        const int k = atomicAdd(p.ovf_n, 1);
        if (k < CG_OVF_CAP) {
          p.ovf_cell[k] = cid;
          p.ovf_cnt[k] = n;
        } else {
          atomicOr(p.err, ERR_COUNT_OVERFLOW);
        }
        v = CG_COUNT_ESC;
      }
      if (h < 4) lo |= v << (16 * h);
      else hi |= v << (16 * (h - 4));
      tot += n;
    }
    *reinterpret_cast<uint4 *>(p.counts + c0) =
        make_uint4((unsigned)lo, (unsigned)(lo >> 32), (unsigned)hi, (unsigned)(hi >> 32));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    tot += __shfl_xor_sync(0xffffffffu, tot, o);
    nfb += __shfl_xor_sync(0xffffffffu, nfb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (tot) atomicAdd(reinterpret_cast<unsigned long long *>(&p.block_sums[blockIdx.x]), (unsigned long long)tot);
    if (nfb) atomicAdd(p.xstats, (unsigned long long)nfb);
  }
}

/* Exclusive scan of the n block totals in place, their sum into *total, in
 * three coalesced passes over tiles of SCAN_T values (a thread holds two
 * neighbours): each tile reduced to its sum (tsum), the tile sums scanned by
 * one block, then every tile scanned from its offset.  (One block walking
 * the whole array took 0.87 ms at 1024^3.) */
constexpr int SCAN_T = 2048;

/* Exclusive scan of x over the block's 1024 threads; *tot = the block sum. */
__device__ __forceinline__ long long block_scan(long long x, long long *ws, long long *tot)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (w == 0) {
    long long y = ws[lane], yi = y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, yi, o);
      if (lane >= o) yi += t;
    }
    ws[lane] = yi - y;
    if (lane == 31) ws[32] = yi;
  }
  __syncthreads();
  const long long ex = ws[w] + inc - x;
  *tot = ws[32];
  __syncthreads(); /* ws is reused by the next call */
  return ex;
}

__global__ void __launch_bounds__(1024) k_scan_tiles(const long long *__restrict__ v, long long n, long long *tsum,
                                                     unsigned int *err)
{
  __shared__ long long ws[33];
  const long long i = (long long)blockIdx.x * SCAN_T + 2 * (long long)threadIdx.x;
  const long long a = i < n ? v[i] : 0, b = i + 1 < n ? v[i + 1] : 0;
  if (a > 0x7fffffffLL || b > 0x7fffffffLL) atomicOr(err, ERR_COUNT_OVERFLOW); /* k_emit scans a block in int */
  long long tot;
  block_scan(a + b, ws, &tot);
  if (threadIdx.x == 0) tsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_top(long long *tsum, long long nt, long long *total)
{
  __shared__ long long ws[33];
  long long carry = 0;
  for (long long c0 = 0; c0 < nt; c0 += 1024) {
    const long long i = c0 + threadIdx.x;
    const long long x = i < nt ? tsum[i] : 0;
    long long tot;
    const long long ex = block_scan(x, ws, &tot);
    if (i < nt) tsum[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(1024) k_scan_apply(long long *v, long long n, const long long *__restrict__ tsum)
{
  __shared__ long long ws[33];
  const long long i = (long long)blockIdx.x * SCAN_T + 2 * (long long)threadIdx.x;
  const long long a = i < n ? v[i] : 0, b = i + 1 < n ? v[i + 1] : 0;
  long long tot;
  const long long off = tsum[blockIdx.x] + block_scan(a + b, ws, &tot);
  if (i < n) v[i] = off;
  if (i + 1 < n) v[i + 1] = off + a;
}

/* Centred potential differences at a cell (get_rvel / get_element VEL). */
__device__ __forceinline__ void grad_phi(const float *__restrict__ phi, int ix, int iy, int iz, int N, float v[3])
{
  int xh = wrap(ix + 1, N), xl = wrap(ix - 1, N);
  int yh = wrap(iy + 1, N), yl = wrap(iy - 1, N);
  int zh = wrap(iz + 1, N), zl = wrap(iz - 1, N);
  v[0] = CG_SUB(__ldg(&phi[pidx(xh, iy, iz, N)]), __ldg(&phi[pidx(xl, iy, iz, N)]));
  v[1] = CG_SUB(__ldg(&phi[pidx(ix, yh, iz, N)]), __ldg(&phi[pidx(ix, yl, iz, N)]));
  v[2] = CG_SUB(__ldg(&phi[pidx(ix, iy, zh, N)]), __ldg(&phi[pidx(ix, iy, zl, N)]));
}

/* Base and count-map pixels of a source by the reference's double
 * arithmetic (vec2pix_ring, srcs.c:268; he_ang2pix of cart2sph); returns the
 * number of pixels decided here.  Out of line: rare. */
__device__ __noinline__ unsigned int pixels_double(const cg_srcs_params &p, float px, float py, float pz, long long *pr,
                                                   long long *pc)
{
  unsigned int k = 0;
  if (*pr < 0) {
    *pr = cgx_vec2pix_ring(p.nside_base, (double)px, (double)py, (double)pz);
    k++;
  }
  if (p.cmap && *pc < 0) {
    double r, cth, ph;
    cgx_cart2sph((double)px, (double)py, (double)pz, &r, &cth, &ph);
    *pc = cgx_ang2pix(p.nside_count, cth, ph);
    k++;
  }
  return k;
}

__global__ void __launch_bounds__(SB, 8) k_emit(const float *__restrict__ phi, cg_srcs_params p)
{
  __shared__ int coff[CPB + 1]; /* exclusive source offset of each cell in the block */
  __shared__ int ws[SB / 32];
  const int N = p.box.N;
  const long long ncell = (long long)N * N * N;
  const long long cb = (long long)blockIdx.x * CPB;
  const long long c0 = cb + (long long)threadIdx.x * CPT;
  int n[CPT];
  int tot = 0;
#pragma unroll
  for (int h = 0; h < CPT; h++) n[h] = 0;
  if (c0 < ncell) {
    const uint4 pk = *reinterpret_cast<const uint4 *>(p.counts + c0);
    const unsigned w4[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
    for (int h = 0; h < CPT; h++) {
      int v = (int)((w4[h >> 1] >> (16 * (h & 1))) & 0xffffu);
      if (v == CG_COUNT_ESC) v = ovf_lookup(p, c0 + h);
      n[h] = v;
      tot += v;
    }
  }
  /* block exclusive scan of per-thread totals */
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  int woff = 0;
  for (int w = 0; w < wid; w++) woff += ws[w];
  int run = woff + inc - tot;
#pragma unroll
  for (int h = 0; h < CPT; h++) {
    coff[threadIdx.x * CPT + h] = run;
    run += n[h];
  }
  if (threadIdx.x == SB - 1) coff[CPB] = run;
  __syncthreads();
  /* the block's sources, spread evenly over its threads: consecutive threads
   * write consecutive catalogue entries */
  const int T = coff[CPB];
  const long long base = p.block_sums[blockIdx.x];
  const float dx = p.box.dx;
  unsigned int nfb = 0; /* pixels decided in double */
  for (int k = threadIdx.x; k < T; k += SB) {
    /* the cell holding source k: the last cell whose offset is <= k (cells
     * without sources share their successor's offset) */
    int lo = 0, hi = CPB - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (coff[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    const int j = k - coff[lo];
    const long long cid = cb + lo;
    const long long id = base + k;
    if (id >= p.capacity) {
      atomicOr(p.err, ERR_CATALOG_OVERFLOW);
      break;
    }
    int ix, iy, iz;
    cell_of(cid, p.box, ix, iy, iz);
    const float x0 = cg_cell_coord(ix, dx, p.box.p0);
    const float y0 = cg_cell_coord(iy, dx, p.box.p1), z0 = cg_cell_coord(iz, dx, p.box.p2);
    const float rr = cg_norm3(x0, y0, z0);
    float v[3];
    grad_phi(phi, ix, iy, iz, N, v);
    const float rvel = CG_MUL(p.factor_vel, cg_rvel(v[0], v[1], v[2], x0, y0, z0, rr, p.box.idx));
    const float dz_rsd = CG_MUL(rvel, bg(p.v1, p.g, rr));
    cg_u32x4 u = cg_philox4x32_10((uint32_t)cid, (uint32_t)(cid >> 32), (uint32_t)j, 0u, p.kq0, p.kq1);
    /* the position of the double arithmetic, stored as float (srcs.c:261-263):
     * in single precision where its rounding is certain, else in double */
    float px, py, pz;
    if (p.force_double || !cg_src_offset_checked(p.pa.xc[ix], p.cl[0][ix], p.dxh, p.dxl, u.v[0], &px))
      px = cgx_src_offset(cgx_coord(ix, p.dx64, p.p64[0]), p.dx64, u.v[0]);
    if (p.force_double || !cg_src_offset_checked(p.pa.yc[iy], p.cl[1][iy], p.dxh, p.dxl, u.v[1], &py))
      py = cgx_src_offset(cgx_coord(iy, p.dx64, p.p64[1]), p.dx64, u.v[1]);
    if (p.force_double || !cg_src_offset_checked(p.pa.zc[iz], p.cl[2][iz], p.dxh, p.dxl, u.v[2], &pz))
      pz = cgx_src_offset(cgx_coord(iz, p.dx64, p.p64[2]), p.dx64, u.v[2]);
    p.pos[id] = make_float4(px, py, pz, dz_rsd);
    float r, cth, ph;
    cg_cart2sph(px, py, pz, &r, &cth, &ph);
    /* the base pixel and the count-map pixel: the reference's double
     * decisions, in single precision where the margins allow */
    long long pr = -1, pc = -1;
    if (!p.force_double) {
      const cg_dir dr = cg_dir_of(px, py, pz, 0.0f);
      pr = cg_pix_checked(&dr, (int)p.nside_base, 0.0f);
      if (p.cmap) pc = cg_pix_checked(&dr, (int)p.nside_count, 0.0f);
    }
    if (pr < 0 || (p.cmap && pc < 0)) {
      nfb += pixels_double(p, px, py, pz, &pr, &pc);
    }
    /* ring2nest costs several 64-bit divisions; nside_base is small, so its
     * table (built on the host with the same function) replaces them */
    p.ipix[id] = p.base_r2n ? __ldg(p.base_r2n + pr) : (int)cg_ring2nest(p.nside_base, pr);
    float *q = p.src + (size_t)id * 9;
    cg_radec(px, py, pz, ph, &q[0], &q[1]);                       /* ra, dec */
    q[2] = bg(p.zt, p.g, r);                                      /* z0  */
    q[3] = p.need_beaming ? 0.0f : dz_rsd;                        /* dz_rsd */
    q[4] = p.need_beaming ? 0.0f : -1.0f;                         /* e1  */
    q[5] = p.need_beaming ? 0.0f : -1.0f;                         /* e2  */
    q[6] = 0.0f;
    q[7] = 0.0f;
    q[8] = 0.0f;
    if (p.cmap) atomicAdd(&p.cmap[pc], 1);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nfb += __shfl_xor_sync(0xffffffffu, nfb, o);
  if ((threadIdx.x & 31) == 0 && nfb) atomicAdd(p.xstats + 1, (unsigned long long)nfb);
}

/* Trilinear potential gradient at a point with corner cells i0/i1 and
 * weights h0/h1 (interpolate_from_grid RETURN_VEL, beaming.c:183-265): per z
 * plane the four corners' central differences weighted and summed with FMAs,
 * then the two planes added. */
__device__ __forceinline__ void cic_grad(const float *__restrict__ phi, const int i0[3], const int i1[3],
                                         const float h0[3], const float h1[3], int N, float v[3])
{
  v[0] = v[1] = v[2] = 0.0f;
#pragma unroll
  for (int hz = 0; hz < 2; hz++) {
    const int zc = hz ? i1[2] : i0[2];
    const float wz = hz ? h0[2] : h1[2];
    float acc[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int yc = (k & 2) ? i1[1] : i0[1], xc = (k & 1) ? i1[0] : i0[0];
      const float w = CG_MUL(CG_MUL(wz, (k & 2) ? h0[1] : h1[1]), (k & 1) ? h0[0] : h1[0]);
      float g[3];
      grad_phi(phi, xc, yc, zc, N, g);
#pragma unroll
      for (int a = 0; a < 3; a++) acc[a] = CG_FMA(g[a], w, acc[a]);
    }
#pragma unroll
    for (int a = 0; a < 3; a++) v[a] = CG_ADD(v[a], acc[a]);
  }
}

/* radial projection 0.5 idx (v . u), srcs.c:503 */
__device__ __forceinline__ float los_vel(const float v[3], const float u[3], float idx)
{
  return CG_MUL(CG_MUL(0.5f, idx), CG_ADD(CG_ADD(CG_MUL(v[0], u[0]), CG_MUL(v[1], u[1])), CG_MUL(v[2], u[2])));
}

/* Line-of-sight RSD at each source: trilinear gradient of the potential
 * (interpolate_from_grid CIC branch, beaming.c:183-265) projected on the
 * line of sight (srcs.c:500-504), then scaled by V1(r(z0)) * factor_vel
 * (srcs.c:657-662). */
__device__ __forceinline__ long long src_count(long long n, const long long *n_dev)
{
  if (n_dev) {
    const long long d = *n_dev;
    if (d < n) n = d;
  }
  return n;
}

__global__ void __launch_bounds__(256) k_beam_rsd(const float *__restrict__ phi, cg_srcs_params p, long long nsrc,
                                                  const long long *nsrc_dev)
{
  const int N = p.box.N;
  nsrc = src_count(nsrc, nsrc_dev);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nsrc;
       i += (long long)gridDim.x * blockDim.x) {
    float4 q = p.pos[i];
    float pos[3] = {q.x, q.y, q.z};
    const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
    float r = cg_norm3(pos[0], pos[1], pos[2]);
    float ir = CG_DIV(1.0f, r > 0.001f ? r : 0.001f);
    float u[3];
    int i0[3], i1[3];
    float h0[3], h1[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float xn = CG_MUL(CG_ADD(pos[a], po[a]), p.box.idx);
      u[a] = CG_MUL(pos[a], ir);
      i0[a] = (int)xn;
      h0[a] = CG_SUB(xn, (float)i0[a]);
      h1[a] = CG_SUB(1.0f, h0[a]);
      i1[a] = wrap(i0[a] + 1, N);
      i0[a] = wrap(i0[a], N);
    }
    float v[3];
    cic_grad(phi, i0, i1, h0, h1, N, v);
    const float vr = los_vel(v, u, p.box.idx);
    float *s = p.src + (size_t)i * 9;
    float z0 = s[2];
    float rz = r_of_z(p.a_a2r, p.r_a2r, p.na, z0);
    s[3] = CG_MUL(vr, CG_MUL(bg(p.v1, p.g, rz), p.factor_vel));
  }
}

/* Direction, distance and last radial step of a source (srcs.c:485-493,
 * 583): r = |pos|, u = pos / max(r, 0.001), i_r_max = min((int)(r/dr + 0.5), nr - 1). */
__device__ __forceinline__ int los_setup(float4 q, const cg_los_params &p, float *r, float u[3])
{
  *r = cg_norm3(q.x, q.y, q.z);
  const float ir = CG_DIV(1.0f, *r > 0.001f ? *r : 0.001f);
  u[0] = CG_MUL(q.x, ir);
  u[1] = CG_MUL(q.y, ir);
  u[2] = CG_MUL(q.z, ir);
  const int k = (int)CG_ADD(CG_MUL(*r, p.idr), 0.5f);
  return k < p.nr - 1 ? k : p.nr - 1;
}

/* Lensing at each source (srcs.c:536-625 without _USE_FAST_LENSING): at
 * each step up to the source the nearest cell's tidal tensor and potential
 * gradient, projected with the source's rotation, weighted by
 * rm pg dr (r - rm) (shear, convergence) and 2 pg dr (r - rm) (deflection),
 * summed with Kahan compensation; the deflections are turned to degrees
 * (srcs.c:721-722). */
__global__ void __launch_bounds__(256) k_src_lensing(const float *__restrict__ phi, cg_los_params p)
{
  extern __shared__ float lsh[];
  for (int i = threadIdx.x; i < 2 * p.nr; i += blockDim.x) lsh[i] = p.lfac[i];
  __syncthreads();
  const float *f0 = lsh, *f1 = lsh + p.nr;
  const int N = p.box.N;
  const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
  const float idx = p.box.idx;
  const long long nsrc = src_count(p.nsrc, p.nsrc_dev);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nsrc;
       i += (long long)gridDim.x * blockDim.x) {
    float r, u[3];
    const int kmax = los_setup(p.pos[i], p, &r, u);
    const float ir = CG_DIV(1.0f, r > 0.001f ? r : 0.001f);
    float ux[3], uy[3], rk[6], re1[6], re2[6];
    cg_lens_rot(u, CG_MUL(CG_MUL(idx, idx), ir), CG_MUL(CG_MUL(0.5f, idx), ir), ux, uy, rk, re1, re2);
    float a[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, c[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k <= kmax; k++) {
      const float rm = CG_MUL(CG_ADD((float)k, 0.5f), p.dr);
      const int x0 = cg_ngp_cell(rm, u[0], po[0], idx, N);
      const int y0 = cg_ngp_cell(rm, u[1], po[1], idx, N);
      const int z0 = cg_ngp_cell(rm, u[2], po[2], idx, N);
      float f[19], t[6];
      stencil19(phi, x0, y0, z0, N, f);
      cg_tidal(f, t);
      const float v[3] = {CG_SUB(f[1], f[2]), CG_SUB(f[3], f[4]), CG_SUB(f[5], f[6])};
      const float dd = CG_SUB(r, rm);
      const float fr = CG_MUL(f1[k], dd), frm = CG_MUL(f0[k], dd);
      cg_kahan_add(&a[0], &c[0], CG_MUL(cg_dot6(re1, t), fr));
      cg_kahan_add(&a[1], &c[1], CG_MUL(cg_dot6(re2, t), fr));
      cg_kahan_add(&a[2], &c[2], CG_MUL(cg_dot6(rk, t), fr));
      cg_kahan_add(&a[3], &c[3], CG_MUL(cg_dot3(ux, v), frm));
      cg_kahan_add(&a[4], &c[4], CG_MUL(cg_dot3(uy, v), frm));
    }
    float *s = p.src + (size_t)i * 9;
    s[4] = a[0];
    s[5] = a[1];
    s[6] = a[2];
    s[7] = CG_MUL(a[4], 57.2957795f); /* dra  = RTOD * dty */
    s[8] = CG_MUL(a[3], 57.2957795f); /* ddec = RTOD * dtx */
  }
}

/* Skewers (srcs.c:509-536, 725-733): at each step up to the source the
 * trilinear density, or the Gaussian field of the eight corner cells, and
 * the trilinear radial velocity times V1(rm) factor_vel; 0 beyond. */
__global__ void __launch_bounds__(256) k_src_skewers(const float *__restrict__ dens, const float *__restrict__ phi,
                                                      cg_los_params p)
{
  extern __shared__ float ssh[];
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) ssh[i] = p.vfac[i];
  __syncthreads();
  const int N = p.box.N;
  const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
  const float idx = p.box.idx;
  const float s2 = p.skw_gauss ? *p.sigma2 : 0.0f;
  const long long nsrc = src_count(p.nsrc, p.nsrc_dev);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nsrc;
       i += (long long)gridDim.x * blockDim.x) {
    float r, u[3];
    const int kmax = los_setup(p.pos[i], p, &r, u);
    float *sd = p.skw_d + (size_t)i * p.nr, *sv = p.skw_v + (size_t)i * p.nr;
    for (int k = 0; k <= kmax; k++) {
      const float rm = CG_MUL(CG_ADD((float)k, 0.5f), p.dr);
      int i0[3], i1[3];
      float h0[3], h1[3];
#pragma unroll
      for (int a = 0; a < 3; a++) cg_cic_axis(rm, u[a], po[a], idx, N, &i0[a], &i1[a], &h0[a], &h1[a]);
      float d;
      if (p.skw_gauss) {
        float gv[8];
#pragma unroll
        for (int b = 0; b < 8; b++) {
          const int ix = (b & 1) ? i1[0] : i0[0], iy = (b & 2) ? i1[1] : i0[1], iz = (b & 4) ? i1[2] : i0[2];
          const float rc = cg_norm3(cg_cell_coord(ix, p.box.dx, p.box.p0), cg_cell_coord(iy, p.box.dx, p.box.p1),
                                    cg_cell_coord(iz, p.box.dx, p.box.p2));
          gv[b] = cg_gauss_of_dens(__ldg(&dens[pidx(ix, iy, iz, N)]), bg(p.d1, p.g, rc), s2);
        }
        d = cg_cic_combine(gv, h0, h1);
      } else {
        d = cg_cic_value(dens, i0, i1, h0, h1, N);
      }
      float v[3];
      cic_grad(phi, i0, i1, h0, h1, N, v);
      sd[k] = d;
      sv[k] = CG_MUL(los_vel(v, u, idx), ssh[k]);
    }
    for (int k = kmax + 1; k < p.nr; k++) {
      sd[k] = 0.0f;
      sv[k] = 0.0f;
    }
  }
}

} /* namespace */

long long cg_srcs_nblocks(int N) { return ((long long)N * N * N + CPB - 1) / CPB; }
long long cg_srcs_scan_room(long long nb) { return (nb + SCAN_T - 1) / SCAN_T; }

cudaError_t cg_srcs_count(cudaStream_t s, const float *grid, const cg_srcs_params *p, long long *total)
{
  long long nb = cg_srcs_nblocks(p->box.N);
  cudaError_t e = cudaMemsetAsync(p->ovf_n, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(p->block_sums, 0, nb * sizeof(long long), s);
  if (e != cudaSuccess) return e;
  k_pois_count<<<(unsigned)nb, SB, 0, s>>>(grid, *p);
  const long long nt = cg_srcs_scan_room(nb);
  long long *tsum = p->block_sums + nb; /* the tile sums, just past the block totals */
  k_scan_tiles<<<(unsigned)nt, 1024, 0, s>>>(p->block_sums, nb, tsum, p->err);
  k_scan_top<<<1, 1024, 0, s>>>(tsum, nt, total);
  k_scan_apply<<<(unsigned)nt, 1024, 0, s>>>(p->block_sums, nb, tsum);
  return cudaGetLastError();
}

cudaError_t cg_srcs_emit(cudaStream_t s, const float *phi, const cg_srcs_params *p)
{
  long long nb = cg_srcs_nblocks(p->box.N);
  k_emit<<<(unsigned)nb, SB, 0, s>>>(phi, *p);
  return cudaGetLastError();
}

cudaError_t cg_srcs_lensing(cudaStream_t s, const float *phi, const cg_los_params *p, int nsm)
{
  if (p->nsrc <= 0) return cudaSuccess;
  long long blocks = (p->nsrc + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  k_src_lensing<<<(unsigned)blocks, 256, 2 * p->nr * sizeof(float), s>>>(phi, *p);
  return cudaGetLastError();
}

cudaError_t cg_srcs_skewers(cudaStream_t s, const float *dens, const float *phi, const cg_los_params *p, int nsm)
{
  if (p->nsrc <= 0) return cudaSuccess;
  long long blocks = (p->nsrc + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  k_src_skewers<<<(unsigned)blocks, 256, p->nr * sizeof(float), s>>>(dens, phi, *p);
  return cudaGetLastError();
}

cudaError_t cg_srcs_beam_rsd(cudaStream_t s, const float *phi, const cg_srcs_params *p, long long nsrc,
                             const long long *nsrc_dev, int nsm)
{
  if (nsrc <= 0) return cudaSuccess;
  long long blocks = (nsrc + 255) / 256;
  if (blocks > (long long)nsm * 16) blocks = (long long)nsm * 16;
  k_beam_rsd<<<(unsigned)blocks, 256, 0, s>>>(phi, *p, nsrc, nsrc_dev);
  return cudaGetLastError();
}
