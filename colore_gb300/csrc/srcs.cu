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
 *   k_scan       : exclusive scan of the block totals (one block).
 *   k_emit       : re-reads the counts, scans them inside the block and writes
 *                  every source at its final catalog index, in cell order (the
 *                  order of the reference run with one thread); the block's
 *                  sources are spread evenly over its threads, each finding
 *                  its cell by binary search on the scanned offsets.  Positions,
 *                  the NGP velocity (get_rvel, srcs.c:87-118), ra/dec/z, the
 *                  base-pixel id and the count-map increment are fused.
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

__device__ __forceinline__ float pois_lambda(const cg_srcs_params &p, float d, float r)
{
  if (!(r < p.rlim)) return 0.0f;
  const BgAt at = bg_at(p.g, r);
  float nd = bgv(p.nz, at);
  if (!(nd > 0.0f)) return 0.0f;
  float b = bgv(p.bz, at);
  float dn = bgv(p.norm, at);
  return cg_src_lambda(nd, p.cell_vol, d, b, dn, p.bias_model);
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

__global__ void __launch_bounds__(SB) k_pois_count(const float *__restrict__ grid, cg_srcs_params p)
{
  const int N = p.box.N;
  const long long ncell = (long long)N * N * N;
  const long long c0 = (long long)blockIdx.x * CPB + (long long)threadIdx.x * CPT;
  long long tot = 0;
  if (c0 < ncell) {
    int ix, iy, iz;
    cell_of(c0, p.box, ix, iy, iz);
    const float *row = grid + pidx(ix, iy, iz, N);
    const float y0 = cg_cell_coord(iy, p.box.dx, p.box.p1), z0 = cg_cell_coord(iz, p.box.dx, p.box.p2);
    unsigned short cnt[CPT];
#pragma unroll
    for (int h = 0; h < CPT; h += 2) {
      float2 dv = *reinterpret_cast<const float2 *>(row + h);
      float dd[2] = {dv.x, dv.y};
#pragma unroll
      for (int e = 0; e < 2; e++) {
        float x0 = cg_cell_coord(ix + h + e, p.box.dx, p.box.p0);
        float r = cg_norm3(x0, y0, z0);
        float lam = pois_lambda(p, dd[e], r);
        int n = 0;
        const long long cid = c0 + h + e;
        if (lam > 1073741824.0f) {
          atomicOr(p.err, ERR_COUNT_OVERFLOW);
        } else if (lam > 0.0f) {
          n = cg_poisson(lam, p.kp0, p.kp1, (uint32_t)cid, (uint32_t)(cid >> 32));
        }
        if (n >= CG_COUNT_ESC) {
          const int k = atomicAdd(p.ovf_n, 1);
          if (k < CG_OVF_CAP) {
            p.ovf_cell[k] = cid;
            p.ovf_cnt[k] = n;
          } else {
            atomicOr(p.err, ERR_COUNT_OVERFLOW);
          }
          cnt[h + e] = (unsigned short)CG_COUNT_ESC;
        } else {
          cnt[h + e] = (unsigned short)n;
        }
        tot += n;
      }
    }
    uint4 pk;
    pk.x = cnt[0] | ((unsigned)cnt[1] << 16);
    pk.y = cnt[2] | ((unsigned)cnt[3] << 16);
    pk.z = cnt[4] | ((unsigned)cnt[5] << 16);
    pk.w = cnt[6] | ((unsigned)cnt[7] << 16);
    *reinterpret_cast<uint4 *>(p.counts + c0) = pk;
  }
  /* block total; k_emit scans a block in int, so it must stay below 2^31 */
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  __shared__ long long ws[SB / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long s = 0;
    for (int w = 0; w < SB / 32; w++) s += ws[w];
    if (s > 0x7fffffffLL) atomicOr(p.err, ERR_COUNT_OVERFLOW);
    p.block_sums[blockIdx.x] = s;
  }
}

/* Exclusive scan of n block totals in place; total into *total. */
__global__ void __launch_bounds__(1024) k_scan(long long *v, long long n, long long *total)
{
  __shared__ long long s[1024];
  const long long per = (n + 1023) / 1024;
  const long long b = (long long)threadIdx.x * per, e = (b + per < n) ? b + per : n;
  long long acc = 0;
  for (long long i = b; i < e; i++) acc += v[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    long long t = (int)threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  long long run = s[threadIdx.x] - acc;
  for (long long i = b; i < e; i++) {
    long long x = v[i];
    v[i] = run;
    run += x;
  }
  if (threadIdx.x == 1023) *total = s[1023];
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

__global__ void __launch_bounds__(SB) k_emit(const float *__restrict__ phi, cg_srcs_params p)
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
    const float px = cg_src_offset(x0, dx, u.v[0]);
    const float py = cg_src_offset(y0, dx, u.v[1]);
    const float pz = cg_src_offset(z0, dx, u.v[2]);
    p.pos[id] = make_float4(px, py, pz, dz_rsd);
    float r, cth, ph;
    cg_cart2sph(px, py, pz, &r, &cth, &ph);
    int64_t pr = cg_ang2pix_ring(p.nside_base, cth, ph);
    p.ipix[id] = (int)cg_ring2nest(p.nside_base, pr);
    float *q = p.src + (size_t)id * 9;
    cg_radec(cth, ph, &q[0], &q[1]);                              /* ra, dec */
    q[2] = bg(p.zt, p.g, r);                                      /* z0  */
    q[3] = p.need_beaming ? 0.0f : dz_rsd;                        /* dz_rsd */
    q[4] = p.need_beaming ? 0.0f : -1.0f;                         /* e1  */
    q[5] = p.need_beaming ? 0.0f : -1.0f;                         /* e2  */
    q[6] = 0.0f;
    q[7] = 0.0f;
    q[8] = 0.0f;
    if (p.cmap) atomicAdd(&p.cmap[cg_ang2pix_ring(p.nside_count, cth, ph)], 1);
  }
}

/* Line-of-sight RSD at each source: trilinear gradient of the potential
 * (interpolate_from_grid CIC branch, beaming.c:183-265) projected on the
 * line of sight (srcs.c:500-504), then scaled by V1(r(z0)) * factor_vel
 * (srcs.c:657-662). */
__global__ void __launch_bounds__(256) k_beam_rsd(const float *__restrict__ phi, cg_srcs_params p, long long nsrc)
{
  const int N = p.box.N;
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
    float v[3] = {0.0f, 0.0f, 0.0f};
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
    float vr = CG_MUL(CG_MUL(0.5f, p.box.idx),
                      CG_ADD(CG_ADD(CG_MUL(v[0], u[0]), CG_MUL(v[1], u[1])), CG_MUL(v[2], u[2])));
    float *s = p.src + (size_t)i * 9;
    float z0 = s[2];
    float rz = r_of_z(p.a_a2r, p.r_a2r, p.na, z0);
    s[3] = CG_MUL(vr, CG_MUL(bg(p.v1, p.g, rz), p.factor_vel));
  }
}

} /* namespace */

long long cg_srcs_nblocks(int N) { return ((long long)N * N * N + CPB - 1) / CPB; }

cudaError_t cg_srcs_count(cudaStream_t s, const float *grid, const cg_srcs_params *p, long long *total)
{
  long long nb = cg_srcs_nblocks(p->box.N);
  cudaError_t e = cudaMemsetAsync(p->ovf_n, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_pois_count<<<(unsigned)nb, SB, 0, s>>>(grid, *p);
  k_scan<<<1, 1024, 0, s>>>(p->block_sums, nb, total);
  return cudaGetLastError();
}

cudaError_t cg_srcs_emit(cudaStream_t s, const float *phi, const cg_srcs_params *p)
{
  long long nb = cg_srcs_nblocks(p->box.N);
  k_emit<<<(unsigned)nb, SB, 0, s>>>(phi, *p);
  return cudaGetLastError();
}

cudaError_t cg_srcs_beam_rsd(cudaStream_t s, const float *phi, const cg_srcs_params *p, long long nsrc, int nsm)
{
  if (nsrc <= 0) return cudaSuccess;
  long long blocks = (nsrc + 255) / 256;
  if (blocks > (long long)nsm * 16) blocks = (long long)nsm * 16;
  k_beam_rsd<<<(unsigned)blocks, 256, 0, s>>>(phi, *p, nsrc);
  return cudaGetLastError();
}
