/*
 * imap.cu -- intensity-map painting (imap_set_cartesian_single,
 * imap.c:135-245).
 *
 * Every cell in the radial range of the shells carries a brightness
 * temp = T(r) bias_model(d, b(r)) norm(r) and a redshift-space shift dr_rsd;
 * it is split into nsub^3 sub-cells whose centres are placed in a shell (by
 * r + dr_rsd) and a RING pixel, where temp is added and a hit counted.
 *
 * The work per cell is nsub^3 and nsub grows as 1/r towards the observer
 * (the sub-cell follows the pixel size r * sqrt(4 pi / npix)): from 8 samples
 * per cell at high redshift to thousands near the observer.  So the cells
 * are first listed and their samples then painted as one even stream:
 *
 *   k_imap_cells  Warps take groups of whole rows from a counter; a lane
 *                 computes one cell's brightness, radial shift, shell and
 *                 nsub and appends the cell to the list (one atomic per warp).
 *                 Cells past the list's capacity are painted here, 32
 *                 consecutive samples of the warp's cells at a time.
 *   k_scan_*      exclusive scan of the listed cells' sample counts: the
 *                 first sample of every listed cell.
 *   k_imap_paint  The listed samples are cut into 8 chunks per warp, taken
 *                 from a counter; a warp finds the first cell of its chunk by
 *                 binary search on the offsets and paints 32 consecutive
 *                 samples at a time, each lane walking forward to its cell.
 *
 * Consecutive samples (x fastest) of a cell often land on the same (shell,
 * pixel); each run of equal keys across the lanes is found with one shuffle
 * and a ballot and added to the maps once, with one float and one integer
 * atomic (data += temp * run, nadd += run).  GB300's L2 sustains these
 * without staging: a shared-memory hash table that merged the runs of a
 * warp before the global atomics was measured slower at every nsub.  Keys
 * (shell * npix + pixel) are 32-bit when nr * npix < 2^32 - 1.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "cg_dev.cuh"
#include "imap_api.h"

namespace {
using namespace cg;

constexpr int IW = 4;          /* warps per block                        */
constexpr int ROWS = 4;        /* rows per fetch in k_imap               */
constexpr int CHUNKS = 8;      /* sample chunks per warp in k_imap_paint */
constexpr int SCAN_T = 256;    /* threads per block of the offset scan    */
constexpr int SCAN_I = 16;     /* records per thread of the offset scan   */

struct CellPar {
  float x0, temp, drr, dxs, inv_ns;
  int nsub, irad0, pad;
};

template <typename K>
__device__ __forceinline__ K empty_key()
{
  return (K)~(K)0;
}

/* Key of sample q (0 <= q < ns^3, x fastest, then y, then z) of cell c, whose
 * corner is (c.x0, y0, z0), or the empty key outside the shells. */
template <typename K>
__device__ __forceinline__ K sample_key(const cg_imap_params &p, const float *r0, const float *rf, const CellPar &c,
                                        float y0, float z0, int q)
{
  const int ns = c.nsub;
  int line, izz;
  if (ns <= 128) {
    /* (q + 1/2)/ns is at least 1/(2 ns) from an integer and the float
     * product is within ns^2 2^-23 of it: exact while ns^3 < 2^22 */
    line = (int)(((float)q + 0.5f) * c.inv_ns);
    izz = (int)(((float)line + 0.5f) * c.inv_ns);
  } else {
    line = q / ns;
    izz = line / ns;
  }
  const int ixx = q - line * ns, iyy = line - izz * ns;
  const float zc = cg_sub_centre(z0, izz, c.dxs);
  const float yc = cg_sub_centre(y0, iyy, c.dxs);
  const float yz2 = cg_yz2(yc, zc);
  const float xc = cg_sub_centre(c.x0, ixx, c.dxs);
  int64_t pix = 0;
  const int ir = cg_imap_sample(xc, yc, zc, yz2, c.drr, r0, rf, p.nr, c.irad0, p.nside, &pix);
  if (ir < 0 || ir >= p.nr) return empty_key<K>();
  if (sizeof(K) == 4) return (K)((unsigned)ir * (unsigned)p.npix + (unsigned)pix);
  return (K)((long long)ir * p.npix + pix);
}

/* The lanes hold consecutive samples: each run of equal (tag, key) is added
 * to the maps once, by its first lane, with its length (data += temp * run,
 * nadd += run).  tag separates cells, whose brightness differs. */
template <typename K>
__device__ __forceinline__ void add_runs(K key, int tag, float temp, int lane, const cg_imap_params &p)
{
  const unsigned FULL = 0xffffffffu;
  const K pk = __shfl_up_sync(FULL, key, 1);
  const int pt = __shfl_up_sync(FULL, tag, 1);
  const bool valid = key != empty_key<K>();
  const bool head = valid && (lane == 0 || pk != key || pt != tag);
  const unsigned bnd = __ballot_sync(FULL, head || !valid);
  if (head) {
    const unsigned above = lane == 31 ? 0u : bnd & (FULL << (lane + 1));
    const int end = above ? __ffs(above) - 1 : 32;
    const unsigned int c = (unsigned int)(end - lane);
    atomicAdd(&p.data[(long long)key], CG_MUL(temp, (float)c));
    atomicAdd(&p.nadd[(long long)key], (int)c);
  }
}

template <typename K>
__global__ void __launch_bounds__(IW * 32, 16) k_imap_cells(const float *__restrict__ dens, const float *__restrict__ phi,
                                                     cg_imap_params p)
{
  extern __shared__ unsigned char sraw[];
  CellPar *cells = reinterpret_cast<CellPar *>(sraw);
  float4 *shp = reinterpret_cast<float4 *>(cells + IW * 32);
  float *r0 = reinterpret_cast<float *>(shp + p.nr + 2);
  float *rf = r0 + p.nr;
  float *rfm = rf + p.nr; /* running maximum of rf, for cg_shell_index0 */
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  CellPar *wc = cells + wid * 32;
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) {
    r0[i] = p.r0[i];
    rf[i] = p.rf[i];
  }
  for (int i = threadIdx.x; i < p.nr + 2; i += blockDim.x) shp[i] = p.shp[i];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < p.nr; i++) rfm[i] = i == 0 ? rf[0] : (rf[i] > rfm[i - 1] ? rf[i] : rfm[i - 1]);
  __syncthreads();
  const int N = p.box.N;
  const int nch = (N + 31) / 32;
  const int nrow = N * N;
  const float dx = p.box.dx;
  const unsigned FULL = 0xffffffffu;
  unsigned long long painted = 0; /* samples of the cells painted by this lane */
  for (;;) {
    int rbeg = 0;
    if (lane == 0) rbeg = (int)atomicAdd(&p.ctr[2], (unsigned long long)ROWS);
    rbeg = __shfl_sync(FULL, rbeg, 0);
    if (rbeg >= nrow) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) painted += __shfl_xor_sync(FULL, painted, o);
      if (lane == 0 && painted) atomicAdd(&p.ctr[3], painted);
      break;
    }
    const int rend = rbeg + ROWS < nrow ? rbeg + ROWS : nrow;
    /* whether a cell is listed depends on its radius alone: count the row
     * group's listed cells first and reserve their slots with one atomic */
    int nlist = 0;
    for (int row = rbeg; row < rend; row++) {
      const int iz = row / N, iy = row - iz * N;
      const float y0 = cg_cell_coord(iy, dx, p.box.p1), z0 = cg_cell_coord(iz, dx, p.box.p2);
      for (int ix = lane; ix < N; ix += 32) {
        const float rc = cg_norm3(cg_cell_coord(ix, dx, p.box.p0), y0, z0);
        nlist += (rc <= p.rmax_here && rc >= p.rmin_here && bgv(p.tz, bg_at(p.g, rc)) > 0.0f) ? 1 : 0;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nlist += __shfl_xor_sync(FULL, nlist, o);
    unsigned long long next = 0; /* the warp's next slot */
    if (lane == 0 && nlist > 0) {
      /* once the list is full the counter overshoots its capacity by at most
       * one row group per warp in flight */
      const unsigned long long cur = *(volatile unsigned long long *)&p.ctr[0];
      next = cur < (unsigned long long)p.list_cap ? atomicAdd(&p.ctr[0], (unsigned long long)nlist)
                                                  : (unsigned long long)p.list_cap;
    }
    next = __shfl_sync(FULL, next, 0);
    for (int row = rbeg; row < rend; row++)
    for (int ch = 0; ch < nch; ch++) {
      const int iz = row / N, iy = row - iz * N;
      const int ix = ch * 32 + lane;
      const float y0 = cg_cell_coord(iy, dx, p.box.p1), z0 = cg_cell_coord(iz, dx, p.box.p2);
      CellPar cp = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0, 0, 0};
      int n = 0;
      bool lst = false; /* the condition counted in the first pass */
      if (ix < N) {
        cp.x0 = cg_cell_coord(ix, dx, p.box.p0);
        const float rc = cg_norm3(cp.x0, y0, z0);
        const BgAt at = bg_at(p.g, rc);
        const float tmean = bgv(p.tz, at);
        lst = rc <= p.rmax_here && rc >= p.rmin_here && tmean > 0.0f;
        if (lst) {
          const float bias = bgv(p.bz, at);
          const float dnorm = bgvn(p.norm, at);
          const int xh = wrap(ix + 1, N), xl = wrap(ix - 1, N);
          const int yh = wrap(iy + 1, N), yl = wrap(iy - 1, N);
          const int zh = wrap(iz + 1, N), zl = wrap(iz - 1, N);
          float v0 = CG_SUB(__ldg(&phi[pidx(xh, iy, iz, N)]), __ldg(&phi[pidx(xl, iy, iz, N)]));
          float v1 = CG_SUB(__ldg(&phi[pidx(ix, yh, iz, N)]), __ldg(&phi[pidx(ix, yl, iz, N)]));
          float v2 = CG_SUB(__ldg(&phi[pidx(ix, iy, zh, N)]), __ldg(&phi[pidx(ix, iy, zl, N)]));
          float rvel = CG_MUL(p.factor_vel, cg_rvel(v0, v1, v2, cp.x0, y0, z0, rc, p.box.idx));
          cp.drr = cg_imap_drsd(rvel, bgv(p.v1, at), bgv(p.ih, at));
          const float d = __ldg(&dens[pidx(ix, iy, iz, N)]);
          cp.temp = cg_imap_temp(tmean, d, bias, dnorm, p.bias_model);
          cp.irad0 = cg_shell_index0(r0, rfm, p.nr, rc);
          /* nsub of the cell's shell (the first one below the shells, the
           * last one beyond or in a gap), with dx / nsub and 1 / nsub */
          const float4 sp = shp[cp.irad0 + 1];
          const int ns = __float_as_int(sp.x);
          if (ns < 1 || ns > 1024) {
            atomicOr(p.err, ERR_IMAP_NSUB);
          } else {
            cp.nsub = ns;
            cp.dxs = sp.y;
            cp.inv_ns = sp.z;
            n = ns * ns * ns;
          }
        }
      }
      /* every cell goes to the list, in the slots reserved above; past its
       * capacity it is painted here */
      const unsigned lm = __ballot_sync(FULL, lst);
      if (lm) {
        const long long slot = (long long)next + __popc(lm & ((1u << lane) - 1u));
        next += (unsigned long long)__popc(lm);
        if (lst && slot < p.list_cap) {
          float4 *q = reinterpret_cast<float4 *>(p.cells + slot);
          q[0] = make_float4(cp.x0, y0, z0, cp.temp);
          q[1] = make_float4(cp.drr, cp.dxs, cp.inv_ns, __int_as_float(cp.nsub | ((cp.irad0 + 1) << 11)));
          p.cell_n[slot] = (unsigned int)n;
          n = 0;
        }
      }
      /* cells painted here keep the warp's sample count below 2^26 */
      if (n > 0 && cp.nsub > 128) {
        atomicOr(p.err, ERR_IMAP_HEAVY);
        n = 0;
      }
      if (!__any_sync(FULL, n > 0)) continue;
      wc[lane] = cp;
      painted += (unsigned long long)n;
      /* inclusive scan of the sample counts (nsub^3 per cell) over the warp */
      int incl = n;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
      }
      const int excl = incl - n;
      const int total = __shfl_sync(FULL, incl, 31);
      __syncwarp();
      for (int base = 0; base < total; base += 32) {
        const int s = base + lane;
        /* owning lane j = number of lanes whose inclusive prefix is <= s */
        int j = 0;
#pragma unroll
        for (int st = 16; st > 0; st >>= 1) {
          int v = __shfl_sync(FULL, incl, j + st - 1);
          if (v <= s) j += st;
        }
        if (j > 31) j = 31;
        const int ex = __shfl_sync(FULL, excl, j);
        K key = empty_key<K>();
        float temp = 0.0f;
        if (s < total) {
          const CellPar c = wc[j];
          key = sample_key<K>(p, r0, rf, c, y0, z0, s - ex);
          temp = c.temp;
        }
        add_runs(key, j, temp, lane, p);
      }
      __syncwarp();
    }
  }
}

/* Sum of the sample counts of each block of SCAN_T * SCAN_I records. */
__global__ void __launch_bounds__(SCAN_T) k_scan_sum(const unsigned int *__restrict__ n, long long H, long long *bsum)
{
  const long long i0 = ((long long)blockIdx.x * SCAN_T + threadIdx.x) * SCAN_I;
  long long t = 0;
  if (i0 + SCAN_I <= H) { /* 16 records, 64 B aligned */
#pragma unroll
    for (int i = 0; i < SCAN_I; i += 4) {
      const uint4 q = __ldg(reinterpret_cast<const uint4 *>(n + i0 + i));
      t += (long long)q.x + q.y + q.z + q.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_I; i++)
      if (i0 + i < H) t += n[i0 + i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  __shared__ long long ws[SCAN_T / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long b = 0;
    for (int w = 0; w < SCAN_T / 32; w++) b += ws[w];
    bsum[blockIdx.x] = b;
  }
}

/* Exclusive scan of the nb block sums in place (one block); total -> *total. */
__global__ void __launch_bounds__(1024) k_scan_top(long long *v, long long nb, unsigned long long *total)
{
  __shared__ long long sm[1024];
  const long long per = (nb + 1023) / 1024;
  const long long b = (long long)threadIdx.x * per, e = b + per < nb ? b + per : nb;
  long long acc = 0;
  for (long long i = b; i < e; i++) acc += v[i];
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const long long t = (int)threadIdx.x >= o ? sm[threadIdx.x - o] : 0;
    __syncthreads();
    sm[threadIdx.x] += t;
    __syncthreads();
  }
  long long run = sm[threadIdx.x] - acc;
  for (long long i = b; i < e; i++) {
    const long long x = v[i];
    v[i] = run;
    run += x;
  }
  if (threadIdx.x == 1023) *total = (unsigned long long)sm[1023];
}

/* First sample of every record: block offset + in-block exclusive scan. */
__global__ void __launch_bounds__(SCAN_T) k_scan_out(const unsigned int *__restrict__ n, long long H,
                                                      const long long *__restrict__ bexcl, long long *off)
{
  const long long i0 = ((long long)blockIdx.x * SCAN_T + threadIdx.x) * SCAN_I;
  const bool full = i0 + SCAN_I <= H; /* a thread's 16 records, 64 B aligned */
  unsigned int v[SCAN_I];
  long long t = 0;
  if (full) {
#pragma unroll
    for (int i = 0; i < SCAN_I; i += 4) {
      const uint4 q = __ldg(reinterpret_cast<const uint4 *>(n + i0 + i));
      v[i] = q.x;
      v[i + 1] = q.y;
      v[i + 2] = q.z;
      v[i + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_I; i++) v[i] = i0 + i < H ? n[i0 + i] : 0u;
  }
#pragma unroll
  for (int i = 0; i < SCAN_I; i++) t += v[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long inc = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  __shared__ long long ws[SCAN_T / 32];
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  long long run = bexcl[blockIdx.x];
  for (int w = 0; w < wid; w++) run += ws[w];
  run += inc - t;
  if (full) {
#pragma unroll
    for (int i = 0; i < SCAN_I; i += 2) {
      const long long a = run;
      run += v[i];
      reinterpret_cast<longlong2 *>(off + i0)[i / 2] = make_longlong2(a, run);
      run += v[i + 1];
    }
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_I; i++) {
      if (i0 + i < H) off[i0 + i] = run;
      run += v[i];
    }
  }
}

template <typename K>
__global__ void __launch_bounds__(IW * 32, 1) k_imap_paint(cg_imap_params p)
{
  extern __shared__ unsigned char sraw[];
  float *r0 = reinterpret_cast<float *>(sraw);
  float *rf = r0 + p.nr;
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) {
    r0[i] = p.r0[i];
    rf[i] = p.rf[i];
  }
  __syncthreads();
  long long H = (long long)*(volatile unsigned long long *)&p.ctr[0];
  if (H > p.list_cap) H = p.list_cap;
  const unsigned long long S = *(volatile unsigned long long *)&p.ctr[4];
  if (H <= 0 || S == 0) return;
  const cg_imap_cell *cl = p.cells;
  const long long *off = p.cell_off;
  const unsigned long long NC = (unsigned long long)gridDim.x * IW * CHUNKS;
  const unsigned FULL = 0xffffffffu;
  for (;;) {
    unsigned long long k = 0;
    if (lane == 0) k = atomicAdd(&p.ctr[1], 1ull);
    k = __shfl_sync(FULL, k, 0);
    if (k >= NC) break;
    const long long s0 = (long long)(S * k / NC), s1 = (long long)(S * (k + 1) / NC);
    if (s0 >= s1) continue;
    /* last record starting at or before s0 */
    long long lo = 0, hi = H - 1;
    while (lo < hi) {
      const long long mid = (lo + hi + 1) >> 1;
      if (__ldg(&off[mid]) <= s0) lo = mid;
      else hi = mid - 1;
    }
    long long hw = lo, ow = __ldg(&off[lo]); /* the warp's current record and its first sample */
    for (long long sb = s0; sb < s1; sb += 32) {
      const long long s = sb + lane;
      long long h = hw, oh = ow;
      K key = empty_key<K>();
      float temp = 0.0f;
      if (s < s1) {
        while (h + 1 < H) {
          const long long nx = __ldg(&off[h + 1]);
          if (nx > s) break;
          h++;
          oh = nx;
        }
        const float4 qa = __ldg(reinterpret_cast<const float4 *>(cl + h));
        const float4 qb = __ldg(reinterpret_cast<const float4 *>(cl + h) + 1);
        const int pk = __float_as_int(qb.w);
        CellPar c;
        c.x0 = qa.x;
        c.temp = qa.w;
        c.drr = qb.x;
        c.dxs = qb.y;
        c.inv_ns = qb.z;
        c.nsub = pk & 2047;
        c.irad0 = (pk >> 11) - 1;
        c.pad = 0;
        key = sample_key<K>(p, r0, rf, c, qa.y, qa.z, (int)(s - oh));
        temp = c.temp;
      }
      add_runs(key, (int)h, temp, lane, p);
      hw = __shfl_sync(FULL, h, 31);
      ow = __shfl_sync(FULL, oh, 31);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) p.ctr[4] = S; /* listed samples, for the caller */
}

template <typename K>
cudaError_t launch(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  size_t smem = IW * 32 * sizeof(CellPar) + (size_t)(p->nr + 2) * sizeof(float4) + (size_t)p->nr * 3 * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_imap_cells<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_imap_cells<K>, IW * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  e = cudaMemsetAsync(p->ctr, 0, 5 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  long long nrow = (long long)p->box.N * p->box.N;
  long long blocks = (nrow + IW * ROWS - 1) / (IW * ROWS);
  if (blocks > (long long)nsm * per_sm) blocks = (long long)nsm * per_sm;
  k_imap_cells<K><<<(unsigned)blocks, IW * 32, smem, s>>>(dens, phi, *p);
  e = cudaGetLastError();
  if (e != cudaSuccess || p->list_cap <= 0) return e;
  /* records listed (the count may overshoot the capacity) */
  unsigned long long h = 0;
  e = cudaMemcpyAsync(&h, p->ctr, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  const long long H = (long long)std::min<unsigned long long>(h, (unsigned long long)p->list_cap);
  if (H == 0) return cudaSuccess;
  const long long nb = (H + SCAN_T * SCAN_I - 1) / (SCAN_T * SCAN_I);
  k_scan_sum<<<(unsigned)nb, SCAN_T, 0, s>>>(p->cell_n, H, p->scan_tmp);
  k_scan_top<<<1, 1024, 0, s>>>(p->scan_tmp, nb, p->ctr + 4);
  k_scan_out<<<(unsigned)nb, SCAN_T, 0, s>>>(p->cell_n, H, p->scan_tmp, p->cell_off);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  /* every warp of the painting pass resident at once */
  const size_t psmem = (size_t)p->nr * 2 * sizeof(float);
  e = cudaFuncSetAttribute(k_imap_paint<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_imap_paint<K>, IW * 32, psmem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  k_imap_paint<K><<<(unsigned)(nsm * per_sm), IW * 32, psmem, s>>>(*p);
  return cudaGetLastError();
}

} /* namespace */

long long cg_imap_scan_blocks(long long cap) { return (cap + SCAN_T * SCAN_I - 1) / (SCAN_T * SCAN_I); }

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  if (!p->ctr) return cudaErrorInvalidValue;
  /* 32-bit keys when every (shell, pixel) index and the empty key fit */
  if ((unsigned long long)p->nr * (unsigned long long)p->npix < 0xffffffffull)
    return launch<unsigned int>(s, dens, phi, p, nsm);
  return launch<unsigned long long>(s, dens, phi, p, nsm);
}
