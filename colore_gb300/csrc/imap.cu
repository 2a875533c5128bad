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
 * (the sub-cell follows the pixel size r * sqrt(4 pi / npix)), so a few
 * cells near the observer hold most of the samples.  Two kernels:
 *
 *   k_imap        Warps take groups of whole rows from a counter; a warp
 *                 handles 32 consecutive cells of a row at a time (one per
 *                 lane) and computes their per-cell quantities.  Cells with
 *                 at least nsub_heavy sub-samples per side are appended to the
 *                 heavy list, with their first sample offset from one 64-bit
 *                 atomic that counts records and samples together, so the
 *                 offsets are an exclusive prefix in list order.  The lanes
 *                 then take the sub-samples of the remaining cells, 32
 *                 consecutive ones at a time.
 *   k_imap_heavy  The heavy samples are cut into 8 chunks per warp, taken
 *                 from a counter; a warp finds the first cell of its chunk by
 *                 binary search on the offsets and paints 32 consecutive
 *                 samples at a time.
 *
 * Consecutive samples (x fastest) of a cell often land on the same (shell,
 * pixel); each run of equal keys across the lanes is found with one shuffle
 * and a ballot and added once.  The runs go to a per-warp shared-memory hash
 * table keyed by (shell, pixel) that sums
 * the brightness (temp * run) and the hits: each pixel receives tens of
 * sub-samples of a cell, and neighbouring cells share pixels, so the table
 * turns one global atomic pair per sub-sample into one per distinct key.
 * The table is flushed (data += sum, nadd += hits) when half full and at the
 * end of each row group or chunk; runs that find it nearly full go straight
 * to global memory.  Keys are 32-bit when nr * npix < 2^32 - 1.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "imap_api.h"

namespace {
using namespace cg;

constexpr int IW = 4;          /* warps per block                        */
constexpr int HT = 512;        /* hash slots per warp                    */
constexpr int HFLUSH = 256;    /* flush after a step with this many used */
constexpr int HCAP = 448;      /* no new keys beyond this many           */
constexpr int ROWS = 4;        /* rows per fetch in k_imap               */
constexpr int CHUNKS = 8;      /* sample chunks per warp in k_imap_heavy */

struct CellPar {
  float x0, temp, drr, dxs, inv_ns;
  int nsub, irad0, pad;
};

template <typename K>
struct Table {
  K key[HT];
  float sum[HT];
  unsigned int cnt[HT];
  unsigned short list[HT];
  int nused;
};

template <typename K>
__device__ __forceinline__ K empty_key()
{
  return (K)~(K)0;
}

template <typename K>
__device__ __forceinline__ unsigned int hslot(K k)
{
  unsigned long long h = (unsigned long long)k * 0x9E3779B97F4A7C15ull;
  return (unsigned int)(h >> 55) & (HT - 1);
}

template <typename K>
__device__ __forceinline__ void init_table(Table<K> &w, int lane)
{
  for (int i = lane; i < HT; i += 32) {
    w.key[i] = empty_key<K>();
    w.sum[i] = 0.0f;
    w.cnt[i] = 0u;
  }
  if (lane == 0) w.nused = 0;
}

template <typename K>
__device__ __forceinline__ void flush(Table<K> &w, int lane, const cg_imap_params &p)
{
  __syncwarp();
  const int n = *(volatile int *)&w.nused;
  for (int i = lane; i < n; i += 32) {
    const int h = w.list[i];
    const long long idx = (long long)w.key[h];
    atomicAdd(&p.data[idx], w.sum[h]);
    atomicAdd(&p.nadd[idx], (int)w.cnt[h]);
    w.key[h] = empty_key<K>();
    w.sum[h] = 0.0f;
    w.cnt[h] = 0u;
  }
  __syncwarp();
  if (lane == 0) w.nused = 0;
  __syncwarp();
}

/* Add c hits of brightness temp to key; new keys go to global memory once
 * the table is nearly full. */
template <typename K>
__device__ __forceinline__ void insert(Table<K> &w, K key, unsigned int c, float temp, const cg_imap_params &p)
{
  const float v = CG_MUL(temp, (float)c);
  unsigned int h = hslot(key);
  volatile K *vk = w.key;
  for (int probe = 0; probe < HT; probe++) {
    const K k = vk[h];
    if (k == key) {
      atomicAdd(&w.sum[h], v);
      atomicAdd(&w.cnt[h], c);
      return;
    }
    if (k == empty_key<K>()) {
      if (*(volatile int *)&w.nused >= HCAP) break;
      const K old = atomicCAS(&w.key[h], empty_key<K>(), key);
      if (old == empty_key<K>()) {
        atomicAdd(&w.sum[h], v);
        atomicAdd(&w.cnt[h], c);
        const int pos = atomicAdd(&w.nused, 1);
        w.list[pos] = (unsigned short)h;
        return;
      }
      if (old == key) {
        atomicAdd(&w.sum[h], v);
        atomicAdd(&w.cnt[h], c);
        return;
      }
    }
    h = (h + 1) & (HT - 1);
  }
  atomicAdd(&p.data[(long long)key], v);
  atomicAdd(&p.nadd[(long long)key], (int)c);
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
  const float yz2 = CG_ADD(CG_MUL(yc, yc), CG_MUL(zc, zc));
  const float xc = cg_sub_centre(c.x0, ixx, c.dxs);
  int64_t pix = 0;
  const int ir = cg_imap_sample(xc, yc, zc, yz2, c.drr, r0, rf, p.nr, c.irad0, p.nside, &pix);
  if (ir < 0 || ir >= p.nr) return empty_key<K>();
  return (K)((long long)ir * p.npix + pix);
}

/* The lanes hold consecutive samples: each run of equal (tag, key) is added
 * once, by its first lane, with its length.  tag separates cells. */
template <typename K>
__device__ __forceinline__ void insert_runs(Table<K> &w, K key, int tag, float temp, int lane,
                                            const cg_imap_params &p)
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
    insert(w, key, (unsigned int)(end - lane), temp, p);
  }
}

constexpr unsigned long long HREC = 1ull << 40;     /* one heavy record    */
constexpr unsigned long long HSMASK = HREC - 1;     /* heavy sample field  */

template <typename K>
__global__ void __launch_bounds__(IW * 32, 1) k_imap(const float *__restrict__ dens, const float *__restrict__ phi,
                                                     cg_imap_params p)
{
  extern __shared__ unsigned char sraw[];
  Table<K> *ws = reinterpret_cast<Table<K> *>(sraw);
  CellPar *cells = reinterpret_cast<CellPar *>(sraw + IW * sizeof(Table<K>));
  float *r0 = reinterpret_cast<float *>(cells + IW * 32);
  float *rf = r0 + p.nr;
  int *nsa = reinterpret_cast<int *>(rf + p.nr);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  Table<K> &w = ws[wid];
  CellPar *wc = cells + wid * 32;
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) {
    r0[i] = p.r0[i];
    rf[i] = p.rf[i];
    nsa[i] = p.nsub[i];
  }
  init_table(w, lane);
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
    for (int row = rbeg; row < rend; row++)
    for (int ch = 0; ch < nch; ch++) {
      const int iz = row / N, iy = row - iz * N;
      const int ix = ch * 32 + lane;
      const float y0 = cg_cell_coord(iy, dx, p.box.p1), z0 = cg_cell_coord(iz, dx, p.box.p2);
      CellPar cp = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0, 0, 0};
      int n = 0;
      if (ix < N) {
        cp.x0 = cg_cell_coord(ix, dx, p.box.p0);
        const float rc = cg_norm3(cp.x0, y0, z0);
        const float tmean = bg(p.tz, p.g, rc);
        if (rc <= p.rmax_here && rc >= p.rmin_here && tmean > 0.0f) {
          const float bias = bg(p.bz, p.g, rc);
          const float dnorm = bg(p.norm, p.g, rc);
          const int xh = wrap(ix + 1, N), xl = wrap(ix - 1, N);
          const int yh = wrap(iy + 1, N), yl = wrap(iy - 1, N);
          const int zh = wrap(iz + 1, N), zl = wrap(iz - 1, N);
          float v0 = CG_SUB(__ldg(&phi[pidx(xh, iy, iz, N)]), __ldg(&phi[pidx(xl, iy, iz, N)]));
          float v1 = CG_SUB(__ldg(&phi[pidx(ix, yh, iz, N)]), __ldg(&phi[pidx(ix, yl, iz, N)]));
          float v2 = CG_SUB(__ldg(&phi[pidx(ix, iy, zh, N)]), __ldg(&phi[pidx(ix, iy, zl, N)]));
          float rvel = CG_MUL(p.factor_vel, cg_rvel(v0, v1, v2, cp.x0, y0, z0, rc, p.box.idx));
          cp.drr = cg_imap_drsd(rvel, bg(p.v1, p.g, rc), bg(p.ih, p.g, rc));
          const float d = __ldg(&dens[pidx(ix, iy, iz, N)]);
          cp.temp = cg_imap_temp(tmean, d, bias, dnorm, p.bias_model);
          cp.irad0 = cg_shell_index(r0, rf, p.nr, rc, 0);
          int ns = cp.irad0 < 0 ? p.nsub_lo : (cp.irad0 >= p.nr ? p.nsub_hi : nsa[cp.irad0]);
          if (ns < 1 || ns > 1024) {
            atomicOr(p.err, ERR_IMAP_NSUB);
            ns = 0;
          }
          cp.nsub = ns;
          if (ns > 0) {
            cp.dxs = CG_DIV(dx, (float)ns);
            cp.inv_ns = 1.0f / (float)ns;
            n = ns * ns * ns;
          }
        }
      }
      /* heavy cells go to the list (one atomic per warp); past its capacity
       * they are painted here */
      const bool hv = n > 0 && p.nsub_heavy > 0 && cp.nsub >= p.nsub_heavy;
      if (__ballot_sync(FULL, hv)) {
        const unsigned long long v = hv ? HREC | (unsigned long long)n : 0ull;
        unsigned long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          unsigned long long t = __shfl_up_sync(FULL, inc, o);
          if (lane >= o) inc += t;
        }
        const unsigned long long wt = __shfl_sync(FULL, inc, 31);
        unsigned long long base = 0;
        int ok = 0;
        if (lane == 0) {
          /* stop appending once the list is full or half the sample field is
           * used, so that neither field can wrap (the overshoot of warps in
           * flight is at most 32 records and 2^35 samples each) */
          const unsigned long long cur = *(volatile unsigned long long *)&p.ctr[0];
          if ((long long)(cur >> 40) < p.heavy_cap && (cur & HSMASK) < (HSMASK >> 1)) {
            base = atomicAdd(&p.ctr[0], wt);
            ok = 1;
            if ((base & HSMASK) + (wt & HSMASK) > HSMASK) atomicOr(p.err, ERR_IMAP_HEAVY);
          }
        }
        ok = __shfl_sync(FULL, ok, 0);
        base = __shfl_sync(FULL, base, 0);
        const unsigned long long mine = base + inc - v;
        const long long slot = (long long)(mine >> 40);
        if (ok && hv && slot < p.heavy_cap) {
          float4 *q = reinterpret_cast<float4 *>(p.heavy + slot);
          q[0] = make_float4(cp.x0, y0, z0, cp.temp);
          q[1] = make_float4(cp.drr, cp.dxs, __int_as_float(cp.nsub), __int_as_float(cp.irad0));
          p.heavy_off[slot] = (long long)(mine & HSMASK);
          n = 0;
        }
      }
      /* cells painted here keep the warp's sample count below 2^26 */
      if (n > 0 && cp.nsub > 128) {
        atomicOr(p.err, ERR_IMAP_HEAVY);
        n = 0;
      }
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
        insert_runs(w, key, j, temp, lane, p);
        __syncwarp();
        if (*(volatile int *)&w.nused >= HFLUSH) flush(w, lane, p);
      }
      __syncwarp();
    }
    flush(w, lane, p);
  }
}

template <typename K>
__global__ void __launch_bounds__(IW * 32, 1) k_imap_heavy(cg_imap_params p)
{
  extern __shared__ unsigned char sraw[];
  Table<K> *ws = reinterpret_cast<Table<K> *>(sraw);
  float *r0 = reinterpret_cast<float *>(sraw + IW * sizeof(Table<K>));
  float *rf = r0 + p.nr;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  Table<K> &w = ws[wid];
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) {
    r0[i] = p.r0[i];
    rf[i] = p.rf[i];
  }
  init_table(w, lane);
  __syncthreads();
  const unsigned long long ctr = *(volatile unsigned long long *)&p.ctr[0];
  long long H = (long long)(ctr >> 40);
  if (H > p.heavy_cap) H = p.heavy_cap;
  if (H <= 0) return;
  const cg_heavy_cell *hl = p.heavy;
  const long long *off = p.heavy_off;
  const long long nlast = hl[H - 1].nsub;
  const unsigned long long S = (unsigned long long)(off[H - 1] + nlast * nlast * nlast);
  if (blockIdx.x == 0 && threadIdx.x == 0) p.ctr[4] = S;
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
      if (off[mid] <= s0) lo = mid;
      else hi = mid - 1;
    }
    for (long long h = lo; h < H && off[h] < s1; h++) {
      const float4 qa = __ldg(reinterpret_cast<const float4 *>(hl + h));
      const float4 qb = __ldg(reinterpret_cast<const float4 *>(hl + h) + 1);
      CellPar c;
      c.x0 = qa.x;
      c.temp = qa.w;
      c.drr = qb.x;
      c.dxs = qb.y;
      c.nsub = __float_as_int(qb.z);
      c.irad0 = __float_as_int(qb.w);
      c.inv_ns = 1.0f / (float)c.nsub;
      c.pad = 0;
      const long long ns = c.nsub, base = off[h];
      const long long qbeg = s0 > base ? s0 - base : 0;
      long long qend = s1 - base;
      if (qend > ns * ns * ns) qend = ns * ns * ns;
      for (long long q0 = qbeg; q0 < qend; q0 += 32) {
        const long long q = q0 + lane;
        const K key = q < qend ? sample_key<K>(p, r0, rf, c, qa.y, qa.z, (int)q) : empty_key<K>();
        insert_runs(w, key, 0, c.temp, lane, p);
        __syncwarp();
        if (*(volatile int *)&w.nused >= HFLUSH) flush(w, lane, p);
      }
    }
    flush(w, lane, p);
  }
}

template <typename K>
cudaError_t launch(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  size_t smem = IW * sizeof(Table<K>) + IW * 32 * sizeof(CellPar) + (size_t)p->nr * (2 * sizeof(float) + sizeof(int));
  cudaError_t e = cudaFuncSetAttribute(k_imap<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_imap<K>, IW * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  e = cudaMemsetAsync(p->ctr, 0, 5 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  long long nrow = (long long)p->box.N * p->box.N;
  long long blocks = (nrow + IW * ROWS - 1) / (IW * ROWS);
  if (blocks > (long long)nsm * per_sm) blocks = (long long)nsm * per_sm;
  k_imap<K><<<(unsigned)blocks, IW * 32, smem, s>>>(dens, phi, *p);
  e = cudaGetLastError();
  if (e != cudaSuccess || p->heavy_cap <= 0) return e;
  size_t hsmem = IW * sizeof(Table<K>) + (size_t)p->nr * 2 * sizeof(float);
  e = cudaFuncSetAttribute(k_imap_heavy<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsmem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_imap_heavy<K>, IW * 32, hsmem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  k_imap_heavy<K><<<(unsigned)(nsm * per_sm), IW * 32, hsmem, s>>>(*p);
  return cudaGetLastError();
}

} /* namespace */

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  if (!p->ctr) return cudaErrorInvalidValue;
  /* 32-bit keys when every (shell, pixel) index and the empty key fit */
  if ((unsigned long long)p->nr * (unsigned long long)p->npix < 0xffffffffull)
    return launch<unsigned int>(s, dens, phi, p, nsm);
  return launch<unsigned long long>(s, dens, phi, p, nsm);
}
