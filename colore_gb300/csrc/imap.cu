/*
 * imap.cu -- intensity-map painting (imap_set_cartesian_single,
 * imap.c:135-245).
 *
 * Every cell in the radial range of the shells carries a brightness
 * temp = T(r) bias_model(d, b(r)) norm(r) and a redshift-space shift dr_rsd;
 * it is split into nsub^3 sub-cells whose centres are placed in a shell (by
 * r + dr_rsd) and a RING pixel, where temp is added and a hit counted.  The
 * shells and pixels are decided as the reference's double arithmetic
 * decides them: in single precision where a bound on the distance to the
 * double value proves the decision, in float-float where that bound fails,
 * and in double only where the float-float bound fails too (cg_exact.h), so
 * the hit counts are those of the double arithmetic.
 *
 * nsub is fixed by the shell of the cell's corner radius and grows towards
 * the observer (from 2 at high redshift to ~20 for the nearest shells), so
 * cells are listed per shell -- one bucket per shell, holding cells of one
 * nsub -- and painted bucket after bucket:
 *
 *   k_imap_list    Warps take groups of rows from a counter; a lane decides
 *                  one cell (listed or not, its shell, brightness, radial
 *                  shift, and whether all its samples certainly stay in one
 *                  shell, which spares them the radial test) and appends it
 *                  to its bucket: one atomic per bucket present in the warp,
 *                  all issued together.  A cell that finds its bucket full is
 *                  painted by its warp on the spot.
 *   k_imap_chunks  One thread cuts each bucket into chunks of about CHS
 *                  samples: whole cells, or slices of one cell.
 *   k_imap_paint   Warps take chunks in bucket order, so the maps' working
 *                  set at any time is a few shells (25 MB per shell at nside
 *                  512) and the atomics stay in L2.  Each lane walks one unit
 *                  sample by sample, keeping two (key, count) run slots that
 *                  it evicts with one float and one integer atomic.  Samples
 *                  whose margins fail are staged per warp in shared memory
 *                  and queued in batches.
 *   k_imap_double  The queued samples: first in float-float, then, for the
 *                  few left, gathered per warp and decided in double 32 at a
 *                  time, the cell's radial shift computed once per run of
 *                  one record.
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "imap_api.h"

namespace {
using namespace cg;

constexpr int IW = 4;     /* warps per block                     */
constexpr int ROWS = 2;   /* rows per fetch in k_imap_list        */
constexpr int CHS = 4096; /* samples per painting chunk           */
constexpr int QB = 256;   /* queue entries staged per painting warp */
constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned F_DOUBLE = 16u; /* flags: mode (2 bits), delta + 1 (2 bits), double */

/* Per-block copies of the species' shell tables. */
struct Sh {
  float *b, *dxs, *invns;
  int *shell_of, *nsub;
  unsigned long long *chunk_off;
};

__host__ __device__ __forceinline__ size_t shell_smem(int nr, int nbk, bool chunks)
{
  size_t n = (size_t)(2 * nr) * 4 + (size_t)(2 * nr + 1) * 4 + 3 * (size_t)(nr + 2) * 4;
  n = (n + 7) & ~(size_t)7;
  if (chunks) n += (size_t)(nbk + 1) * 8;
  return n;
}

/* Where the tables sit in the block's shared memory. */
__device__ __forceinline__ Sh shells_at(const cg_imap_params &p, unsigned char *raw)
{
  const int nr = p.nr;
  Sh s;
  s.b = reinterpret_cast<float *>(raw);
  s.shell_of = reinterpret_cast<int *>(s.b + 2 * nr);
  s.nsub = s.shell_of + 2 * nr + 1;
  s.dxs = reinterpret_cast<float *>(s.nsub + nr + 2);
  s.invns = s.dxs + nr + 2;
  s.chunk_off = reinterpret_cast<unsigned long long *>(raw + shell_smem(nr, p.nbk, false));
  return s;
}

/* The painting warps' queue stages follow the tables. */
__host__ __device__ __forceinline__ size_t paint_stage_off(int nr, int nbk) { return (shell_smem(nr, nbk, true) + 15) & ~(size_t)15; }
__host__ __device__ __forceinline__ size_t paint_smem(int nr, int nbk) { return paint_stage_off(nr, nbk) + (size_t)IW * QB * 8; }
/* The double pass keeps the buckets' bases where the painting keeps its
 * chunk table; its per-warp gathers (64 entries) follow. */
__host__ __device__ __forceinline__ size_t double_stage_off(int nr, int nbk) { return (shell_smem(nr, nbk, true) + 15) & ~(size_t)15; }

__device__ __forceinline__ Sh load_shells(const cg_imap_params &p, unsigned char *raw, bool chunks)
{
  const int nb = p.a.sh.nb, nr = p.nr;
  const Sh s = shells_at(p, raw);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s.b[i] = p.a.sh.b[i];
  for (int i = threadIdx.x; i <= nb; i += blockDim.x) s.shell_of[i] = p.a.sh.shell_of[i];
  for (int i = threadIdx.x; i < nr + 2; i += blockDim.x) {
    s.nsub[i] = p.a.nsub[i];
    s.dxs[i] = p.a.dxs[i];
    s.invns[i] = 1.0f / (float)p.a.nsub[i];
  }
  if (chunks)
    for (int i = threadIdx.x; i <= p.nbk; i += blockDim.x) s.chunk_off[i] = p.chunk_off[i];
  return s;
}

__device__ __forceinline__ cg_imap_args args_with(const cg_imap_params &p, const Sh &s)
{
  cg_imap_args A = p.a;
  A.sh.b = s.b;
  A.sh.shell_of = s.shell_of;
  A.nsub = s.nsub;
  A.dxs = s.dxs;
  return A;
}

template <typename K>
__device__ __forceinline__ K empty_key()
{
  return (K)~(K)0;
}

template <typename K>
__device__ __forceinline__ K key_of(const cg_imap_params &p, int s, long long pix)
{
  if (s < 0 || s >= p.nr) return empty_key<K>();
  if (sizeof(K) == 4) return (K)((unsigned)s * (unsigned)p.npix + (unsigned)pix);
  return (K)((long long)s * p.npix + pix);
}

/* The lanes hold consecutive samples: each run of equal (tag, key) is added
 * to the maps once, by its first lane, with its length (data += temp * run,
 * nadd += run).  tag separates cells, whose brightness differs. */
template <typename K>
__device__ __forceinline__ void add_runs(K key, int tag, float temp, int lane, const cg_imap_params &p)
{
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

/* Sub-cell (sx, sy, sz) of sample q < ns^3, x fastest. */
__device__ __forceinline__ void sub_of(int q, int ns, float inv_ns, int *sx, int *sy, int *sz)
{
  int line, z;
  if (ns <= 128) {
    /* (q + 1/2)/ns is at least 1/(2 ns) from an integer and the float
     * product is within ns^2 2^-23 of it: exact while ns^3 < 2^22 */
    line = (int)(((float)q + 0.5f) * inv_ns);
    z = (int)(((float)line + 0.5f) * inv_ns);
  } else {
    line = q / ns;
    z = line / ns;
  }
  *sx = q - line * ns;
  *sy = line - z * ns;
  *sz = z;
}

/* Centred potential differences at a cell (get_rvel, imap.c:43-74): float
 * minus float, as the reference forms them from its float grid. */
__device__ __forceinline__ void grad_phi(const float *__restrict__ phi, int ix, int iy, int iz, int N, float v[3])
{
  v[0] = CG_SUB(__ldg(&phi[pidx(wrap(ix + 1, N), iy, iz, N)]), __ldg(&phi[pidx(wrap(ix - 1, N), iy, iz, N)]));
  v[1] = CG_SUB(__ldg(&phi[pidx(ix, wrap(iy + 1, N), iz, N)]), __ldg(&phi[pidx(ix, wrap(iy - 1, N), iz, N)]));
  v[2] = CG_SUB(__ldg(&phi[pidx(ix, iy, wrap(iz + 1, N), N)]), __ldg(&phi[pidx(ix, iy, wrap(iz - 1, N), N)]));
}

/* Brightness of a cell whose decisions were taken in double (imap.c:199,
 * 201), in single precision like every other cell's. */
__device__ __forceinline__ float temp32(const cg_imap_args &A, int ix, int iy, int iz, float d)
{
  const float x0 = A.xc[ix], y0 = A.yc[iy], z0 = A.zc[iz];
  const float r2 = CG_FMA(z0, z0, CG_FMA(y0, y0, CG_MUL(x0, x0)));
  const float rc = CG_MUL(r2, cg_rsqrt_fast(r2));
  const float tm = cg_tab_at(A.tz, A.na, A.idr, A.r, rc, 0.0f).v;
  const float b = cg_tab_at(A.bz, A.na, A.idr, A.r, rc, 0.0f).v;
  const float dn = cg_tab_at(A.norm, A.na, A.idr, A.r, rc, 0.0f).v;
  return CG_MUL(CG_MUL(tm, cg_bias_model(d, b, A.bias_model)), dn);
}

__device__ __forceinline__ cg_imap_rec pack(int ix, int iy, int iz, const cg_imap_cell &c, unsigned flags)
{
  cg_imap_rec r;
  r.ixy = (unsigned)ix | ((unsigned)iy << 16);
  const unsigned short eh = __half_as_ushort(__float2half_ru(c.edrr));
  r.izf = (unsigned)iz | (flags << 11) | ((unsigned)eh << 16);
  r.temp = c.temp;
  r.drr = c.drr;
  return r;
}

__device__ __forceinline__ cg_imap_cell unpack(const cg_imap_rec &r, int j, int *ix, int *iy, int *iz, int *dbl)
{
  cg_imap_cell c;
  *ix = (int)(r.ixy & 0xffffu);
  *iy = (int)(r.ixy >> 16);
  *iz = (int)(r.izf & 0x7ffu);
  const unsigned f = (r.izf >> 11) & 0x1fu;
  c.mode = (int)(f & 3u);
  c.delta = (int)((f >> 2) & 3u) - 1;
  *dbl = (f & F_DOUBLE) ? 1 : 0;
  c.edrr = __half2float(__ushort_as_half((unsigned short)(r.izf >> 16)));
  c.temp = r.temp;
  c.drr = r.drr;
  c.j = j;
  return c;
}

/* A sample of a cell the listing kernel paints itself: its double decision,
 * when needed, on the spot. */
template <typename K>
__device__ __noinline__ K sample_key_inline(const cg_imap_params &p, const cg_imap_args &A, const float *phi, int ix,
                                            int iy, int iz, const cg_imap_cell &c, int dbl, int ns, int q,
                                            float inv_ns)
{
  int sx, sy, sz, s = -1;
  long long pix = 0;
  sub_of(q, ns, inv_ns, &sx, &sy, &sz);
  if (dbl || p.force_double || !cg_imap_sample_checked(&A, ix, iy, iz, &c, ns, sx, sy, sz, &s, &pix)) {
    float v[3];
    grad_phi(phi, ix, iy, iz, p.box.N, v);
    int j;
    double drr = 0;
    cgx_imap_cell(&A, ix, iy, iz, v, &j, &drr);
    cgx_imap_sample(&A, ix, iy, iz, ns, drr, sx, sy, sz, &s, &pix);
    atomicAdd(p.xstats + 3, 1ull);
  }
  return key_of<K>(p, s, pix);
}

template <typename K>
__global__ void __launch_bounds__(IW * 32) k_imap_list(const float *__restrict__ dens, const float *__restrict__ phi,
                                                       cg_imap_params p)
{
  extern __shared__ __align__(16) unsigned char sraw[];
  const Sh sh = load_shells(p, sraw, false);
  __syncthreads();
  const cg_imap_args A = args_with(p, sh);
  const int lane = threadIdx.x & 31;
  const int N = p.box.N;
  const int nrow = N * N, nch = (N + 31) / 32;
  const float rlo = A.rmin - 1.0f, rhi = A.rmax + 1.0f;
  unsigned long long drawn = 0, ndbl = 0;
  for (;;) {
    int rbeg = 0;
    if (lane == 0) rbeg = (int)atomicAdd(&p.ctr[1], (unsigned long long)ROWS);
    rbeg = __shfl_sync(FULL, rbeg, 0);
    if (rbeg >= nrow) break;
    const int rend = rbeg + ROWS < nrow ? rbeg + ROWS : nrow;
    for (int row = rbeg; row < rend; row++)
      for (int ch = 0; ch < nch; ch++) {
        const int iz = row / N, iy = row - iz * N;
        const int ix = ch * 32 + lane;
        cg_imap_cell c;
        bool want = false; /* listed and painted */
        int dbl = 0;
        float d = 0.0f;
        if (ix < N) {
          const float x0 = A.xc[ix], y0 = A.yc[iy], z0 = A.zc[iz];
          const float r2 = CG_FMA(z0, z0, CG_FMA(y0, y0, CG_MUL(x0, x0)));
          if (r2 >= rlo * rlo * (rlo > 0.0f ? 1.0f : 0.0f) && r2 <= rhi * rhi) {
            d = __ldg(&dens[pidx(ix, iy, iz, N)]);
            float v[3];
            grad_phi(phi, ix, iy, iz, N, v);
            int st = cg_imap_cell_checked(&A, ix, iy, iz, d, v, &c);
            if (p.force_double && st == 1) st = 2;
            if (st == 2) {
              ndbl++;
              int j;
              double drr;
              if (cgx_imap_cell(&A, ix, iy, iz, v, &j, &drr)) {
                c.j = j;
                c.temp = temp32(A, ix, iy, iz, d);
                c.drr = (float)drr;
                c.edrr = 0.0f;
                c.mode = CG_SH_WALK;
                c.delta = 0;
                dbl = 1;
                st = 1;
              } else {
                st = 0;
              }
            }
            if (st == 1) {
              const int ns = A.nsub[c.j + 1];
              drawn += (unsigned long long)ns * ns * ns;
              const int sfin = c.j + c.delta;
              want = !(c.mode == CG_SH_SINGLE && (sfin < 0 || sfin >= p.nr));
            }
          }
        }
        /* nothing to append (a chunk outside the shells' radial range, about
         * half of them): skip the bucket reservation */
        if (!__any_sync(FULL, want)) continue;
        /* append to the buckets: one atomic per bucket present in the warp,
         * issued together by each bucket's first lane (one round trip) */
        bool over = false;
        long long slot = 0;
        const int bk = want ? c.j + 1 : -1;
        const unsigned same = __match_any_sync(FULL, bk);
        const int leader = __ffs(same) - 1;
        unsigned long long old = 0;
        if (want && lane == leader) old = atomicAdd(&p.cnt[bk], (unsigned long long)__popc(same));
        old = __shfl_sync(FULL, old, leader);
        if (want) {
          const long long k = (long long)old + __popc(same & ((1u << lane) - 1u));
          if (k < p.cap[bk]) slot = p.base[bk] + k;
          else over = true;
        }
        if (want && !over)
          p.recs[slot] = pack(ix, iy, iz, c, (unsigned)c.mode | ((unsigned)(c.delta + 1) << 2) | (dbl ? F_DOUBLE : 0u));
        /* cells past their bucket's room: painted here by the warp */
        unsigned om = __ballot_sync(FULL, want && over);
        while (om) {
          const int l = __ffs(om) - 1;
          om &= om - 1;
          const int cx = __shfl_sync(FULL, ix, l);
          cg_imap_cell cc;
          cc.j = __shfl_sync(FULL, c.j, l);
          cc.temp = __shfl_sync(FULL, c.temp, l);
          cc.drr = __shfl_sync(FULL, c.drr, l);
          cc.edrr = __shfl_sync(FULL, c.edrr, l);
          cc.mode = __shfl_sync(FULL, c.mode, l);
          cc.delta = __shfl_sync(FULL, c.delta, l);
          const int cd = __shfl_sync(FULL, dbl, l);
          const int ns = A.nsub[cc.j + 1];
          const int n3 = ns * ns * ns;
          const float inv = sh.invns[cc.j + 1];
          const int tag = cx;
          for (int q0 = 0; q0 < n3; q0 += 32) {
            const int q = q0 + lane;
            K key = empty_key<K>();
            if (q < n3) key = sample_key_inline<K>(p, A, phi, cx, iy, iz, cc, cd, ns, q, inv);
            add_runs(key, tag, cc.temp, lane, p);
          }
          if (lane == 0) atomicAdd(&p.ctr[3], (unsigned long long)n3);
        }
      }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    drawn += __shfl_xor_sync(FULL, drawn, o);
    ndbl += __shfl_xor_sync(FULL, ndbl, o);
  }
  if (lane == 0) {
    if (drawn) atomicAdd(&p.ctr[2], drawn);
    if (ndbl) atomicAdd(p.xstats + 2, ndbl);
  }
}

/* Work units of a bucket of nsub ns: whole cells for ns <= 4 (8 to 64
 * samples), one z-slab of a cell for ns <= 32 (ns^2 samples), one x-line
 * beyond; each lane of a warp walks one unit. */
__host__ __device__ __forceinline__ long long units_per_cell(int ns)
{
  return ns <= 4 ? 1 : (ns <= 32 ? ns : (long long)ns * ns);
}

/* Unit groups of 32 per chunk so that a chunk is about CHS samples per lane
 * count: G = max(1, CHS / (32 x samples per unit)). */
__host__ __device__ __forceinline__ int groups_per_chunk(int ns)
{
  const int su = ns <= 4 ? ns * ns * ns : (ns <= 32 ? ns * ns : ns); /* samples per unit */
  const int g = CHS / (32 * su);
  return g > 1 ? g : 1;
}

/* Chunks of every bucket: 32 G units each. */
__global__ void k_imap_chunks(cg_imap_params p)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long acc = 0;
  for (int b = 0; b < p.nbk; b++) {
    p.chunk_off[b] = acc;
    const unsigned long long n = p.cnt[b] < (unsigned long long)p.cap[b] ? p.cnt[b] : (unsigned long long)p.cap[b];
    const int ns = p.a.nsub[b];
    const unsigned long long nu = n * (unsigned long long)units_per_cell(ns);
    const unsigned long long per = 32ull * (unsigned long long)groups_per_chunk(ns);
    acc += (nu + per - 1) / per;
  }
  p.chunk_off[p.nbk] = acc;
}

/* One sample for the double pass, queued on its own. */
__device__ __noinline__ void queue_one(const cg_imap_params &p, long long rec, int q)
{
  const unsigned long long k = atomicAdd(&p.ctr[4], 1ull);
  if ((long long)k < p.queue_cap) p.queue[k] = ((unsigned long long)rec << 30) | (unsigned long long)q;
  else atomicOr(p.err, ERR_IMAP_QUEUE);
}

/* This warp's queue stage in the painting kernel's shared memory. */
__device__ __forceinline__ unsigned long long *stage_of(const cg_imap_params &p)
{
  extern __shared__ __align__(16) unsigned char sraw[];
  return reinterpret_cast<unsigned long long *>(sraw + paint_stage_off(p.nr, p.nbk)) + (size_t)(threadIdx.x >> 5) * QB;
}

/* The warp's staged queue entries (qn of them, in shared memory) to the
 * double queue: one atomic per QB - 128 or more entries. */
__device__ __forceinline__ void queue_flush(const cg_imap_params &p, const unsigned long long *qb, int qn, int lane)
{
  __syncwarp();
  unsigned long long q0 = 0;
  if (lane == 0) q0 = atomicAdd(&p.ctr[4], (unsigned long long)qn);
  q0 = __shfl_sync(FULL, q0, 0);
  for (int i = lane; i < qn; i += 32) {
    if ((long long)(q0 + i) < p.queue_cap) p.queue[q0 + i] = qb[i];
    else atomicOr(p.err, ERR_IMAP_QUEUE);
  }
  __syncwarp();
}

/* Add a run of cnt samples of brightness temp to key k. */
template <typename K>
__device__ __forceinline__ void flush(const cg_imap_params &p, K k, unsigned cnt, float temp)
{
  if (cnt) {
    atomicAdd(&p.data[(long long)k], CG_MUL(temp, (float)cnt));
    atomicAdd(&p.nadd[(long long)k], (int)cnt);
  }
}

/* One sample at float position (x, y, z), sub-cell index q, of the lane's
 * cell: added to the lane's two (key, count) slots -- a key in a slot adds to
 * it, another key evicts the older slot to the maps -- or, when only double
 * can decide it, held (up to four per unit) or queued. */
template <typename K>
__device__ __forceinline__ void paint_sample(const cg_imap_params &p, const cg_imap_args &A, const cg_imap_cell &c,
                                             int dbl, long long rec, float x, float y, float z, int q, K &k0,
                                             unsigned &n0, K &k1, unsigned &n1, int &nf, int &f0, int &f1, int &f2,
                                             int &f3)
{
  int s = -1;
  long long pix = 0;
  if (dbl || !cg_imap_decide(&A, &c, x, y, z, &s, &pix)) {
    if (nf == 0) f0 = q;
    else if (nf == 1) f1 = q;
    else if (nf == 2) f2 = q;
    else if (nf == 3) f3 = q;
    else queue_one(p, rec, q);
    nf++;
    return;
  }
  const K key = key_of<K>(p, s, pix);
  if (key == empty_key<K>()) return;
  if (key == k0) {
    n0++;
  } else if (key == k1) {
    n1++;
  } else {
    flush<K>(p, k1, n1, c.temp);
    k1 = k0;
    n1 = n0;
    k0 = key;
    n0 = 1;
  }
}

/* The G unit groups of one chunk of bucket b (nsub ns).  Each lane walks one
 * unit (a cell, a slab or a line) sample by sample with its row coordinates
 * and the cell's fields held in registers.  Every lane of a warp runs the same sample loop,
 * so the samples that only double can decide are staged per warp in shared
 * memory (qb, qn entries) and queued in batches. */
template <typename K>
__device__ __forceinline__ void paint_chunk(const cg_imap_params &p, const cg_imap_args &A, int b, int ns,
                                            unsigned long long u0, int G, unsigned long long nu, float dxs, int lane,
                                            int &qn)
{
  const int U = (int)units_per_cell(ns);
  /* the chunk's first unit as (record, unit within it); later units are
   * within 32 G of it, so their offsets divide in 32 bits */
  const long long r0 = (long long)(u0 / (unsigned long long)U);
  const unsigned w0 = (unsigned)(u0 - (unsigned long long)r0 * (unsigned long long)U);
  for (int g = 0; g < G; g++) {
    const unsigned long long u = u0 + (unsigned long long)g * 32ull + (unsigned long long)lane;
    const bool valid = u < nu;
    /* the unit: record and its range of (sz, sy) */
    long long rl = 0;
    int z0 = 0, z1 = ns, y0 = 0, y1 = ns;
    if (valid) {
      if (U == 1) {
        rl = (long long)u;
      } else {
        const unsigned t = w0 + (unsigned)(g * 32 + lane);
        const unsigned dr = t / (unsigned)U;
        const int w = (int)(t - dr * (unsigned)U);
        rl = r0 + (long long)dr;
        if (ns <= 32) {
          z0 = w;
          z1 = w + 1;
        } else {
          z0 = w / ns;
          z1 = z0 + 1;
          y0 = w - z0 * ns;
          y1 = y0 + 1;
        }
      }
    }
    const long long rec = p.base[b] + rl;
    cg_imap_cell c;
    int ix = 0, iy = 0, iz = 0, dbl = 0;
    float xc = 0.0f, xl = 0.0f, yc = 0.0f, yl = 0.0f, zc = 0.0f, zl = 0.0f;
    if (valid) {
      c = unpack(p.recs[rec], b - 1, &ix, &iy, &iz, &dbl);
      dbl |= p.force_double;
      xc = A.xc[ix];
      xl = A.xl[ix];
      yc = A.yc[iy];
      yl = A.yl[iy];
      zc = A.zc[iz];
      zl = A.zl[iz];
    } else {
      c.temp = 0.0f;
      c.drr = 0.0f;
      c.edrr = 0.0f;
      c.j = b - 1;
      c.mode = CG_SH_SINGLE;
      c.delta = 0;
    }
    K k0 = empty_key<K>(), k1 = empty_key<K>();
    unsigned n0 = 0, n1 = 0;
    /* samples only double can decide: up to four per lane held here and
     * queued after the unit, the rest queued at once */
    int nf = 0, f0 = 0, f1 = 0, f2 = 0, f3 = 0;
    if (valid) {
      for (int sz = z0; sz < z1; sz++) {
        const float z = CG_ADD(zc, CG_FMA(CG_ADD((float)sz, 0.5f), dxs, zl));
        for (int sy = y0; sy < y1; sy++) {
          const float y = CG_ADD(yc, CG_FMA(CG_ADD((float)sy, 0.5f), dxs, yl));
          float fsx = 0.5f; /* sx + 1/2, exact, without a conversion per sample */
          /* unrolled by 3: half the samples of a 1024^3 run are in cells of
           * nsub 2 and 3; copies per nsub, or unrolled by 2 or 4, measured
           * slower (instruction fetch) */
#pragma unroll 3
          for (int sx = 0; sx < ns; sx++, fsx = CG_ADD(fsx, 1.0f))
            paint_sample<K>(p, A, c, dbl, rec, CG_ADD(xc, CG_FMA(fsx, dxs, xl)), y, z, sx + ns * (sy + ns * sz), k0,
                            n0, k1, n1, nf, f0, f1, f2, f3);
        }
      }
    }
    flush<K>(p, k0, n0, c.temp);
    flush<K>(p, k1, n1, c.temp);
    /* the held samples (most units hold none) to the warp's stage; at most
     * 128 per group, so a stage past QB - 128 entries is queued first */
    const int held = nf < 4 ? nf : 4;
    if (__any_sync(FULL, held > 0)) {
      int incl = held;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
      }
      const int tot = __shfl_sync(FULL, incl, 31);
      unsigned long long *qb = stage_of(p);
      if (qn + tot > QB) {
        queue_flush(p, qb, qn, lane);
        qn = 0;
      }
      const int o = qn + incl - held;
      for (int h = 0; h < held; h++)
        qb[o + h] = ((unsigned long long)rec << 30) | (unsigned long long)(h == 0 ? f0 : (h == 1 ? f1 : (h == 2 ? f2 : f3)));
      qn += tot;
    }
  }
}

/* Warps take chunks in bucket order; paint_chunk paints one. */
template <typename K>
__global__ void __launch_bounds__(IW * 32, 8) k_imap_paint(cg_imap_params p)
{
  extern __shared__ __align__(16) unsigned char sraw[];
  const Sh sh = load_shells(p, sraw, true);
  __syncthreads();
  const cg_imap_args A = args_with(p, sh);
  const int lane = threadIdx.x & 31;
  const unsigned long long total = sh.chunk_off[p.nbk];
  int qn = 0;
  for (;;) {
    unsigned long long ck = 0;
    if (lane == 0) ck = atomicAdd(&p.ctr[0], 1ull);
    ck = __shfl_sync(FULL, ck, 0);
    if (ck >= total) break;
    /* the bucket: last b with chunk_off[b] <= ck */
    int lo = 0, hi = p.nbk - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sh.chunk_off[mid] <= ck) lo = mid;
      else hi = mid - 1;
    }
    const int b = lo;
    const unsigned long long nrec =
        p.cnt[b] < (unsigned long long)p.cap[b] ? p.cnt[b] : (unsigned long long)p.cap[b];
    const int ns = sh.nsub[b];
    const unsigned long long nu = nrec * (unsigned long long)units_per_cell(ns);
    const int G = groups_per_chunk(ns);
    const float dxs = sh.dxs[b];
    const unsigned long long u0 = (ck - sh.chunk_off[b]) * 32ull * (unsigned long long)G;
    paint_chunk<K>(p, A, b, ns, u0, G, nu, dxs, lane, qn);
  }
  if (qn) queue_flush(p, stage_of(p), qn, lane);
}

/* The samples of one warp batch (n <= 32 entries of the queue's form) in
 * double: the cell's radial shift (imap.c:196-198), taken by the first lane
 * of each run of one record and handed to the rest of the run, then the
 * sample's shell and pixel (imap.c:210-231). */
__device__ __forceinline__ void double_batch(const float *__restrict__ phi, const cg_imap_params &p,
                                             const cg_imap_args &A, const Sh &sh, const long long *sbase,
                                             unsigned long long e, bool valid, int lane)
{
  const long long rec = (long long)(e >> 30);
  const int q = (int)(e & ((1ull << 30) - 1));
  const long long prev = __shfl_up_sync(FULL, rec, 1);
  const bool lead = valid && (lane == 0 || prev != rec);
  const unsigned lm = __ballot_sync(FULL, lead);
  const unsigned le = lm & (lane == 31 ? FULL : ((2u << lane) - 1u));
  const int src = valid ? 31 - __clz(le) : lane;
  int lo = 0, ix = 0, iy = 0, iz = 0;
  float temp = 0.0f;
  double drr = 0;
  if (lead) {
    /* the record's bucket: last b with base[b] <= rec */
    int hi = p.nbk - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sbase[mid] <= rec) lo = mid;
      else hi = mid - 1;
    }
    int dbl;
    const cg_imap_cell c = unpack(p.recs[rec], lo - 1, &ix, &iy, &iz, &dbl);
    temp = c.temp;
    float v[3];
    grad_phi(phi, ix, iy, iz, p.box.N, v);
    int j;
    cgx_imap_cell(&A, ix, iy, iz, v, &j, &drr);
  }
  lo = __shfl_sync(FULL, lo, src);
  ix = __shfl_sync(FULL, ix, src);
  iy = __shfl_sync(FULL, iy, src);
  iz = __shfl_sync(FULL, iz, src);
  temp = __shfl_sync(FULL, temp, src);
  drr = __shfl_sync(FULL, drr, src);
  if (!valid) return;
  const int ns = sh.nsub[lo];
  int s = -1, sx, sy, sz;
  sub_of(q, ns, sh.invns[lo], &sx, &sy, &sz);
  long long pix = 0;
  cgx_imap_sample(&A, ix, iy, iz, ns, drr, sx, sy, sz, &s, &pix);
  if (s >= 0 && s < p.nr) {
    const long long key = (long long)s * p.npix + pix;
    atomicAdd(&p.data[key], temp);
    atomicAdd(&p.nadd[key], 1);
  }
}

constexpr int DB_WARPS = 8; /* warps per block of k_imap_double */

/* The queued samples: first again in float-float (cg_imap_decide_ff), which
 * settles all but ~1e-9 of the pixels the float margins left open; the rest
 * -- shells within the float radial shift's bound of an edge, and every
 * sample of a cell listed in double -- are gathered per warp in shared
 * memory and decided in double 32 at a time, so that the FP64 work runs in
 * full warps. */
__global__ void __launch_bounds__(DB_WARPS * 32) k_imap_double(const float *__restrict__ phi, cg_imap_params p)
{
  extern __shared__ __align__(16) unsigned char sraw[];
  const Sh sh = load_shells(p, sraw, false);
  long long *sbase = reinterpret_cast<long long *>(sh.chunk_off); /* the buckets' first records */
  for (int i = threadIdx.x; i < p.nbk; i += blockDim.x) sbase[i] = p.base[i];
  __syncthreads();
  const cg_imap_args A = args_with(p, sh);
  unsigned long long *db = reinterpret_cast<unsigned long long *>(sraw + double_stage_off(p.nr, p.nbk)) +
                           (size_t)(threadIdx.x >> 5) * 64;
  const unsigned long long nq0 = p.ctr[4];
  const long long nq = (long long)nq0 < p.queue_cap ? (long long)nq0 : p.queue_cap;
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  int dn = 0; /* entries gathered for double (warp-uniform) */
  unsigned long long ndbl = 0;
  for (long long kb = (long long)blockIdx.x * blockDim.x + threadIdx.x - lane; kb < nq; kb += stride) {
    const long long k = kb + lane;
    const bool valid = k < nq;
    const unsigned long long e = valid ? p.queue[k] : ~0ull;
    bool need = valid;
    if (valid && !p.force_double) {
      const long long rec = (long long)(e >> 30);
      const int q = (int)(e & ((1ull << 30) - 1));
      int lo = 0, hi = p.nbk - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sbase[mid] <= rec) lo = mid;
        else hi = mid - 1;
      }
      int ix, iy, iz, dbl;
      const cg_imap_cell c = unpack(p.recs[rec], lo - 1, &ix, &iy, &iz, &dbl);
      if (!dbl) {
        const int ns = sh.nsub[lo];
        int s = -1, sx, sy, sz;
        long long pix = 0;
        sub_of(q, ns, sh.invns[lo], &sx, &sy, &sz);
        if (cg_imap_decide_ff(&A, &c, ix, iy, iz, sx, sy, sz, &s, &pix)) {
          need = false;
          if (s >= 0 && s < p.nr) {
            const long long key = (long long)s * p.npix + pix;
            atomicAdd(&p.data[key], c.temp);
            atomicAdd(&p.nadd[key], 1);
          }
        }
      }
    }
    const unsigned nm = __ballot_sync(FULL, need);
    if (!nm) continue;
    if (need) db[dn + __popc(nm & ((1u << lane) - 1u))] = e;
    dn += __popc(nm);
    ndbl += lane == 0 ? (unsigned long long)__popc(nm) : 0ull;
    __syncwarp();
    if (dn >= 32) {
      double_batch(phi, p, A, sh, sbase, db[lane], true, lane);
      __syncwarp();
      if (lane < dn - 32) db[lane] = db[lane + 32];
      dn -= 32;
      __syncwarp();
    }
  }
  if (dn > 0) double_batch(phi, p, A, sh, sbase, lane < dn ? db[lane] : ~0ull, lane < dn, lane);
  if (ndbl) atomicAdd(p.xstats + 3, ndbl);
}

template <typename K>
cudaError_t launch(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  cudaError_t e = cudaMemsetAsync(p->ctr, 0, 5 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(p->cnt, 0, (size_t)p->nbk * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const size_t sm_list = shell_smem(p->nr, p->nbk, false), sm_paint = paint_smem(p->nr, p->nbk);
  const size_t sm_double = double_stage_off(p->nr, p->nbk) + (size_t)DB_WARPS * 64 * 8;
  if ((e = cudaFuncSetAttribute(k_imap_list<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_list)) ||
      (e = cudaFuncSetAttribute(k_imap_paint<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_paint)) ||
      (e = cudaFuncSetAttribute(k_imap_double, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_double)))
    return e;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_imap_list<K>, IW * 32, sm_list))) return e;
  const long long nrow = (long long)p->box.N * p->box.N;
  long long blocks = (nrow + IW * ROWS - 1) / (IW * ROWS);
  if (blocks > (long long)nsm * (per_sm > 0 ? per_sm : 1)) blocks = (long long)nsm * (per_sm > 0 ? per_sm : 1);
  k_imap_list<K><<<(unsigned)blocks, IW * 32, sm_list, s>>>(dens, phi, *p);
  k_imap_chunks<<<1, 32, 0, s>>>(*p);
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_imap_paint<K>, IW * 32, sm_paint))) return e;
  k_imap_paint<K><<<(unsigned)(nsm * (per_sm > 0 ? per_sm : 1)), IW * 32, sm_paint, s>>>(*p);
  k_imap_double<<<(unsigned)(nsm * 4), DB_WARPS * 32, sm_double, s>>>(phi, *p);
  return cudaGetLastError();
}

/* RING pixels of float directions by the margin-checked single-precision
 * decision, on the device. */
__global__ void k_pix_checked(int nside, const float *__restrict__ xyz, long long n, float ein, long long *pix)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    cg_dir d = cg_dir_of(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
    d.ecth = CG_FMA(2.0f, ein, d.ecth);
    pix[i] = cg_pix_checked(&d, nside, ein);
  }
}

} /* namespace */

cudaError_t cg_pix_checked_dev(cudaStream_t s, int nside, const float *xyz, long long n, float ein, long long *pix,
                               int nsm)
{
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  k_pix_checked<<<(unsigned)blocks, 256, 0, s>>>(nside, xyz, n, ein, pix);
  return cudaGetLastError();
}

size_t cg_imap_shell_smem(int nr, int nbk) { return paint_smem(nr, nbk); }

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  if (!p->ctr || !p->recs || !p->queue) return cudaErrorInvalidValue;
  /* 32-bit keys when every (shell, pixel) index and the empty key fit */
  if ((unsigned long long)p->nr * (unsigned long long)p->npix < 0xffffffffull)
    return launch<unsigned int>(s, dens, phi, p, nsm);
  return launch<unsigned long long>(s, dens, phi, p, nsm);
}
