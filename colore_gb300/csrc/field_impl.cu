/*
 * field_impl.cu -- Gaussian field (fourier.c:285-423) and 1LPT displacement
 * transforms (density.c:376-445) for one grid size N = CG_N.
 *
 * This file is compiled once per supported grid size with -DCG_N=<N>; the
 * dispatcher in capi.cu selects the instantiation.  Three passes make the
 * 3-D c2r transform of the half spectrum H[kz][ky][kx] (kx in [0, N/2],
 * fastest) into the padded real grid, in place:
 *
 *   1. fill + z : a block owns TX consecutive kx at one ky and all kz.  It
 *                 generates the modes of every output field from one set of
 *                 Philox draws (fields after the first are parked in shared
 *                 memory), transforms along z and writes the result.  The
 *                 spectrum is never read back from HBM.
 *   2. y        : the same column transform along y, read-modify-write.
 *   3. x (c2r)  : a group of threads owns one row of N/2+1 complex values;
 *                 the Hermitian even/odd split turns the length-N real
 *                 inverse into a length-N/2 complex one.  The block's rows
 *                 (contiguous in HBM) are staged into shared memory by one
 *                 bulk copy of the copy engine.  The normalisation
 *                 (sqrt(2 pi)/L)^3 (fourier.c:383-398) and the partial sums
 *                 of <d> and <d^2> (fourier.c:24-79) are fused here.
 *
 * FFTW's c2r semantics for the kx = 0 and kx = N/2 planes (the imaginary
 * parts of each row's DC and Nyquist terms are ignored after the y and z
 * transforms) are reproduced by dropping those imaginary parts in pass 3.
 *
 * 2LPT (density.c:646-1031) adds the forward transform of the second-order
 * source: an r2c row pass along x, the forward y pass, and a z pass that
 * transforms forward, forms Psi2_a = -i k_a S_k / (N^3 k^2) for the three
 * axes and transforms each back along z; the inverse y and x passes follow.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "cg_tma.cuh"
#include "fft.cuh"
#include "field_api.h"
#include "fft_plans.h"

#ifndef CG_N
#error "compile with -DCG_N=<grid size>"
#endif

namespace {

using namespace cg;


constexpr int N = CG_N;
constexpr int NH = N / 2 + 1;
using PL = Plan<N>;
constexpr int P = N / PL::CR;       /* threads per column transform (y pass)      */
constexpr int PF = N / PL::FR;      /* threads per column transform (fill + z)    */
constexpr int LH = N / 2;           /* row transform length         */
constexpr int PR = LH / PL::RR;     /* threads per row transform    */
constexpr int ROWS = (NH > LH + LH / 32 + 1) ? NH : (LH + LH / 32 + 1); /* smem per row */

/* P(k) at log10 k, pk_linear0 (cosmo.c:291-308).  The interpolation branch
 * stops at numk-2: the reference also takes it for ik = numk-1 and then
 * reads one element past the table. */
__device__ __forceinline__ float pk_lin(const FillParams &p, float lgk)
{
  int ik = (int)((lgk - p.logkmin) * p.idlogk);
  if (ik < 0) return __ldg(&p.pk[0]) * exp10f(p.n_scal * (lgk - p.logkmin));
  if (ik < p.numk - 1) {
    float lk = p.logkmin + (float)ik / p.idlogk;
    float a = __ldg(&p.pk[ik]), b = __ldg(&p.pk[ik + 1]);
    return a + (lgk - lk) * (b - a) * p.idlogk;
  }
  return __ldg(&p.pk[p.numk - 1]) * exp10f(-3.0f * (lgk - p.logkmax));
}

__device__ __forceinline__ float kcomp(int i, int n, float dk) { return (float)(2 * i <= n ? i : i - n) * dk; }

/* Unsmoothed Gaussian mode (rng_delta_gauss, common.c:191-201, with
 * sigma^2 = P(k)/dk^3, fourier.c:343) and its |k|^2 and smoothing factor. */
__device__ __forceinline__ float2 gen_mode(const FillParams &p, int kx, int ky, int kz, float &k2, float &sm)
{
  float kxf = (float)kx * p.dk, kyf = kcomp(ky, N, p.dk), kzf = kcomp(kz, N, p.dk);
  k2 = kxf * kxf + kyf * kyf + kzf * kzf;
  sm = 1.0f;
  if (!(k2 > 0.0f)) return make_float2(0.0f, 0.0f);
  float lgk = 0.5f * log10f(k2);
  float s2 = pk_lin(p, lgk) * p.idk3;
  uint64_t m = (uint64_t)kx + (uint64_t)NH * ((uint64_t)ky + (uint64_t)N * (uint64_t)kz);
  cg_u32x4 w = cg_philox4x32_10((uint32_t)m, (uint32_t)(m >> 32), 0u, 0u, p.key0, p.key1);
  float u1 = cg_u01f(w.v[0]), u2 = cg_u01f(w.v[1]);
  float s, c;
  sincospif(2.0f * u1, &s, &c);
  float mod = sqrtf(-s2 * logf(1.0f - u2));
  if (p.do_smooth) sm = expf(-0.5f * p.r2s * k2);
  return make_float2(mod * c, mod * s);
}

/* Field values of one mode of the two-field fill: (delta_k, phi_k)
 * (fourier.c:337-352). */
template <int F>
__device__ __forceinline__ void gen_fields(const FillParams &p, int kx, int ky, int kz, float2 *f)
{
  static_assert(F == 2, "the three-field fills use lpt_base and lpt_field");
  float k2, sm;
  float2 d = gen_mode(p, kx, ky, kz, k2, sm);
  if (!(k2 > 0.0f)) {
#pragma unroll
    for (int j = 0; j < F; j++) f[j] = make_float2(0.0f, 0.0f);
    return;
  }
  float g = -p.prefac / k2;
  float2 phi = make_float2(g * d.x, g * d.y);
  if (p.do_smooth) {
    d.x *= sm;
    d.y *= sm;
    if (p.smooth_pot) {
      phi.x *= sm;
      phi.y *= sm;
    }
  }
  f[0] = d;
  f[1] = phi;
}

/* Pass 1: fill + z transform of F fields.  grid = (ceil(NH/TX), N).
 * Each thread first generates, in a rolled loop, the modes its stage-0
 * loads will read and parks every field in shared memory (one copy of the
 * generator in the instruction stream: inlined per register element it
 * overflowed the instruction cache); field 0's slot is also the exchange
 * buffer of the transforms, safe because a transform reads all its inputs
 * before its first exchange write. */
template <int F, int TX>
__global__ void __launch_bounds__(TX *PF) k_fill_z(float2 *o0, float2 *o1, float2 *o2, FillParams p,
                                                  const float2 *__restrict__ twN)
{
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % TX, t = threadIdx.x / TX;
  const int kx = blockIdx.x * TX + c, ky = blockIdx.y;
  const bool ok = kx < NH;
#pragma unroll 1
  for (int e = 0; e < PL::FR; e++) {
    const int i = e / PL::F0, q = e - i * PL::F0;
    const int pos = t + (N / PL::FR) * i + q * (N / PL::F0); /* cgfft::in_pos of stage 0 */
    float2 f[F];
    if (ok) {
      gen_fields<F>(p, kx, ky, pos, f);
    } else {
#pragma unroll
      for (int jj = 0; jj < F; jj++) f[jj] = make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int jj = 0; jj < F; jj++) smem[(size_t)jj * N * TX + pos * TX + c] = f[jj];
  }
  float2 *outs[3] = {o0, o1, o2};
  auto sm = [&](int pos) -> float2 & { return smem[pos * TX + c]; };
#pragma unroll
  for (int j = 0; j < F; j++) {
    auto ld = [&](int pos) -> float2 { return smem[(size_t)j * N * TX + pos * TX + c]; };
    float2 *o = outs[j];
    auto st = [&](int pos, float2 v) {
      if (ok) o[((size_t)pos * N + ky) * NH + kx] = v;
    };
    cgfft::transform<N, PL::FR, PL::F0, PL::F1, PL::F2, 1>(t, twN, ld, st, sm);
    __syncthreads();
  }
}

/* The three-field fills: 1LPT displacements i k_a delta'_k / (N^3 k^2)
 * (density.c:430-436), where delta'_k = r2c(delta_G) = N^3 norm H(delta_k)
 * and H is the Hermitian projection that the c2r applied on the kx = 0 and
 * kx = N/2 planes; with lpt_kind 1 or 2 the second derivatives
 * i k_i (i k_j delta'_k / (N^3 k^2)) of 2LPT (density.c:704-709), xx xy xz
 * or yy yz zz.  One value per mode is kept, b = delta'_k / (N^3 k^2) with
 * the smoothing (0 at k = 0), and each field is formed from it as the
 * transform loads it. */
__device__ __forceinline__ float2 lpt_base(const FillParams &p, int kx, int ky, int kz)
{
  float k2, sm;
  float2 d = gen_mode(p, kx, ky, kz, k2, sm);
  if (!(k2 > 0.0f)) return make_float2(0.0f, 0.0f);
  d.x *= sm;
  d.y *= sm;
  if (kx == 0 || kx == N / 2) {
    int ky2 = ky == 0 ? 0 : N - ky, kz2 = kz == 0 ? 0 : N - kz;
    float k2b, smb;
    float2 e = gen_mode(p, kx, ky2, kz2, k2b, smb);
    e.x *= smb;
    e.y *= smb;
    d = make_float2(0.5f * (d.x + e.x), 0.5f * (d.y - e.y));
  }
  const float s = p.lpt_norm / k2;
  return make_float2(s * d.x, s * d.y);
}

__device__ __forceinline__ float2 lpt_field(const FillParams &p, int j, int kx, int ky, int kz, float2 b)
{
  const float kv[3] = {(float)kx * p.dk, kcomp(ky, N, p.dk), kcomp(kz, N, p.dk)};
  if (p.lpt_kind == 0) return make_float2(-kv[j] * b.y, kv[j] * b.x);
  const float ki[3] = {p.lpt_kind == 1 ? kv[0] : kv[1], p.lpt_kind == 1 ? kv[0] : kv[1], p.lpt_kind == 1 ? kv[0] : kv[2]};
  const float kj[3] = {p.lpt_kind == 1 ? kv[0] : kv[1], p.lpt_kind == 1 ? kv[1] : kv[2], kv[2]};
  const float g = -ki[j] * kj[j];
  return make_float2(g * b.x, g * b.y);
}

/* Pass 1 of the three-field fills: as k_fill_z, but each thread parks one
 * value per mode (lpt_base) in the second shared-memory slot and the first
 * stage of each transform forms the field from it (lpt_field); the first
 * slot is the exchange buffer.  Two slots instead of three per block, so
 * three blocks fit on an SM. */
template <int TX>
__global__ void __launch_bounds__(TX *PF, 3) k_fill_z3(float2 *o0, float2 *o1, float2 *o2, FillParams p,
                                                       const float2 *__restrict__ twN)
{
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % TX, t = threadIdx.x / TX;
  const int kx = blockIdx.x * TX + c, ky = blockIdx.y;
  const bool ok = kx < NH;
  float2 *base = smem + (size_t)N * TX;
#pragma unroll 1
  for (int e = 0; e < PL::FR; e++) {
    const int i = e / PL::F0, q = e - i * PL::F0;
    const int pos = t + (N / PL::FR) * i + q * (N / PL::F0); /* cgfft::in_pos of stage 0 */
    base[pos * TX + c] = ok ? lpt_base(p, kx, ky, pos) : make_float2(0.0f, 0.0f);
  }
  float2 *outs[3] = {o0, o1, o2};
  auto sm = [&](int pos) -> float2 & { return smem[pos * TX + c]; };
#pragma unroll
  for (int j = 0; j < 3; j++) {
    auto ld = [&](int pos) -> float2 { return lpt_field(p, j, kx, ky, pos, base[pos * TX + c]); };
    float2 *o = outs[j];
    auto st = [&](int pos, float2 v) {
      if (ok) o[((size_t)pos * N + ky) * NH + kx] = v;
    };
    cgfft::transform<N, PL::FR, PL::F0, PL::F1, PL::F2, 1>(t, twN, ld, st, sm);
    __syncthreads();
  }
}

/* Pass 2: in-place column transform along y (inverse, S = 1, or forward,
 * S = -1).  grid = (ceil(NH/TX), N, nf). */
template <int TX, int S>
__global__ void __launch_bounds__(TX *P) k_col_y(float2 *f0, float2 *f1, float2 *f2,
                                                 const float2 *__restrict__ twN)
{
  extern __shared__ float2 smem[];
  const int c = threadIdx.x % TX, t = threadIdx.x / TX;
  const int kx = blockIdx.x * TX + c, z = blockIdx.y;
  const bool ok = kx < NH;
  float2 *f = blockIdx.z == 0 ? f0 : (blockIdx.z == 1 ? f1 : f2);
  float2 *base = f + (size_t)z * N * NH + kx;
  auto sm = [&](int pos) -> float2 & { return smem[pos * TX + c]; };
  auto ld = [&](int pos) -> float2 { return ok ? base[(size_t)pos * NH] : make_float2(0.0f, 0.0f); };
  auto st = [&](int pos, float2 v) {
    if (ok) base[(size_t)pos * NH] = v;
  };
  cgfft::transform<N, PL::CR, PL::C0, PL::C1, PL::C2, S>(t, twN, ld, st, sm);
}

/* Forward pass 1 of the 2LPT source: row r2c along x, in place.  A row's N
 * reals are read as N/2 complex z_j = x_2j + i x_2j+1, transformed forward,
 * and split into the N/2 + 1 modes
 *   X_k = (E_k - i e^{-2 pi i k/N} O_k) / 2,  E_k = Z_k + conj Z_{N/2-k},
 *   O_k = Z_k - conj Z_{N/2-k}  (Z_{N/2} = Z_0).
 * The half-length spectrum goes to its own shared buffer: the exchange
 * buffer may still be read by other threads when the last stage stores. */
__global__ void __launch_bounds__(PL::RB *PR) k_row_r2c(float2 *f, const float2 *__restrict__ twN,
                                                        const float2 *__restrict__ twH, unsigned int *err)
{
  extern __shared__ __align__(16) float2 smem[];
  __shared__ uint64_t bar;
  float2 *zb = smem + PL::RB * ROWS;
  const int t = threadIdx.x % PR, rl = threadIdx.x / PR;
  const size_t row0 = (size_t)blockIdx.x * PL::RB;
  if (!cgtma::stage_rows(smem, f + row0 * NH, (unsigned)(PL::RB * NH * sizeof(float2)), &bar, err)) return;
  const float2 *rin = smem + rl * NH;
  float2 *row = smem + rl * ROWS;
  float2 *z = zb + rl * LH;
  auto ld = [&](int j) -> float2 { return rin[j]; };
  auto sm = [&](int pos) -> float2 & { return row[pos + (pos >> 5)]; };
  auto st = [&](int n, float2 v) { z[n] = v; };
  cgfft::transform<LH, PL::RR, PL::R0, PL::R1, PL::R2, -1>(t, twH, ld, st, sm);
  __syncthreads();
  float2 *dst = f + (row0 + rl) * NH;
  for (int k = t; k <= LH; k += PR) {
    const float2 a = z[k == LH ? 0 : k], b = z[k == 0 ? 0 : LH - k];
    const float2 e = make_float2(a.x + b.x, a.y - b.y), o = make_float2(a.x - b.x, a.y + b.y);
    const float2 w = __ldg(&twN[k]); /* exp(+2 pi i k/N); the split takes its conjugate */
    const float2 wo = make_float2(w.x * o.x + w.y * o.y, w.x * o.y - w.y * o.x);
    dst[k] = make_float2(0.5f * (e.x + wo.y), 0.5f * (e.y - wo.x));
  }
}

/* Forward z pass of the 2LPT source with the second-order displacement
 * fill (density.c:764-809): per column (kx, ky) the forward transform along
 * z into shared memory, then for each axis a the product
 * -i k_a S_k / (N^3 k^2) (0 at k = 0) transformed back along z.
 * grid = (ceil(NH/TX), N). */
template <int TX>
__global__ void __launch_bounds__(TX *PF) k_z_lpt2(const float2 *__restrict__ src, float2 *o0, float2 *o1,
                                                   float2 *o2, float dk, float inv_n3,
                                                   const float2 *__restrict__ twN)
{
  extern __shared__ float2 smem[];
  float2 *X = smem + (size_t)N * TX;
  const int c = threadIdx.x % TX, t = threadIdx.x / TX;
  const int kx = blockIdx.x * TX + c, ky = blockIdx.y;
  const bool ok = kx < NH;
  auto sm = [&](int pos) -> float2 & { return smem[pos * TX + c]; };
  auto ld = [&](int pos) -> float2 { return ok ? src[((size_t)pos * N + ky) * NH + kx] : make_float2(0.0f, 0.0f); };
  auto stx = [&](int pos, float2 v) { X[pos * TX + c] = v; };
  cgfft::transform<N, PL::FR, PL::F0, PL::F1, PL::F2, -1>(t, twN, ld, stx, sm);
  __syncthreads();
  float2 *outs[3] = {o0, o1, o2};
  const float kxf = (float)kx * dk, kyf = kcomp(ky, N, dk);
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    auto ld2 = [&](int pos) -> float2 {
      const float kzf = kcomp(pos, N, dk);
      const float k2 = kxf * kxf + kyf * kyf + kzf * kzf;
      if (!(k2 > 0.0f)) return make_float2(0.0f, 0.0f);
      const float ka = a == 0 ? kxf : (a == 1 ? kyf : kzf);
      const float g = ka * inv_n3 / k2;
      const float2 v = X[pos * TX + c];
      return make_float2(g * v.y, -g * v.x); /* -i g v */
    };
    float2 *o = outs[a];
    auto st = [&](int pos, float2 v) {
      if (ok) o[((size_t)pos * N + ky) * NH + kx] = v;
    };
    cgfft::transform<N, PL::FR, PL::F0, PL::F1, PL::F2, 1>(t, twN, ld2, st, sm);
    __syncthreads();
  }
}

/* Pass 3: row c2r along x with normalisation and optional moment sums,
 * RB rows per block.  grid = (N*N/RB, nf).  partials[blockIdx.x] =
 * (sum d, sum d^2). */
template <bool STATS, int RB>
__global__ void __launch_bounds__(RB *PR) k_row_c2r(float2 *f0, float2 *f1, float2 *f2, float norm,
                                                        double2 *partials, const float2 *__restrict__ twN,
                                                        const float2 *__restrict__ twH, unsigned int *err)
{
  extern __shared__ __align__(16) float2 smem[];
  __shared__ uint64_t bar;
  const int t = threadIdx.x % PR, rl = threadIdx.x / PR;
  float2 *f = blockIdx.y == 0 ? f0 : (blockIdx.y == 1 ? f1 : f2);
  const size_t row0 = (size_t)blockIdx.x * RB;
  /* the block's rows, contiguous in HBM (RB NH float2, a multiple of 16
   * bytes at a 16-byte boundary since RB is even), in one bulk copy; they
   * land at a stride of NH and the transform then exchanges through the
   * same buffer at the padded stride ROWS, once every input is loaded */
  if (!cgtma::stage_rows(smem, f + row0 * NH, (unsigned)(RB * NH * sizeof(float2)), &bar, err)) return;
  const float2 *rin = smem + rl * NH;
  float2 *row = smem + rl * ROWS;
  float2 *dst = f + (row0 + rl) * NH;
  auto ld = [&](int j) -> float2 {
    float2 a = rin[j], b = rin[LH - j];
    if (j == 0) {
      a.y = 0.0f;
      b.y = 0.0f;
    }
    float2 e = make_float2(a.x + b.x, a.y - b.y);
    float2 o = make_float2(a.x - b.x, a.y + b.y);
    float2 w = __ldg(&twN[j]);
    float2 ow = make_float2(o.x * w.x - o.y * w.y, o.x * w.y + o.y * w.x);
    return make_float2(e.x - ow.y, e.y + ow.x);
  };
  auto sm = [&](int pos) -> float2 & { return row[pos + (pos >> 5)]; };
  float s1 = 0.0f, s2 = 0.0f;
  auto st = [&](int n, float2 v) {
    float2 r = make_float2(v.x * norm, v.y * norm);
    dst[n] = r;
    if (STATS) {
      s1 += r.x + r.y;
      s2 += r.x * r.x + r.y * r.y;
    }
  };
  cgfft::transform<LH, PL::RR, PL::R0, PL::R1, PL::R2, 1>(t, twH, ld, st, sm);
  if (STATS) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    __shared__ double red[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
      red[0][wid] = (double)s1;
      red[1][wid] = (double)s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < (RB * PR + 31) / 32; w++) {
        a += red[0][w];
        b += red[1][w];
      }
      partials[blockIdx.x] = make_double2(a, b);
    }
  }
}

template <class K>
cudaError_t prep(K kern, size_t smem)
{
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

/* ---- tile candidates of the autotuner ----------------------------------
 * Each pass has up to three tile widths: variant 0 is the plan's (fft_plans.h),
 * 1 half of it, 2 twice it.  A variant is valid when its shared memory fits
 * in 200 KiB and its block in 1024 threads (x pass: an even row count, for
 * the 16-byte bulk copy).  Only the block shape changes: every column and
 * row goes through the same transform, so all variants give the same bits.
 * The x pass that also sums the moments keeps the plan's RB, since the
 * per-block partial sums depend on it. */
constexpr size_t SMEM_MAX = 200u * 1024u;
constexpr int tile_of(int def, int v) { return v == 1 ? def / 2 : (v == 2 ? def * 2 : def); }
constexpr bool fill_ok(int T) { return T >= 1 && (size_t)2 * N * T * sizeof(float2) <= SMEM_MAX && T * PF <= 1024; }
constexpr bool y_ok(int T) { return T >= 1 && (size_t)N * T * sizeof(float2) <= SMEM_MAX && T * P <= 1024; }
constexpr bool x_ok(int R)
{
  return R >= 2 && R % 2 == 0 && ((size_t)N * N) % R == 0 && (size_t)R * ROWS * sizeof(float2) <= SMEM_MAX &&
         R * PR <= 1024;
}
static_assert(fill_ok(PL::TX2) && fill_ok(PL::TX3) && y_ok(PL::TXY) && x_ok(PL::RB), "plan out of limits");

template <int T>
cudaError_t fill2(const cg_field_launch *L)
{
  if constexpr (!fill_ok(T)) {
    return cudaErrorInvalidValue;
  } else {
    const size_t sm = (size_t)2 * N * T * sizeof(float2);
    cudaError_t e = prep(k_fill_z<2, T>, sm);
    if (e != cudaSuccess) return e;
    dim3 g((NH + T - 1) / T, N);
    k_fill_z<2, T><<<g, T * PF, sm, L->stream>>>(L->f[0], L->f[1], nullptr, L->fill, L->twN);
    return cudaGetLastError();
  }
}

template <int T>
cudaError_t fill3(const cg_field_launch *L)
{
  if constexpr (!fill_ok(T)) {
    return cudaErrorInvalidValue;
  } else {
    const size_t sm = (size_t)2 * N * T * sizeof(float2); /* one value per mode + the exchange buffer */
    cudaError_t e = prep(k_fill_z3<T>, sm);
    if (e != cudaSuccess) return e;
    dim3 g((NH + T - 1) / T, N);
    k_fill_z3<T><<<g, T * PF, sm, L->stream>>>(L->f[0], L->f[1], L->f[2], L->fill, L->twN);
    return cudaGetLastError();
  }
}

template <int T, int S>
cudaError_t ypass(const cg_field_launch *L, float2 *a, float2 *b, float2 *c, int nf)
{
  if constexpr (!y_ok(T)) {
    return cudaErrorInvalidValue;
  } else {
    const size_t sm = (size_t)N * T * sizeof(float2);
    cudaError_t e = prep(k_col_y<T, S>, sm);
    if (e != cudaSuccess) return e;
    dim3 g((NH + T - 1) / T, N, nf);
    k_col_y<T, S><<<g, T * P, sm, L->stream>>>(a, b, c, L->twN);
    return cudaGetLastError();
  }
}

template <bool STATS, int R>
cudaError_t xpass(const cg_field_launch *L, float2 *a, float2 *b, float2 *c, int nf, float norm, double2 *part)
{
  if constexpr (!x_ok(R)) {
    return cudaErrorInvalidValue;
  } else {
    const size_t sm = (size_t)R * ROWS * sizeof(float2);
    cudaError_t e = prep(k_row_c2r<STATS, R>, sm);
    if (e != cudaSuccess) return e;
    dim3 g((unsigned)((size_t)N * N / R), nf);
    k_row_c2r<STATS, R><<<g, R * PR, sm, L->stream>>>(a, b, c, norm, part, L->twN, L->twH, L->err);
    return cudaGetLastError();
  }
}

cudaError_t fill2_v(const cg_field_launch *L, int v)
{
  switch (v) {
    case 1: return fill2<tile_of(PL::TX2, 1)>(L);
    case 2: return fill2<tile_of(PL::TX2, 2)>(L);
    default: return fill2<PL::TX2>(L);
  }
}

cudaError_t fill3_v(const cg_field_launch *L, int v)
{
  switch (v) {
    case 1: return fill3<tile_of(PL::TX3, 1)>(L);
    case 2: return fill3<tile_of(PL::TX3, 2)>(L);
    default: return fill3<PL::TX3>(L);
  }
}

template <int S>
cudaError_t ypass_v(const cg_field_launch *L, int v, float2 *a, float2 *b, float2 *c, int nf)
{
  switch (v) {
    case 1: return ypass<tile_of(PL::TXY, 1), S>(L, a, b, c, nf);
    case 2: return ypass<tile_of(PL::TXY, 2), S>(L, a, b, c, nf);
    default: return ypass<PL::TXY, S>(L, a, b, c, nf);
  }
}

cudaError_t xpass_v(const cg_field_launch *L, int v, float2 *a, float2 *b, float2 *c, int nf)
{
  switch (v) {
    case 1: return xpass<false, tile_of(PL::RB, 1)>(L, a, b, c, nf, L->norm, nullptr);
    case 2: return xpass<false, tile_of(PL::RB, 2)>(L, a, b, c, nf, L->norm, nullptr);
    default: return xpass<false, PL::RB>(L, a, b, c, nf, L->norm, nullptr);
  }
}

} /* namespace */

#define CG_CAT2(a, b) a##b
#define CG_CAT(a, b) CG_CAT2(a, b)

/* Gaussian density and potential: passes 1-3 on both grids. */
extern "C" cudaError_t CG_CAT(cg_field_gauss_, CG_N)(const cg_field_launch *L)
{
  using namespace cg;
  cudaError_t e;
  if ((e = fill2_v(L, L->var[CG_PASS_FILL2])) != cudaSuccess) return e;
  if (L->ev) cudaEventRecord(L->ev[0], L->stream);
  if ((e = ypass_v<1>(L, L->var[CG_PASS_Y], L->f[0], L->f[1], nullptr, 2)) != cudaSuccess) return e;
  if (L->ev) cudaEventRecord(L->ev[1], L->stream);
  if ((e = xpass<true, PL::RB>(L, L->f[0], nullptr, nullptr, 1, L->norm, L->partials)) != cudaSuccess) return e;
  if ((e = xpass_v(L, L->var[CG_PASS_X], L->f[1], nullptr, nullptr, 1)) != cudaSuccess) return e;
  if (L->ev) cudaEventRecord(L->ev[2], L->stream);
  return cudaGetLastError();
}

/* 1LPT displacement fields Psi_x,y,z: passes 1-3 on three grids. */
extern "C" cudaError_t CG_CAT(cg_field_lpt_, CG_N)(const cg_field_launch *L)
{
  using namespace cg;
  cudaError_t e;
  if ((e = fill3_v(L, L->var[CG_PASS_FILL3])) != cudaSuccess) return e;
  if (L->ev) cudaEventRecord(L->ev[0], L->stream);
  if ((e = ypass_v<1>(L, L->var[CG_PASS_Y], L->f[0], L->f[1], L->f[2], 3)) != cudaSuccess) return e;
  if (L->ev) cudaEventRecord(L->ev[1], L->stream);
  if ((e = xpass_v(L, L->var[CG_PASS_X], L->f[0], L->f[1], L->f[2], 3)) != cudaSuccess) return e;
  if (L->ev) cudaEventRecord(L->ev[2], L->stream);
  return cudaGetLastError();
}

/* 2LPT second-order displacements from the source grid L->src (padded
 * real, overwritten): r2c along x, forward y, the fused z pass into
 * L->f[0..2], then the inverse y and x passes of those three grids. */
extern "C" cudaError_t CG_CAT(cg_field_lpt2_, CG_N)(const cg_field_launch *L)
{
  using namespace cg;
  constexpr int TX3 = PL::TX3;
  size_t smr = (size_t)PL::RB * (ROWS + LH) * sizeof(float2);
  size_t smz = (size_t)2 * N * TX3 * sizeof(float2);
  cudaError_t e;
  if ((e = prep(k_row_r2c, smr)) != cudaSuccess) return e;
  if ((e = prep(k_z_lpt2<TX3>, smz)) != cudaSuccess) return e;
  dim3 gr((unsigned)((size_t)N * N / PL::RB), 1);
  k_row_r2c<<<gr, PL::RB * PR, smr, L->stream>>>(L->src, L->twN, L->twH, L->err);
  if ((e = ypass_v<-1>(L, L->var[CG_PASS_Y], L->src, nullptr, nullptr, 1)) != cudaSuccess) return e;
  dim3 gz((NH + TX3 - 1) / TX3, N);
  const float inv_n3 = 1.0f / ((float)N * (float)N * (float)N);
  k_z_lpt2<TX3><<<gz, TX3 * PF, smz, L->stream>>>(L->src, L->f[0], L->f[1], L->f[2], L->fill.dk, inv_n3, L->twN);
  if ((e = ypass_v<1>(L, L->var[CG_PASS_Y], L->f[0], L->f[1], L->f[2], 3)) != cudaSuccess) return e;
  cg_field_launch L1 = *L;
  L1.norm = 1.0f;
  if ((e = xpass_v(&L1, L->var[CG_PASS_X], L->f[0], L->f[1], L->f[2], 3)) != cudaSuccess) return e;
  return cudaGetLastError();
}

/* Number of blocks of the moment-sum pass (size of the partials array). */
extern "C" size_t CG_CAT(cg_field_npartials_, CG_N)(void) { return (size_t)N * N / PL::RB; }

/* Tile width of variant v of a pass (CG_PASS_*), or 0 when the variant is
 * not valid at this size. */
extern "C" int CG_CAT(cg_field_tile_, CG_N)(int pass, int v)
{
  if (v < 0 || v > 2) return 0;
  switch (pass) {
    case CG_PASS_FILL2: return fill_ok(tile_of(PL::TX2, v)) ? tile_of(PL::TX2, v) : 0;
    case CG_PASS_FILL3: return fill_ok(tile_of(PL::TX3, v)) ? tile_of(PL::TX3, v) : 0;
    case CG_PASS_Y: return y_ok(tile_of(PL::TXY, v)) ? tile_of(PL::TXY, v) : 0;
    case CG_PASS_X: return x_ok(tile_of(PL::RB, v)) ? tile_of(PL::RB, v) : 0;
  }
  return 0;
}

/* One pass alone with variant v, for timing: the fills write f[0..1] (two
 * fields) or f[0..2] (three); the y and x passes transform f[0..nf-1] in
 * place (inverse, no moment sums). */
extern "C" cudaError_t CG_CAT(cg_field_pass_, CG_N)(const cg_field_launch *L, int pass, int v, int nf)
{
  switch (pass) {
    case CG_PASS_FILL2: return fill2_v(L, v);
    case CG_PASS_FILL3: return fill3_v(L, v);
    case CG_PASS_Y: return ypass_v<1>(L, v, L->f[0], nf > 1 ? L->f[1] : nullptr, nf > 2 ? L->f[2] : nullptr, nf);
    case CG_PASS_X: return xpass_v(L, v, L->f[0], nf > 1 ? L->f[1] : nullptr, nf > 2 ? L->f[2] : nullptr, nf);
  }
  return cudaErrorInvalidValue;
}
