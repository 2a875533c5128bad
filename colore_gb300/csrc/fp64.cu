/*
 * fp64.cu -- the plain FP64 path of the driver sequence (src/main.c:66-125)
 * on the same GPU: the baseline that the FP32 path is measured against.
 *
 * Every per-element quantity is computed in double precision, one thread per
 * Fourier mode, cell, source, intensity-map cell or convergence pixel, with
 * the CUDA double-precision math library; transforms use cuFFT; no stage is
 * fused with another, so each reads and writes its grids in HBM.  The steps
 * and formulas are those of the reference:
 *
 *   k64_fill      create_grids_fourier            fourier.c:285-359
 *   c2r / r2c     cuFFT: a batched 2-D complex transform over (kz, ky) and a
 *                 batched 1-D real transform along x, so that the imaginary
 *                 parts of the kx = 0 and N/2 coefficients are dropped after
 *                 the (kz, ky) transforms, as the FFTW c2r of the reference
 *   k64_scale     normalisation and <d>, <d^2>    fourier.c:24-79, 401-423
 *   k64_density   lognormalize / densclip         density.c:1034-1103
 *   k64_lpt_mult, k64_cic   1LPT and its CIC      density.c:376-644, 64-105
 *   k64_bins      redshift-bin sums               density.c:1128-1211
 *   (host)        normalisation tables            density.c:1227-1355
 *   k64_count, k64_emit     Poisson sources       srcs.c:120-283, 386-416
 *   k64_beam_rsd  RSD at the sources              srcs.c:425-504, 634-662
 *   k64_imap      intensity maps, one atomic pair per sub-sample
 *                                                 imap.c:135-245
 *   k64_kappa     convergence                     kappa.c:78-175
 *
 * Random numbers come from the Philox streams of the FP32 path; the Poisson
 * deviate is drawn in double from the same uniforms (inversion below 10,
 * PTRS above), so a cell whose mean agrees draws the same count.  Sources
 * are written in an unspecified order (one atomic cursor).
 */
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/colore_cuda.h"
#include "cg_math.h"
#include "cg_cell.h"
#include "cg_exact.h"

struct cg64_ctx {
  cg_config cfg;
  int device = 0, N = 0, NH = 0, nsm = 0;
  cudaStream_t stream = nullptr;
  char err[512] = {0};
  /* FP64 tables on the device: r, z, D1, V1, 1/H, a(a2r), r(a2r), then per
   * population nz, bz, and per species tz, bz; then the norm tables */
  double *d_tab = nullptr;
  /* grids: padded real layout [z][y][2(N/2+1)] shared with the complex one */
  double *d_dens = nullptr, *d_npot = nullptr, *d_disp[3] = {nullptr, nullptr, nullptr}, *d_out = nullptr;
  double *d_stats = nullptr;
  unsigned long long *d_ncount = nullptr;
  double *d_zsum = nullptr, *d_bsum = nullptr;
  int *d_counts = nullptr;
  unsigned long long *d_total = nullptr;
  float4 *d_pos = nullptr;
  float *d_src = nullptr;
  long long cap = 0;
  long long nsrc[CG_NPOP_MAX] = {0};
  double *d_imap[CG_NPOP_MAX] = {nullptr};
  int *d_nadd[CG_NPOP_MAX] = {nullptr};
  int *d_cmap[CG_NPOP_MAX] = {nullptr};
  double *d_kmap = nullptr;
  unsigned int *d_err = nullptr;
  cufftHandle p2 = 0, p1c2r = 0, p1r2c = 0;
  std::vector<double> h_norm;   /* tracer tables, CG_NA each */
  std::vector<double> h_norm0f; /* edges per tracer          */
  float ms_last = 0.0f;
};

namespace {

constexpr int NA = CG_NA;

int fail(cg64_ctx *c, int code, const char *fmt, ...)
{
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

#define CU(c, call)                                                                                   \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) return fail((c), CG_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));       \
  } while (0)
#define CF(c, call)                                                                                   \
  do {                                                                                                \
    cufftResult r_ = (call);                                                                          \
    if (r_ != CUFFT_SUCCESS) return fail((c), CG_ECUDA, "%s: cufft error %d", #call, (int)r_);        \
  } while (0)

/* table slots in d_tab */
enum { T_R = 0, T_Z, T_D1, T_V1, T_IH, T_A, T_RA, T_BASE };

struct P64 {
  int N, NH;
  double L, dx, idx, pos[3], glob_idr, r_last;
  const double *tab;
  int ntr; /* tracers: n_srcs + n_imap */
};

__device__ __forceinline__ const double *tb(const P64 &p, int k) { return p.tab + (size_t)k * NA; }

/* get_bg, cosmo.c:30-38 */
__device__ double bg64(const P64 &p, int k, double f0, double ff, double r)
{
  if (r <= 0) return f0;
  if (r >= p.r_last) return ff;
  const double *f = tb(p, k), *ra = tb(p, T_R);
  int ir = (int)(r * p.glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - ra[ir]) * p.glob_idr;
}

__device__ double bias64(double d, double b, int model) /* common.h:414-431 */
{
  if (d <= -1) return 0;
  if (model == CG_BIAS_MODEL_EXPLIN) return d < 0 ? exp(b * d / (1 + d)) : 1 + b * d;
  if (model == CG_BIAS_MODEL_LIN) return 1 + b * d > 0 ? 1 + b * d : 0;
  return pow(1 + d, b);
}

__device__ __forceinline__ size_t pid(const P64 &p, int ix, int iy, int iz)
{
  return (size_t)ix + (size_t)(2 * p.NH) * ((size_t)iy + (size_t)p.N * iz);
}

__device__ __forceinline__ double kc(int i, int n, double dk) { return (2 * i <= n ? i : -(n - i)) * dk; }

struct Fill64 {
  int numk;
  double logkmin, logkmax, idlogk, n_scal, prefac, r2s;
  int smooth, smooth_pot;
  const double *pk;
  uint32_t k0, k1;
};

__global__ void k64_fill(P64 p, Fill64 f, double2 *dk, double2 *pk)
{
  const int N = p.N, NH = p.NH;
  const size_t nh = (size_t)N * N * NH;
  const double dkk = 2 * M_PI / p.L, idk3 = 1. / (dkk * dkk * dkk);
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nh; idx += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % NH), ky = (int)((idx / NH) % N), kz = (int)(idx / ((size_t)NH * N));
    const double x = kx * dkk, y = kc(ky, N, dkk), z = kc(kz, N, dkk);
    const double k2 = x * x + y * y + z * z;
    if (k2 <= 0) {
      dk[idx] = make_double2(0, 0);
      pk[idx] = make_double2(0, 0);
      continue;
    }
    /* pk_linear0, cosmo.c:291-308 (guarded at numk-1) */
    const double lgk = 0.5 * log10(k2);
    const int ik = (int)((lgk - f.logkmin) * f.idlogk);
    double pkv;
    if (ik < 0) pkv = f.pk[0] * pow(10., f.n_scal * (lgk - f.logkmin));
    else if (ik < f.numk - 1) {
      const double lk = f.logkmin + ik / f.idlogk;
      pkv = f.pk[ik] + (lgk - lk) * (f.pk[ik + 1] - f.pk[ik]) * f.idlogk;
    } else pkv = f.pk[f.numk - 1] * pow(10., -3 * (lgk - f.logkmax));
    const double s2 = pkv * idk3;
    const cg_u32x4 w = cg_philox4x32_10((uint32_t)idx, (uint32_t)((uint64_t)idx >> 32), 0u, 0u, f.k0, f.k1);
    const double ph = 2 * M_PI * (double)cg_u01f(w.v[0]);
    const double u = cg_u01f(w.v[1]);
    const double mod = sqrt(-s2 * log(1 - u)); /* rng_delta_gauss, common.c:191-201 */
    double sn, cs;
    sincos(ph, &sn, &cs);
    double dr = mod * cs, di = mod * sn;
    double pr = -f.prefac * dr / k2, pi = -f.prefac * di / k2;
    if (f.smooth) {
      const double sm = exp(-0.5 * f.r2s * k2);
      dr *= sm;
      di *= sm;
      if (f.smooth_pot) {
        pr *= sm;
        pi *= sm;
      }
    }
    dk[idx] = make_double2(dr, di);
    pk[idx] = make_double2(pr, pi);
  }
}

__global__ void k64_scale(P64 p, double *a, double *b, double norm, double *stats)
{
  const int N = p.N;
  const size_t ncell = (size_t)N * N * N;
  double s1 = 0, s2 = 0;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(c % N), iy = (int)((c / N) % N), iz = (int)(c / ((size_t)N * N));
    const size_t i = pid(p, ix, iy, iz);
    const double d = a[i] * norm;
    a[i] = d;
    b[i] *= norm;
    s1 += d;
    s2 += d * d;
  }
  __shared__ double r1[256], r2[256];
  r1[threadIdx.x] = s1;
  r2[threadIdx.x] = s2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      r1[threadIdx.x] += r1[threadIdx.x + s];
      r2[threadIdx.x] += r2[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&stats[0], r1[0]);
    atomicAdd(&stats[1], r2[0]);
  }
}

__device__ __forceinline__ void cell_xyz(const P64 &p, size_t c, int &ix, int &iy, int &iz, double &x0, double &y0,
                                         double &z0)
{
  const int N = p.N;
  ix = (int)(c % N);
  iy = (int)((c / N) % N);
  iz = (int)(c / ((size_t)N * N));
  x0 = ix * p.dx - p.pos[0];
  y0 = iy * p.dx - p.pos[1];
  z0 = iz * p.dx - p.pos[2];
}

__global__ void k64_density(P64 p, double *dens, const double *stats, int mode)
{
  const size_t ncell = (size_t)p.N * p.N * p.N;
  const double s1 = stats[0], s2 = stats[1], mean = s1 / ncell, sig2 = s2 / ncell - mean * mean;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    double x0, y0, z0;
    cell_xyz(p, c, ix, iy, iz, x0, y0, z0);
    const double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
    const double dg = bg64(p, T_D1, 1, tb(p, T_D1)[NA - 1], r);
    const size_t i = pid(p, ix, iy, iz);
    const double d = dens[i];
    if (mode == CG_DENS_CLIP) dens[i] = fmax(1 + dg * d, 0.0) - 1;
    else dens[i] = exp(dg * (d - 0.5 * dg * sig2)) - 1;
  }
}

/* c = i k_ax dk / (N^3 k^2), density.c:408-440 */
__global__ void k64_lpt_mult(P64 p, const double2 *dk, double2 *ck, int ax)
{
  const int N = p.N, NH = p.NH;
  const size_t nh = (size_t)N * N * NH;
  const double dkk = 2 * M_PI / p.L, fftnorm = (double)N * N * N;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nh; idx += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % NH), ky = (int)((idx / NH) % N), kz = (int)(idx / ((size_t)NH * N));
    const double kv[3] = {kx * dkk, kc(ky, N, dkk), kc(kz, N, dkk)};
    const double k2 = fftnorm * (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
    if (k2 <= 0) {
      ck[idx] = make_double2(0, 0);
      continue;
    }
    const double2 d = dk[idx];
    const double f = kv[ax] / k2;
    ck[idx] = make_double2(-f * d.y, f * d.x);
  }
}

__global__ void k64_zero(double *a, size_t n)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = 0;
}

/* positions (density.c:473-501) and CIC (density.c:64-105) */
__global__ void k64_cic(P64 p, const double *d0, const double *d1, const double *d2, double *out)
{
  const int N = p.N;
  const size_t ncell = (size_t)N * N * N;
  const double iag = N / p.L;
  const double *disp[3] = {d0, d1, d2};
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    double xv[3];
    cell_xyz(p, c, ix, iy, iz, xv[0], xv[1], xv[2]);
    const double r = sqrt(xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2]);
    const double g = bg64(p, T_D1, 1, tb(p, T_D1)[NA - 1], r);
    const size_t id = pid(p, ix, iy, iz);
    int i0[3], i1[3];
    double a0[3], a1[3];
    for (int ax = 0; ax < 3; ax++) {
      double q = xv[ax] + g * disp[ax][id] + p.pos[ax];
      if (q < 0) q += p.L;
      if (q >= p.L) q -= p.L;
      i0[ax] = (int)(q * iag);
      a1[ax] = q * iag - i0[ax];
      a0[ax] = 1 - a1[ax];
      i1[ax] = i0[ax] + 1;
      i0[ax] %= N;
      i1[ax] %= N;
      if (i0[ax] < 0) i0[ax] += N;
      if (i1[ax] < 0) i1[ax] += N;
    }
    atomicAdd(&out[pid(p, i0[0], i0[1], i0[2])], a0[0] * a0[1] * a0[2]);
    atomicAdd(&out[pid(p, i1[0], i0[1], i0[2])], a1[0] * a0[1] * a0[2]);
    atomicAdd(&out[pid(p, i0[0], i1[1], i0[2])], a0[0] * a1[1] * a0[2]);
    atomicAdd(&out[pid(p, i1[0], i1[1], i0[2])], a1[0] * a1[1] * a0[2]);
    atomicAdd(&out[pid(p, i0[0], i0[1], i1[2])], a0[0] * a0[1] * a1[2]);
    atomicAdd(&out[pid(p, i1[0], i0[1], i1[2])], a1[0] * a0[1] * a1[2]);
    atomicAdd(&out[pid(p, i0[0], i1[1], i1[2])], a0[0] * a1[1] * a1[2]);
    atomicAdd(&out[pid(p, i1[0], i1[1], i1[2])], a1[0] * a1[1] * a1[2]);
  }
}

__global__ void k64_minus1(P64 p, double *a)
{
  const size_t ncell = (size_t)p.N * p.N * p.N;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    const int N = p.N;
    a[pid(p, (int)(c % N), (int)((c / N) % N), (int)(c / ((size_t)N * N)))] -= 1;
  }
}

/* collect_density_normalization_from_grid, density.c:1128-1211 */
__global__ void k64_bins(P64 p, const double *dens, int nz, double idz, int bias_model, unsigned long long *ncount,
                         double *zsum, double *bsum)
{
  const size_t ncell = (size_t)p.N * p.N * p.N;
  const int nt = p.ntr;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    double x0, y0, z0;
    cell_xyz(p, c, ix, iy, iz, x0, y0, z0);
    const double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
    const double z = bg64(p, T_Z, 0, tb(p, T_Z)[NA - 1], r);
    const int b = (int)(z * idz) + 1;
    if (b < 0 || b >= nz) continue;
    const double d = dens[pid(p, ix, iy, iz)];
    atomicAdd(&ncount[b], 1ull);
    atomicAdd(&zsum[b], z);
    for (int t = 0; t < nt; t++) {
      const int k = T_BASE + 2 * t + 1; /* bz of tracer t */
      atomicAdd(&bsum[(size_t)t * nz + b], bias64(d, bg64(p, k, tb(p, k)[0], 1, r), bias_model));
    }
  }
}

/* Poisson deviate in double from the FP32 path's streams (cg_exact.h): the
 * cell's uniform from its word of the shared Philox block, inversion below
 * 10, PTRS (Hormann 1993) above. */
__device__ long long poisson64(double lam, uint32_t k0, uint32_t k1, long long cid)
{
  if (!(lam > 0)) return 0;
  return cgx_poisson(lam, (double)cg_u01f(cg_pois_word(cid, k0, k1)), cid, k0, k1);
}

struct Src64 {
  int ipop, bias_model, need_beaming, nside_base, nside_count;
  double rlim, cvol, fvel;
  uint32_t kp0, kp1, kq0, kq1;
};

__global__ void k64_count(P64 p, Src64 s, const double *dens, int *counts, unsigned long long *total,
                          unsigned int *err)
{
  const size_t ncell = (size_t)p.N * p.N * p.N;
  const int knz = T_BASE + 2 * s.ipop, kbz = knz + 1, knrm = T_BASE + 2 * p.ntr + s.ipop;
  unsigned long long t = 0;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    double x0, y0, z0;
    cell_xyz(p, c, ix, iy, iz, x0, y0, z0);
    const double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
    long long n = 0;
    if (r < s.rlim) {
      const double nd = bg64(p, knz, 0, 0, r);
      if (nd > 0) {
        const double lam = nd * s.cvol * bias64(dens[pid(p, ix, iy, iz)], bg64(p, kbz, tb(p, kbz)[0], 1, r), s.bias_model) *
                           bg64(p, knrm, p.tab[(size_t)(T_BASE + 3 * p.ntr) * NA + 2 * s.ipop],
                                p.tab[(size_t)(T_BASE + 3 * p.ntr) * NA + 2 * s.ipop + 1], r);
        n = poisson64(lam, s.kp0, s.kp1, (long long)c);
      }
    }
    if (n > 0x7fffffffLL) {
      atomicOr(err, 1u);
      n = 0;
    }
    counts[c] = (int)n;
    t += (unsigned long long)n;
  }
  atomicAdd(total, t);
}

__device__ void cart2sph64(double x, double y, double z, double *r, double *cth, double *phi)
{
  *r = sqrt(x * x + y * y + z * z);
  if (*r == 0) {
    *cth = 1;
    *phi = 0;
    return;
  }
  *cth = z / *r;
  *phi = atan2(y / *r, x / *r);
  if (*phi < 0) *phi += 2 * M_PI;
}

/* he_ang2pix in double, healpix_extra.c:118-172 */
__device__ long long ang2pix64(long long nside, double cth, double phi)
{
  const double ctha = fabs(cth), tp2 = 2 * M_PI;
  double ph = phi >= 0 ? (phi < tp2 ? phi : fmod(phi, tp2)) : fmod(phi, tp2) + tp2;
  if (ph == tp2) ph = 0;
  const double tt = ph * (2 / M_PI);
  if (ctha <= 2. / 3.) {
    const double t1 = nside * (0.5 + tt), t2 = nside * cth * 0.75;
    const long long jp = (long long)(t1 - t2), jm = (long long)(t1 + t2);
    const long long ir = nside + 1 + jp - jm, ks = 1 - (ir & 1);
    long long ip = (jp + jm - nside + ks + 1) / 2;
    ip %= 4 * nside;
    if (ip < 0) ip += 4 * nside;
    return nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip;
  }
  const double tp = tt - (long long)tt, tmp = nside * sqrt(3 * (1 - ctha));
  const long long jp = (long long)(tp * tmp), jm = (long long)((1.0 - tp) * tmp), ir = jp + jm + 1;
  long long ip = (long long)(tt * ir);
  ip %= 4 * ir;
  if (ip < 0) ip += 4 * ir;
  return cth > 0 ? 2 * ir * (ir - 1) + ip : 12 * nside * nside - 2 * ir * (ir + 1) + ip;
}

__device__ double rvel64(const P64 &p, const double *npot, int ix, int iy, int iz, double x0, double y0, double z0,
                         double rr)
{
  const int N = p.N;
  const int xh = (ix + 1) % N, xl = (ix + N - 1) % N, yh = (iy + 1) % N, yl = (iy + N - 1) % N, zh = (iz + 1) % N,
            zl = (iz + N - 1) % N;
  const double v0 = npot[pid(p, xh, iy, iz)] - npot[pid(p, xl, iy, iz)];
  const double v1 = npot[pid(p, ix, yh, iz)] - npot[pid(p, ix, yl, iz)];
  const double v2 = npot[pid(p, ix, iy, zh)] - npot[pid(p, ix, iy, zl)];
  const double u0 = x0 / rr, u1 = y0 / rr, u2 = z0 / rr; /* get_rvel, imap.c:65-73 */
  return 0.5 * p.idx * (v0 * u0 + v1 * u1 + v2 * u2);
}

/* srcs_set_cartesian_single pass 2 (srcs.c:186-283) with the local
 * properties of srcs_get_local_properties (srcs.c:386-416). */
__global__ void k64_emit(P64 p, Src64 s, const double *npot, const int *counts, unsigned long long *cursor,
                         long long cap, float4 *pos, float *src, int *cmap, unsigned int *err)
{
  const size_t ncell = (size_t)p.N * p.N * p.N;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    const int n = counts[c];
    if (n == 0) continue;
    int ix, iy, iz;
    double x0, y0, z0;
    cell_xyz(p, c, ix, iy, iz, x0, y0, z0);
    const double rr = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
    const double rv = s.fvel * rvel64(p, npot, ix, iy, iz, x0, y0, z0, rr);
    const double dz = rv * bg64(p, T_V1, tb(p, T_V1)[0], tb(p, T_V1)[NA - 1], rr);
    const unsigned long long id0 = atomicAdd(cursor, (unsigned long long)n);
    for (int j = 0; j < n; j++) {
      const long long id = (long long)id0 + j;
      if (id >= cap) {
        atomicOr(err, 2u);
        return;
      }
      const cg_u32x4 u = cg_philox4x32_10((uint32_t)c, (uint32_t)((uint64_t)c >> 32), (uint32_t)j, 0u, s.kq0, s.kq1);
      const double px = x0 + p.dx * ((double)cg_u01f(u.v[0]) - 0.5);
      const double py = y0 + p.dx * ((double)cg_u01f(u.v[1]) - 0.5);
      const double pz = z0 + p.dx * ((double)cg_u01f(u.v[2]) - 0.5);
      pos[id] = make_float4((float)px, (float)py, (float)pz, (float)dz);
      double r, cth, ph;
      cart2sph64(px, py, pz, &r, &cth, &ph);
      float *q = src + (size_t)id * 9;
      q[0] = (float)(ph * (180.0 / M_PI));
      q[1] = (float)(90.0 - acos(cth) * (180.0 / M_PI));
      q[2] = (float)bg64(p, T_Z, 0, tb(p, T_Z)[NA - 1], r);
      q[3] = s.need_beaming ? 0.0f : (float)dz;
      q[4] = s.need_beaming ? 0.0f : -1.0f;
      q[5] = s.need_beaming ? 0.0f : -1.0f;
      q[6] = q[7] = q[8] = 0.0f;
      if (cmap) atomicAdd(&cmap[ang2pix64(s.nside_count, cth, ph)], 1);
    }
  }
}

/* RSD at each source from the trilinear potential gradient (beaming.c:183-265,
 * srcs.c:500-504, 657-662). */
__global__ void k64_beam_rsd(P64 p, Src64 s, const double *npot, long long n, const float4 *pos, float *src)
{
  const int N = p.N;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 q = pos[i];
    const double x[3] = {q.x, q.y, q.z};
    const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    const double ir = 1.0 / (r > 0.001 ? r : 0.001);
    int i0[3], i1[3];
    double h0[3], h1[3], u[3];
    for (int a = 0; a < 3; a++) {
      const double xn = (x[a] + p.pos[a]) * p.idx;
      u[a] = x[a] * ir;
      i0[a] = (int)xn;
      h0[a] = xn - i0[a];
      h1[a] = 1 - h0[a];
      i1[a] = ((i0[a] + 1) % N + N) % N;
      i0[a] = (i0[a] % N + N) % N;
    }
    double v[3] = {0, 0, 0};
    for (int k = 0; k < 8; k++) {
      const int xc = (k & 1) ? i1[0] : i0[0], yc = (k & 2) ? i1[1] : i0[1], zc = (k & 4) ? i1[2] : i0[2];
      const double w = ((k & 1) ? h0[0] : h1[0]) * ((k & 2) ? h0[1] : h1[1]) * ((k & 4) ? h0[2] : h1[2]);
      v[0] += w * (npot[pid(p, (xc + 1) % N, yc, zc)] - npot[pid(p, (xc + N - 1) % N, yc, zc)]);
      v[1] += w * (npot[pid(p, xc, (yc + 1) % N, zc)] - npot[pid(p, xc, (yc + N - 1) % N, zc)]);
      v[2] += w * (npot[pid(p, xc, yc, (zc + 1) % N)] - npot[pid(p, xc, yc, (zc + N - 1) % N)]);
    }
    const double vr = 0.5 * p.idx * (v[0] * u[0] + v[1] * u[1] + v[2] * u[2]);
    float *q9 = src + (size_t)i * 9;
    /* r_of_z, cosmo.c:101-112 */
    const double z0 = q9[2], a = 1 / (1 + z0);
    double rz = 0;
    if (a < 1) {
      const double *aa = tb(p, T_A), *ra = tb(p, T_RA);
      const int ia = (int)(a * (NA - 1));
      rz = ra[ia] + (ra[ia + 1] - ra[ia]) * (a - aa[ia]) * (NA - 1);
    }
    q9[3] = (float)(vr * bg64(p, T_V1, tb(p, T_V1)[0], tb(p, T_V1)[NA - 1], rz) * s.fvel);
  }
}

struct Imap64 {
  int ipop, nr, nsub_lo, nsub_hi, bias_model;
  long long nside, npix;
  double rmin, rmax, fvel;
  const double *r0, *rf; /* sorted shells */
  const int *nsub;
};

__device__ int walk64(const Imap64 &m, double r, int start)
{
  int q = start < 0 ? 0 : (start >= m.nr ? m.nr - 1 : start);
  for (int it = 0; it < 2 * m.nr + 4; it++) {
    if (q == -1 || q == m.nr) return q;
    if (r < m.r0[q]) q--;
    else if (r >= m.rf[q]) q++;
    else return q;
  }
  return -1;
}

/* imap_set_cartesian_single, imap.c:135-245: one thread per cell, one
 * atomic pair per sub-sample */
__global__ void k64_imap(P64 p, Imap64 m, const double *dens, const double *npot, double *data, int *nadd)
{
  const size_t ncell = (size_t)p.N * p.N * p.N;
  const int kt = T_BASE + 2 * m.ipop, kb = kt + 1, knrm = T_BASE + 2 * p.ntr + m.ipop;
  const double *edge = p.tab + (size_t)(T_BASE + 3 * p.ntr) * NA;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    double x0, y0, z0;
    cell_xyz(p, c, ix, iy, iz, x0, y0, z0);
    const double rc = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
    const double tm = bg64(p, kt, 0, 0, rc);
    if (!(rc <= m.rmax && rc >= m.rmin && tm > 0)) continue;
    const double b = bg64(p, kb, tb(p, kb)[0], 1, rc);
    const double dn = bg64(p, knrm, edge[2 * m.ipop], edge[2 * m.ipop + 1], rc);
    const double rv = m.fvel * rvel64(p, npot, ix, iy, iz, x0, y0, z0, rc);
    const double drr = rv * bg64(p, T_V1, tb(p, T_V1)[0], tb(p, T_V1)[NA - 1], rc) *
                       bg64(p, T_IH, tb(p, T_IH)[0], tb(p, T_IH)[NA - 1], rc);
    const double temp = tm * bias64(dens[pid(p, ix, iy, iz)], b, m.bias_model) * dn;
    int irad = walk64(m, rc, 0);
    const int nsh = irad < 0 ? m.nsub_lo : (irad >= m.nr ? m.nsub_hi : m.nsub[irad]);
    const double dxs = p.dx / nsh;
    for (int izz = 0; izz < nsh; izz++)
      for (int iyy = 0; iyy < nsh; iyy++)
        for (int ixx = 0; ixx < nsh; ixx++) {
          double r, cth, ph;
          cart2sph64(x0 + (ixx + 0.5) * dxs, y0 + (iyy + 0.5) * dxs, z0 + (izz + 0.5) * dxs, &r, &cth, &ph);
          irad = walk64(m, r + drr, irad);
          if (irad >= 0 && irad < m.nr) {
            const long long k = irad * m.npix + ang2pix64(m.nside, cth, ph);
            atomicAdd(&data[k], temp);
            atomicAdd(&nadd[k], 1);
          }
        }
  }
}

struct Kap64 {
  int np, nr;
  long long nside, npix;
  double dr;
  int irmin[CG_NPLANES_MAX], irmax[CG_NPLANES_MAX];
  double inv[CG_NPLANES_MAX];
};

/* kappa_get_beam_properties, kappa.c:78-175: one thread per pixel */
__global__ void k64_kappa(P64 p, Kap64 k, const double *npot, double *map)
{
  const int N = p.N;
  for (long long ip = (long long)blockIdx.x * blockDim.x + threadIdx.x; ip < k.npix; ip += (long long)gridDim.x * blockDim.x) {
    int64_t jr, jp, nrg, ks;
    cg_nest_ringpos(k.nside, ip, &jr, &jp, &nrg, &ks);
    const double fact2 = 4.0 / (12.0 * k.nside * k.nside);
    double z;
    if (jr < k.nside) z = 1 - nrg * nrg * fact2;
    else if (jr > 3 * k.nside) z = nrg * nrg * fact2 - 1;
    else z = (2 * k.nside - jr) * 2.0 / (3.0 * k.nside);
    const double phi = (jp - (ks + 1) * 0.5) * (M_PI / 2) / nrg;
    const double sthz = sqrt((1 - z) * (1 + z));
    const double u[3] = {sthz * cos(phi), sthz * sin(phi), z};
    const double cth = u[2] > 1 ? 1 : (u[2] < -1 ? -1 : u[2]), sth = sqrt((1 - cth) * (1 + cth));
    double cph = 1, sph = 0;
    if (sth != 0) {
      cph = u[0] / sth;
      sph = u[1] / sth;
    }
    const double pf = p.idx * p.idx;
    const double rot[6] = {(cth * cth * cph * cph + sph * sph) * pf, (2 * cph * sph * (cth * cth - 1)) * pf,
                           (-2 * cth * sth * cph) * pf,            (cth * cth * sph * sph + cph * cph) * pf,
                           (-2 * cth * sth * sph) * pf,            (sth * sth) * pf};
    const long long ring = cg_nest2ring(k.nside, ip);
    double k1 = 0, k2 = 0;
    for (int pl = 0; pl < k.np; pl++) {
      for (int irr = k.irmin[pl]; irr <= k.irmax[pl]; irr++) {
        const double rm = (irr + 0.5) * k.dr;
        int cc[3];
        for (int a = 0; a < 3; a++) {
          const long long q = (long long)((rm * u[a] + p.pos[a]) * p.idx + 0.5);
          cc[a] = (int)(q >= N ? q - N : (q < 0 ? q + N : q));
        }
        const int x0 = cc[0], y0 = cc[1], z0 = cc[2];
        const int xh = (x0 + 1) % N, xl = (x0 + N - 1) % N, yh = (y0 + 1) % N, yl = (y0 + N - 1) % N,
                  zh = (z0 + 1) % N, zl = (z0 + N - 1) % N;
#define PP(X, Y, Z) npot[pid(p, X, Y, Z)]
        double t[6];
        t[0] = PP(xh, y0, z0) + PP(xl, y0, z0) - 2 * PP(x0, y0, z0);
        t[3] = PP(x0, yh, z0) + PP(x0, yl, z0) - 2 * PP(x0, y0, z0);
        t[5] = PP(x0, y0, zh) + PP(x0, y0, zl) - 2 * PP(x0, y0, z0);
        t[1] = 0.25 * (PP(xh, yh, z0) + PP(xl, yl, z0) - PP(xh, yl, z0) - PP(xl, yh, z0));
        t[2] = 0.25 * (PP(xh, y0, zh) + PP(xl, y0, zl) - PP(xh, y0, zl) - PP(xl, y0, zh));
        t[4] = 0.25 * (PP(x0, yh, zh) + PP(x0, yl, zl) - PP(x0, yh, zl) - PP(x0, yl, zh));
#undef PP
        double dot = 0;
        for (int a = 0; a < 6; a++) dot += rot[a] * t[a];
        const double pg = bg64(p, T_D1, 1, tb(p, T_D1)[NA - 1], rm) * (1 + bg64(p, T_Z, 0, tb(p, T_Z)[NA - 1], rm));
        k1 += dot * rm * pg * k.dr;
        k2 += dot * rm * rm * pg * k.dr;
      }
      map[(long long)pl * k.npix + ring] = k1 - k.inv[pl] * k2;
    }
  }
}

unsigned grid_for(long long n, int nsm) { return (unsigned)std::min<long long>((n + 255) / 256, (long long)nsm * 32); }

/* host get_bg in double (cosmo.c:30-38) */
double hbg(const cg_config &c, const double *f, double f0, double ff, double r)
{
  if (r <= 0) return f0;
  if (r >= c.r_arr_r2z[NA - 1]) return ff;
  int ir = (int)(r * c.glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - c.r_arr_r2z[ir]) * c.glob_idr;
}

P64 params(const cg64_ctx *c)
{
  P64 p;
  p.N = c->N;
  p.NH = c->NH;
  p.L = c->cfg.l_box;
  p.dx = c->cfg.l_box / c->N;
  p.idx = c->N / c->cfg.l_box;
  for (int a = 0; a < 3; a++) p.pos[a] = c->cfg.pos_obs[a];
  p.glob_idr = c->cfg.glob_idr;
  p.r_last = c->cfg.r_arr_r2z[NA - 1];
  p.tab = c->d_tab;
  p.ntr = c->cfg.n_srcs + c->cfg.n_imap;
  return p;
}

/* inverse (c2r) or forward (r2c) 3-D transform of the padded grid a */
int fft3(cg64_ctx *c, double *a, bool inverse)
{
  if (inverse) {
    CF(c, cufftExecZ2Z(c->p2, (cufftDoubleComplex *)a, (cufftDoubleComplex *)a, CUFFT_INVERSE));
    CF(c, cufftExecZ2D(c->p1c2r, (cufftDoubleComplex *)a, (cufftDoubleReal *)a));
  } else {
    CF(c, cufftExecD2Z(c->p1r2c, (cufftDoubleReal *)a, (cufftDoubleComplex *)a));
    CF(c, cufftExecZ2Z(c->p2, (cufftDoubleComplex *)a, (cufftDoubleComplex *)a, CUFFT_FORWARD));
  }
  return CG_OK;
}

int dalloc(cg64_ctx *c, void **p, size_t bytes)
{
  if (*p) return CG_OK;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return fail(c, CG_ENOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  return CG_OK;
}

/* Gaussian field and potential (create_cartesian_fields, fourier.c:361-423):
 * the fill, the two c2r transforms and the normalisation with the moments. */
int run_fields(cg64_ctx *c)
{
  const cg_config &cf = c->cfg;
  const int N = c->N, NH = c->NH, nsm = c->nsm;
  const size_t ncell = (size_t)N * N * N, nh = (size_t)N * N * NH, gbytes = nh * sizeof(double2);
  cudaStream_t s = c->stream;
  P64 p = params(c);
  int rc;
  if ((rc = dalloc(c, (void **)&c->d_dens, gbytes)) || (rc = dalloc(c, (void **)&c->d_npot, gbytes)) ||
      (rc = dalloc(c, (void **)&c->d_stats, 4 * sizeof(double))))
    return rc;
  /* Gaussian field and potential */
  Fill64 f;
  f.numk = cf.numk;
  f.logkmin = cf.logkmin;
  f.logkmax = cf.logkmax;
  f.idlogk = cf.idlogk;
  f.n_scal = cf.n_scal;
  f.prefac = cf.prefac_lensing;
  f.r2s = cf.r2_smooth;
  f.smooth = cf.do_smoothing;
  f.smooth_pot = cf.smooth_potential;
  f.pk = c->d_tab + (size_t)(T_BASE + 3 * p.ntr) * NA + 2 * CG_NPOP_MAX * 2;
  f.k0 = (uint32_t)cf.seed;
  f.k1 = (uint32_t)(cf.seed >> 32) ^ CG_STREAM_FIELD;
  k64_fill<<<grid_for((long long)nh, nsm), 256, 0, s>>>(p, f, (double2 *)c->d_dens, (double2 *)c->d_npot);
  CU(c, cudaGetLastError());
  if ((rc = fft3(c, c->d_dens, true)) || (rc = fft3(c, c->d_npot, true))) return rc;
  CU(c, cudaMemsetAsync(c->d_stats, 0, 4 * sizeof(double), s));
  const double norm = pow(sqrt(2 * M_PI) / cf.l_box, 3);
  k64_scale<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, c->d_dens, c->d_npot, norm, c->d_stats);
  CU(c, cudaGetLastError());
  return CG_OK;
}

int run(cg64_ctx *c)
{
  const cg_config &cf = c->cfg;
  const int N = c->N, NH = c->NH, nsm = c->nsm;
  const size_t ncell = (size_t)N * N * N, nh = (size_t)N * N * NH, gbytes = nh * sizeof(double2);
  cudaStream_t s = c->stream;
  P64 p = params(c);
  int rc;
  if ((rc = run_fields(c))) return rc;
  /* physical density */
  if (cf.dens_type == CG_DENS_1LPT) {
    for (int a = 0; a < 3; a++)
      if ((rc = dalloc(c, (void **)&c->d_disp[a], gbytes))) return rc;
    if ((rc = dalloc(c, (void **)&c->d_out, gbytes))) return rc;
    if ((rc = fft3(c, c->d_dens, false))) return rc; /* density.c:392 */
    for (int a = 0; a < 3; a++) {
      k64_lpt_mult<<<grid_for((long long)nh, nsm), 256, 0, s>>>(p, (const double2 *)c->d_dens, (double2 *)c->d_disp[a], a);
      CU(c, cudaGetLastError());
      if ((rc = fft3(c, c->d_disp[a], true))) return rc;
    }
    k64_zero<<<grid_for((long long)(2 * nh), nsm), 256, 0, s>>>(c->d_out, 2 * nh);
    k64_cic<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, c->d_disp[0], c->d_disp[1], c->d_disp[2], c->d_out);
    k64_minus1<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, c->d_out);
    CU(c, cudaGetLastError());
    std::swap(c->d_dens, c->d_out);
  } else {
    k64_density<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, c->d_dens, c->d_stats, cf.dens_type);
    CU(c, cudaGetLastError());
  }
  /* normalisation (density.c:1227-1355) */
  const int nts = cf.n_srcs, nti = cf.n_imap, nt = nts + nti;
  const double zmax = hbg(cf, cf.z_arr_r2z, 0, cf.z_arr_r2z[NA - 1], cf.l_box * 0.5);
  const int nz = (int)(zmax / 0.05) + 2;
  const double idz = (nz - 2) / zmax;
  if ((rc = dalloc(c, (void **)&c->d_ncount, 4096 * sizeof(unsigned long long))) ||
      (rc = dalloc(c, (void **)&c->d_zsum, 4096 * sizeof(double))) ||
      (rc = dalloc(c, (void **)&c->d_bsum, (size_t)4096 * 2 * CG_NPOP_MAX * sizeof(double))))
    return rc;
  if (nz > 4096) return fail(c, CG_EINVAL, "nz=%d", nz);
  CU(c, cudaMemsetAsync(c->d_ncount, 0, nz * sizeof(unsigned long long), s));
  CU(c, cudaMemsetAsync(c->d_zsum, 0, nz * sizeof(double), s));
  CU(c, cudaMemsetAsync(c->d_bsum, 0, (size_t)std::max(nt, 1) * nz * sizeof(double), s));
  k64_bins<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, c->d_dens, nz, idz, cf.bias_model, c->d_ncount,
                                                          c->d_zsum, c->d_bsum);
  CU(c, cudaGetLastError());
  std::vector<unsigned long long> narr(nz);
  std::vector<double> zz(nz), y((size_t)std::max(nt, 1) * nz);
  CU(c, cudaMemcpyAsync(narr.data(), c->d_ncount, nz * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CU(c, cudaMemcpyAsync(zz.data(), c->d_zsum, nz * sizeof(double), cudaMemcpyDeviceToHost, s));
  CU(c, cudaMemcpyAsync(y.data(), c->d_bsum, y.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CU(c, cudaStreamSynchronize(s));
  for (int iz = 0; iz < nz; iz++)
    if (narr[iz] > 0) {
      zz[iz] /= narr[iz];
      for (int t = 0; t < nt; t++) y[(size_t)t * nz + iz] = narr[iz] / y[(size_t)t * nz + iz];
    }
  zz[0] = 0;
  zz[nz - 1] = zmax;
  c->h_norm.assign((size_t)std::max(nt, 1) * NA, 0.0);
  c->h_norm0f.assign(2 * std::max(nt, 1), 0.0);
  for (int t = 0; t < nt; t++) {
    double *yt = y.data() + (size_t)t * nz;
    yt[0] = yt[1];
    yt[nz - 1] = yt[nz - 2];
    c->h_norm0f[2 * t] = yt[0];
    c->h_norm0f[2 * t + 1] = yt[nz - 1];
    for (int i = 0; i < NA; i++) {
      const double z = hbg(cf, cf.z_arr_r2z, 0, cf.z_arr_r2z[NA - 1], cf.r_arr_r2z[i]);
      double nm;
      if (z < zz[0]) nm = yt[0];
      else if (z >= zz[nz - 1]) nm = yt[nz - 1];
      else {
        int lo = 0, hi = nz - 1;
        while (hi > lo + 1) {
          int mid = (lo + hi) / 2;
          if (zz[mid] > z) hi = mid;
          else lo = mid;
        }
        nm = yt[lo] + (z - zz[lo]) * (yt[hi] - yt[lo]) / (zz[hi] - zz[lo]);
      }
      c->h_norm[(size_t)t * NA + i] = nm;
    }
  }
  if (nt > 0) {
    CU(c, cudaMemcpyAsync(c->d_tab + (size_t)(T_BASE + 2 * nt) * NA, c->h_norm.data(), (size_t)nt * NA * sizeof(double),
                          cudaMemcpyHostToDevice, s));
    CU(c, cudaMemcpyAsync(c->d_tab + (size_t)(T_BASE + 3 * nt) * NA, c->h_norm0f.data(), 2 * nt * sizeof(double),
                          cudaMemcpyHostToDevice, s));
  }
  /* sources */
  if ((rc = dalloc(c, (void **)&c->d_err, sizeof(unsigned int)))) return rc;
  unsigned int *d_err = c->d_err;
  CU(c, cudaMemsetAsync(d_err, 0, sizeof(unsigned int), s));
  if (nts > 0) {
    if ((rc = dalloc(c, (void **)&c->d_counts, ncell * sizeof(int))) ||
        (rc = dalloc(c, (void **)&c->d_total, 2 * sizeof(unsigned long long))))
      return rc;
  }
  for (int ip = 0; ip < nts; ip++) {
    Src64 sp;
    sp.ipop = ip;
    sp.bias_model = cf.bias_model;
    sp.need_beaming = cf.need_beaming;
    sp.nside_base = cf.nside_base;
    sp.nside_count = cf.nside_count[ip];
    sp.rlim = cf.l_box / 2 + 20.;
    sp.cvol = p.dx * p.dx * p.dx;
    sp.fvel = -cf.fgrowth_0 / (1.5 * cf.hubble_0 * cf.omega_m);
    sp.kp0 = (uint32_t)cf.seed;
    sp.kp1 = (uint32_t)(cf.seed >> 32) ^ (CG_STREAM_POIS + (uint32_t)ip);
    sp.kq0 = (uint32_t)cf.seed;
    sp.kq1 = (uint32_t)(cf.seed >> 32) ^ (CG_STREAM_POS + (uint32_t)ip);
    CU(c, cudaMemsetAsync(c->d_total, 0, 2 * sizeof(unsigned long long), s));
    k64_count<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, sp, c->d_dens, c->d_counts, c->d_total, d_err);
    CU(c, cudaGetLastError());
    unsigned long long tot = 0;
    CU(c, cudaMemcpyAsync(&tot, c->d_total, sizeof(tot), cudaMemcpyDeviceToHost, s));
    CU(c, cudaStreamSynchronize(s));
    if ((long long)tot > c->cap) {
      if (c->d_pos) cudaFree(c->d_pos);
      if (c->d_src) cudaFree(c->d_src);
      c->d_pos = nullptr;
      c->d_src = nullptr;
      const long long cap = (long long)tot + (long long)tot / 8 + 1024;
      if ((rc = dalloc(c, (void **)&c->d_pos, cap * sizeof(float4))) ||
          (rc = dalloc(c, (void **)&c->d_src, (size_t)cap * 9 * sizeof(float))))
        return rc;
      c->cap = cap;
    }
    c->nsrc[ip] = (long long)tot;
    int *cmap = nullptr;
    if (sp.nside_count > 0) {
      const size_t np = 12ull * sp.nside_count * sp.nside_count;
      if ((rc = dalloc(c, (void **)&c->d_cmap[ip], np * sizeof(int)))) return rc;
      cmap = c->d_cmap[ip];
      CU(c, cudaMemsetAsync(cmap, 0, np * sizeof(int), s));
    }
    k64_emit<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, sp, c->d_npot, c->d_counts, c->d_total + 1, c->cap,
                                                            c->d_pos, c->d_src, cmap, d_err);
    CU(c, cudaGetLastError());
    if (cf.need_beaming && tot > 0) {
      k64_beam_rsd<<<grid_for((long long)tot, nsm), 256, 0, s>>>(p, sp, c->d_npot, (long long)tot, c->d_pos, c->d_src);
      CU(c, cudaGetLastError());
    }
  }
  /* intensity maps */
  for (int ip = 0; ip < nti; ip++) {
    const int nr = cf.imap_nr[ip];
    const long long nside = cf.nside_imap[ip], npix = 12LL * nside * nside;
    std::vector<int> ord(nr);
    for (int i = 0; i < nr; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return cf.imap_r0[ip][a] < cf.imap_r0[ip][b]; });
    std::vector<double> sh(2 * nr);
    std::vector<int> ns(nr);
    const double ps = sqrt(4 * M_PI / npix);
    for (int i = 0; i < nr; i++) {
      const double a = cf.imap_r0[ip][ord[i]], b = cf.imap_rf[ip][ord[i]];
      sh[i] = a;
      sh[nr + i] = b;
      const double vol = (b * b * b - a * a * a) * ps * ps / 3;
      ns[i] = (int)(p.dx / fmin(pow(vol, 0.333333), fmin(a * ps, b - a)) + 0.5) + 1;
    }
    double *d_sh = nullptr;
    int *d_ns = nullptr;
    CU(c, cudaMallocAsync((void **)&d_sh, 2 * nr * sizeof(double), s));
    CU(c, cudaMallocAsync((void **)&d_ns, nr * sizeof(int), s));
    CU(c, cudaMemcpyAsync(d_sh, sh.data(), 2 * nr * sizeof(double), cudaMemcpyHostToDevice, s));
    CU(c, cudaMemcpyAsync(d_ns, ns.data(), nr * sizeof(int), cudaMemcpyHostToDevice, s));
    if ((rc = dalloc(c, (void **)&c->d_imap[ip], (size_t)nr * npix * sizeof(double))) ||
        (rc = dalloc(c, (void **)&c->d_nadd[ip], (size_t)nr * npix * sizeof(int))))
      return rc;
    CU(c, cudaMemsetAsync(c->d_imap[ip], 0, (size_t)nr * npix * sizeof(double), s));
    CU(c, cudaMemsetAsync(c->d_nadd[ip], 0, (size_t)nr * npix * sizeof(int), s));
    Imap64 m;
    m.ipop = nts + ip;
    m.nr = nr;
    m.nsub_lo = ns[0];
    m.nsub_hi = ns[nr - 1];
    m.bias_model = cf.bias_model;
    m.nside = nside;
    m.npix = npix;
    m.rmin = sh[0] - 20.;
    m.rmax = sh[nr + nr - 1] + 20.;
    m.fvel = -cf.fgrowth_0 / (1.5 * cf.hubble_0 * cf.omega_m);
    m.r0 = d_sh;
    m.rf = d_sh + nr;
    m.nsub = d_ns;
    k64_imap<<<grid_for((long long)ncell, nsm), 256, 0, s>>>(p, m, c->d_dens, c->d_npot, c->d_imap[ip], c->d_nadd[ip]);
    CU(c, cudaGetLastError());
    CU(c, cudaFreeAsync(d_sh, s));
    CU(c, cudaFreeAsync(d_ns, s));
  }
  /* convergence */
  if (cf.do_kappa) {
    Kap64 k;
    k.np = cf.n_kappa;
    k.nr = N / 2;
    k.nside = cf.nside_kappa;
    k.npix = 12LL * k.nside * k.nside;
    k.dr = cf.r_max / k.nr;
    double rp[CG_NPLANES_MAX];
    for (int i = 0; i < k.np; i++) rp[i] = (float)cf.kappa_r[i];
    std::sort(rp, rp + k.np);
    for (int i = 0; i < k.np; i++) {
      const int irh = (int)(rp[i] / k.dr + 0.5);
      k.inv[i] = 1. / (irh * k.dr);
      k.irmax[i] = irh < k.nr - 1 ? irh : k.nr - 1;
    }
    k.irmin[0] = 0;
    for (int i = 1; i < k.np; i++) k.irmin[i] = k.irmax[i - 1] + 1;
    if ((rc = dalloc(c, (void **)&c->d_kmap, (size_t)k.np * k.npix * sizeof(double)))) return rc;
    k64_kappa<<<grid_for(k.npix, nsm), 256, 0, s>>>(p, k, c->d_npot, c->d_kmap);
    CU(c, cudaGetLastError());
  }
  unsigned int herr = 0;
  CU(c, cudaMemcpyAsync(&herr, d_err, sizeof(herr), cudaMemcpyDeviceToHost, s));
  CU(c, cudaStreamSynchronize(s));
  if (herr) return fail(c, CG_EDEVICE, "device error flags 0x%x", herr);
  return CG_OK;
}

} /* namespace */

extern "C" int cg64_create(cg64_ctx **out, const cg_config *cfg, int device)
{
  if (!out || !cfg) return CG_EINVAL;
  *out = nullptr;
  if (cfg->n_grid < 8 || cfg->n_grid % 2) return CG_EINVAL;
  cg64_ctx *c = new cg64_ctx();
  c->cfg = *cfg;
  c->device = device;
  c->N = cfg->n_grid;
  c->NH = c->N / 2 + 1;
  auto bad = [&](int code) {
    cg64_destroy(c);
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bad(CG_ECUDA);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return bad(CG_ECUDA);
  c->nsm = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bad(CG_ECUDA);
  /* tables: 7 background, 2 per tracer, norm per tracer, edges, P(k) */
  const int nt = cfg->n_srcs + cfg->n_imap;
  std::vector<double> h((size_t)(T_BASE + 3 * nt) * NA + 2 * CG_NPOP_MAX * 2 + cfg->numk, 0.0);
  const double *bgs[T_BASE] = {cfg->r_arr_r2z, cfg->z_arr_r2z, cfg->growth_d_arr, cfg->growth_v_arr, cfg->ihub_arr,
                               cfg->a_arr_a2r, cfg->r_arr_a2r};
  for (int t = 0; t < T_BASE; t++) memcpy(h.data() + (size_t)t * NA, bgs[t], NA * sizeof(double));
  for (int t = 0; t < nt; t++) {
    const double *a = t < cfg->n_srcs ? cfg->srcs_nz_arr[t] : cfg->imap_tz_arr[t - cfg->n_srcs];
    const double *b = t < cfg->n_srcs ? cfg->srcs_bz_arr[t] : cfg->imap_bz_arr[t - cfg->n_srcs];
    memcpy(h.data() + (size_t)(T_BASE + 2 * t) * NA, a, NA * sizeof(double));
    memcpy(h.data() + (size_t)(T_BASE + 2 * t + 1) * NA, b, NA * sizeof(double));
  }
  memcpy(h.data() + (size_t)(T_BASE + 3 * nt) * NA + 2 * CG_NPOP_MAX * 2, cfg->pkarr, cfg->numk * sizeof(double));
  if (cudaMalloc((void **)&c->d_tab, h.size() * sizeof(double)) != cudaSuccess) return bad(CG_ENOMEM);
  if (cudaMemcpy(c->d_tab, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    return bad(CG_ECUDA);
  /* cuFFT plans: 2-D complex over (kz, ky) for every kx; 1-D real along x */
  const int N = c->N, NH = c->NH;
  int n2[2] = {N, N}, e2[2] = {N, N};
  if (cufftPlanMany(&c->p2, 2, n2, e2, NH, 1, e2, NH, 1, CUFFT_Z2Z, NH) != CUFFT_SUCCESS) return bad(CG_ECUDA);
  int n1[1] = {N}, ec[1] = {NH}, er[1] = {2 * NH};
  if (cufftPlanMany(&c->p1c2r, 1, n1, ec, 1, NH, er, 1, 2 * NH, CUFFT_Z2D, N * N) != CUFFT_SUCCESS) return bad(CG_ECUDA);
  if (cufftPlanMany(&c->p1r2c, 1, n1, er, 1, 2 * NH, ec, 1, NH, CUFFT_D2Z, N * N) != CUFFT_SUCCESS) return bad(CG_ECUDA);
  cufftSetStream(c->p2, c->stream);
  cufftSetStream(c->p1c2r, c->stream);
  cufftSetStream(c->p1r2c, c->stream);
  *out = c;
  return CG_OK;
}

extern "C" void cg64_destroy(cg64_ctx *c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->p2) cufftDestroy(c->p2);
  if (c->p1c2r) cufftDestroy(c->p1c2r);
  if (c->p1r2c) cufftDestroy(c->p1r2c);
  void *ptrs[] = {c->d_tab, c->d_dens, c->d_npot, c->d_disp[0], c->d_disp[1], c->d_disp[2], c->d_out, c->d_stats,
                  c->d_ncount, c->d_zsum, c->d_bsum, c->d_counts, c->d_total, c->d_pos, c->d_src, c->d_kmap};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int i = 0; i < CG_NPOP_MAX; i++) {
    if (c->d_imap[i]) cudaFree(c->d_imap[i]);
    if (c->d_nadd[i]) cudaFree(c->d_nadd[i]);
    if (c->d_cmap[i]) cudaFree(c->d_cmap[i]);
  }
  if (c->d_err) cudaFree(c->d_err);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" const char *cg64_last_error(const cg64_ctx *c) { return c ? c->err : "null context"; }

extern "C" int cg64_run_mock(cg64_ctx *c, float *ms)
{
  if (!c) return CG_EINVAL;
  if (c->cfg.dens_type == CG_DENS_1LPT && c->cfg.lpt_interp_type != 1)
    return fail(c, CG_EINVAL, "the FP64 baseline deposits 1LPT particles with CIC only");
  if (c->cfg.n_cstm > 0 || c->cfg.do_isw) return fail(c, CG_EINVAL, "the FP64 baseline has no custom or ISW maps");
  if (c->cfg.dens_type == CG_DENS_2LPT) return fail(c, CG_EINVAL, "the FP64 baseline has no 2LPT");
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, CG_ECUDA, "cudaSetDevice");
  cudaEvent_t a, b;
  CU(c, cudaEventCreate(&a));
  CU(c, cudaEventCreate(&b));
  CU(c, cudaEventRecord(a, c->stream));
  int rc = run(c);
  if (rc) {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
  }
  CU(c, cudaEventRecord(b, c->stream));
  CU(c, cudaEventSynchronize(b));
  float t = 0;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  c->ms_last = t;
  if (ms) *ms = t;
  return CG_OK;
}

extern "C" int cg64_create_cartesian_fields(cg64_ctx *c)
{
  if (!c) return CG_EINVAL;
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, CG_ECUDA, "cudaSetDevice");
  int rc = run_fields(c);
  if (rc) return rc;
  CU(c, cudaStreamSynchronize(c->stream));
  return CG_OK;
}

extern "C" long long cg64_num_sources(const cg64_ctx *c, int ipop)
{
  return (c && ipop >= 0 && ipop < c->cfg.n_srcs) ? c->nsrc[ipop] : -1;
}

/* what: 0 density, 1 potential (N^3 doubles, unpadded [z][y][x]); 2 intensity
 * map data (nr * npix doubles, RING, summed temperatures) and 3 its hit
 * counts (ints) of species ipop; 4 convergence (n_kappa * npix doubles,
 * RING); 5 normalisation tables (CG_NA doubles of tracer ipop, sources
 * first); 6 source count map of population ipop (12 nside_count^2 ints,
 * RING). */
extern "C" int cg64_download(cg64_ctx *c, int what, int ipop, void *dst)
{
  if (!c || !dst) return CG_EINVAL;
  const int N = c->N, NH = c->NH;
  CU(c, cudaStreamSynchronize(c->stream));
  if (what == 0 || what == 1) {
    const double *g = what == 0 ? c->d_dens : c->d_npot;
    if (!g) return fail(c, CG_ESTATE, "not run");
    CU(c, cudaMemcpy2D(dst, N * sizeof(double), g, 2 * NH * sizeof(double), N * sizeof(double), (size_t)N * N,
                       cudaMemcpyDefault));
    return CG_OK;
  }
  if (what == 2 || what == 3) {
    if (ipop < 0 || ipop >= c->cfg.n_imap || !c->d_imap[ipop]) return fail(c, CG_ESTATE, "no intensity map %d", ipop);
    const size_t m = (size_t)c->cfg.imap_nr[ipop] * 12 * c->cfg.nside_imap[ipop] * c->cfg.nside_imap[ipop];
    if (what == 2) CU(c, cudaMemcpy(dst, c->d_imap[ipop], m * sizeof(double), cudaMemcpyDeviceToHost));
    else CU(c, cudaMemcpy(dst, c->d_nadd[ipop], m * sizeof(int), cudaMemcpyDeviceToHost));
    return CG_OK;
  }
  if (what == 4) {
    if (!c->d_kmap) return fail(c, CG_ESTATE, "no convergence maps");
    const size_t m = (size_t)c->cfg.n_kappa * 12 * c->cfg.nside_kappa * c->cfg.nside_kappa;
    CU(c, cudaMemcpy(dst, c->d_kmap, m * sizeof(double), cudaMemcpyDeviceToHost));
    return CG_OK;
  }
  if (what == 6) {
    if (ipop < 0 || ipop >= c->cfg.n_srcs || !c->d_cmap[ipop]) return fail(c, CG_ESTATE, "no count map %d", ipop);
    const size_t m = 12ull * c->cfg.nside_count[ipop] * c->cfg.nside_count[ipop];
    CU(c, cudaMemcpy(dst, c->d_cmap[ipop], m * sizeof(int), cudaMemcpyDeviceToHost));
    return CG_OK;
  }
  if (what == 5) {
    const int nt = c->cfg.n_srcs + c->cfg.n_imap;
    if (ipop < 0 || ipop >= nt || c->h_norm.empty()) return fail(c, CG_ESTATE, "no table %d", ipop);
    memcpy(dst, c->h_norm.data() + (size_t)ipop * NA, NA * sizeof(double));
    return CG_OK;
  }
  return CG_EINVAL;
}
