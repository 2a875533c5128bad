/*
 * imap.cu -- intensity-map painting (imap_set_cartesian_single,
 * imap.c:135-245).
 *
 * Every cell in the radial range of the shells carries a brightness
 * temp = T(r) bias_model(d, b(r)) norm(r) and a redshift-space shift dr_rsd;
 * it is split into nsub^3 sub-cells whose centres are placed in a shell (by
 * r + dr_rsd) and a RING pixel, where temp is added and a hit counted.
 *
 * A warp takes 32 consecutive cells of a row (one per lane), computes their
 * per-cell quantities, and then walks the concatenated list of all their
 * sub-samples 32 at a time, so that lanes stay busy whatever nsub is.  Lanes
 * whose samples land on the same (cell, shell, pixel) are merged with
 * __match_any_sync before the atomic updates.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "imap_api.h"

namespace {
using namespace cg;

constexpr int IW = 8; /* warps per block */

__global__ void __launch_bounds__(IW * 32) k_imap(const float *__restrict__ dens, const float *__restrict__ phi,
                                                  cg_imap_params p)
{
  extern __shared__ float ssh[];
  float *r0 = ssh, *rf = ssh + p.nr;
  int *nsa = reinterpret_cast<int *>(ssh + 2 * p.nr);
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) {
    r0[i] = p.r0[i];
    rf[i] = p.rf[i];
    nsa[i] = p.nsub[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int N = p.box.N;
  const int nch = (N + 31) / 32;
  const long long ntask = (long long)nch * N * N;
  const float dx = p.box.dx;
  const unsigned FULL = 0xffffffffu;
  for (long long task = (long long)blockIdx.x * IW + wid; task < ntask; task += (long long)gridDim.x * IW) {
    const int ch = (int)(task % nch);
    const long long row = task / nch;
    const int iy = (int)(row % N), iz = (int)(row / N);
    const int ix = ch * 32 + lane;
    const float y0 = cg_cell_coord(iy, dx, p.box.p1), z0 = cg_cell_coord(iz, dx, p.box.p2);
    float x0 = 0.0f, temp = 0.0f, drr = 0.0f, dxs = 0.0f;
    int nsub = 0, irad0 = 0, n = 0;
    if (ix < N) {
      x0 = cg_cell_coord(ix, dx, p.box.p0);
      const float rc = cg_norm3(x0, y0, z0);
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
        float rvel = CG_MUL(p.factor_vel, cg_rvel(v0, v1, v2, x0, y0, z0, rc, p.box.idx));
        drr = cg_imap_drsd(rvel, bg(p.v1, p.g, rc), bg(p.ih, p.g, rc));
        const float d = __ldg(&dens[pidx(ix, iy, iz, N)]);
        temp = cg_imap_temp(tmean, d, bias, dnorm, p.bias_model);
        irad0 = cg_shell_index(r0, rf, p.nr, rc, 0);
        nsub = irad0 < 0 ? p.nsub_lo : (irad0 >= p.nr ? p.nsub_hi : nsa[irad0]);
        if (nsub < 1 || nsub > 1024) {
          atomicOr(p.err, ERR_IMAP_NSUB);
          nsub = 0;
        }
        dxs = CG_DIV(dx, (float)nsub);
        n = nsub * nsub * nsub;
      }
    }
    /* inclusive scan of the sample counts over the warp */
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    const int excl = incl - n;
    const int total = __shfl_sync(FULL, incl, 31);
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
      const int ns = __shfl_sync(FULL, nsub, j);
      const int ex = __shfl_sync(FULL, excl, j);
      const float cx = __shfl_sync(FULL, x0, j);
      const float ct = __shfl_sync(FULL, temp, j);
      const float cd = __shfl_sync(FULL, drr, j);
      const float cs = __shfl_sync(FULL, dxs, j);
      const int cr = __shfl_sync(FULL, irad0, j);
      unsigned long long key = ~0ull;
      if (s < total) {
        const int l = s - ex;
        const int nn = ns * ns;
        const int izz = l / nn, rem = l - izz * nn;
        const int iyy = rem / ns, ixx = rem - iyy * ns;
        const float zc = cg_sub_centre(z0, izz, cs);
        const float yc = cg_sub_centre(y0, iyy, cs);
        const float xc = cg_sub_centre(cx, ixx, cs);
        float r, cth, ph;
        cg_cart2sph(xc, yc, zc, &r, &cth, &ph);
        const int ir = cg_shell_index(r0, rf, p.nr, CG_ADD(r, cd), cr);
        if (ir >= 0 && ir < p.nr) {
          const long long pix = cg_ang2pix_ring(p.nside, cth, ph);
          key = ((unsigned long long)j << 58) | (unsigned long long)((long long)ir * p.npix + pix);
        }
      }
      const unsigned act = __ballot_sync(FULL, key != ~0ull);
      if (key != ~0ull) {
        const unsigned grp = __match_any_sync(act, key);
        if (lane == __ffs(grp) - 1) {
          const int c = __popc(grp);
          const long long idx = (long long)(key & ((1ull << 58) - 1));
          atomicAdd(&p.data[idx], CG_MUL(ct, (float)c));
          atomicAdd(&p.nadd[idx], c);
        }
      }
    }
  }
}

} /* namespace */

cudaError_t cg_imap_paint(cudaStream_t s, const float *dens, const float *phi, const cg_imap_params *p, int nsm)
{
  size_t smem = (size_t)p->nr * (2 * sizeof(float) + sizeof(int));
  cudaError_t e = cudaFuncSetAttribute(k_imap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  long long ntask = (long long)((p->box.N + 31) / 32) * p->box.N * p->box.N;
  long long blocks = (ntask + IW - 1) / IW;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  k_imap<<<(unsigned)blocks, IW * 32, smem, s>>>(dens, phi, *p);
  return cudaGetLastError();
}
