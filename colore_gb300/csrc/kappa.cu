/*
 * kappa.cu -- lensing convergence on source planes
 * (kappa_get_beam_properties, kappa.c:78-175).
 *
 * One thread per HEALPix pixel (NEST id, as listed by hp_shell_alloc,
 * common.c:505-552) marches the N/2 radial steps of the line of sight,
 * samples the tidal tensor of the potential at the nearest grid cell
 * (get_element, beaming.c:84-116; interpolate_from_grid NGP branch,
 * beaming.c:148-182), projects it on the transverse directions and
 * accumulates the two radial moments.  At each source-plane boundary it
 * writes kappa_1 - kappa_2 / r_plane straight into RING order (the
 * nest-to-ring reordering of write_kappa, io.c:826-873).  Threads of a warp
 * hold neighbouring NEST pixels, so their rays stay close and the 19-point
 * stencil reads hit L1/L2.  The radial sums use Kahan compensation.
 * k_isw integrates the ISW maps along the same rays, k_cstm the custom maps.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_dev.cuh"
#include "kappa_api.h"

namespace {
using namespace cg;

__global__ void __launch_bounds__(256) k_kappa(const float *__restrict__ phi, cg_kappa_params p)
{
  extern __shared__ float ksh[];
  float *f1 = ksh, *f2 = ksh + p.nr;
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) {
    f1[i] = p.fac1[i];
    f2[i] = p.fac2[i];
  }
  __syncthreads();
  const long long ip = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= p.npix) return;
  const int N = p.box.N;
  float u[3], rot[6];
  cg_pix2vec_nest(p.nside, ip, u);
  cg_kappa_rot(u, CG_MUL(p.box.idx, p.box.idx), rot);
  const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
  const long long ring = cg_nest2ring(p.nside, ip);
  float k1 = 0.0f, k1c = 0.0f, k2 = 0.0f, k2c = 0.0f;
  for (int pl = 0; pl < p.nplanes; pl++) {
    const int irmin = p.ir_min[pl], irmax = p.ir_max[pl];
    for (int irr = irmin; irr <= irmax; irr++) {
      const float rm = CG_MUL(CG_ADD((float)irr, 0.5f), p.dr);
      const int x0 = cg_ngp_cell(rm, u[0], po[0], p.box.idx, N);
      const int y0 = cg_ngp_cell(rm, u[1], po[1], p.box.idx, N);
      const int z0 = cg_ngp_cell(rm, u[2], po[2], p.box.idx, N);
      float f[19];
      stencil19(phi, x0, y0, z0, N, f);
      float t[6];
      cg_tidal(f, t);
      const float dot = cg_dot6(rot, t);
      cg_kahan_add(&k1, &k1c, CG_MUL(dot, f1[irr]));
      cg_kahan_add(&k2, &k2c, CG_MUL(dot, f2[irr]));
    }
    p.map[(long long)pl * p.npix + ring] = CG_SUB(k1, CG_MUL(p.inv_r_max[pl], k2));
  }
}

/* isw_get_beam_properties (isw.c:78-147): the same rays, the potential at the
 * nearest cell (RETURN_PDOT, beaming.c:81-82, 145-180) weighted by
 * fac1 = 2 PD(r) dr, cumulative over the sorted planes. */
__global__ void __launch_bounds__(256) k_isw(const float *__restrict__ phi, cg_kappa_params p)
{
  extern __shared__ float ksh[];
  float *f1 = ksh;
  for (int i = threadIdx.x; i < p.nr; i += blockDim.x) f1[i] = p.fac1[i];
  __syncthreads();
  const long long ip = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= p.npix) return;
  const int N = p.box.N;
  const int ngx = 2 * (N / 2 + 1);
  const size_t plane = (size_t)ngx * N;
  float u[3];
  cg_pix2vec_nest(p.nside, ip, u);
  const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
  const long long ring = cg_nest2ring(p.nside, ip);
  float acc = 0.0f, cmp = 0.0f;
  for (int pl = 0; pl < p.nplanes; pl++) {
    const int irmin = p.ir_min[pl], irmax = p.ir_max[pl];
    for (int irr = irmin; irr <= irmax; irr++) {
      const float rm = CG_MUL(CG_ADD((float)irr, 0.5f), p.dr);
      const int x0 = cg_ngp_cell(rm, u[0], po[0], p.box.idx, N);
      const int y0 = cg_ngp_cell(rm, u[1], po[1], p.box.idx, N);
      const int z0 = cg_ngp_cell(rm, u[2], po[2], p.box.idx, N);
      const float pd = __ldg(phi + (size_t)z0 * plane + y0 * ngx + x0);
      cg_kahan_add(&acc, &cmp, CG_MUL(pd, f1[irr]));
    }
    p.map[(long long)pl * p.npix + ring] = acc;
  }
}

/* cstm_get_beam_properties (cstm.c:68-145): one NEST pixel per thread, the
 * density interpolated trilinearly at each step centre of the kernel's
 * support, written back in NEST order as write_cstm stores it
 * (io.c:754-800 copies the shell data without reordering). */
__global__ void __launch_bounds__(256) k_cstm(const float *__restrict__ dens, cg_cstm_params p)
{
  extern __shared__ float csh[];
  const int ns = p.ir_max - p.ir_min + 1;
  float *kz = csh, *bz = csh + ns, *nm = csh + 2 * ns;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) {
    const int irr = p.ir_min + i;
    kz[i] = p.kz[irr];
    bz[i] = p.bz[irr];
    nm[i] = bgn(p.norm, p.g, CG_MUL(CG_ADD((float)irr, 0.5f), p.dr));
  }
  __syncthreads();
  const long long ip = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= p.npix) return;
  const int N = p.box.N;
  float u[3];
  cg_pix2vec_nest(p.nside, ip, u);
  const float po[3] = {p.box.p0, p.box.p1, p.box.p2};
  float acc = 0.0f, cmp = 0.0f;
  for (int i = 0; i < ns; i++) {
    const float rm = CG_MUL(CG_ADD((float)(p.ir_min + i), 0.5f), p.dr);
    int i0[3], i1[3];
    float h0[3], h1[3];
#pragma unroll
    for (int a = 0; a < 3; a++) cg_cic_axis(rm, u[a], po[a], p.box.idx, N, &i0[a], &i1[a], &h0[a], &h1[a]);
    const float d = cg_cic_value(dens, i0, i1, h0, h1, N);
    cg_kahan_add(&acc, &cmp, CG_MUL(kz[i], CG_SUB(CG_MUL(cg_bias_model(d, bz[i], p.bias_model), nm[i]), 1.0f)));
  }
  p.map[ip] = CG_MUL(acc, p.dr);
}

} /* namespace */

cudaError_t cg_cstm_integrate(cudaStream_t s, const float *dens, const cg_cstm_params *p)
{
  long long blocks = (p->npix + 255) / 256;
  const size_t smem = 3 * sizeof(float) * (size_t)(p->ir_max - p->ir_min + 1);
  k_cstm<<<(unsigned)blocks, 256, smem, s>>>(dens, *p);
  return cudaGetLastError();
}

cudaError_t cg_isw_integrate(cudaStream_t s, const float *phi, const cg_kappa_params *p)
{
  size_t smem = (size_t)p->nr * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_isw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  long long blocks = (p->npix + 255) / 256;
  k_isw<<<(unsigned)blocks, 256, smem, s>>>(phi, *p);
  return cudaGetLastError();
}

cudaError_t cg_kappa_integrate(cudaStream_t s, const float *phi, const cg_kappa_params *p)
{
  size_t smem = (size_t)2 * p->nr * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_kappa, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  long long blocks = (p->npix + 255) / 256;
  k_kappa<<<(unsigned)blocks, 256, smem, s>>>(phi, *p);
  return cudaGetLastError();
}
