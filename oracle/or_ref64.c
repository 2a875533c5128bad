/*
 * or_ref64.c -- ORACLE (test infrastructure only).  The reference's hot path
 * restated in double precision with libm, loop by loop; the tolerance
 * oracle for every floating-point output and the timed CPU baseline.
 *
 *   or_fill64        create_grids_fourier          fourier.c:285-359
 *   or_field64       create_cartesian_fields       fourier.c:361-423 (+ compute_sigma_dens 24-79)
 *   or_density64     lognormalize / densclip       density.c:1034-1103
 *   or_lpt64         lpt_1 + pos_2_dens            density.c:376-644, 37-187 (literal r2c path)
 *   or_bins64        collect_density_normalization_from_grid density.c:1128-1211
 *   or_norm_tables64 compute_density_normalization density.c:1227-1355
 *   or_lambda64      Poisson mean per cell         srcs.c:156-178
 *   or_imap64        imap_set_cartesian_single     imap.c:135-245
 *   or_kappa64       kappa_get_beam_properties     kappa.c:78-175
 *   or_isw64         isw_get_beam_properties       isw.c:78-147
 *   or_cstm_steps    custom-map step tables        cstm.c:81-116
 *   or_cstm64        cstm_get_beam_properties      cstm.c:68-145
 *   or_lpt2_64       2LPT displacements + deposit  density.c:646-1031
 *   or_lens64        source lensing along the LOS  srcs.c:452-625, 715-723
 *   or_skw64         source skewers                srcs.c:509-536, 725-733
 *   or_run_mock64    the driver sequence of main.c:66-125 for timing.
 * Random numbers: the Philox streams of the GPU path (uniforms identical
 * bit for bit), since GSL's MT19937 streams cannot be reproduced here.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../colore_gb300/csrc/cg_cell.h"
#include "oracle.h"

static double bg(const cg_config *c, const double *f, double f0, double ff, double r) /* cosmo.c:30-38 */
{
  if (r <= 0) return f0;
  if (r >= c->r_arr_r2z[CG_NA - 1]) return ff;
  int ir = (int)(r * c->glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - c->r_arr_r2z[ir]) * c->glob_idr;
}
#define BG_Z(c, r) bg((c), (c)->z_arr_r2z, 0, (c)->z_arr_r2z[CG_NA - 1], (r))
#define BG_D1(c, r) bg((c), (c)->growth_d_arr, 1, (c)->growth_d_arr[CG_NA - 1], (r))
#define BG_V1(c, r) bg((c), (c)->growth_v_arr, (c)->growth_v_arr[0], (c)->growth_v_arr[CG_NA - 1], (r))
#define BG_IH(c, r) bg((c), (c)->ihub_arr, (c)->ihub_arr[0], (c)->ihub_arr[CG_NA - 1], (r))
#define BG_D2(c, r) bg((c), (c)->growth_d2_arr, (c)->growth_d2_arr[0], (c)->growth_d2_arr[CG_NA - 1], (r))

static double bias_model64(double d, double b, int model) /* common.h:414-431 */
{
  if (d <= -1) return 0;
  if (model == CG_BIAS_MODEL_EXPLIN) return d < 0 ? exp(b * d / (1 + d)) : 1 + b * d;
  if (model == CG_BIAS_MODEL_LIN) return 1 + b * d > 0 ? 1 + b * d : 0;
  return pow(1 + d, b);
}

static double pk_lin0(const cg_config *c, double lgk) /* cosmo.c:291-308, guarded at numk-1 */
{
  int ik = (int)((lgk - c->logkmin) * c->idlogk);
  if (ik < 0) return c->pkarr[0] * pow(10, c->n_scal * (lgk - c->logkmin));
  if (ik < c->numk - 1) {
    double lk = c->logkmin + ik / c->idlogk;
    return c->pkarr[ik] + (lgk - lk) * (c->pkarr[ik + 1] - c->pkarr[ik]) * c->idlogk;
  }
  return c->pkarr[c->numk - 1] * pow(10, -3 * (lgk - c->logkmax));
}

static double kc(int i, int n, double dk) { return (2 * i <= n ? i : -(n - i)) * dk; }

int or_fill64(const cg_config *c, double complex *dk, double complex *pk)
{
  const int N = c->n_grid, NH = N / 2 + 1;
  const double dkk = 2 * M_PI / c->l_box, idk3 = 1. / (dkk * dkk * dkk);
  const uint32_t k0 = (uint32_t)c->seed, k1 = (uint32_t)(c->seed >> 32) ^ CG_STREAM_FIELD;
#pragma omp parallel for schedule(static)
  for (int kz = 0; kz < N; kz++) {
    double z = kc(kz, N, dkk);
    for (int ky = 0; ky < N; ky++) {
      double y = kc(ky, N, dkk);
      for (int kx = 0; kx <= N / 2; kx++) {
        double x = kx * dkk;
        size_t idx = kx + (size_t)NH * (ky + (size_t)N * kz);
        double k2 = x * x + y * y + z * z;
        if (k2 <= 0) {
          dk[idx] = 0;
          if (pk) pk[idx] = 0;
          continue;
        }
        double lgk = 0.5 * log10(k2);
        double s2 = pk_lin0(c, lgk) * idk3;
        uint64_t m = (uint64_t)idx;
        cg_u32x4 w = cg_philox4x32_10((uint32_t)m, (uint32_t)(m >> 32), 0u, 0u, k0, k1);
        double ph = 2 * M_PI * (double)cg_u01f(w.v[0]);
        double u = cg_u01f(w.v[1]);
        double mod = sqrt(-s2 * log(1 - u)); /* rng_delta_gauss, common.c:191-201 */
        double complex d = mod * cexp(I * ph);
        double complex p = -c->prefac_lensing * d / k2;
        if (c->do_smoothing) {
          double sm = exp(-0.5 * c->r2_smooth * k2);
          d *= sm;
          if (c->smooth_potential) p *= sm;
        }
        dk[idx] = d;
        if (pk) pk[idx] = p;
      }
    }
  }
  return 0;
}

int or_field64(const cg_config *c, double *dens, double *npot, double stats[4])
{
  const int N = c->n_grid, NH = N / 2 + 1;
  const size_t nh = (size_t)N * N * NH, ncell = (size_t)N * N * N;
  double complex *dk = malloc(nh * sizeof(double complex)), *pk = malloc(nh * sizeof(double complex));
  if (!dk || !pk) return -1;
  or_fill64(c, dk, pk);
  or_c2r_3d(N, dk, dens);
  or_c2r_3d(N, pk, npot);
  free(dk);
  free(pk);
  const double norm = pow(sqrt(2 * M_PI) / c->l_box, 3);
  double s1 = 0, s2 = 0;
#pragma omp parallel for schedule(static) reduction(+ : s1, s2)
  for (size_t i = 0; i < ncell; i++) {
    dens[i] *= norm;
    npot[i] *= norm;
    s1 += dens[i];
    s2 += dens[i] * dens[i];
  }
  double mean = s1 / ncell, sig2 = s2 / ncell - mean * mean;
  stats[0] = s1;
  stats[1] = s2;
  stats[2] = mean;
  stats[3] = sig2;
  return 0;
}

int or_density64(const cg_config *c, double *dens, double sigma2)
{
  const int N = c->n_grid;
  const double dx = c->l_box / N;
#pragma omp parallel for schedule(static)
  for (int iz = 0; iz < N; iz++) {
    double z0 = iz * dx - c->pos_obs[2];
    for (int iy = 0; iy < N; iy++) {
      double y0 = iy * dx - c->pos_obs[1];
      for (int ix = 0; ix < N; ix++) {
        double x0 = ix * dx - c->pos_obs[0];
        double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        double dg = BG_D1(c, r);
        size_t id = ix + (size_t)N * (iy + (size_t)N * iz);
        double d = dens[id];
        if (c->dens_type == CG_DENS_CLIP) dens[id] = fmax(1 + dg * d, 0) - 1;
        else dens[id] = exp(dg * (d - 0.5 * dg * sigma2)) - 1;
      }
    }
  }
  return 0;
}

/* Particle positions q + D1 Psi1 (+ D2 Psi2 for 2LPT, density.c:890) and
 * the mass assignment of pos_2_dens (density.c:178-187): NGP (37-62), CIC
 * (64-105) or TSC (107-176); then rho - 1 (density.c:621, 1015). */
static void lpt_deposit64(const cg_config *c, const double *disp, const double *disp2, double *dens_out)
{
  const int N = c->n_grid;
  const size_t ncell = (size_t)N * N * N;
  const double dx = c->l_box / N;
  memset(dens_out, 0, ncell * sizeof(double));
  /* positions (density.c:473-501) and the deposit of pos_2_dens
   * (density.c:178-187): NGP (37-62), CIC (64-105) or TSC (107-176) */
  const double iag = N / c->l_box;
  const int S = c->lpt_interp_type;
  for (int iz = 0; iz < N; iz++)
    for (int iy = 0; iy < N; iy++)
      for (int ix = 0; ix < N; ix++) {
        double xv[3] = {ix * dx - c->pos_obs[0], iy * dx - c->pos_obs[1], iz * dx - c->pos_obs[2]};
        double r = sqrt(xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2]);
        double g = BG_D1(c, r), g2 = disp2 ? BG_D2(c, r) : 0;
        size_t id = ix + (size_t)N * (iy + (size_t)N * iz);
        int ib[3], K = S + 1;
        double w[3][3];
        for (int ax = 0; ax < 3; ax++) {
          double q = xv[ax] + g * disp[(size_t)ax * ncell + id] +
                     (disp2 ? g2 * disp2[(size_t)ax * ncell + id] : 0) + c->pos_obs[ax];
          if (q < 0) q += c->l_box;
          if (q >= c->l_box) q -= c->l_box;
          double u = q * iag;
          int i0;
          if (S == 0) {
            i0 = (int)(u + 0.5);
            w[ax][0] = 1;
          } else if (S == 1) {
            i0 = (int)u;
            w[ax][1] = u - i0;
            w[ax][0] = 1 - w[ax][1];
          } else {
            i0 = (int)floor(u + 0.5);
            double a0 = u - i0;
            w[ax][0] = 0.5 * (0.5 - a0) * (0.5 - a0);
            w[ax][1] = 0.75 - a0 * a0;
            w[ax][2] = 0.5 * (0.5 + a0) * (0.5 + a0);
            i0 -= 1;
          }
          ib[ax] = ((i0 % N) + N) % N;
        }
        for (int cz = 0; cz < K; cz++)
          for (int cy = 0; cy < K; cy++)
            for (int cx = 0; cx < K; cx++) {
              int gx = (ib[0] + cx) % N, gy = (ib[1] + cy) % N, gz = (ib[2] + cz) % N;
              dens_out[gx + (size_t)N * (gy + (size_t)N * gz)] += w[0][cx] * w[1][cy] * w[2][cz];
            }
      }
  for (size_t i = 0; i < ncell; i++) dens_out[i] -= 1;
}

int or_lpt64(const cg_config *c, const double *dg_in, double *dens_out, double *disp)
{
  const int N = c->n_grid, NH = N / 2 + 1;
  const size_t nh = (size_t)N * N * NH, ncell = (size_t)N * N * N;
  double complex *dk = malloc(nh * sizeof(double complex)), *ck = malloc(nh * sizeof(double complex));
  if (!dk || !ck) return -1;
  or_r2c_3d(N, dg_in, dk); /* density.c:392 */
  const double dkk = 2 * M_PI / c->l_box, fftnorm = (double)N * N * N;
  for (int ax = 0; ax < 3; ax++) { /* density.c:408-440 */
#pragma omp parallel for schedule(static)
    for (int kz = 0; kz < N; kz++)
      for (int ky = 0; ky < N; ky++)
        for (int kx = 0; kx <= N / 2; kx++) {
          double kv[3] = {kx * dkk, kc(ky, N, dkk), kc(kz, N, dkk)};
          double k2 = fftnorm * (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
          size_t idx = kx + (size_t)NH * (ky + (size_t)N * kz);
          ck[idx] = k2 <= 0 ? 0 : I * kv[ax] * dk[idx] / k2;
        }
    or_c2r_3d(N, ck, disp + (size_t)ax * ncell);
  }
  free(dk);
  free(ck);
  lpt_deposit64(c, disp, NULL, dens_out);
  return 0;
}

/* lpt_2 (density.c:646-1031) in double precision: r2c of the Gaussian
 * density, the six second derivatives of the first-order potential, the
 * source xx yy + xx zz + yy zz - xy^2 - xz^2 - yz^2, its r2c, the
 * second-order displacements -i k S_k / (N^3 k^2), the first-order ones,
 * positions q + D1 Psi1 + D2 Psi2 and the deposit.  disp, disp2: 3 N^3 each. */
int or_lpt2_64(const cg_config *c, const double *dg_in, double *dens_out, double *disp, double *disp2)
{
  const int N = c->n_grid, NH = N / 2 + 1;
  const size_t nh = (size_t)N * N * NH, ncell = (size_t)N * N * N;
  double complex *dk = malloc(nh * sizeof(double complex)), *ck = malloc(nh * sizeof(double complex));
  double *dig = malloc(6 * ncell * sizeof(double));
  if (!dk || !ck || !dig) return -1;
  or_r2c_3d(N, dg_in, dk); /* density.c:667 */
  const double dkk = 2 * M_PI / c->l_box, fftnorm = (double)N * N * N;
  const int pi_[6] = {0, 0, 0, 1, 1, 2}, pj_[6] = {0, 1, 2, 1, 2, 2};
  for (int m = 0; m < 6; m++) { /* density.c:688-709, 712-714 */
#pragma omp parallel for schedule(static)
    for (int kz = 0; kz < N; kz++)
      for (int ky = 0; ky < N; ky++)
        for (int kx = 0; kx <= N / 2; kx++) {
          double kv[3] = {kx * dkk, kc(ky, N, dkk), kc(kz, N, dkk)};
          double k2 = fftnorm * (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
          size_t idx = kx + (size_t)NH * (ky + (size_t)N * kz);
          double complex cd = k2 <= 0 ? 0 : I * kv[pi_[m]] * dk[idx] / k2;
          ck[idx] = I * kv[pj_[m]] * cd;
        }
    or_c2r_3d(N, ck, dig + (size_t)m * ncell);
  }
  double *src = malloc(ncell * sizeof(double));
  if (!src) return -1;
  for (size_t i = 0; i < ncell; i++) { /* density.c:749-755 */
    const double *g = dig + i;
    src[i] = g[0] * g[3 * ncell] + g[0] * g[5 * ncell] + g[3 * ncell] * g[5 * ncell] - g[ncell] * g[ncell] -
             g[2 * ncell] * g[2 * ncell] - g[4 * ncell] * g[4 * ncell];
  }
  free(dig);
  double complex *sk = malloc(nh * sizeof(double complex));
  if (!sk) return -1;
  or_r2c_3d(N, src, sk); /* density.c:763 */
  free(src);
  for (int ax = 0; ax < 3; ax++) {
#pragma omp parallel for schedule(static)
    for (int kz = 0; kz < N; kz++)
      for (int ky = 0; ky < N; ky++)
        for (int kx = 0; kx <= N / 2; kx++) {
          double kv[3] = {kx * dkk, kc(ky, N, dkk), kc(kz, N, dkk)};
          double k2 = fftnorm * (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
          size_t idx = kx + (size_t)NH * (ky + (size_t)N * kz);
          ck[idx] = k2 <= 0 ? 0 : -I * kv[ax] * sk[idx] / k2; /* density.c:802-805 */
        }
    or_c2r_3d(N, ck, disp2 + (size_t)ax * ncell);
#pragma omp parallel for schedule(static)
    for (int kz = 0; kz < N; kz++)
      for (int ky = 0; ky < N; ky++)
        for (int kx = 0; kx <= N / 2; kx++) {
          double kv[3] = {kx * dkk, kc(ky, N, dkk), kc(kz, N, dkk)};
          double k2 = fftnorm * (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
          size_t idx = kx + (size_t)NH * (ky + (size_t)N * kz);
          ck[idx] = k2 <= 0 ? 0 : I * kv[ax] * dk[idx] / k2; /* density.c:700-704 */
        }
    or_c2r_3d(N, ck, disp + (size_t)ax * ncell);
  }
  free(sk);
  free(dk);
  free(ck);
  lpt_deposit64(c, disp, disp2, dens_out);
  return 0;
}

int or_bins64(const cg_config *c, const double *dens, int nz, double idz, unsigned long long *narr, double *zarr,
              double *bsum)
{
  const int N = c->n_grid, nts = c->n_srcs, nti = c->n_imap, nt = nts + nti + c->n_cstm;
  const double dx = c->l_box / N;
  memset(narr, 0, nz * sizeof(unsigned long long));
  memset(zarr, 0, nz * sizeof(double));
  memset(bsum, 0, (size_t)nt * nz * sizeof(double));
  for (int iz = 0; iz < N; iz++) {
    double z0 = iz * dx - c->pos_obs[2];
    for (int iy = 0; iy < N; iy++) {
      double y0 = iy * dx - c->pos_obs[1];
      for (int ix = 0; ix < N; ix++) {
        double x0 = ix * dx - c->pos_obs[0];
        double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        double z = BG_Z(c, r);
        int b = (int)(z * idz) + 1;
        if (b < 0 || b >= nz) continue;
        double d = dens[ix + (size_t)N * (iy + (size_t)N * iz)];
        narr[b]++;
        zarr[b] += z;
        for (int t = 0; t < nt; t++) {
          const double *bt = t < nts ? c->srcs_bz_arr[t]
                                     : (t < nts + nti ? c->imap_bz_arr[t - nts] : c->cstm_bz_arr[t - nts - nti]);
          bsum[(size_t)t * nz + b] += bias_model64(d, bg(c, bt, bt[0], 1, r), c->bias_model);
        }
      }
    }
  }
  return 0;
}

int or_norm_tables64(const cg_config *c, double *tabs, double *e0f, int *nz_out, unsigned long long *narr,
                     double *zarr, double *bsum, const double *dens)
{
  const int nt = c->n_srcs + c->n_imap + c->n_cstm;
  double zmax = BG_Z(c, c->l_box * 0.5);
  int nz = (int)(zmax / 0.05) + 2;
  double idz = (nz - 2) / zmax;
  if (nz_out) *nz_out = nz;
  if (dens) or_bins64(c, dens, nz, idz, narr, zarr, bsum);
  double *zz = malloc(nz * sizeof(double)), *y = malloc((size_t)nt * nz * sizeof(double));
  memcpy(zz, zarr, nz * sizeof(double));
  memcpy(y, bsum, (size_t)nt * nz * sizeof(double));
  for (int iz = 0; iz < nz; iz++)
    if (narr[iz] > 0) {
      zz[iz] /= narr[iz];
      for (int t = 0; t < nt; t++) y[(size_t)t * nz + iz] = narr[iz] / y[(size_t)t * nz + iz];
    }
  zz[0] = 0;
  zz[nz - 1] = BG_Z(c, 0.5 * c->l_box);
  for (int t = 0; t < nt; t++) {
    y[(size_t)t * nz] = y[(size_t)t * nz + 1];
    y[(size_t)t * nz + nz - 1] = y[(size_t)t * nz + nz - 2];
    e0f[2 * t] = y[(size_t)t * nz];
    e0f[2 * t + 1] = y[(size_t)t * nz + nz - 1];
    for (int i = 0; i < CG_NA; i++) {
      double z = BG_Z(c, c->r_arr_r2z[i]), nm;
      const double *yt = y + (size_t)t * nz;
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
      tabs[(size_t)t * CG_NA + i] = nm;
    }
  }
  free(zz);
  free(y);
  return 0;
}

int or_lambda64(const cg_config *c, int ipop, const double *dens, const double *nt_, double n0, double nf,
                double *lambda)
{
  const int N = c->n_grid;
  const double dx = c->l_box / N, cv = dx * dx * dx;
  const double *nzt = c->srcs_nz_arr[ipop], *bzt = c->srcs_bz_arr[ipop];
#pragma omp parallel for schedule(static)
  for (int iz = 0; iz < N; iz++) {
    double z0 = iz * dx - c->pos_obs[2];
    for (int iy = 0; iy < N; iy++) {
      double y0 = iy * dx - c->pos_obs[1];
      for (int ix = 0; ix < N; ix++) {
        double x0 = ix * dx - c->pos_obs[0];
        double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        size_t id = ix + (size_t)N * (iy + (size_t)N * iz);
        double lam = 0;
        if (r < c->l_box / 2 + 20.) {
          double nd = bg(c, nzt, 0, 0, r);
          if (nd > 0)
            lam = nd * cv * bias_model64(dens[id], bg(c, bzt, bzt[0], 1, r), c->bias_model) * bg(c, nt_, n0, nf, r);
        }
        lambda[id] = lam;
      }
    }
  }
  return 0;
}

/* he_ang2pix in double, healpix_extra.c:118-172 */
static long ang2pix64(long nside, double cth, double phi)
{
  double ctha = fabs(cth), tp2 = 2 * M_PI;
  double ph = phi >= 0 ? (phi < tp2 ? phi : fmod(phi, tp2)) : fmod(phi, tp2) + tp2;
  if (ph == tp2) ph = 0;
  double tt = ph * (2 / M_PI);
  if (ctha <= 2. / 3.) {
    double t1 = nside * (0.5 + tt), t2 = nside * cth * 0.75;
    int jp = (int)(t1 - t2), jm = (int)(t1 + t2);
    int ir = nside + 1 + jp - jm, ks = 1 - (ir & 1);
    int ip = (jp + jm - nside + ks + 1) / 2;
    ip %= 4 * nside;
    if (ip < 0) ip += 4 * nside;
    return nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip;
  }
  double tp = tt - (int)tt, tmp = nside * sqrt(3 * (1 - ctha));
  int jp = (int)(tp * tmp), jm = (int)((1.0 - tp) * tmp), ir = jp + jm + 1;
  int ip = (int)(tt * ir);
  ip %= 4 * ir;
  if (ip < 0) ip += 4 * ir;
  return cth > 0 ? 2 * ir * (ir - 1) + ip : 12 * nside * nside - 2 * ir * (ir + 1) + ip;
}

static void cart2sph64(double x, double y, double z, double *r, double *cth, double *phi)
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

/* RING pixel of he_ang2pix after cart2sph (imap.c:210-231, srcs.c:404-409)
 * for each double direction (independent restatement). */
void or_pix64(long nside, const double *xyz, long n, long long *pix)
{
  for (long i = 0; i < n; i++) {
    double r, cth, ph;
    cart2sph64(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], &r, &cth, &ph);
    pix[i] = ang2pix64(nside, cth, ph);
  }
}

/* get_rvel (imap.c:43-74, srcs.c:87-118): the unit vector x0/rr is formed
 * before the products; with sprec (the reference built with _SPREC, float
 * grids) the potential's centred differences are float - float. */
static double rvel64(const cg_config *c, const double *p, int ix, int iy, int iz, double x0, double y0, double z0,
                     double rr, int sprec)
{
  const int N = c->n_grid;
  const double idx = c->n_grid / c->l_box;
#define P(X, Y, Z) p[(X) + (size_t)N * ((Y) + (size_t)N * (Z))]
  int xh = (ix + 1) % N, xl = (ix + N - 1) % N, yh = (iy + 1) % N, yl = (iy + N - 1) % N, zh = (iz + 1) % N,
      zl = (iz + N - 1) % N;
  double v0 = P(xh, iy, iz) - P(xl, iy, iz), v1 = P(ix, yh, iz) - P(ix, yl, iz), v2 = P(ix, iy, zh) - P(ix, iy, zl);
  if (sprec) { /* float grid: the difference is a float */
    v0 = (float)v0;
    v1 = (float)v1;
    v2 = (float)v2;
  }
#undef P
  double u0 = x0 / rr, u1 = y0 / rr, u2 = z0 / rr;
  return 0.5 * idx * (v0 * u0 + v1 * u1 + v2 * u2);
}

int or_imap64_part(const cg_config *c, int ipop, const double *dens, const double *npot, const double *nrm,
                   double n0, double nf, int iz_stride, double *data, int *nadd, long long *nsamp, int sprec)
{
  long long ns_tot = 0;
  const int N = c->n_grid, nr = c->imap_nr[ipop], nside = c->nside_imap[ipop];
  const long npix = 12L * nside * nside;
  double *r0 = malloc(nr * sizeof(double)), *rf = malloc(nr * sizeof(double));
  int *ns = malloc(nr * sizeof(int)), *ord = malloc(nr * sizeof(int));
  for (int i = 0; i < nr; i++) ord[i] = i;
  for (int i = 1; i < nr; i++) /* insertion sort by r0 (stable) */
    for (int j = i; j > 0 && c->imap_r0[ipop][ord[j]] < c->imap_r0[ipop][ord[j - 1]]; j--) {
      int t = ord[j];
      ord[j] = ord[j - 1];
      ord[j - 1] = t;
    }
  for (int i = 0; i < nr; i++) { /* the shells are flouble: float with _SPREC */
    r0[i] = sprec ? (float)c->imap_r0[ipop][ord[i]] : c->imap_r0[ipop][ord[i]];
    rf[i] = sprec ? (float)c->imap_rf[ipop][ord[i]] : c->imap_rf[ipop][ord[i]];
  }
  const double dx = c->l_box / N, ps = sqrt(4 * M_PI / npix);
  for (int i = 0; i < nr; i++) {
    double vol = (rf[i] * rf[i] * rf[i] - r0[i] * r0[i] * r0[i]) * ps * ps / 3;
    ns[i] = (int)(dx / fmin(pow(vol, 0.333333), fmin(r0[i] * ps, rf[i] - r0[i])) + 0.5) + 1;
  }
  const double rmin = r0[0] - 20., rmax = rf[nr - 1] + 20.;
  const double fvel = -c->fgrowth_0 / (1.5 * c->hubble_0 * c->omega_m);
  memset(data, 0, (size_t)nr * npix * sizeof(double));
  memset(nadd, 0, (size_t)nr * npix * sizeof(int));
  const double *tz = c->imap_tz_arr[ipop], *bz = c->imap_bz_arr[ipop];
  for (int iz = 0; iz < N; iz += iz_stride) {
    int irad = 0;
    double z0 = iz * dx - c->pos_obs[2];
    for (int iy = 0; iy < N; iy++) {
      double y0 = iy * dx - c->pos_obs[1];
      for (int ix = 0; ix < N; ix++) {
        double x0 = ix * dx - c->pos_obs[0];
        double rc = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        double tm = bg(c, tz, 0, 0, rc);
        if (!(rc <= rmax && rc >= rmin && tm > 0)) continue;
        double b = bg(c, bz, bz[0], 1, rc), dn = bg(c, nrm, n0, nf, rc);
        double rv = fvel * rvel64(c, npot, ix, iy, iz, x0, y0, z0, rc, sprec);
        double drr = rv * BG_V1(c, rc) * BG_IH(c, rc);
        size_t id = ix + (size_t)N * (iy + (size_t)N * iz);
        double temp = tm * bias_model64(dens[id], b, c->bias_model) * dn;
        /* get_r_index_imap walk (imap.c:76-103), bounded */
#define WALK(R, START)                                                   \
  ({                                                                     \
    int q = (START) < 0 ? 0 : ((START) >= nr ? nr - 1 : (START));        \
    for (int it = 0; it < 2 * nr + 4; it++) {                           \
      if (q == -1 || q == nr) break;                                     \
      if ((R) < r0[q]) q--;                                              \
      else if ((R) >= rf[q]) q++;                                        \
      else break;                                                        \
    }                                                                    \
    q;                                                                   \
  })
        irad = WALK(rc, irad);
        int nsh = irad < 0 ? ns[0] : (irad >= nr ? ns[nr - 1] : ns[irad]);
        ns_tot += (long long)nsh * nsh * nsh;
        double dxs = dx / nsh;
        for (int izz = 0; izz < nsh; izz++)
          for (int iyy = 0; iyy < nsh; iyy++)
            for (int ixx = 0; ixx < nsh; ixx++) {
              double r, cth, ph;
              cart2sph64(x0 + (ixx + 0.5) * dxs, y0 + (iyy + 0.5) * dxs, z0 + (izz + 0.5) * dxs, &r, &cth, &ph);
              irad = WALK(r + drr, irad);
              if (irad >= 0 && irad < nr) {
                long k = irad * npix + ang2pix64(nside, cth, ph);
                data[k] += temp;
                nadd[k]++;
              }
            }
#undef WALK
      }
    }
  }
  free(r0);
  free(rf);
  free(ns);
  free(ord);
  if (nsamp) *nsamp = ns_tot;
  return 0;
}

int or_imap64(const cg_config *c, int ipop, const double *dens, const double *npot, const double *nrm, double n0,
              double nf, double *data, int *nadd, int sprec)
{
  return or_imap64_part(c, ipop, dens, npot, nrm, n0, nf, 1, data, nadd, NULL, sprec);
}

/* Number of sub-samples imap_set_cartesian_single draws for species ipop at
 * the configuration's grid size (cells in the shells' range with T > 0,
 * times nsub^3), from the geometry alone. */
long long or_imap_samples(const cg_config *c, int ipop)
{
  const int N = c->n_grid, nr = c->imap_nr[ipop], nside = c->nside_imap[ipop];
  const long npix = 12L * nside * nside;
  double r0min = 1e300, rfmax = -1e300;
  double *r0 = malloc(nr * sizeof(double)), *rf = malloc(nr * sizeof(double));
  int *ns = malloc(nr * sizeof(int));
  int *ord = malloc(nr * sizeof(int));
  for (int i = 0; i < nr; i++) ord[i] = i;
  for (int i = 1; i < nr; i++)
    for (int j = i; j > 0 && (float)c->imap_r0[ipop][ord[j]] < (float)c->imap_r0[ipop][ord[j - 1]]; j--) {
      int t = ord[j];
      ord[j] = ord[j - 1];
      ord[j - 1] = t;
    }
  for (int i = 0; i < nr; i++) { /* the shells are flouble (float) in the reference */
    r0[i] = (float)c->imap_r0[ipop][ord[i]];
    rf[i] = (float)c->imap_rf[ipop][ord[i]];
  }
  const double dx = c->l_box / N, ps = sqrt(4 * M_PI / npix);
  for (int i = 0; i < nr; i++) {
    double vol = (rf[i] * rf[i] * rf[i] - r0[i] * r0[i] * r0[i]) * ps * ps / 3;
    ns[i] = (int)(dx / fmin(pow(vol, 0.333333), fmin(r0[i] * ps, rf[i] - r0[i])) + 0.5) + 1;
    if (r0[i] < r0min) r0min = r0[i];
    if (rf[i] > rfmax) rfmax = rf[i];
  }
  const double rmin = r0[0] - 20., rmax = rf[nr - 1] + 20.;
  const double *tz = c->imap_tz_arr[ipop];
  long long tot = 0;
#pragma omp parallel for schedule(dynamic) reduction(+ : tot)
  for (int iz = 0; iz < N; iz++) {
    double z0 = iz * dx - c->pos_obs[2];
    int q = 0;
    for (int iy = 0; iy < N; iy++) {
      double y0 = iy * dx - c->pos_obs[1];
      for (int ix = 0; ix < N; ix++) {
        double x0 = ix * dx - c->pos_obs[0];
        double rc = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        if (!(rc <= rmax && rc >= rmin)) continue;
        if (!(bg(c, tz, 0, 0, rc) > 0)) continue;
        for (int it = 0; it < 2 * nr + 4; it++) {
          if (q == -1 || q == nr) break;
          if (rc < r0[q]) q--;
          else if (rc >= rf[q]) q++;
          else break;
        }
        int nsh = q < 0 ? ns[0] : (q >= nr ? ns[nr - 1] : ns[q]);
        if (q < 0) q = 0;
        if (q >= nr) q = nr - 1;
        tot += (long long)nsh * nsh * nsh;
      }
    }
  }
  free(r0);
  free(rf);
  free(ns);
  free(ord);
  return tot;
}

static void pix2vec_nest64(long nside, long ip, double v[3])
{
  int64_t jr, jp, nr, ks;
  cg_nest_ringpos(nside, ip, &jr, &jp, &nr, &ks);
  double fact2 = 4.0 / (12.0 * nside * nside), z;
  if (jr < nside) z = 1 - nr * nr * fact2;
  else if (jr > 3 * nside) z = nr * nr * fact2 - 1;
  else z = (2 * nside - jr) * 2.0 / (3.0 * nside);
  double phi = (jp - (ks + 1) * 0.5) * (M_PI / 2) / nr;
  double sth = sqrt((1 - z) * (1 + z));
  v[0] = sth * cos(phi);
  v[1] = sth * sin(phi);
  v[2] = z;
}

int or_kappa64_part(const cg_config *c, const double *p, int pix_stride, double *map)
{
  const int N = c->n_grid, np = c->n_kappa, nside = c->nside_kappa;
  const long npix = 12L * nside * nside;
  const int nr = N / 2;
  const double dr = c->r_max / nr, idr = 1. / dr, idx = N / c->l_box;
  double rp[CG_NPLANES_MAX];
  for (int i = 0; i < np; i++) rp[i] = (float)c->kappa_r[i]; /* stored as flouble */
  for (int i = 1; i < np; i++)
    for (int j = i; j > 0 && rp[j] < rp[j - 1]; j--) {
      double t = rp[j];
      rp[j] = rp[j - 1];
      rp[j - 1] = t;
    }
  int irmin[CG_NPLANES_MAX], irmax[CG_NPLANES_MAX];
  double inv[CG_NPLANES_MAX];
  for (int i = 0; i < np; i++) {
    int irh = (int)(rp[i] * idr + 0.5);
    inv[i] = 1. / (irh * dr);
    irmax[i] = irh < nr - 1 ? irh : nr - 1;
  }
  irmin[0] = 0;
  for (int i = 1; i < np; i++) irmin[i] = irmax[i - 1] + 1;
  double *f1 = malloc(nr * sizeof(double)), *f2 = malloc(nr * sizeof(double));
  for (int i = 0; i < nr; i++) {
    double rm = (i + 0.5) * dr, pg = BG_D1(c, rm) * (1 + BG_Z(c, rm));
    f1[i] = rm * pg * dr;
    f2[i] = rm * rm * pg * dr;
  }
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < npix; ip += pix_stride) {
    double u[3];
    pix2vec_nest64(nside, ip, u);
    double cth = u[2] > 1 ? 1 : (u[2] < -1 ? -1 : u[2]), sth = sqrt((1 - cth) * (1 + cth)), cph = 1, sph = 0;
    if (sth != 0) {
      cph = u[0] / sth;
      sph = u[1] / sth;
    }
    double pf = idx * idx, rot[6] = {(cth * cth * cph * cph + sph * sph) * pf, (2 * cph * sph * (cth * cth - 1)) * pf,
                                     (-2 * cth * sth * cph) * pf,            (cth * cth * sph * sph + cph * cph) * pf,
                                     (-2 * cth * sth * sph) * pf,            (sth * sth) * pf};
    long ring = cg_nest2ring(nside, ip);
    double k1 = 0, k2 = 0;
    for (int pl = 0; pl < np; pl++) {
      for (int irr = irmin[pl]; irr <= irmax[pl]; irr++) {
        double rm = (irr + 0.5) * dr;
        int cc[3];
        for (int a = 0; a < 3; a++) {
          long q = (long)((rm * u[a] + c->pos_obs[a]) * idx + 0.5);
          cc[a] = (int)(q >= N ? q - N : (q < 0 ? q + N : q));
        }
        int x0 = cc[0], y0 = cc[1], z0 = cc[2];
        int xh = (x0 + 1) % N, xl = (x0 + N - 1) % N, yh = (y0 + 1) % N, yl = (y0 + N - 1) % N, zh = (z0 + 1) % N,
            zl = (z0 + N - 1) % N;
#define P(X, Y, Z) p[(X) + (size_t)N * ((Y) + (size_t)N * (Z))]
        double t[6];
        t[0] = P(xh, y0, z0) + P(xl, y0, z0) - 2 * P(x0, y0, z0);
        t[3] = P(x0, yh, z0) + P(x0, yl, z0) - 2 * P(x0, y0, z0);
        t[5] = P(x0, y0, zh) + P(x0, y0, zl) - 2 * P(x0, y0, z0);
        t[1] = 0.25 * (P(xh, yh, z0) + P(xl, yl, z0) - P(xh, yl, z0) - P(xl, yh, z0));
        t[2] = 0.25 * (P(xh, y0, zh) + P(xl, y0, zl) - P(xh, y0, zl) - P(xl, y0, zh));
        t[4] = 0.25 * (P(x0, yh, zh) + P(x0, yl, zl) - P(x0, yh, zl) - P(x0, yl, zh));
#undef P
        double dot = 0;
        for (int a = 0; a < 6; a++) dot += rot[a] * t[a];
        k1 += dot * f1[irr];
        k2 += dot * f2[irr];
      }
      map[(long)pl * npix + ring] = k1 - inv[pl] * k2;
    }
  }
  free(f1);
  free(f2);
  return 0;
}

int or_kappa64(const cg_config *c, const double *p, double *map) { return or_kappa64_part(c, p, 1, map); }

/* isw_beams_preproc + isw_get_beam_properties, isw.c:38-147: per NEST pixel,
 * the potential at the nearest cell (RETURN_PDOT with the NGP lensing
 * interpolation, beaming.c:81-82,145-180) times 2 PD(r) dr, summed along the
 * ray and written at each plane (cumulative), in RING order (write_isw,
 * io.c:946-1010). */
int or_isw64(const cg_config *c, const double *p, double *map)
{
  const int N = c->n_grid, np = c->n_isw, nside = c->nside_isw;
  const long npix = 12L * nside * nside;
  const int nr = N / 2;
  const double dr = c->r_max / nr, idr = 1. / dr, idx = N / c->l_box;
  double rp[CG_NPLANES_MAX];
  for (int i = 0; i < np; i++) rp[i] = (float)c->isw_r[i]; /* stored as flouble */
  for (int i = 1; i < np; i++)
    for (int j = i; j > 0 && rp[j] < rp[j - 1]; j--) {
      double t = rp[j];
      rp[j] = rp[j - 1];
      rp[j - 1] = t;
    }
  int irmin[CG_NPLANES_MAX], irmax[CG_NPLANES_MAX];
  for (int i = 0; i < np; i++) {
    int irh = (int)(rp[i] * idr + 0.5);
    irmax[i] = irh < nr - 1 ? irh : nr - 1;
  }
  irmin[0] = 0;
  for (int i = 1; i < np; i++) irmin[i] = irmax[i - 1] + 1;
  double *fac = malloc(nr * sizeof(double));
  const double *pd = c->growth_pd_arr;
  for (int i = 0; i < nr; i++) fac[i] = 2 * bg(c, pd, pd[0], pd[CG_NA - 1], (i + 0.5) * dr) * dr;
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < npix; ip++) {
    double u[3];
    pix2vec_nest64(nside, ip, u);
    long ring = cg_nest2ring(nside, ip);
    double isw = 0;
    for (int pl = 0; pl < np; pl++) {
      for (int irr = irmin[pl]; irr <= irmax[pl]; irr++) {
        double rm = (irr + 0.5) * dr;
        int cc[3];
        for (int a = 0; a < 3; a++) {
          long q = (long)((rm * u[a] + c->pos_obs[a]) * idx + 0.5);
          cc[a] = (int)(q >= N ? q - N : (q < 0 ? q + N : q));
        }
        isw += p[cc[0] + (size_t)N * (cc[1] + (size_t)N * cc[2])] * fac[irr];
      }
      map[(long)pl * npix + ring] = isw;
    }
  }
  free(fac);
  return 0;
}

/* The Poisson stream of the build (gsl_ran_poisson's MT19937 stream cannot
 * be reproduced): the uniform of cell cid is word cid % 4 of the Philox block
 * with counter (cid / 4, 0, 0, 0), its top 24 bits times 2^-24; the PTRS
 * pairs of cell cid come from counter (cid, iteration, 1, 0). */
static double pois_u(long long cid, uint32_t k0, uint32_t k1)
{
  unsigned long long m = (unsigned long long)cid >> 2;
  cg_u32x4 w = cg_philox4x32_10((uint32_t)m, (uint32_t)(m >> 32), 0u, 0u, k0, k1);
  return (double)(w.v[cid & 3] >> 8) * 5.9604644775390625e-08;
}

/* PTRS transformed rejection (Hormann 1993) for lam >= 10, in double. */
static int ptrs64(double lam, long long cid, uint32_t k0, uint32_t k1)
{
  double slam = sqrt(lam), loglam = log(lam);
  double b = 2.53 * slam + 0.931;
  double a = 0.02483 * b + -0.059;
  double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (uint32_t it = 0; it < 64u; it++) {
    cg_u32x4 w = cg_philox4x32_10((uint32_t)cid, (uint32_t)((unsigned long long)cid >> 32), it, 1u, k0, k1);
    double U = (double)(w.v[0] >> 8) * 5.9604644775390625e-08 - 0.5;
    double V = (double)(w.v[1] >> 8) * 5.9604644775390625e-08;
    double us = 0.5 - fabs(U);
    double kd = floor(((2.0 * a / us + b) * U + lam) + 0.43);
    if (us >= 0.07 && V <= vr) return (int)kd;
    if (kd < 0 || (us < 0.013 && V > us)) continue;
    double lhs = log(V) + (log(invalpha) - log(a / (us * us) + b));
    double rhs = (kd * loglam - lam) - lgamma(kd + 1.0);
    if (lhs <= rhs) return (int)kd;
  }
  return (int)floor(lam);
}

/* Poisson deviate in double: inversion by sequential search for lam < 10,
 * PTRS above. */
static int poisson64(double lam, uint32_t k0, uint32_t k1, long long cid)
{
  if (!(lam > 0)) return 0;
  if (lam >= 10) return ptrs64(lam, cid, k0, k1);
  double u = pois_u(cid, k0, k1), p = exp(-lam), F = p;
  int k = 0;
  while (u >= F && k < 200) {
    k++;
    p *= lam / k;
    F += p;
  }
  return k;
}

/* Counts of every cell of population ipop (srcs_set_cartesian_single pass 1,
 * srcs.c:156-183) in double from the float density dens (unpadded, as
 * doubles) and the normalisation table normtab (CG_NA values, then the two
 * edge values). */
int or_counts64(const cg_config *c, int ipop, const double *dens, const double *normtab, int *counts,
                long long *total)
{
  const size_t ncell = (size_t)c->n_grid * c->n_grid * c->n_grid;
  double *lam = malloc(ncell * sizeof(double));
  if (!lam) return -1;
  or_lambda64(c, ipop, dens, normtab, normtab[CG_NA], normtab[CG_NA + 1], lam);
  const uint32_t k0 = (uint32_t)c->seed, k1 = (uint32_t)(c->seed >> 32) ^ (CG_STREAM_POIS + (uint32_t)ipop);
  long long t = 0;
#pragma omp parallel for schedule(static) reduction(+ : t)
  for (size_t i = 0; i < ncell; i++) {
    int n = poisson64(lam[i], k0, k1, (long long)i);
    if (counts) counts[i] = n;
    t += n;
  }
  free(lam);
  *total = t;
  return 0;
}

/* The catalogue of population ipop in double (srcs_set_cartesian_single
 * pass 2, srcs.c:238-276; srcs_get_local_properties_single, srcs.c:386-416):
 * sources in cell order; pos4 = x, y, z, dz_rsd as the reference's float
 * CatalogCartesian.pos; ipix the NEST base pixel of vec2pix_ring of the float
 * position; src9 the Src record (ra, dec, z0, dz_rsd, e1, e2, then 0s); cmap
 * the count map at nside_count (he_ang2pix of cart2sph of the float
 * position).  counts: the cell counts (or_counts64).  Returns -1 when more
 * than cap sources. */
#define RTOD64 57.2957795 /* RTOD, common.h:124 */
int or_emit64(const cg_config *c, int ipop, const double *npot, const int *counts, long long cap, float *pos4,
              int *ipix, float *src9, int *cmap, long long *nsrc)
{
  const int N = c->n_grid;
  const double dx = c->l_box / N, idx = c->n_grid / c->l_box;
  const double fvel = -c->fgrowth_0 / (1.5 * c->hubble_0 * c->omega_m);
  const uint32_t kq0 = (uint32_t)c->seed, kq1 = (uint32_t)(c->seed >> 32) ^ (CG_STREAM_POS + (uint32_t)ipop);
  const long nsb = c->nside_base, nsc = c->nside_count[ipop];
  long long id = 0;
  for (int iz = 0; iz < N; iz++) {
    double z0 = (iz + 0.0) * dx - c->pos_obs[2];
    for (int iy = 0; iy < N; iy++) {
      double y0 = (iy + 0.0) * dx - c->pos_obs[1];
      for (int ix = 0; ix < N; ix++) {
        size_t cid = ix + (size_t)N * (iy + (size_t)N * iz);
        int n = counts[cid];
        if (n <= 0) continue;
        double x0 = (ix + 0.0) * dx - c->pos_obs[0];
        double rr = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
        /* get_rvel (srcs.c:87-118): float differences of the float grid */
        int xh = (ix + 1) % N, xl = (ix + N - 1) % N, yh = (iy + 1) % N, yl = (iy + N - 1) % N;
        int zh = (iz + 1) % N, zl = (iz + N - 1) % N;
#define P(X, Y, Z) npot[(X) + (size_t)N * ((Y) + (size_t)N * (Z))]
        double v0 = (float)(P(xh, iy, iz) - P(xl, iy, iz)), v1 = (float)(P(ix, yh, iz) - P(ix, yl, iz));
        double v2 = (float)(P(ix, iy, zh) - P(ix, iy, zl));
#undef P
        double u0 = x0 / rr, u1 = y0 / rr, u2 = z0 / rr;
        double rvel = fvel * (0.5 * idx * (v0 * u0 + v1 * u1 + v2 * u2));
        double dz_rsd = rvel * BG_V1(c, rr);
        for (int j = 0; j < n; j++, id++) {
          if (id >= cap) return -1;
          cg_u32x4 u = cg_philox4x32_10((uint32_t)cid, (uint32_t)((unsigned long long)cid >> 32), (uint32_t)j, 0u,
                                        kq0, kq1);
          float p[4];
          p[0] = (float)(x0 + dx * ((double)(u.v[0] >> 8) * 5.9604644775390625e-08 - 0.5));
          p[1] = (float)(y0 + dx * ((double)(u.v[1] >> 8) * 5.9604644775390625e-08 - 0.5));
          p[2] = (float)(z0 + dx * ((double)(u.v[2] >> 8) * 5.9604644775390625e-08 - 0.5));
          p[3] = (float)dz_rsd;
          if (pos4) memcpy(pos4 + 4 * id, p, sizeof(p));
          double v[3] = {p[0], p[1], p[2]};
          double vlen = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
          if (ipix) ipix[id] = (int)cg_ring2nest(nsb, ang2pix64(nsb, v[2] / vlen, atan2(v[1], v[0])));
          double r, cth, ph;
          cart2sph64(v[0], v[1], v[2], &r, &cth, &ph);
          if (src9) {
            float *q = src9 + 9 * id;
            q[0] = (float)(RTOD64 * ph);
            q[1] = (float)(90 - RTOD64 * acos(cth));
            q[2] = (float)BG_Z(c, r);
            q[3] = c->need_beaming ? 0.0f : p[3];
            q[4] = c->need_beaming ? 0.0f : -1.0f;
            q[5] = c->need_beaming ? 0.0f : -1.0f;
            q[6] = q[7] = q[8] = 0.0f;
          }
          if (cmap && nsc > 0) cmap[ang2pix64(nsc, cth, ph)]++;
        }
      }
    }
  }
  *nsrc = id;
  return 0;
}

long long or_poisson_total64(const cg_config *c, int ipop, const double *lam)
{
  const size_t ncell = (size_t)c->n_grid * c->n_grid * c->n_grid;
  const uint32_t k0 = (uint32_t)c->seed, k1 = (uint32_t)(c->seed >> 32) ^ (CG_STREAM_POIS + (uint32_t)ipop);
  long long t = 0;
#pragma omp parallel for schedule(static) reduction(+ : t)
  for (size_t i = 0; i < ncell; i++) t += poisson64(lam[i], k0, k1, (long long)i);
  return t;
}

int or_run_mock64(const cg_config *c, int nthreads_hint, long long *nsrc_total, double *checksum)
{
  (void)nthreads_hint;
  const int N = c->n_grid;
  const size_t ncell = (size_t)N * N * N;
  double *dens = malloc(ncell * sizeof(double)), *npot = malloc(ncell * sizeof(double));
  if (!dens || !npot) return -1;
  double st[4];
  or_field64(c, dens, npot, st);
  if (c->dens_type == CG_DENS_1LPT) {
    double *d2 = malloc(ncell * sizeof(double)), *disp = malloc(3 * ncell * sizeof(double));
    or_lpt64(c, dens, d2, disp);
    memcpy(dens, d2, ncell * sizeof(double));
    free(d2);
    free(disp);
  } else {
    or_density64(c, dens, st[3]);
  }
  const int nt = c->n_srcs + c->n_imap + c->n_cstm;
  double *tabs = malloc((size_t)(nt > 0 ? nt : 1) * CG_NA * sizeof(double)), e0f[2 * 3 * CG_NPOP_MAX];
  unsigned long long narr[4096];
  double zarr[4096], *bsum = malloc((size_t)(nt > 0 ? nt : 1) * 4096 * sizeof(double));
  int nz;
  or_norm_tables64(c, tabs, e0f, &nz, narr, zarr, bsum, dens);
  double cs = 0;
  long long tot = 0;
  double *lam = malloc(ncell * sizeof(double));
  for (int p = 0; p < c->n_srcs; p++) {
    or_lambda64(c, p, dens, tabs + (size_t)p * CG_NA, e0f[2 * p], e0f[2 * p + 1], lam);
    const uint32_t k0 = (uint32_t)c->seed, k1 = (uint32_t)(c->seed >> 32) ^ (CG_STREAM_POIS + (uint32_t)p);
    long long t = 0;
#pragma omp parallel for schedule(static) reduction(+ : t)
    for (size_t i = 0; i < ncell; i++) t += poisson64(lam[i], k0, k1, (long long)i);
    tot += t;
  }
  free(lam);
  for (int p = 0; p < c->n_imap; p++) {
    long npix = 12L * c->nside_imap[p] * c->nside_imap[p];
    double *data = malloc((size_t)c->imap_nr[p] * npix * sizeof(double));
    int *nadd = malloc((size_t)c->imap_nr[p] * npix * sizeof(int));
    or_imap64(c, p, dens, npot, tabs + (size_t)(c->n_srcs + p) * CG_NA, e0f[2 * (c->n_srcs + p)],
              e0f[2 * (c->n_srcs + p) + 1], data, nadd, 1);
    for (long i = 0; i < (long)c->imap_nr[p] * npix; i++) cs += nadd[i];
    free(data);
    free(nadd);
  }
  if (c->do_kappa) {
    long npix = 12L * c->nside_kappa * c->nside_kappa;
    double *map = malloc((size_t)c->n_kappa * npix * sizeof(double));
    or_kappa64(c, npot, map);
    for (long i = 0; i < (long)c->n_kappa * npix; i++) cs += map[i];
    free(map);
  }
  free(tabs);
  free(bsum);
  free(dens);
  free(npot);
  if (nsrc_total) *nsrc_total = tot;
  if (checksum) *checksum = cs + st[3];
  return 0;
}

/* Step tables of cstm_get_beam_properties (cstm.c:81-116): kz = K(r)/IH(r)
 * and b(r) at the N/2 step centres, and the integration range where
 * |kz| > 1e-4 max|kz|.  Returns -1 when the kernel has no support. */
int or_cstm_steps(const cg_config *c, int ipop, double *kz, double *bz, int *ir_min, int *ir_max)
{
  const int nr = c->n_grid / 2;
  const double dr = c->r_max / nr;
  const double *kt = c->cstm_kz_arr[ipop], *bt = c->cstm_bz_arr[ipop];
  double kmax = -1e100;
  for (int i = 0; i < nr; i++) {
    const double rm = (i + 0.5) * dr;
    kz[i] = bg(c, kt, 0, 0, rm) / BG_IH(c, rm);
    bz[i] = bg(c, bt, bt[0], 1, rm);
    if (fabs(kz[i]) > kmax) kmax = fabs(kz[i]);
  }
  *ir_min = 0;
  *ir_max = nr - 1;
  for (int i = 0; i < nr; i++)
    if (fabs(kz[i]) > 1e-4 * kmax) {
      *ir_min = i;
      break;
    }
  for (int i = nr - 1; i >= 0; i--)
    if (fabs(kz[i]) > 1e-4 * kmax) {
      *ir_max = i;
      break;
    }
  return *ir_max < *ir_min ? -1 : 0;
}

/* cstm_get_beam_properties (cstm.c:68-145) in double precision: per NEST
 * pixel, dr * sum over the support of kz (bias_model(d, bz) norm - 1), d the
 * trilinear density at (rm u + pos_obs) idx (interpolate_from_grid,
 * beaming.c:183-262).  dens: N^3 unpadded; map: NEST order (write_cstm,
 * io.c:754-800, writes the shell data without reordering). */
int or_cstm64(const cg_config *c, int ipop, const double *dens, const double *normtab, double n0, double nf,
              double *map)
{
  const int N = c->n_grid, nr = N / 2, nside = c->nside_cstm[ipop];
  const long npix = 12L * nside * nside;
  const double dr = c->r_max / nr, idx = N / c->l_box;
  double *kz = malloc(3 * (size_t)nr * sizeof(double)), *bz = kz + nr, *nm = bz + nr;
  int lo, hi;
  if (or_cstm_steps(c, ipop, kz, bz, &lo, &hi)) {
    free(kz);
    return -1;
  }
  for (int i = 0; i < nr; i++) nm[i] = bg(c, normtab, n0, nf, (i + 0.5) * dr);
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < npix; ip++) {
    double u[3], cval = 0;
    pix2vec_nest64(nside, ip, u);
    for (int irr = lo; irr <= hi; irr++) {
      const double rm = (irr + 0.5) * dr;
      long i0[3], i1[3];
      double h0[3], h1[3];
      for (int a = 0; a < 3; a++) {
        const double x = (rm * u[a] + c->pos_obs[a]) * idx;
        i0[a] = (long)x;
        h0[a] = x - i0[a];
        h1[a] = 1 - h0[a];
        i1[a] = i0[a] + 1;
        if (i0[a] >= N) i0[a] -= N;
        else if (i0[a] < 0) i0[a] += N;
        if (i1[a] >= N) i1[a] -= N;
        else if (i1[a] < 0) i1[a] += N;
      }
#define D(X, Y, Z) dens[(X) + (size_t)N * ((Y) + (size_t)N * (Z))]
      const double d = (D(i0[0], i0[1], i0[2]) * h1[2] * h1[1] * h1[0] + D(i1[0], i0[1], i0[2]) * h1[2] * h1[1] * h0[0] +
                        D(i0[0], i1[1], i0[2]) * h1[2] * h0[1] * h1[0] + D(i1[0], i1[1], i0[2]) * h1[2] * h0[1] * h0[0]) +
                       (D(i0[0], i0[1], i1[2]) * h0[2] * h1[1] * h1[0] + D(i1[0], i0[1], i1[2]) * h0[2] * h1[1] * h0[0] +
                        D(i0[0], i1[1], i1[2]) * h0[2] * h0[1] * h1[0] + D(i1[0], i1[1], i1[2]) * h0[2] * h0[1] * h0[0]);
#undef D
      cval += kz[irr] * (bias_model64(d, bz[irr], c->bias_model) * nm[irr] - 1);
    }
    map[ip] = cval * dr;
  }
  free(kz);
  return 0;
}

/* per-source direction and last step of srcs_get_beam_properties_single
 * (srcs.c:485-493, 583): r from the float position, u = pos / max(r, 0.001) */
static int los64_setup(const cg_config *c, const float *pos, double *r, double u[3])
{
  const int nr = c->n_grid / 2;
  const double idr = nr / c->r_max;
  *r = sqrt((double)pos[0] * pos[0] + (double)pos[1] * pos[1] + (double)pos[2] * pos[2]);
  const double ir = 1. / (*r > 0.001 ? *r : 0.001);
  for (int a = 0; a < 3; a++) u[a] = pos[a] * ir;
  const int k = (int)(*r * idr + 0.5);
  return k < nr - 1 ? k : nr - 1;
}

#define P64(G, X, Y, Z) (G)[(X) + (size_t)N * ((Y) + (size_t)N * (Z))]

/* srcs_get_beam_properties_single, lensing branch without _USE_FAST_LENSING
 * (srcs.c:465-478, 536-625), and the degree conversion of the deflections in
 * srcs_beams_postproc_single (srcs.c:721-722).  npot: N^3 unpadded;
 * pos4: 4 floats per source; out: 5 per source (e1, e2, kappa, dra, ddec). */
int or_lens64(const cg_config *c, const double *p, long long n, const float *pos4, double *out)
{
  const int N = c->n_grid, nr = N / 2;
  const double dr = c->r_max / nr, idx = N / c->l_box;
  double *f0 = malloc(3 * (size_t)nr * sizeof(double)), *f1 = f0 + nr, *f2 = f1 + nr;
  for (int i = 0; i < nr; i++) {
    const double rm = (i + 0.5) * dr, pg = BG_D1(c, rm) * (1 + BG_Z(c, rm));
    f0[i] = pg * dr;
    f1[i] = rm * pg * dr;
    f2[i] = rm * rm * pg * dr;
  }
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    double r, u[3];
    const int kmax = los64_setup(c, pos4 + 4 * i, &r, u);
    const double ir = 1. / (r > 0.001 ? r : 0.001);
    double cth = u[2] >= 1 ? 1 : (u[2] <= -1 ? -1 : u[2]), sth = sqrt((1 - cth) * (1 + cth)), cph = 1, sph = 0;
    if (sth != 0) {
      cph = u[0] / sth;
      sph = u[1] / sth;
    }
    const double pf = idx * idx * ir, pm = 0.5 * idx * ir;
    const double ux[3] = {cth * cph * pm, cth * sph * pm, -sth * pm}, uy[3] = {-sph * pm, cph * pm, 0};
    const double rk[6] = {(cth * cth * cph * cph + sph * sph) * pf, (2 * cph * sph * (cth * cth - 1)) * pf,
                          (-2 * cth * sth * cph) * pf,            (cth * cth * sph * sph + cph * cph) * pf,
                          (-2 * cth * sth * sph) * pf,            (sth * sth) * pf};
    const double re1[6] = {(cth * cth * cph * cph - sph * sph) * pf, (2 * cph * sph * (cth * cth + 1)) * pf,
                           (-2 * cth * sth * cph) * pf,            (cth * cth * sph * sph - cph * cph) * pf,
                           (-2 * cth * sth * sph) * pf,            (sth * sth) * pf};
    const double re2[6] = {(-2 * cth * cph * sph) * pf, (2 * cth * (cph * cph - sph * sph)) * pf,
                           (2 * sth * sph) * pf,        (2 * cth * sph * cph) * pf,
                           (-2 * sth * cph) * pf,       0};
    double e1 = 0, e2 = 0, kp = 0, dtx = 0, dty = 0;
    for (int k = 0; k <= kmax; k++) {
      const double rm = (k + 0.5) * dr;
      int cc[3];
      for (int a = 0; a < 3; a++) {
        long q = (long)((rm * u[a] + c->pos_obs[a]) * idx + 0.5);
        cc[a] = (int)(q >= N ? q - N : (q < 0 ? q + N : q));
      }
      const int x0 = cc[0], y0 = cc[1], z0 = cc[2];
      const int xh = (x0 + 1) % N, xl = (x0 + N - 1) % N, yh = (y0 + 1) % N, yl = (y0 + N - 1) % N,
                zh = (z0 + 1) % N, zl = (z0 + N - 1) % N;
      double t[6], v[3];
      v[0] = P64(p, xh, y0, z0) - P64(p, xl, y0, z0);
      v[1] = P64(p, x0, yh, z0) - P64(p, x0, yl, z0);
      v[2] = P64(p, x0, y0, zh) - P64(p, x0, y0, zl);
      t[0] = P64(p, xh, y0, z0) + P64(p, xl, y0, z0) - 2 * P64(p, x0, y0, z0);
      t[3] = P64(p, x0, yh, z0) + P64(p, x0, yl, z0) - 2 * P64(p, x0, y0, z0);
      t[5] = P64(p, x0, y0, zh) + P64(p, x0, y0, zl) - 2 * P64(p, x0, y0, z0);
      t[1] = 0.25 * (P64(p, xh, yh, z0) + P64(p, xl, yl, z0) - P64(p, xh, yl, z0) - P64(p, xl, yh, z0));
      t[2] = 0.25 * (P64(p, xh, y0, zh) + P64(p, xl, y0, zl) - P64(p, xh, y0, zl) - P64(p, xl, y0, zh));
      t[4] = 0.25 * (P64(p, x0, yh, zh) + P64(p, x0, yl, zl) - P64(p, x0, yh, zl) - P64(p, x0, yl, zh));
      const double fr = f1[k] * r - f2[k], frm = 2 * (f0[k] * r - f1[k]);
      double d1 = 0, d2 = 0, dk = 0, dvx = 0, dvy = 0;
      for (int a = 0; a < 6; a++) {
        d1 += re1[a] * t[a];
        d2 += re2[a] * t[a];
        dk += rk[a] * t[a];
      }
      for (int a = 0; a < 3; a++) {
        dvx += ux[a] * v[a];
        dvy += uy[a] * v[a];
      }
      e1 += d1 * fr;
      e2 += d2 * fr;
      kp += dk * fr;
      dtx += dvx * frm;
      dty += dvy * frm;
    }
    double *o = out + 5 * i;
    o[0] = e1;
    o[1] = e2;
    o[2] = kp;
    o[3] = dty * (180. / M_PI);
    o[4] = dtx * (180. / M_PI);
  }
  free(f0);
  return 0;
}

/* Skewers (srcs.c:509-536 with INTERP_TYPE_SKW = CIC, beaming.c:183-265; the
 * velocity scaling of srcs.c:725-733): density (or, with gauss, the
 * Gaussian field log(1 + d)/D(r_cell) + D(r_cell) sigma^2/2 of each corner
 * cell, beaming.c:54-66) and the radial velocity times V1(rm) factor_vel at
 * every step up to the source, 0 beyond.  dens, npot: N^3 unpadded. */
int or_skw64(const cg_config *c, const double *dens, const double *p, int gauss, double sigma2, long long n,
             const float *pos4, double *dout, double *vout)
{
  const int N = c->n_grid, nr = N / 2;
  const double dr = c->r_max / nr, idx = N / c->l_box, dx = c->l_box / N;
  const double fv = -c->fgrowth_0 / (1.5 * c->hubble_0 * c->omega_m);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    double r, u[3];
    const int kmax = los64_setup(c, pos4 + 4 * i, &r, u);
    double *od = dout + (size_t)i * nr, *ov = vout + (size_t)i * nr;
    for (int k = 0; k < nr; k++) od[k] = ov[k] = 0;
    for (int k = 0; k <= kmax; k++) {
      const double rm = (k + 0.5) * dr;
      long i0[3], i1[3];
      double h0[3], h1[3];
      for (int a = 0; a < 3; a++) {
        const double x = (rm * u[a] + c->pos_obs[a]) * idx;
        i0[a] = (long)x;
        h0[a] = x - i0[a];
        h1[a] = 1 - h0[a];
        i1[a] = i0[a] + 1;
        if (i0[a] >= N) i0[a] -= N;
        else if (i0[a] < 0) i0[a] += N;
        if (i1[a] >= N) i1[a] -= N;
        else if (i1[a] < 0) i1[a] += N;
      }
      double d = 0, v[3] = {0, 0, 0};
      for (int b = 0; b < 8; b++) {
        const long ix = (b & 1) ? i1[0] : i0[0], iy = (b & 2) ? i1[1] : i0[1], iz = (b & 4) ? i1[2] : i0[2];
        const double w = ((b & 4) ? h0[2] : h1[2]) * ((b & 2) ? h0[1] : h1[1]) * ((b & 1) ? h0[0] : h1[0]);
        double val = P64(dens, ix, iy, iz);
        if (gauss) {
          const double x0 = ix * dx - c->pos_obs[0], y0 = iy * dx - c->pos_obs[1], z0 = iz * dx - c->pos_obs[2];
          const double dg = BG_D1(c, sqrt(x0 * x0 + y0 * y0 + z0 * z0));
          val = log(1 + val) / dg + dg * sigma2 * 0.5;
        }
        d += val * w;
        const long xh = (ix + 1) % N, xl = (ix + N - 1) % N, yh = (iy + 1) % N, yl = (iy + N - 1) % N,
                   zh = (iz + 1) % N, zl = (iz + N - 1) % N;
        v[0] += (P64(p, xh, iy, iz) - P64(p, xl, iy, iz)) * w;
        v[1] += (P64(p, ix, yh, iz) - P64(p, ix, yl, iz)) * w;
        v[2] += (P64(p, ix, iy, zh) - P64(p, ix, iy, zl)) * w;
      }
      od[k] = d;
      ov[k] = 0.5 * idx * (v[0] * u[0] + v[1] * u[1] + v[2] * u[2]) * BG_V1(c, rm) * fv;
    }
  }
  return 0;
}
#undef P64
