/*
 * or_dev32.c -- ORACLE (test infrastructure only).  CPU restatement of the
 * per-cell stages of CoLoRe evaluated with the single-precision arithmetic
 * the GPU kernels define (colore_gb300/csrc/cg_cell.h), in the reference's
 * loop order, so that integer results can be compared bit for bit:
 *   or_density32  lognormalize / densclip / 1LPT rho-1   density.c:1034-1103, 610-624
 *   or_bins32     collect_density_normalization_from_grid density.c:1128-1211
 *   or_counts32   srcs_set_cartesian_single, pass 1       srcs.c:156-184
 *   or_emit32     srcs_set_cartesian_single, pass 2, and
 *                 srcs_get_local_properties_single        srcs.c:238-276, 386-416
 *   or_beam_rsd32 srcs beam RSD (pre/get/postproc)        srcs.c:437-504, 656-662
 *   or_imap32     imap_set_cartesian_single               imap.c:135-245
 *   or_kappa32    kappa_get_beam_properties               kappa.c:78-175
 *   or_isw32      isw_get_beam_properties                 isw.c:78-147
 *   or_cstm32     cstm_get_beam_properties                cstm.c:68-145
 *   or_lens32     source lensing along the line of sight  srcs.c:452-625, 715-723
 *   or_skw32      source skewers                          srcs.c:509-536, 725-733
 * Tables are rebuilt from the config with the same double->float roundings
 * as the GPU upload.  The Poisson and position streams are the Philox
 * streams of the GPU path (the reference's GSL MT19937 streams depend on the
 * OpenMP thread count and cannot be reproduced).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../colore_gb300/csrc/cg_exact.h"
#include "oracle.h"

typedef struct {
  const float *f;
  float f0, ff;
} T32;

typedef struct {
  int N;
  float dx, idx, L, p[3];
  float *tabs, *r, r_last, idr;
  T32 zt, d1, v1, ih;
  float *a_a2r, *r_a2r;
  T32 nz[CG_NPOP_MAX], bz[CG_NPOP_MAX], tz[CG_NPOP_MAX], bzi[CG_NPOP_MAX], bzc[CG_NPOP_MAX];
} S32;

static void s32_init(S32 *s, const cg_config *c)
{
  const int na = CG_NA;
  const int ntab = 9 + 2 * c->n_srcs + 2 * c->n_imap + c->n_cstm;
  s->tabs = malloc((size_t)ntab * na * sizeof(float));
  const double *src[9] = {c->r_arr_r2z, c->z_arr_r2z, c->growth_d_arr, c->growth_d2_arr, c->growth_v_arr,
                          c->growth_pd_arr, c->ihub_arr, c->a_arr_a2r, c->r_arr_a2r};
  int k = 0;
  for (int t = 0; t < 9; t++, k++)
    for (int i = 0; i < na; i++) s->tabs[(size_t)k * na + i] = (float)src[t][i];
  for (int p = 0; p < c->n_srcs; p++) {
    for (int i = 0; i < na; i++) s->tabs[(size_t)k * na + i] = (float)c->srcs_nz_arr[p][i];
    for (int i = 0; i < na; i++) s->tabs[(size_t)(k + 1) * na + i] = (float)c->srcs_bz_arr[p][i];
    s->nz[p] = (T32){s->tabs + (size_t)k * na, 0.0f, 0.0f};
    s->bz[p] = (T32){s->tabs + (size_t)(k + 1) * na, (float)c->srcs_bz_arr[p][0], 1.0f};
    k += 2;
  }
  for (int p = 0; p < c->n_imap; p++) {
    for (int i = 0; i < na; i++) s->tabs[(size_t)k * na + i] = (float)c->imap_tz_arr[p][i];
    for (int i = 0; i < na; i++) s->tabs[(size_t)(k + 1) * na + i] = (float)c->imap_bz_arr[p][i];
    s->tz[p] = (T32){s->tabs + (size_t)k * na, 0.0f, 0.0f};
    s->bzi[p] = (T32){s->tabs + (size_t)(k + 1) * na, (float)c->imap_bz_arr[p][0], 1.0f};
    k += 2;
  }
  for (int p = 0; p < c->n_cstm; p++, k++) {
    for (int i = 0; i < na; i++) s->tabs[(size_t)k * na + i] = (float)c->cstm_bz_arr[p][i];
    s->bzc[p] = (T32){s->tabs + (size_t)k * na, (float)c->cstm_bz_arr[p][0], 1.0f};
  }
  float *T = s->tabs;
  s->r = T;
  s->r_last = (float)c->r_arr_r2z[na - 1];
  s->idr = (float)c->glob_idr;
  s->zt = (T32){T + 1 * na, 0.0f, (float)c->z_arr_r2z[na - 1]};
  s->d1 = (T32){T + 2 * na, 1.0f, (float)c->growth_d_arr[na - 1]};
  s->v1 = (T32){T + 4 * na, (float)c->growth_v_arr[0], (float)c->growth_v_arr[na - 1]};
  s->ih = (T32){T + 6 * na, (float)c->ihub_arr[0], (float)c->ihub_arr[na - 1]};
  s->a_a2r = T + 7 * na;
  s->r_a2r = T + 8 * na;
  s->N = c->n_grid;
  s->dx = (float)(c->l_box / c->n_grid);
  s->idx = (float)(c->n_grid / c->l_box);
  s->L = (float)c->l_box;
  for (int i = 0; i < 3; i++) s->p[i] = (float)c->pos_obs[i];
}

static void s32_free(S32 *s) { free(s->tabs); }

static float bg32(const S32 *s, T32 t, float r) { return cg_bg_eval(t.f, s->r, t.f0, t.ff, r, s->r_last, s->idr); }

static long long pidx(int ix, int iy, int iz, int N)
{
  return (long long)ix + (long long)(2 * (N / 2 + 1)) * ((long long)iy + (long long)N * iz);
}

static int wrapi(int i, int N) { return i >= N ? i - N : (i < 0 ? i + N : i); }

int or_density32(const cg_config *cfg, float *dens, float s2f, int mode)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N;
#pragma omp parallel for schedule(static)
  for (int iz = 0; iz < N; iz++) {
    float z0 = cg_cell_coord(iz, s.dx, s.p[2]);
    for (int iy = 0; iy < N; iy++) {
      float y0 = cg_cell_coord(iy, s.dx, s.p[1]);
      for (int ix = 0; ix < N; ix++) {
        float x0 = cg_cell_coord(ix, s.dx, s.p[0]);
        float r = cg_norm3(x0, y0, z0);
        long long id = pidx(ix, iy, iz, N);
        dens[id] = cg_dens_transform(mode, dens[id], bg32(&s, s.d1, r), s2f);
      }
    }
  }
  s32_free(&s);
  return 0;
}

int or_bins32(const cg_config *cfg, const float *dens, int nz, double idz, unsigned long long *narr, double *zarr,
              double *bsum)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N, nts = cfg->n_srcs, nti = cfg->n_imap, nt = nts + nti + cfg->n_cstm;
  const float idzf = (float)idz;
  memset(narr, 0, nz * sizeof(unsigned long long));
  memset(zarr, 0, nz * sizeof(double));
  memset(bsum, 0, (size_t)nt * nz * sizeof(double));
  for (int iz = 0; iz < N; iz++) {
    float z0 = cg_cell_coord(iz, s.dx, s.p[2]);
    for (int iy = 0; iy < N; iy++) {
      float y0 = cg_cell_coord(iy, s.dx, s.p[1]);
      for (int ix = 0; ix < N; ix++) {
        float x0 = cg_cell_coord(ix, s.dx, s.p[0]);
        float r = cg_norm3(x0, y0, z0);
        float z = bg32(&s, s.zt, r);
        int b = (int)CG_MUL(z, idzf) + 1;
        if (b < 0 || b >= nz) continue;
        float d = dens[pidx(ix, iy, iz, N)];
        narr[b]++;
        zarr[b] += z;
        for (int t = 0; t < nt; t++) {
          T32 tb = t < nts ? s.bz[t] : (t < nts + nti ? s.bzi[t - nts] : s.bzc[t - nts - nti]);
          bsum[(size_t)t * nz + b] += cg_bias_model(d, bg32(&s, tb, r), cfg->bias_model);
        }
      }
    }
  }
  s32_free(&s);
  return 0;
}

static void src_keys(const cg_config *c, int ipop, uint32_t *kp0, uint32_t *kp1, uint32_t *kq0, uint32_t *kq1)
{
  *kp0 = (uint32_t)c->seed;
  *kp1 = (uint32_t)(c->seed >> 32) ^ (CG_STREAM_POIS + (uint32_t)ipop);
  *kq0 = (uint32_t)c->seed;
  *kq1 = (uint32_t)(c->seed >> 32) ^ (CG_STREAM_POS + (uint32_t)ipop);
}

/* The arguments of cg_count_cell for population ipop, as the GPU builds
 * them: float tables and corners, double tables for the decisions that the
 * float margins leave open.  norm32 / norm64: CG_NA values and two edges. */
typedef struct {
  cg_pois_args a;
  float *corner;
} PoisArgs;

static void pois_args(PoisArgs *P, const cg_config *cfg, const S32 *s, int ipop, const float *norm32,
                      const double *norm64)
{
  cg_pois_args *a = &P->a;
  const int N = cfg->n_grid;
  memset(a, 0, sizeof(*a));
  a->r = s->r;
  a->nz = s->nz[ipop].f;
  a->bz = s->bz[ipop].f;
  a->norm = norm32;
  a->idr = s->idr;
  a->r_last = s->r_last;
  a->bz0 = s->bz[ipop].f0;
  a->na = CG_NA;
  a->bias_model = cfg->bias_model;
  const double dx = cfg->l_box / N;
  a->cell_vol = (float)(dx * dx * dx);
  a->rlim = (float)(cfg->l_box / 2 + 20.);
  P->corner = malloc(3 * (size_t)N * sizeof(float));
  for (int k = 0; k < 3; k++)
    for (int i = 0; i < N; i++) P->corner[k * N + i] = (float)cgx_coord(i, dx, cfg->pos_obs[k]);
  a->xc = P->corner;
  a->yc = P->corner + N;
  a->zc = P->corner + 2 * N;
  cgx_srcs_tabs *x = &a->x;
  x->r = cfg->r_arr_r2z;
  x->nz = cfg->srcs_nz_arr[ipop];
  x->bz = cfg->srcs_bz_arr[ipop];
  x->norm = norm64;
  x->idr = cfg->glob_idr;
  x->r_last = cfg->r_arr_r2z[CG_NA - 1];
  x->bz0 = cfg->srcs_bz_arr[ipop][0];
  x->dx = dx;
  x->cell_vol = dx * dx * dx;
  x->rlim = cfg->l_box / 2 + 20.;
  for (int k = 0; k < 3; k++) x->p[k] = cfg->pos_obs[k];
  x->bias_model = cfg->bias_model;
}

/* Counts of population ipop as the GPU computes them (cg_count_cell: float
 * margins, double decisions where they do not hold); *fallbacks counts the
 * cells decided in double. */
int or_counts32(const cg_config *cfg, int ipop, const float *dens, const float *norm32, const double *norm64,
                int *counts, long long *total, long long *fallbacks)
{
  S32 s;
  s32_init(&s, cfg);
  PoisArgs P;
  pois_args(&P, cfg, &s, ipop, norm32, norm64);
  const int N = s.N;
  uint32_t kp0, kp1, kq0, kq1;
  src_keys(cfg, ipop, &kp0, &kp1, &kq0, &kq1);
  long long tot = 0, nfb = 0;
#pragma omp parallel for schedule(static) reduction(+ : tot, nfb)
  for (int iz = 0; iz < N; iz++)
    for (int iy = 0; iy < N; iy++)
      for (int ix = 0; ix < N; ix++) {
        const long long cid = (long long)ix + (long long)N * ((long long)iy + (long long)N * iz);
        int fb = 0;
        const int n = cg_count_cell(&P.a, ix, iy, iz, dens[pidx(ix, iy, iz, N)], cid, cg_pois_word(cid, kp0, kp1),
                                    kp0, kp1, &fb);
        if (counts) counts[cid] = n;
        tot += n;
        nfb += fb;
      }
  *total = tot;
  if (fallbacks) *fallbacks = nfb;
  free(P.corner);
  s32_free(&s);
  return 0;
}

/* The catalogue as the GPU writes it: positions in double rounded to float
 * (the reference's), the base and count-map pixels by cg_src_pixels, the
 * velocity, RA, Dec and redshift in single precision. */
int or_emit32(const cg_config *cfg, int ipop, const float *dens, const float *npot, const float *norm32,
              const double *norm64, long long cap, float *pos4, int *ipix, float *src9, int *cmap, long long *nsrc,
              long long *fallbacks)
{
  S32 s;
  s32_init(&s, cfg);
  PoisArgs P;
  pois_args(&P, cfg, &s, ipop, norm32, norm64);
  const int N = s.N;
  uint32_t kp0, kp1, kq0, kq1;
  src_keys(cfg, ipop, &kp0, &kp1, &kq0, &kq1);
  const double dxd = cfg->l_box / N;
  const float fvel = (float)(-cfg->fgrowth_0 / (1.5 * cfg->hubble_0 * cfg->omega_m));
  const int nsb = cfg->nside_base, nsc = cfg->nside_count[ipop];
  long long id = 0, nfb = 0;
  for (int iz = 0; iz < N; iz++) {
    float z0 = cg_cell_coord(iz, s.dx, s.p[2]);
    for (int iy = 0; iy < N; iy++) {
      float y0 = cg_cell_coord(iy, s.dx, s.p[1]);
      for (int ix = 0; ix < N; ix++) {
        const long long cid = (long long)ix + (long long)N * ((long long)iy + (long long)N * iz);
        int fb = 0;
        const int n = cg_count_cell(&P.a, ix, iy, iz, dens[pidx(ix, iy, iz, N)], cid, cg_pois_word(cid, kp0, kp1),
                                    kp0, kp1, &fb);
        if (n == 0) continue;
        float x0 = cg_cell_coord(ix, s.dx, s.p[0]);
        float rr = cg_norm3(x0, y0, z0);
        int xh = wrapi(ix + 1, N), xl = wrapi(ix - 1, N), yh = wrapi(iy + 1, N), yl = wrapi(iy - 1, N);
        int zh = wrapi(iz + 1, N), zl = wrapi(iz - 1, N);
        float v0 = CG_SUB(npot[pidx(xh, iy, iz, N)], npot[pidx(xl, iy, iz, N)]);
        float v1 = CG_SUB(npot[pidx(ix, yh, iz, N)], npot[pidx(ix, yl, iz, N)]);
        float v2 = CG_SUB(npot[pidx(ix, iy, zh, N)], npot[pidx(ix, iy, zl, N)]);
        float rvel = CG_MUL(fvel, cg_rvel(v0, v1, v2, x0, y0, z0, rr, s.idx));
        float dz = CG_MUL(rvel, bg32(&s, s.v1, rr));
        const float dxh = (float)dxd, dxl = (float)(dxd - (double)(float)dxd);
        const double x0d = cgx_coord(ix, dxd, cfg->pos_obs[0]), y0d = cgx_coord(iy, dxd, cfg->pos_obs[1]);
        const double z0d = cgx_coord(iz, dxd, cfg->pos_obs[2]);
        for (int j = 0; j < n; j++, id++) {
          if (id >= cap) {
            free(P.corner);
            s32_free(&s);
            return -1;
          }
          cg_u32x4 u = cg_philox4x32_10((uint32_t)cid, (uint32_t)(cid >> 32), (uint32_t)j, 0u, kq0, kq1);
          /* the kernel's route: single precision where certain, else double */
          float px, py, pz;
          if (!cg_src_offset_checked((float)x0d, (float)(x0d - (double)(float)x0d), dxh, dxl, u.v[0], &px))
            px = cgx_src_offset(x0d, dxd, u.v[0]);
          if (!cg_src_offset_checked((float)y0d, (float)(y0d - (double)(float)y0d), dxh, dxl, u.v[1], &py))
            py = cgx_src_offset(y0d, dxd, u.v[1]);
          if (!cg_src_offset_checked((float)z0d, (float)(z0d - (double)(float)z0d), dxh, dxl, u.v[2], &pz))
            pz = cgx_src_offset(z0d, dxd, u.v[2]);
          if (pos4) {
            pos4[4 * id + 0] = px;
            pos4[4 * id + 1] = py;
            pos4[4 * id + 2] = pz;
            pos4[4 * id + 3] = dz;
          }
          long long pb = 0, pc = 0;
          int pfb = 0;
          cg_src_pixels(px, py, pz, nsb, cmap ? nsc : 0, &pb, &pc, &pfb);
          nfb += pfb;
          if (ipix) ipix[id] = (int)cg_ring2nest(nsb, pb);
          float r, cth, ph;
          cg_cart2sph(px, py, pz, &r, &cth, &ph);
          if (src9) {
            float *q = src9 + 9 * id;
            cg_radec(px, py, pz, ph, &q[0], &q[1]);
            q[2] = bg32(&s, s.zt, r);
            q[3] = cfg->need_beaming ? 0.0f : dz;
            q[4] = cfg->need_beaming ? 0.0f : -1.0f;
            q[5] = cfg->need_beaming ? 0.0f : -1.0f;
            q[6] = q[7] = q[8] = 0.0f;
          }
          if (cmap && nsc > 0) cmap[pc]++;
        }
      }
    }
  }
  *nsrc = id;
  if (fallbacks) *fallbacks = nfb;
  free(P.corner);
  s32_free(&s);
  return 0;
}

static void grad32(const float *phi, int ix, int iy, int iz, int N, float v[3])
{
  int xh = wrapi(ix + 1, N), xl = wrapi(ix - 1, N), yh = wrapi(iy + 1, N), yl = wrapi(iy - 1, N);
  int zh = wrapi(iz + 1, N), zl = wrapi(iz - 1, N);
  v[0] = CG_SUB(phi[pidx(xh, iy, iz, N)], phi[pidx(xl, iy, iz, N)]);
  v[1] = CG_SUB(phi[pidx(ix, yh, iz, N)], phi[pidx(ix, yl, iz, N)]);
  v[2] = CG_SUB(phi[pidx(ix, iy, zh, N)], phi[pidx(ix, iy, zl, N)]);
}

static float r_of_z32(const S32 *s, float z)
{
  float a = CG_DIV(1.0f, CG_ADD(1.0f, z));
  if (a >= 1.0f) return 0.0f;
  if (a <= 0.0f) return s->r_a2r[0];
  float nm1 = (float)(CG_NA - 1);
  int ia = (int)CG_MUL(a, nm1);
  return CG_FMA(CG_SUB(s->r_a2r[ia + 1], s->r_a2r[ia]), CG_MUL(CG_SUB(a, s->a_a2r[ia]), nm1), s->r_a2r[ia]);
}

int or_beam_rsd32(const cg_config *cfg, const float *npot, long long n, const float *pos4, float *src9)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N;
  const float fvel = (float)(-cfg->fgrowth_0 / (1.5 * cfg->hubble_0 * cfg->omega_m));
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    const float pos[3] = {pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]};
    float r = cg_norm3(pos[0], pos[1], pos[2]);
    float ir = CG_DIV(1.0f, r > 0.001f ? r : 0.001f);
    float u[3], h0[3], h1[3];
    int i0[3], i1[3];
    for (int a = 0; a < 3; a++) {
      float xn = CG_MUL(CG_ADD(pos[a], s.p[a]), s.idx);
      u[a] = CG_MUL(pos[a], ir);
      i0[a] = (int)xn;
      h0[a] = CG_SUB(xn, (float)i0[a]);
      h1[a] = CG_SUB(1.0f, h0[a]);
      i1[a] = wrapi(i0[a] + 1, N);
      i0[a] = wrapi(i0[a], N);
    }
    float v[3] = {0.0f, 0.0f, 0.0f};
    for (int hz = 0; hz < 2; hz++) {
      const int zc = hz ? i1[2] : i0[2];
      const float wz = hz ? h0[2] : h1[2];
      float acc[3] = {0.0f, 0.0f, 0.0f};
      for (int k = 0; k < 4; k++) {
        const int yc = (k & 2) ? i1[1] : i0[1], xc = (k & 1) ? i1[0] : i0[0];
        const float w = CG_MUL(CG_MUL(wz, (k & 2) ? h0[1] : h1[1]), (k & 1) ? h0[0] : h1[0]);
        float g[3];
        grad32(npot, xc, yc, zc, N, g);
        for (int a = 0; a < 3; a++) acc[a] = CG_FMA(g[a], w, acc[a]);
      }
      for (int a = 0; a < 3; a++) v[a] = CG_ADD(v[a], acc[a]);
    }
    float vr = CG_MUL(CG_MUL(0.5f, s.idx), CG_ADD(CG_ADD(CG_MUL(v[0], u[0]), CG_MUL(v[1], u[1])), CG_MUL(v[2], u[2])));
    float *q = src9 + 9 * i;
    float rz = r_of_z32(&s, q[2]);
    q[3] = CG_MUL(vr, CG_MUL(bg32(&s, s.v1, rz), fvel));
  }
  s32_free(&s);
  return 0;
}

static int cmp_float_idx(const void *a, const void *b)
{
  const float *x = a, *y = b;
  return (x[0] < y[0]) ? -1 : (x[0] > y[0] ? 1 : (x[1] < y[1] ? -1 : 1));
}

/* The arguments of the intensity-map decisions for species ipop, as the GPU
 * builds them (cg_imap_args); the buffers are owned by *B. */
typedef struct {
  cg_imap_args a;
  float *corner, *r0f, *rff, *b, *dxs, *dxsl;
  int *shell_of, *nsub;
  float att[2 * (CG_ATT_N + 1)];
} ImapArgs;

static void imap_args(ImapArgs *B, const cg_config *cfg, const S32 *s, int ipop, const float *norm32,
                      const double *norm64)
{
  cg_imap_args *a = &B->a;
  memset(a, 0, sizeof(*a));
  const int N = cfg->n_grid, nr = cfg->imap_nr[ipop], na = CG_NA;
  const double dx = cfg->l_box / N;
  B->corner = malloc(6 * (size_t)N * sizeof(float));
  for (int k = 0; k < 3; k++)
    for (int i = 0; i < N; i++) {
      const double c = cgx_coord(i, dx, cfg->pos_obs[k]);
      B->corner[k * N + i] = (float)c;
      B->corner[(3 + k) * N + i] = (float)(c - (double)(float)c);
    }
  a->xc = B->corner;
  a->yc = B->corner + N;
  a->zc = B->corner + 2 * N;
  a->xl = B->corner + 3 * N;
  a->yl = B->corner + 4 * N;
  a->zl = B->corner + 5 * N;
  B->r0f = malloc(nr * sizeof(float));
  B->rff = malloc(nr * sizeof(float));
  B->b = malloc(2 * nr * sizeof(float));
  B->shell_of = malloc((2 * nr + 1) * sizeof(int));
  B->nsub = malloc((nr + 2) * sizeof(int));
  B->dxs = malloc((nr + 2) * sizeof(float));
  const long long npix = 12LL * cfg->nside_imap[ipop] * cfg->nside_imap[ipop];
  const int nb = cg_imap_shells(cfg->imap_r0[ipop], cfg->imap_rf[ipop], nr, dx, npix, B->r0f, B->rff, B->b,
                                B->shell_of, B->nsub, B->dxs);
  a->sh.b = B->b;
  a->sh.shell_of = B->shell_of;
  a->sh.nb = nb;
  a->sh.nr = nr;
  a->sh.contig = cg_imap_contig(B->r0f, B->rff, nr, nb);
  a->nsub = B->nsub;
  a->dxs = B->dxs;
  B->dxsl = malloc((nr + 2) * sizeof(float));
  for (int i = 0; i < nr + 2; i++) B->dxsl[i] = (float)(dx / B->nsub[i] - (double)B->dxs[i]);
  a->dxsl = B->dxsl;
  cg_att_table(B->att);
  a->att = B->att;
  a->r = s->r;
  a->tz = s->tz[ipop].f;
  a->bz = s->bzi[ipop].f;
  a->norm = norm32;
  a->v1 = s->v1.f;
  a->ih = s->ih.f;
  a->idr = s->idr;
  a->r_last = s->r_last;
  a->na = na;
  a->bias_model = cfg->bias_model;
  a->nside = cfg->nside_imap[ipop];
  a->dx = (float)dx;
  const double fv = -cfg->fgrowth_0 / (1.5 * cfg->hubble_0 * cfg->omega_m);
  a->fvh = (float)(fv * (0.5 * (cfg->n_grid / cfg->l_box)));
  a->rmin64 = (double)B->r0f[0] - 20.;
  a->rmax64 = (double)B->rff[nr - 1] + 20.;
  a->rmin = (float)a->rmin64;
  a->rmax = (float)a->rmax64;
  a->r64 = cfg->r_arr_r2z;
  a->tz64 = cfg->imap_tz_arr[ipop];
  a->bz64 = cfg->imap_bz_arr[ipop];
  a->norm64 = norm64;
  a->v164 = cfg->growth_v_arr;
  a->ih64 = cfg->ihub_arr;
  a->idr64 = cfg->glob_idr;
  a->r_last64 = cfg->r_arr_r2z[na - 1];
  a->dx64 = dx;
  for (int k = 0; k < 3; k++) a->p64[k] = cfg->pos_obs[k];
  a->idx64 = cfg->n_grid / cfg->l_box;
  a->fv64 = fv;
}

static void imap_args_free(ImapArgs *B)
{
  free(B->corner);
  free(B->r0f);
  free(B->rff);
  free(B->b);
  free(B->shell_of);
  free(B->nsub);
  free(B->dxs);
  free(B->dxsl);
}

/* The intensity map of species ipop as the GPU paints it: cells and samples
 * decided in single precision where the margins hold, then in float-float,
 * and in double otherwise (cg_exact.h); brightness summed in cell order in
 * float.  stats:
 * [0] cells and [1] samples decided in double, [2] samples drawn (may be
 * NULL).  norm32 / norm64: the normalisation table with its two edges. */
int or_imap32(const cg_config *cfg, int ipop, const float *dens, const float *npot, const float *norm32,
              const double *norm64, float *data, int *nadd, long long *stats)
{
  S32 s;
  s32_init(&s, cfg);
  ImapArgs B;
  imap_args(&B, cfg, &s, ipop, norm32, norm64);
  const cg_imap_args *a = &B.a;
  const int N = s.N, nr = cfg->imap_nr[ipop];
  const long long npix = 12LL * cfg->nside_imap[ipop] * cfg->nside_imap[ipop];
  const float fvel = (float)(-cfg->fgrowth_0 / (1.5 * cfg->hubble_0 * cfg->omega_m));
  memset(data, 0, (size_t)nr * npix * sizeof(float));
  memset(nadd, 0, (size_t)nr * npix * sizeof(int));
  long long st[3] = {0, 0, 0};
  for (int iz = 0; iz < N; iz++)
    for (int iy = 0; iy < N; iy++)
      for (int ix = 0; ix < N; ix++) {
        float v[3];
        grad32(npot, ix, iy, iz, N, v);
        const float d = dens[pidx(ix, iy, iz, N)];
        cg_imap_cell c;
        int k = cg_imap_cell_checked(a, ix, iy, iz, d, v, &c);
        double drr64 = 0;
        int dbl = 0;
        if (k == 2) {
          st[0]++;
          int j;
          if (!cgx_imap_cell(a, ix, iy, iz, v, &j, &drr64)) continue;
          /* listed: the float fields, with the double shell of the corner */
          float x0 = cg_cell_coord(ix, s.dx, s.p[0]), y0 = cg_cell_coord(iy, s.dx, s.p[1]),
                z0 = cg_cell_coord(iz, s.dx, s.p[2]);
          float rc = cg_norm3(x0, y0, z0);
          c.j = j;
          c.mode = CG_SH_WALK;
          c.delta = 0;
          c.temp = cg_imap_temp(bg32(&s, s.tz[ipop], rc), d, bg32(&s, s.bzi[ipop], rc),
                                cg_bg_eval(norm32, s.r, norm32[CG_NA], norm32[CG_NA + 1], rc, s.r_last, s.idr),
                                cfg->bias_model);
          dbl = 1;
        } else if (k == 0) {
          continue;
        }
        (void)fvel;
        const int ns = a->nsub[c.j + 1];
        st[2] += (long long)ns * ns * ns;
        for (int sz = 0; sz < ns; sz++)
          for (int sy = 0; sy < ns; sy++)
            for (int sx = 0; sx < ns; sx++) {
              int sh = -1;
              long long pix = 0;
              if (dbl || (!cg_imap_sample_checked(a, ix, iy, iz, &c, ns, sx, sy, sz, &sh, &pix) &&
                          !cg_imap_decide_ff(a, &c, ix, iy, iz, sx, sy, sz, &sh, &pix))) {
                if (!dbl) {
                  int j2;
                  cgx_imap_cell(a, ix, iy, iz, v, &j2, &drr64);
                  dbl = 2;
                }
                cgx_imap_sample(a, ix, iy, iz, ns, drr64, sx, sy, sz, &sh, &pix);
                st[1]++;
                if (dbl == 2) dbl = 0; /* keep the float path for the cell's other samples */
              }
              if (sh >= 0 && sh < nr) {
                const long long q = (long long)sh * npix + pix;
                data[q] += c.temp;
                nadd[q]++;
              }
            }
      }
  if (stats) memcpy(stats, st, sizeof(st));
  imap_args_free(&B);
  s32_free(&s);
  return 0;
}

static int cmp_float(const void *a, const void *b)
{
  float x = *(const float *)a, y = *(const float *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

static double bg64(const cg_config *c, const double *f, double f0, double ff, double r)
{
  if (r <= 0) return f0;
  if (r >= c->r_arr_r2z[CG_NA - 1]) return ff;
  int ir = (int)(r * c->glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - c->r_arr_r2z[ir]) * c->glob_idr;
}

int or_kappa32(const cg_config *cfg, const float *npot, float *map)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N, np = cfg->n_kappa, nside = cfg->nside_kappa;
  const long long npix = 12LL * nside * nside;
  const int nr = N / 2;
  const double dr = cfg->r_max / nr, idr = 1. / dr;
  float *rp = malloc(np * sizeof(float));
  for (int i = 0; i < np; i++) rp[i] = (float)cfg->kappa_r[i];
  qsort(rp, np, sizeof(float), cmp_float);
  int *irmin = malloc(np * sizeof(int)), *irmax = malloc(np * sizeof(int));
  float *inv = malloc(np * sizeof(float)), *f1 = malloc(nr * sizeof(float)), *f2 = malloc(nr * sizeof(float));
  for (int i = 0; i < np; i++) {
    int irh = (int)((double)rp[i] * idr + 0.5);
    inv[i] = (float)(1. / (irh * dr));
    irmax[i] = irh < nr - 1 ? irh : nr - 1;
  }
  irmin[0] = 0;
  for (int i = 1; i < np; i++) irmin[i] = irmax[i - 1] + 1;
  for (int i = 0; i < nr; i++) {
    double rm = (i + 0.5) * dr;
    double pg = bg64(cfg, cfg->growth_d_arr, 1, cfg->growth_d_arr[CG_NA - 1], rm) *
                (1 + bg64(cfg, cfg->z_arr_r2z, 0, cfg->z_arr_r2z[CG_NA - 1], rm));
    f1[i] = (float)(rm * pg * dr);
    f2[i] = (float)(rm * rm * pg * dr);
  }
  const float drf = (float)dr;
#pragma omp parallel for schedule(static)
  for (long long ip = 0; ip < npix; ip++) {
    float u[3], rot[6];
    cg_pix2vec_nest(nside, ip, u);
    cg_kappa_rot(u, CG_MUL(s.idx, s.idx), rot);
    long long ring = cg_nest2ring(nside, ip);
    float k1 = 0, k1c = 0, k2 = 0, k2c = 0;
    for (int pl = 0; pl < np; pl++) {
      for (int irr = irmin[pl]; irr <= irmax[pl]; irr++) {
        float rm = CG_MUL(CG_ADD((float)irr, 0.5f), drf);
        int x0 = cg_ngp_cell(rm, u[0], s.p[0], s.idx, N), y0 = cg_ngp_cell(rm, u[1], s.p[1], s.idx, N),
            z0 = cg_ngp_cell(rm, u[2], s.p[2], s.idx, N);
        int xh = wrapi(x0 + 1, N), xl = wrapi(x0 - 1, N), yh = wrapi(y0 + 1, N), yl = wrapi(y0 - 1, N);
        int zh = wrapi(z0 + 1, N), zl = wrapi(z0 - 1, N);
#define PHI(X, Y, Z) npot[pidx((X), (Y), (Z), N)]
        const float f[19] = {PHI(x0, y0, z0), PHI(xh, y0, z0), PHI(xl, y0, z0), PHI(x0, yh, z0), PHI(x0, yl, z0),
                             PHI(x0, y0, zh), PHI(x0, y0, zl), PHI(xh, yh, z0), PHI(xl, yl, z0), PHI(xh, yl, z0),
                             PHI(xl, yh, z0), PHI(xh, y0, zh), PHI(xl, y0, zl), PHI(xh, y0, zl), PHI(xl, y0, zh),
                             PHI(x0, yh, zh), PHI(x0, yl, zl), PHI(x0, yh, zl), PHI(x0, yl, zh)};
#undef PHI
        float t[6];
        cg_tidal(f, t);
        float dot = cg_dot6(rot, t);
        cg_kahan_add(&k1, &k1c, CG_MUL(dot, f1[irr]));
        cg_kahan_add(&k2, &k2c, CG_MUL(dot, f2[irr]));
      }
      map[(long long)pl * npix + ring] = CG_SUB(k1, CG_MUL(inv[pl], k2));
    }
  }
  free(rp);
  free(irmin);
  free(irmax);
  free(inv);
  free(f1);
  free(f2);
  s32_free(&s);
  return 0;
}


/* isw_get_beam_properties (isw.c:78-147) in the GPU's FP32 arithmetic:
 * FP64-built weights 2 PD(r) dr rounded to float, the cell of cg_ngp_cell,
 * compensated sum. */
int or_isw32(const cg_config *cfg, const float *npot, float *map)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N, np = cfg->n_isw, nside = cfg->nside_isw;
  const long long npix = 12LL * nside * nside;
  const int nr = N / 2;
  const double dr = cfg->r_max / nr, idr = 1. / dr;
  float *rp = malloc(np * sizeof(float));
  for (int i = 0; i < np; i++) rp[i] = (float)cfg->isw_r[i];
  qsort(rp, np, sizeof(float), cmp_float);
  int *irmin = malloc(np * sizeof(int)), *irmax = malloc(np * sizeof(int));
  float *f1 = malloc(nr * sizeof(float));
  for (int i = 0; i < np; i++) {
    int irh = (int)((double)rp[i] * idr + 0.5);
    irmax[i] = irh < nr - 1 ? irh : nr - 1;
  }
  irmin[0] = 0;
  for (int i = 1; i < np; i++) irmin[i] = irmax[i - 1] + 1;
  const double *pd = cfg->growth_pd_arr;
  for (int i = 0; i < nr; i++) f1[i] = (float)(2 * bg64(cfg, pd, pd[0], pd[CG_NA - 1], (i + 0.5) * dr) * dr);
  const float drf = (float)dr;
#pragma omp parallel for schedule(static)
  for (long long ip = 0; ip < npix; ip++) {
    float u[3];
    cg_pix2vec_nest(nside, ip, u);
    long long ring = cg_nest2ring(nside, ip);
    float acc = 0, cmp = 0;
    for (int pl = 0; pl < np; pl++) {
      for (int irr = irmin[pl]; irr <= irmax[pl]; irr++) {
        float rm = CG_MUL(CG_ADD((float)irr, 0.5f), drf);
        int x0 = cg_ngp_cell(rm, u[0], s.p[0], s.idx, N), y0 = cg_ngp_cell(rm, u[1], s.p[1], s.idx, N),
            z0 = cg_ngp_cell(rm, u[2], s.p[2], s.idx, N);
        cg_kahan_add(&acc, &cmp, CG_MUL(npot[pidx(x0, y0, z0, N)], f1[irr]));
      }
      map[(long long)pl * npix + ring] = acc;
    }
  }
  free(rp);
  free(irmin);
  free(irmax);
  free(f1);
  s32_free(&s);
  return 0;
}

/* k_cstm: step tables kz, bz from the FP64 tables rounded to float, the
 * FP32 normalisation table evaluated at the float step centre, trilinear
 * density and Kahan sum along the ray; NEST order. */
int or_cstm32(const cg_config *cfg, int ipop, const float *dens, const float *normtab, float n0, float nf,
              float *map)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N, nr = N / 2, nside = cfg->nside_cstm[ipop];
  const long long npix = 12LL * nside * nside;
  double *kzd = malloc(2 * (size_t)nr * sizeof(double)), *bzd = kzd + nr;
  int lo, hi;
  if (or_cstm_steps(cfg, ipop, kzd, bzd, &lo, &hi)) {
    free(kzd);
    s32_free(&s);
    return -1;
  }
  const float drf = (float)(cfg->r_max / nr);
  float *kz = malloc(3 * (size_t)nr * sizeof(float)), *bz = kz + nr, *nm = bz + nr;
  const T32 nt = {normtab, n0, nf};
  for (int i = 0; i < nr; i++) {
    kz[i] = (float)kzd[i];
    bz[i] = (float)bzd[i];
    nm[i] = bg32(&s, nt, CG_MUL(CG_ADD((float)i, 0.5f), drf));
  }
#pragma omp parallel for schedule(static)
  for (long long ip = 0; ip < npix; ip++) {
    float u[3];
    cg_pix2vec_nest(nside, ip, u);
    float acc = 0, cmp = 0;
    for (int irr = lo; irr <= hi; irr++) {
      const float rm = CG_MUL(CG_ADD((float)irr, 0.5f), drf);
      int i0[3], i1[3];
      float h0[3], h1[3];
      for (int a = 0; a < 3; a++) cg_cic_axis(rm, u[a], s.p[a], s.idx, N, &i0[a], &i1[a], &h0[a], &h1[a]);
      const float d = cg_cic_value(dens, i0, i1, h0, h1, N);
      cg_kahan_add(&acc, &cmp, CG_MUL(kz[irr], CG_SUB(CG_MUL(cg_bias_model(d, bz[irr], cfg->bias_model), nm[irr]), 1.0f)));
    }
    map[ip] = CG_MUL(acc, drf);
  }
  free(kzd);
  free(kz);
  s32_free(&s);
  return 0;
}

/* direction and last step, as los_setup in srcs.cu */
static int los32_setup(const S32 *s, const float *pos, int nr, float idr, float *r, float u[3])
{
  *r = cg_norm3(pos[0], pos[1], pos[2]);
  const float ir = CG_DIV(1.0f, *r > 0.001f ? *r : 0.001f);
  for (int a = 0; a < 3; a++) u[a] = CG_MUL(pos[a], ir);
  const int k = (int)CG_ADD(CG_MUL(*r, idr), 0.5f);
  (void)s;
  return k < nr - 1 ? k : nr - 1;
}

/* k_src_lensing: writes e1 e2 kappa dra ddec (src9[4..8]) of each source */
int or_lens32(const cg_config *cfg, const float *npot, long long n, const float *pos4, float *src9)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N, nr = N / 2;
  const double dr = cfg->r_max / nr;
  float *f0 = malloc(2 * (size_t)nr * sizeof(float)), *f1 = f0 + nr;
  for (int i = 0; i < nr; i++) {
    const double rm = (i + 0.5) * dr;
    const double pg = bg64(cfg, cfg->growth_d_arr, 1, cfg->growth_d_arr[CG_NA - 1], rm) *
                      (1 + bg64(cfg, cfg->z_arr_r2z, 0, cfg->z_arr_r2z[CG_NA - 1], rm));
    f0[i] = (float)(2 * pg * dr);
    f1[i] = (float)(rm * pg * dr);
  }
  const float drf = (float)dr, idrf = (float)(nr / cfg->r_max);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    float r, u[3];
    const int kmax = los32_setup(&s, pos4 + 4 * i, nr, idrf, &r, u);
    const float ir = CG_DIV(1.0f, r > 0.001f ? r : 0.001f);
    float ux[3], uy[3], rk[6], re1[6], re2[6];
    cg_lens_rot(u, CG_MUL(CG_MUL(s.idx, s.idx), ir), CG_MUL(CG_MUL(0.5f, s.idx), ir), ux, uy, rk, re1, re2);
    float a[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k <= kmax; k++) {
      const float rm = CG_MUL(CG_ADD((float)k, 0.5f), drf);
      const int x0 = cg_ngp_cell(rm, u[0], s.p[0], s.idx, N), y0 = cg_ngp_cell(rm, u[1], s.p[1], s.idx, N),
                z0 = cg_ngp_cell(rm, u[2], s.p[2], s.idx, N);
      const int xh = wrapi(x0 + 1, N), xl = wrapi(x0 - 1, N), yh = wrapi(y0 + 1, N), yl = wrapi(y0 - 1, N);
      const int zh = wrapi(z0 + 1, N), zl = wrapi(z0 - 1, N);
#define PHI(X, Y, Z) npot[pidx((X), (Y), (Z), N)]
      const float f[19] = {PHI(x0, y0, z0), PHI(xh, y0, z0), PHI(xl, y0, z0), PHI(x0, yh, z0), PHI(x0, yl, z0),
                           PHI(x0, y0, zh), PHI(x0, y0, zl), PHI(xh, yh, z0), PHI(xl, yl, z0), PHI(xh, yl, z0),
                           PHI(xl, yh, z0), PHI(xh, y0, zh), PHI(xl, y0, zl), PHI(xh, y0, zl), PHI(xl, y0, zh),
                           PHI(x0, yh, zh), PHI(x0, yl, zl), PHI(x0, yh, zl), PHI(x0, yl, zh)};
#undef PHI
      float t[6];
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
    float *q = src9 + 9 * i;
    q[4] = a[0];
    q[5] = a[1];
    q[6] = a[2];
    q[7] = CG_MUL(a[4], 57.2957795f);
    q[8] = CG_MUL(a[3], 57.2957795f);
  }
  free(f0);
  s32_free(&s);
  return 0;
}

/* k_src_skewers: nr values per source of the density (or Gaussian field)
 * and the scaled radial velocity, 0 beyond the source's last step */
int or_skw32(const cg_config *cfg, const float *dens, const float *npot, int gauss, float sigma2f, long long n,
             const float *pos4, float *dout, float *vout)
{
  S32 s;
  s32_init(&s, cfg);
  const int N = s.N, nr = N / 2;
  const double dr = cfg->r_max / nr;
  const double fv = -cfg->fgrowth_0 / (1.5 * cfg->hubble_0 * cfg->omega_m);
  float *vf = malloc((size_t)nr * sizeof(float));
  for (int i = 0; i < nr; i++)
    vf[i] = (float)(bg64(cfg, cfg->growth_v_arr, cfg->growth_v_arr[0], cfg->growth_v_arr[CG_NA - 1], (i + 0.5) * dr) *
                    fv);
  const float drf = (float)dr, idrf = (float)(nr / cfg->r_max);
  const T32 d1 = s.d1;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    float r, u[3];
    const int kmax = los32_setup(&s, pos4 + 4 * i, nr, idrf, &r, u);
    float *od = dout + (size_t)i * nr, *ov = vout + (size_t)i * nr;
    for (int k = 0; k <= kmax; k++) {
      const float rm = CG_MUL(CG_ADD((float)k, 0.5f), drf);
      int i0[3], i1[3];
      float h0[3], h1[3];
      for (int a = 0; a < 3; a++) cg_cic_axis(rm, u[a], s.p[a], s.idx, N, &i0[a], &i1[a], &h0[a], &h1[a]);
      float d;
      if (gauss) {
        float gv[8];
        for (int b = 0; b < 8; b++) {
          const int ix = (b & 1) ? i1[0] : i0[0], iy = (b & 2) ? i1[1] : i0[1], iz = (b & 4) ? i1[2] : i0[2];
          const float rc = cg_norm3(cg_cell_coord(ix, s.dx, s.p[0]), cg_cell_coord(iy, s.dx, s.p[1]),
                                    cg_cell_coord(iz, s.dx, s.p[2]));
          gv[b] = cg_gauss_of_dens(dens[pidx(ix, iy, iz, N)], bg32(&s, d1, rc), sigma2f);
        }
        d = cg_cic_combine(gv, h0, h1);
      } else {
        d = cg_cic_value(dens, i0, i1, h0, h1, N);
      }
      float v[3] = {0.0f, 0.0f, 0.0f};
      for (int hz = 0; hz < 2; hz++) {
        const int zc = hz ? i1[2] : i0[2];
        const float wz = hz ? h0[2] : h1[2];
        float acc[3] = {0.0f, 0.0f, 0.0f};
        for (int k2 = 0; k2 < 4; k2++) {
          const int yc = (k2 & 2) ? i1[1] : i0[1], xc = (k2 & 1) ? i1[0] : i0[0];
          const float w = CG_MUL(CG_MUL(wz, (k2 & 2) ? h0[1] : h1[1]), (k2 & 1) ? h0[0] : h1[0]);
          float g[3];
          grad32(npot, xc, yc, zc, N, g);
          for (int a = 0; a < 3; a++) acc[a] = CG_FMA(g[a], w, acc[a]);
        }
        for (int a = 0; a < 3; a++) v[a] = CG_ADD(v[a], acc[a]);
      }
      const float vr =
          CG_MUL(CG_MUL(0.5f, s.idx), CG_ADD(CG_ADD(CG_MUL(v[0], u[0]), CG_MUL(v[1], u[1])), CG_MUL(v[2], u[2])));
      od[k] = d;
      ov[k] = CG_MUL(vr, vf[k]);
    }
    for (int k = kmax + 1; k < nr; k++) od[k] = ov[k] = 0.0f;
  }
  free(vf);
  s32_free(&s);
  return 0;
}
