/*
 * capi.cu -- the C ABI of libcolore_cuda.so (declared in colore_cuda.h):
 * context, device tables, stage orchestration and host mirrors.
 *
 * The host-side parts of the stages (bias-normalisation spline,
 * density.c:1272-1355; shell sub-sampling factors, imap.c:153-174; kappa
 * radial kernels, kappa.c:87-116) run here in FP64 on the small tables they
 * need, exactly as the reference computes them, and are uploaded in FP32.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/colore_cuda.h"
#include "cg_dev.cuh"
#include "dens_api.h"
#include "field_api.h"
#include "imap_api.h"
#include "kappa_api.h"
#include "srcs_api.h"

using namespace cg;

namespace {

struct HostTab { /* double copy of one background table */
  std::vector<double> v;
  double f0 = 0, ff = 0;
};

struct Cat {
  float4 *pos = nullptr;
  int *ipix = nullptr;
  float *src = nullptr;
  long long n = 0, cap = 0;
  int *cmap = nullptr;
  long long cmap_npix = 0;
  float *skw_d = nullptr, *skw_v = nullptr; /* skewers: n x nr each */
  long long skw_cap = 0;                   /* sources the skewer buffers hold */
  long long skw_n = -1;                    /* sources of the last skewer pass */
};

struct Imap {
  int nr = 0, nside = 0;
  long long npix = 0;
  /* shells (cg_imap_shells): edges, shell of each interval, nsub and
   * dx/nsub per bucket; bucket slots and counts */
  float *b = nullptr, *dxs = nullptr, *dxsl = nullptr;
  int *shell_of = nullptr, *nsub = nullptr;
  long long *base = nullptr, *cap = nullptr;
  unsigned long long *cnt = nullptr, *chunk_off = nullptr;
  float *data = nullptr;
  int *nadd = nullptr;
  unsigned long long *ctr = nullptr; /* the kernels' counters (5) */
  unsigned long long samples = 0;    /* sub-samples drawn by the last run */
  bool samples_stale = false;        /* a run since samples was read */
  /* the species' tables were built for table generation gen (0: never) */
  unsigned long long gen = 0;
  int nb = 0, contig = 0;
  double rmin = 0, rmax = 0;
};

} /* namespace */

struct cg_ctx {
  int device = 0, nsm = 0;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  cg_config cfg;
  int N = 0, NH = 0;
  size_t grid_floats = 0;
  /* host double tables */
  std::vector<double> h_r, h_z, h_d1, h_v1, h_ih, h_a, h_ra, h_pd;
  std::vector<unsigned char> cfg_sig; /* the last uploaded configuration and tables */
  /* device tables */
  float *d_tabs = nullptr;
  Grid1 g;
  Tab zt, d1, d2, v1, pd, ih;
  const float *a_a2r = nullptr, *r_a2r = nullptr;
  Tab nz[CG_NPOP_MAX], bz[CG_NPOP_MAX], norm[CG_NPOP_MAX];
  Tab tz[CG_NPOP_MAX], bzi[CG_NPOP_MAX], normi[CG_NPOP_MAX];
  Tab kzc[CG_NPOP_MAX], bzc[CG_NPOP_MAX], normc[CG_NPOP_MAX]; /* custom maps */
  float *d_norm = nullptr; /* (n_srcs + n_imap + n_cstm) tables of NA values and their 2 edge values */
  /* the same tables in double, for the decisions that the float margins
   * leave to the reference's double arithmetic (cg_exact.h): background r,
   * z, V1, 1/H, then n(r), b(r) per source population and T(r), b(r) per
   * intensity species; the normalisation tables with their edges; the cell
   * corners i*dx - p per axis rounded once to float; and the counts of
   * decisions taken in double (cg_exact_stats) */
  double *d_tabs64 = nullptr, *d_norm64 = nullptr;
  float *d_corner = nullptr;
  float *d_att = nullptr; /* cg_att_table, for the float-float decisions */
  unsigned long long *d_xstats = nullptr;
  int force_double = 0;
  /* normalisation bins (density.c:1233-1245): z(r_i) of the table radii,
   * z(L/2), the bin count and width; bin buffers keep their capacity */
  double *d_zr = nullptr;
  int *d_r2n = nullptr; /* RING -> NEST ids at nside_base (base pixels of the sources) */
  double norm_zlast = 0, norm_idz = 0;
  int norm_nz = 0;
  int bins_nz_cap = 0, bins_nt_cap = 0;
  float *d_pk = nullptr;
  float2 *d_twN = nullptr, *d_twH = nullptr;
  Box box;
  FillParams fill;
  /* grids */
  float *d_dens = nullptr, *d_npot = nullptr, *d_disp[3] = {nullptr, nullptr, nullptr};
  /* 2LPT work grids: the six second derivatives, then the source in [5]
   * and the second-order displacements in [0..2] */
  float *d_lpt2[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double2 *d_part = nullptr;
  size_t npart = 0;
  double *d_stats = nullptr;
  float *d_s2f = nullptr;
  unsigned int *d_err = nullptr;
  /* normalisation bins */
  unsigned long long *d_ncount = nullptr;
  double *d_zsum = nullptr, *d_bsum = nullptr;
  unsigned long long *d_bacc = nullptr; /* fixed-point accumulators of the bin sums */
  int pending_mode = CG_DMODE_NONE;
  /* sources */
  unsigned short *d_counts = nullptr;
  long long *d_bsums = nullptr, *d_total = nullptr, *d_ovf_cell = nullptr;
  int *d_ovf_cnt = nullptr, *d_ovf_n = nullptr;
  Cat cat[CG_NPOP_MAX];
  /* intensity maps */
  Imap im[CG_NPOP_MAX];
  float *d_tmpmap = nullptr;
  size_t tmpmap_n = 0;
  cg_imap_rec *d_recs = nullptr;         /* listed cells of one species */
  unsigned long long *d_imap_queue = nullptr; /* samples for the double pass */
  /* bumped by cg_upload_tables: stage tables built from the host tables
   * (convergence, ISW, custom-map, line-of-sight, intensity shells) are
   * rebuilt when their generation is older */
  unsigned long long tab_gen = 1, kgen = 0, igen = 0, cgen = 0, losgen = 0;
  int cir[2 * CG_NPOP_MAX] = {0}; /* custom maps' radial step ranges */
  long long list_cap = 0, queue_cap = 0;
  long long list_cap_max = 0; /* cg_set_imap_list_cap; 0: by free memory */
  /* kappa */
  float *d_kmap = nullptr, *d_kfac = nullptr, *d_kinv = nullptr;
  /* ISW */
  float *d_imap_isw = nullptr, *d_ifac = nullptr;
  /* custom maps: host copies of K(z) and b(z), device maps and step tables */
  std::vector<double> h_kzc[CG_NPOP_MAX], h_bzc[CG_NPOP_MAX];
  float *d_cmap[CG_NPOP_MAX] = {nullptr}, *d_cfac = nullptr;
  /* source lensing and skewer step tables (2 nr + nr floats) */
  float *d_losfac = nullptr;
  int losnr = 0;
  long long cnpix[CG_NPOP_MAX] = {0};
  int cnr = 0;
  int *d_iir = nullptr;
  int ipl = 0, inr = 0;
  long long inpix = 0;
  int *d_kir = nullptr;
  int knr = 0, kpl = 0;
  float kdr = 0;
  long long knpix = 0;
  /* optional per-kernel event log */
  int profiling = 0;
  int fforce[4] = {-1, -1, -1, -1}; /* forced tile variant per pass (CG_PASS_*), -1: the tuner's */
  struct Ev {
    const char *name;
    cudaEvent_t a, b;
    bool own_a; /* false when a is the previous entry's b */
  };
  std::vector<Ev> evlog;
  /* state */
  int have_fields = 0, have_density = 0, have_norm = 0, have_srcs = 0;
  long long launches = 0;
  /* graph of the whole sequence (cg_graph_capture) */
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t graph_done = nullptr;
  long long graph_launches = 0; /* kernels per replay */
  /* cg_set_host_*: page-locked host destinations that the stages fill as
   * each output becomes final, with copy-engine transfers on a copy stream
   * that overlap the stages still to run (no SM is taken from them); one
   * event per output kind orders the next writer of its source after the
   * copy (0 catalogues, 1 maps, 2 kappa) */
  float *h_src[CG_NPOP_MAX] = {};
  long long *h_n[CG_NPOP_MAX] = {};
  long long h_cap[CG_NPOP_MAX] = {};
  float *h_imap[CG_NPOP_MAX] = {};
  float *d_imap_out[CG_NPOP_MAX] = {}; /* data/nadd staged for the copy */
  long long imap_out_n[CG_NPOP_MAX] = {};
  float *h_kappa = nullptr;
  cudaStream_t ostream = nullptr;
  cudaEvent_t oev[4] = {};
  bool opend[3] = {false, false, false};
  char err[1024];
};

/* ------------------------------------------------------------------------ */
/* errors                                                                   */
/* ------------------------------------------------------------------------ */
static int fail(cg_ctx *c, int code, const char *fmt, ...)
{
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

#define CUDA_TRY(c, call)                                                                        \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail((c), CG_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                     \
  } while (0)

static void graph_free(cg_ctx *c);
static void out_wait_all(cg_ctx *c);

/* (Re)allocate a device buffer.  A captured graph holds the old addresses,
 * so any reallocation drops the graph: replaying it would touch freed
 * memory. */
template <class T>
static int dalloc(cg_ctx *c, T **p, size_t n)
{
  graph_free(c);
  out_wait_all(c); /* a host copy may still read the old buffer */
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (n == 0) return CG_OK;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(c, CG_ENOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
  }
  return CG_OK;
}

static int check_device_errors(cg_ctx *c)
{
  unsigned int h = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&h, c->d_err, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (h) {
    CUDA_TRY(c, cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), c->stream));
    return fail(c, CG_EDEVICE, "device error flags 0x%x (1: source count overflow, 2: catalog overflow, "
                               "4: shell search, 8: imap sub-sampling, 16: imap double-decision queue full, 32: bulk copy timeout, "
                               "64: particle deposit overflow)",
                h);
  }
  return CG_OK;
}

/* Event pair around a launch group when profiling is on. */
struct ProfScope {
  cg_ctx *c;
  size_t i;
  ProfScope(cg_ctx *c_, const char *name) : c(c_), i((size_t)-1)
  {
    if (!c->profiling) return;
    cg_ctx::Ev e;
    e.name = name;
    e.own_a = true;
    cudaEventCreate(&e.a);
    cudaEventCreate(&e.b);
    cudaEventRecord(e.a, c->stream);
    c->evlog.push_back(e);
    i = c->evlog.size() - 1;
  }
  ~ProfScope()
  {
    if (i != (size_t)-1) cudaEventRecord(c->evlog[i].b, c->stream);
  }
};

/* When profiling, events around the three passes of a 3-D transform: the
 * start, then one after each pass (recorded by the launcher), logged as
 * three entries <base>_fill, <base>_y, <base>_x that share their boundary
 * events.  base is one of a fixed set of names with static storage. */
struct PassEvents {
  cg_ctx *c;
  const char *names[3];
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  PassEvents(cg_ctx *c_, const char *n_fill, const char *n_y, const char *n_x) : c(c_), names{n_fill, n_y, n_x}
  {
    if (!c->profiling) return;
    for (cudaEvent_t &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], c->stream);
  }
  cudaEvent_t *after() { return c->profiling ? ev + 1 : nullptr; }
  ~PassEvents()
  {
    if (!c->profiling) return;
    for (int k = 0; k < 3; k++) c->evlog.push_back(cg_ctx::Ev{names[k], ev[k], ev[k + 1], k == 0});
  }
};

/* get_bg on the host double tables (cosmo.c:30-38) */
static double host_bg(const cg_ctx *c, const std::vector<double> &f, double f0, double ff, double r)
{
  const int na = CG_NA;
  if (r <= 0) return f0;
  if (r >= c->h_r[na - 1]) return ff;
  int ir = (int)(r * c->cfg.glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - c->h_r[ir]) * c->cfg.glob_idr;
}

static bool size_supported(int n)
{
  switch (n) {
#define X(k) case k:
    CG_FIELD_SIZES(X)
#undef X
    return true;
    default:
      return false;
  }
}

static cudaError_t run_gauss(int n, const cg_field_launch *L)
{
  switch (n) {
#define X(k) \
  case k:    \
    return cg_field_gauss_##k(L);
    CG_FIELD_SIZES(X)
#undef X
  }
  return cudaErrorInvalidValue;
}

static cudaError_t run_lpt(int n, const cg_field_launch *L)
{
  switch (n) {
#define X(k) \
  case k:    \
    return cg_field_lpt_##k(L);
    CG_FIELD_SIZES(X)
#undef X
  }
  return cudaErrorInvalidValue;
}

static cudaError_t run_lpt2(int n, const cg_field_launch *L)
{
  switch (n) {
#define X(k) \
  case k:    \
    return cg_field_lpt2_##k(L);
    CG_FIELD_SIZES(X)
#undef X
  }
  return cudaErrorInvalidValue;
}

static int field_tile(int n, int pass, int v)
{
  switch (n) {
#define X(k) \
  case k:    \
    return cg_field_tile_##k(pass, v);
    CG_FIELD_SIZES(X)
#undef X
  }
  return 0;
}

static cudaError_t field_pass(int n, const cg_field_launch *L, int pass, int v, int nf)
{
  switch (n) {
#define X(k) \
  case k:    \
    return cg_field_pass_##k(L, pass, v, nf);
    CG_FIELD_SIZES(X)
#undef X
  }
  return cudaErrorInvalidValue;
}

/* ---- tile autotuner of the transform passes ------------------------------
 * The first time a grid size runs on a device, each pass (the two fills,
 * the y and the x pass) is timed with every valid tile variant on the
 * context's own grids (before the real passes overwrite them): one launch to
 * warm up, then the mean of three with CUDA events.  The fastest variant is
 * kept for the life of the process, for every context of that size on that
 * device.  Variants differ only in block shape, so the choice never changes
 * a result.  COLORE_GB300_TUNE=0 keeps the plans' tiles. */
struct FieldTune {
  bool done[4] = {false, false, false, false};
  int var[4] = {0, 0, 0, 0};
  float ms[4][3] = {{-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}};
};
static std::mutex g_tune_mu;
static std::vector<std::pair<long long, FieldTune>> g_tune; /* key: device * 65536 + N */

static FieldTune *tune_entry(int device, int n)
{
  const long long key = (long long)device * 65536 + n;
  for (auto &e : g_tune)
    if (e.first == key) return &e.second;
  g_tune.emplace_back(key, FieldTune());
  return &g_tune.back().second;
}

static bool tuning_enabled()
{
  const char *e = getenv("COLORE_GB300_TUNE");
  return !(e && e[0] == '0');
}

/* Tune the passes listed (nf grids each) unless done; fills L->var. */
static int tune_field_passes(cg_ctx *c, cg_field_launch *L, const int *passes, const int *nfs, int np)
{
  std::lock_guard<std::mutex> lock(g_tune_mu);
  FieldTune *t = tune_entry(c->device, c->N);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CUDA_TRY(c, cudaStreamIsCapturing(c->stream, &cs));
  const bool can = tuning_enabled() && cs == cudaStreamCaptureStatusNone;
  for (int i = 0; i < np && can; i++) {
    const int pass = passes[i];
    if (t->done[pass]) continue;
    cudaEvent_t e0, e1;
    CUDA_TRY(c, cudaEventCreate(&e0));
    CUDA_TRY(c, cudaEventCreate(&e1));
    float best = 3.0e38f;
    int bv = 0;
    for (int v = 0; v < 3; v++) {
      t->ms[pass][v] = -1.0f;
      if (!field_tile(c->N, pass, v)) continue;
      cudaError_t e = field_pass(c->N, L, pass, v, nfs[i]);
      if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
      for (int r = 0; r < 3 && e == cudaSuccess; r++) e = field_pass(c->N, L, pass, v, nfs[i]);
      if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) { /* a variant the device refuses (resources) is skipped */
        cudaGetLastError();
        continue;
      }
      t->ms[pass][v] = ms / 3.0f;
      if (t->ms[pass][v] < best) {
        best = t->ms[pass][v];
        bv = v;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    t->var[pass] = bv;
    t->done[pass] = true;
  }
  for (int p = 0; p < 4; p++) L->var[p] = c->fforce[p] >= 0 ? c->fforce[p] : t->var[p];
  return CG_OK;
}

extern "C" int cg_set_field_variant(cg_ctx *c, int pass, int v)
{
  if (!c) return CG_EINVAL;
  if (pass < 0 || pass > 3 || v < -1 || v > 2) return fail(c, CG_EINVAL, "pass %d, variant %d out of range", pass, v);
  if (v >= 0 && !field_tile(c->N, pass, v))
    return fail(c, CG_EINVAL, "variant %d of pass %d is not valid at %d^3", v, pass, c->N);
  c->fforce[pass] = v;
  return CG_OK;
}

extern "C" int cg_field_plan(cg_ctx *c, char *buf, size_t len)
{
  if (!c || !buf || !len) return CG_EINVAL;
  static const char *names[4] = {"fill2", "fill3", "y", "x"};
  static const char *tiles[4] = {"TX", "TX", "TXY", "RB"};
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const FieldTune *t = tune_entry(c->device, c->N);
  size_t o = (size_t)snprintf(buf, len, "{\"n_grid\": %d, \"tuned\": %s", c->N, tuning_enabled() ? "true" : "false");
  for (int p = 0; p < 4 && o < len; p++) {
    const int v = c->fforce[p] >= 0 ? c->fforce[p] : t->var[p];
    o += (size_t)snprintf(buf + o, len - o, ", \"%s\": {\"%s\": %d, \"timed\": %s, \"ms\": {", names[p], tiles[p],
                          field_tile(c->N, p, v), t->done[p] ? "true" : "false");
    bool first = true;
    for (int w = 0; w < 3 && o < len; w++) {
      const int tw = field_tile(c->N, p, w);
      if (!tw || t->ms[p][w] < 0) continue;
      o += (size_t)snprintf(buf + o, len - o, "%s\"%d\": %.4f", first ? "" : ", ", tw, t->ms[p][w]);
      first = false;
    }
    if (o < len) o += (size_t)snprintf(buf + o, len - o, "}}");
  }
  if (o < len) snprintf(buf + o, len - o, "}");
  return o < len ? CG_OK : fail(c, CG_EINVAL, "buffer of %zu bytes too short", len);
}

static size_t npartials(int n)
{
  switch (n) {
#define X(k) \
  case k:    \
    return cg_field_npartials_##k();
    CG_FIELD_SIZES(X)
#undef X
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* tables                                                                   */
/* ------------------------------------------------------------------------ */
static int validate(const cg_config *cfg, char *msg, size_t len)
{
  if (!cfg) return snprintf(msg, len, "NULL config"), CG_EINVAL;
  if (cfg->precision != CG_PREC_F32)
    return snprintf(msg, len, "precision %d: this library builds the FP32 path only", cfg->precision), CG_EINVAL;
  if (!size_supported(cfg->n_grid))
    return snprintf(msg, len, "n_grid=%d unsupported (2^a 3^b sizes 64..2048 in field_api.h)", cfg->n_grid),
           CG_EINVAL;
  if (!(cfg->l_box > 0)) return snprintf(msg, len, "l_box must be > 0"), CG_EINVAL;
  if (cfg->numk < 2 || !cfg->pkarr) return snprintf(msg, len, "P(k) table missing"), CG_EINVAL;
  if (cfg->n_srcs < 0 || cfg->n_srcs > CG_NPOP_MAX || cfg->n_imap < 0 || cfg->n_imap > CG_NPOP_MAX)
    return snprintf(msg, len, "population count out of range"), CG_EINVAL;
  if (cfg->do_kappa && (cfg->n_kappa < 1 || cfg->n_kappa > CG_NPLANES_MAX || cfg->nside_kappa < 1))
    return snprintf(msg, len, "kappa planes or nside out of range"), CG_EINVAL;
  if (cfg->do_isw && (cfg->n_isw < 1 || cfg->n_isw > CG_NPLANES_MAX || cfg->nside_isw < 1))
    return snprintf(msg, len, "ISW planes or nside out of range"), CG_EINVAL;
  if (cfg->n_cstm < 0 || cfg->n_cstm > CG_NPOP_MAX)
    return snprintf(msg, len, "custom-map count out of range"), CG_EINVAL;
  for (int i = 0; i < cfg->n_cstm; i++)
    if (!cfg->cstm_kz_arr[i] || !cfg->cstm_bz_arr[i] || cfg->nside_cstm[i] < 1)
      return snprintf(msg, len, "custom-map table missing or nside < 1"), CG_EINVAL;
  if ((cfg->dens_type == CG_DENS_1LPT || cfg->dens_type == CG_DENS_2LPT) &&
      (cfg->lpt_interp_type < 0 || cfg->lpt_interp_type > 2))
    return snprintf(msg, len, "lpt_interp_type %d: 0 (NGP), 1 (CIC) or 2 (TSC)", cfg->lpt_interp_type), CG_EINVAL;
  if (cfg->dens_type != CG_DENS_LGNR && cfg->dens_type != CG_DENS_1LPT && cfg->dens_type != CG_DENS_2LPT &&
      cfg->dens_type != CG_DENS_CLIP)
    return snprintf(msg, len, "dens_type %d not supported", cfg->dens_type), CG_EINVAL;
  const double *req[] = {cfg->r_arr_r2z, cfg->z_arr_r2z, cfg->growth_d_arr, cfg->growth_d2_arr, cfg->growth_v_arr,
                         cfg->growth_pd_arr, cfg->ihub_arr, cfg->a_arr_a2r, cfg->r_arr_a2r};
  for (const double *p : req)
    if (!p) return snprintf(msg, len, "background table missing"), CG_EINVAL;
  for (int i = 0; i < cfg->n_srcs; i++)
    if (!cfg->srcs_nz_arr[i] || !cfg->srcs_bz_arr[i]) return snprintf(msg, len, "source table missing"), CG_EINVAL;
  for (int i = 0; i < cfg->n_imap; i++) {
    if (!cfg->imap_tz_arr[i] || !cfg->imap_bz_arr[i] || !cfg->imap_r0[i] || !cfg->imap_rf[i] ||
        cfg->imap_nr[i] < 1 || cfg->nside_imap[i] < 1)
      return snprintf(msg, len, "intensity-map table missing"), CG_EINVAL;
  }
  if (cfg->n_srcs > 0 && cfg->nside_base < 1) return snprintf(msg, len, "nside_base must be >= 1"), CG_EINVAL;
  for (int i = 0; i < cfg->n_srcs; i++) /* get_element, beaming.c:56-57 */
    if (cfg->skw_srcs[i] && cfg->skw_gauss[i] && cfg->dens_type != CG_DENS_LGNR)
      return snprintf(msg, len, "Cannot write Gaussian skewers with density type %d", cfg->dens_type), CG_EINVAL;
  return CG_OK;
}

/* The configuration's bytes and the contents of every table it points to. */
static std::vector<unsigned char> config_signature(const cg_config *cfg)
{
  std::vector<unsigned char> v;
  auto put = [&](const void *p, size_t n) {
    if (!p || !n) return;
    const unsigned char *b = static_cast<const unsigned char *>(p);
    v.insert(v.end(), b, b + n);
  };
  put(cfg, sizeof(*cfg));
  const size_t na = CG_NA * sizeof(double);
  const double *tabs[] = {cfg->r_arr_r2z, cfg->z_arr_r2z, cfg->growth_d_arr, cfg->growth_d2_arr, cfg->growth_v_arr,
                          cfg->growth_pd_arr, cfg->ihub_arr, cfg->a_arr_a2r, cfg->r_arr_a2r};
  for (const double *t : tabs) put(t, na);
  put(cfg->pkarr, (size_t)(cfg->numk > 0 ? cfg->numk : 0) * sizeof(double));
  for (int i = 0; i < cfg->n_srcs && i < CG_NPOP_MAX; i++) {
    put(cfg->srcs_nz_arr[i], na);
    put(cfg->srcs_bz_arr[i], na);
  }
  for (int i = 0; i < cfg->n_imap && i < CG_NPOP_MAX; i++) {
    put(cfg->imap_tz_arr[i], na);
    put(cfg->imap_bz_arr[i], na);
    put(cfg->imap_r0[i], (size_t)(cfg->imap_nr[i] > 0 ? cfg->imap_nr[i] : 0) * sizeof(double));
    put(cfg->imap_rf[i], (size_t)(cfg->imap_nr[i] > 0 ? cfg->imap_nr[i] : 0) * sizeof(double));
  }
  for (int i = 0; i < cfg->n_cstm && i < CG_NPOP_MAX; i++) {
    put(cfg->cstm_kz_arr[i], na);
    put(cfg->cstm_bz_arr[i], na);
  }
  return v;
}

extern "C" int cg_upload_tables(cg_ctx *c, const cg_config *cfg)
{
  if (!c) return CG_EINVAL;
  if (int rc = validate(cfg, c->err, sizeof(c->err))) return rc;
  if (cfg->n_grid != c->N) return fail(c, CG_EINVAL, "n_grid differs from the context's");
  c->cfg = *cfg;
  {
    /* the stage tables derived from these are rebuilt only when something changed */
    std::vector<unsigned char> sig = config_signature(cfg);
    if (sig != c->cfg_sig) {
      c->cfg_sig.swap(sig);
      c->tab_gen++;
    }
  }
  const int na = CG_NA;
  auto cp = [&](std::vector<double> &v, const double *src) { v.assign(src, src + na); };
  cp(c->h_r, cfg->r_arr_r2z);
  cp(c->h_z, cfg->z_arr_r2z);
  cp(c->h_d1, cfg->growth_d_arr);
  cp(c->h_v1, cfg->growth_v_arr);
  cp(c->h_ih, cfg->ihub_arr);
  cp(c->h_pd, cfg->growth_pd_arr);
  cp(c->h_a, cfg->a_arr_a2r);
  cp(c->h_ra, cfg->r_arr_a2r);
  for (int p = 0; p < cfg->n_cstm; p++) {
    cp(c->h_kzc[p], cfg->cstm_kz_arr[p]);
    cp(c->h_bzc[p], cfg->cstm_bz_arr[p]);
  }
  /* packed float tables: 9 background + 2 per population, species and custom map */
  const int ntab = 9 + 2 * cfg->n_srcs + 2 * cfg->n_imap + 2 * cfg->n_cstm;
  std::vector<float> h((size_t)ntab * na);
  const double *srcs[9] = {cfg->r_arr_r2z, cfg->z_arr_r2z, cfg->growth_d_arr, cfg->growth_d2_arr, cfg->growth_v_arr,
                           cfg->growth_pd_arr, cfg->ihub_arr, cfg->a_arr_a2r, cfg->r_arr_a2r};
  int k = 0;
  for (int t = 0; t < 9; t++, k++)
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)srcs[t][i];
  for (int p = 0; p < cfg->n_srcs; p++) {
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)cfg->srcs_nz_arr[p][i];
    k++;
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)cfg->srcs_bz_arr[p][i];
    k++;
  }
  for (int p = 0; p < cfg->n_imap; p++) {
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)cfg->imap_tz_arr[p][i];
    k++;
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)cfg->imap_bz_arr[p][i];
    k++;
  }
  for (int p = 0; p < cfg->n_cstm; p++) {
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)cfg->cstm_kz_arr[p][i];
    k++;
    for (int i = 0; i < na; i++) h[(size_t)k * na + i] = (float)cfg->cstm_bz_arr[p][i];
    k++;
  }
  if (int rc = dalloc(c, &c->d_tabs, h.size())) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(c->d_tabs, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  const float *T = c->d_tabs;
  auto tab = [&](int i) { return T + (size_t)i * na; };
  auto last = [&](const double *a) { return (float)a[na - 1]; };
  c->g.r = tab(0);
  c->g.r_last = (float)cfg->r_arr_r2z[na - 1];
  c->g.idr = (float)cfg->glob_idr;
  /* edge values of get_bg, cosmo.c:42-57 */
  c->zt = Tab{tab(1), 0.0f, last(cfg->z_arr_r2z)};
  c->d1 = Tab{tab(2), 1.0f, last(cfg->growth_d_arr)};
  c->d2 = Tab{tab(3), (float)cfg->growth_d2_arr[0], last(cfg->growth_d2_arr)};
  c->v1 = Tab{tab(4), (float)cfg->growth_v_arr[0], last(cfg->growth_v_arr)};
  c->pd = Tab{tab(5), (float)cfg->growth_pd_arr[0], last(cfg->growth_pd_arr)};
  c->ih = Tab{tab(6), (float)cfg->ihub_arr[0], last(cfg->ihub_arr)};
  c->a_a2r = tab(7);
  c->r_a2r = tab(8);
  k = 9;
  for (int p = 0; p < cfg->n_srcs; p++) {
    c->nz[p] = Tab{tab(k), 0.0f, 0.0f};                                  /* cosmo.c:58-59 */
    c->bz[p] = Tab{tab(k + 1), (float)cfg->srcs_bz_arr[p][0], 1.0f};     /* cosmo.c:60-61 */
    k += 2;
  }
  for (int p = 0; p < cfg->n_imap; p++) {
    c->tz[p] = Tab{tab(k), 0.0f, 0.0f};                                  /* cosmo.c:66-67 */
    c->bzi[p] = Tab{tab(k + 1), (float)cfg->imap_bz_arr[p][0], 1.0f};    /* cosmo.c:68-69 */
    k += 2;
  }
  for (int p = 0; p < cfg->n_cstm; p++) {
    c->kzc[p] = Tab{tab(k), 0.0f, 0.0f};                                 /* cosmo.c:74-75 */
    c->bzc[p] = Tab{tab(k + 1), (float)cfg->cstm_bz_arr[p][0], 1.0f};    /* cosmo.c:76-77 */
    k += 2;
  }
  /* normalisation tables (NA values, then the two edges) start at 1 until
   * compute_density_normalization */
  const int nnorm = cfg->n_srcs + cfg->n_imap + cfg->n_cstm, nas = na + 2;
  if (nnorm > 0) {
    std::vector<float> ones((size_t)nnorm * nas, 1.0f);
    if (int rc = dalloc(c, &c->d_norm, ones.size())) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_norm, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice,
                                c->stream));
    for (int p = 0; p < cfg->n_srcs; p++) c->norm[p] = Tab{c->d_norm + (size_t)p * nas, 1.0f, 1.0f};
    for (int p = 0; p < cfg->n_imap; p++) c->normi[p] = Tab{c->d_norm + (size_t)(cfg->n_srcs + p) * nas, 1.0f, 1.0f};
    for (int p = 0; p < cfg->n_cstm; p++)
      c->normc[p] = Tab{c->d_norm + (size_t)(cfg->n_srcs + cfg->n_imap + p) * nas, 1.0f, 1.0f};
  }
  /* double tables and float corners for the exact decisions */
  {
    const int nd = 4 + 2 * cfg->n_srcs + 2 * cfg->n_imap;
    std::vector<double> hd((size_t)nd * na);
    const double *bgd[4] = {cfg->r_arr_r2z, cfg->z_arr_r2z, cfg->growth_v_arr, cfg->ihub_arr};
    for (int t = 0; t < 4; t++) memcpy(hd.data() + (size_t)t * na, bgd[t], na * sizeof(double));
    for (int p = 0; p < cfg->n_srcs; p++) {
      memcpy(hd.data() + (size_t)(4 + 2 * p) * na, cfg->srcs_nz_arr[p], na * sizeof(double));
      memcpy(hd.data() + (size_t)(5 + 2 * p) * na, cfg->srcs_bz_arr[p], na * sizeof(double));
    }
    for (int p = 0; p < cfg->n_imap; p++) {
      memcpy(hd.data() + (size_t)(4 + 2 * cfg->n_srcs + 2 * p) * na, cfg->imap_tz_arr[p], na * sizeof(double));
      memcpy(hd.data() + (size_t)(5 + 2 * cfg->n_srcs + 2 * p) * na, cfg->imap_bz_arr[p], na * sizeof(double));
    }
    if (int rc = dalloc(c, &c->d_tabs64, hd.size())) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_tabs64, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice,
                                c->stream));
    const int N = cfg->n_grid;
    const double dx = cfg->l_box / N;
    /* per axis the corner rounded to float, then (three more rows) the rest
     * corner - rounded corner, a double-float pair */
    std::vector<float> cr((size_t)6 * N);
    for (int k3 = 0; k3 < 3; k3++)
      for (int i = 0; i < N; i++) {
        const double cd = cgx_coord(i, dx, cfg->pos_obs[k3]);
        cr[(size_t)k3 * N + i] = (float)cd;
        cr[(size_t)(3 + k3) * N + i] = (float)(cd - (double)(float)cd);
      }
    if (int rc = dalloc(c, &c->d_corner, cr.size())) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_corner, cr.data(), cr.size() * sizeof(float), cudaMemcpyHostToDevice,
                                c->stream));
    std::vector<float> att(2 * (CG_ATT_N + 1));
    cg_att_table(att.data());
    if (!c->d_att)
      if (int rc = dalloc(c, &c->d_att, att.size())) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_att, att.data(), att.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    if (nnorm > 0) {
      std::vector<double> ones((size_t)nnorm * nas, 1.0);
      if (int rc = dalloc(c, &c->d_norm64, ones.size())) return rc;
      CUDA_TRY(c, cudaMemcpyAsync(c->d_norm64, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  c->stream));
    }
    if (!c->d_xstats) {
      if (int rc = dalloc(c, &c->d_xstats, (size_t)4)) return rc;
      CUDA_TRY(c, cudaMemsetAsync(c->d_xstats, 0, 4 * sizeof(unsigned long long), c->stream));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vectors */
  }
  /* RING -> NEST table of the base pixels (srcs.c:268-270) */
  if (cfg->n_srcs > 0 && cfg->nside_base <= 1024) {
    const long long nb = 12LL * cfg->nside_base * cfg->nside_base;
    std::vector<int> t((size_t)nb);
    for (long long i = 0; i < nb; i++) t[(size_t)i] = (int)cg_ring2nest(cfg->nside_base, i);
    if (int rc = dalloc(c, &c->d_r2n, (size_t)nb)) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_r2n, t.data(), nb * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vector */
  }
  /* redshift bins of compute_density_normalization (density.c:1233-1245) and
   * z at the table radii, for the device-side tables */
  {
    c->norm_zlast = host_bg(c, c->h_z, 0, c->h_z[na - 1], 0.5 * cfg->l_box);
    c->norm_nz = (int)(c->norm_zlast / 0.05) + 2;
    c->norm_idz = (c->norm_nz - 2) / c->norm_zlast;
    std::vector<double> zr(na);
    for (int i = 0; i < na; i++) zr[i] = host_bg(c, c->h_z, 0, c->h_z[na - 1], c->h_r[i]);
    if (int rc = dalloc(c, &c->d_zr, (size_t)na)) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_zr, zr.data(), na * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vectors */
  }
  /* P(k) */
  std::vector<float> pk(cfg->numk);
  for (int i = 0; i < cfg->numk; i++) pk[i] = (float)cfg->pkarr[i];
  if (int rc = dalloc(c, &c->d_pk, pk.size())) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(c->d_pk, pk.data(), pk.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  /* box and fill parameters */
  const double L = cfg->l_box;
  const int N = c->N;
  c->box.N = N;
  c->box.mN = ~0ull / (unsigned long long)N + 1ull;
  c->box.dx = (float)(L / N);
  c->box.idx = (float)(N / L);
  c->box.L = (float)L;
  c->box.hL = (float)(0.5 * L);
  c->box.p0 = (float)cfg->pos_obs[0];
  c->box.p1 = (float)cfg->pos_obs[1];
  c->box.p2 = (float)cfg->pos_obs[2];
  const double dk = 2 * M_PI / L;
  FillParams &f = c->fill;
  f.N = N;
  f.NH = N / 2 + 1;
  f.dk = (float)dk;
  f.idk3 = (float)(1.0 / (dk * dk * dk));
  f.prefac = (float)cfg->prefac_lensing;
  f.r2s = (float)cfg->r2_smooth;
  f.do_smooth = cfg->do_smoothing;
  f.smooth_pot = cfg->smooth_potential;
  f.pk = c->d_pk;
  f.numk = cfg->numk;
  f.logkmin = (float)cfg->logkmin;
  f.logkmax = (float)cfg->logkmax;
  f.idlogk = (float)cfg->idlogk;
  f.n_scal = (float)cfg->n_scal;
  f.key0 = (uint32_t)cfg->seed;
  f.key1 = (uint32_t)(cfg->seed >> 32) ^ CG_STREAM_FIELD;
  f.lpt_norm = (float)std::pow(std::sqrt(2 * M_PI) / L, 3);
  c->have_fields = c->have_density = c->have_norm = c->have_srcs = 0;
  return CG_OK;
}

/* ------------------------------------------------------------------------ */
/* lifetime                                                                 */
/* ------------------------------------------------------------------------ */
extern "C" const char *cg_last_error(const cg_ctx *c) { return c ? c->err : "NULL context"; }

extern "C" int cg_memory_estimate(const cg_config *cfg, unsigned long long *bytes)
{
  char msg[256];
  if (!bytes) return CG_EINVAL;
  if (int rc = validate(cfg, msg, sizeof(msg))) return rc;
  const unsigned long long N = cfg->n_grid, NH = N / 2 + 1;
  unsigned long long grid = N * N * NH * 8ull;
  unsigned long long b = 2 * grid;
  if (cfg->dens_type == CG_DENS_1LPT) b += 3 * grid;
  if (cfg->dens_type == CG_DENS_2LPT) b += 9 * grid;
  if (cfg->n_srcs > 0) b += N * N * N * 2ull;
  for (int i = 0; i < cfg->n_imap; i++)
    b += (unsigned long long)cfg->imap_nr[i] * 12ull * cfg->nside_imap[i] * cfg->nside_imap[i] * 8ull;
  if (cfg->do_kappa) b += (unsigned long long)cfg->n_kappa * 12ull * cfg->nside_kappa * cfg->nside_kappa * 4ull;
  if (cfg->do_isw) b += (unsigned long long)cfg->n_isw * 12ull * cfg->nside_isw * cfg->nside_isw * 4ull;
  for (int i = 0; i < cfg->n_cstm; i++) b += 12ull * cfg->nside_cstm[i] * cfg->nside_cstm[i] * 4ull;
  *bytes = b;
  return CG_OK;
}

/* write_imap's normalisation (io.c:738-741): data/nadd where nadd > 0. */
__device__ __forceinline__ float div_nadd(float d, int k) { return k > 0 ? d / (float)k : d; }

/* data/nadd of m pixels (16-byte vectors; the buffers are cudaMalloc'd). */
__global__ void k_div_nadd(const float *__restrict__ d, const int *__restrict__ n, float *out, long long m)
{
  const long long m4 = m >> 2, stride = (long long)gridDim.x * blockDim.x;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long i = t; i < m4; i += stride) {
    const float4 a = reinterpret_cast<const float4 *>(d)[i];
    const int4 k = reinterpret_cast<const int4 *>(n)[i];
    reinterpret_cast<float4 *>(out)[i] = make_float4(div_nadd(a.x, k.x), div_nadd(a.y, k.y), div_nadd(a.z, k.z),
                                                     div_nadd(a.w, k.w));
  }
  for (long long i = 4 * m4 + t; i < m; i += stride) out[i] = div_nadd(d[i], n[i]);
}

/* ---- host outputs (cg_set_host_*) ---- */
static void out_wait_all(cg_ctx *c)
{
  if (c->ostream && (c->opend[0] || c->opend[1] || c->opend[2])) cudaStreamSynchronize(c->ostream);
  c->opend[0] = c->opend[1] = c->opend[2] = false;
}

/* The next writer of output kind k waits (on the device) for its copy. */
static void out_join(cg_ctx *c, int k)
{
  if (c->opend[k]) {
    cudaStreamWaitEvent(c->stream, c->oev[k], 0);
    c->opend[k] = false;
  }
}

/* Start copies of output kind k: the copy stream waits for the work queued
 * so far on the context's stream. */
static int out_begin(cg_ctx *c)
{
  if (!c->ostream) {
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c->ostream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : c->oev) CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  CUDA_TRY(c, cudaEventRecord(c->oev[3], c->stream));
  CUDA_TRY(c, cudaStreamWaitEvent(c->ostream, c->oev[3], 0));
  return CG_OK;
}

static int out_end(cg_ctx *c, int k)
{
  CUDA_TRY(c, cudaEventRecord(c->oev[k], c->ostream));
  c->opend[k] = true;
  return CG_OK;
}

/* Device view of page-locked host memory, or an error. */
static int host_view(cg_ctx *c, const void *p, void **dv)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer) {
    cudaGetLastError();
    return fail(c, CG_EINVAL, "host output buffers must be page-locked (cudaHostAlloc)");
  }
  *dv = a.devicePointer;
  return CG_OK;
}

static void graph_free(cg_ctx *c)
{
  if (!c->gexec && !c->graph) return;
  if (c->graph_done) cudaEventSynchronize(c->graph_done);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
}

extern "C" void cg_destroy(cg_ctx *c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ostream) {
    cudaStreamSynchronize(c->ostream);
    cudaStreamDestroy(c->ostream);
    c->ostream = nullptr;
    for (cudaEvent_t &e : c->oev)
      if (e) cudaEventDestroy(e);
  }
  c->opend[0] = c->opend[1] = c->opend[2] = false;
  graph_free(c); /* waits for a replay still running */
  if (c->graph_done) {
    cudaEventDestroy(c->graph_done);
    c->graph_done = nullptr;
  }
  for (float *q : c->d_lpt2)
    if (q) cudaFree(q);
  for (float *q : c->d_imap_out)
    if (q) cudaFree(q);
  void *ptrs[] = {c->d_tabs, c->d_norm, c->d_tabs64, c->d_norm64, c->d_corner, c->d_att, c->d_xstats, c->d_zr, c->d_r2n, c->d_pk, c->d_twN, c->d_twH, c->d_dens, c->d_npot, c->d_disp[0],
                  c->d_disp[1], c->d_disp[2], c->d_part, c->d_stats, c->d_s2f, c->d_err, c->d_ncount,
                  c->d_zsum, c->d_bsum, c->d_bacc, c->d_counts, c->d_bsums, c->d_total, c->d_tmpmap, c->d_kmap,
                  c->d_kfac, c->d_kinv, c->d_kir, c->d_ovf_cell, c->d_ovf_cnt, c->d_ovf_n,
                  c->d_recs, c->d_imap_queue,
                  c->d_imap_isw, c->d_ifac, c->d_iir, c->d_cfac, c->d_losfac};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int i = 0; i < CG_NPOP_MAX; i++) {
    void *q[] = {c->cat[i].pos, c->cat[i].ipix, c->cat[i].src, c->cat[i].cmap, c->im[i].b, c->im[i].dxs,
                 c->im[i].dxsl, c->im[i].shell_of, c->im[i].nsub, c->im[i].base, c->im[i].cap, c->im[i].cnt, c->im[i].chunk_off,
                 c->im[i].data, c->im[i].nadd, c->im[i].ctr, c->d_cmap[i], c->cat[i].skw_d, c->cat[i].skw_v};
    for (void *p : q)
      if (p) cudaFree(p);
  }
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

extern "C" int cg_create(cg_ctx **out, const cg_config *cfg, int device)
{
  if (!out) return CG_EINVAL;
  *out = nullptr;
  cg_ctx *c = new (std::nothrow) cg_ctx();
  if (!c) return CG_ENOMEM;
  c->err[0] = 0;
  int rc = validate(cfg, c->err, sizeof(c->err));
  if (rc) {
    fprintf(stderr, "cg_create: %s\n", c->err);
    delete c;
    return rc;
  }
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    fprintf(stderr, "cg_create: no usable CUDA device %d\n", device);
    cudaGetLastError();
    delete c;
    return CG_ECUDA;
  }
  c->stream = c->own_stream;
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  c->N = cfg->n_grid;
  c->NH = c->N / 2 + 1;
  c->grid_floats = (size_t)c->N * c->N * 2 * c->NH;
  *out = c;
  /* twiddles in double, rounded once */
  {
    const int N = c->N, H = N / 2;
    std::vector<float2> tw(N), th(H);
    for (int j = 0; j < N; j++) tw[j] = make_float2((float)cos(2 * M_PI * j / N), (float)sin(2 * M_PI * j / N));
    for (int j = 0; j < H; j++) th[j] = make_float2((float)cos(2 * M_PI * j / H), (float)sin(2 * M_PI * j / H));
    if ((rc = dalloc(c, &c->d_twN, (size_t)N)) || (rc = dalloc(c, &c->d_twH, (size_t)H))) return rc;
    CUDA_TRY(c, cudaMemcpy(c->d_twN, tw.data(), N * sizeof(float2), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_twH, th.data(), H * sizeof(float2), cudaMemcpyHostToDevice));
  }
  if ((rc = dalloc(c, &c->d_dens, c->grid_floats)) || (rc = dalloc(c, &c->d_npot, c->grid_floats))) return rc;
  c->npart = npartials(c->N);
  if ((rc = dalloc(c, &c->d_part, c->npart)) || (rc = dalloc(c, &c->d_stats, (size_t)4)) ||
      (rc = dalloc(c, &c->d_s2f, (size_t)1)) || (rc = dalloc(c, &c->d_err, (size_t)1)))
    return rc;
  CUDA_TRY(c, cudaMemset(c->d_err, 0, sizeof(unsigned int)));
  if ((rc = cg_upload_tables(c, cfg))) return rc;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return CG_OK;
}

extern "C" int cg_set_stream(cg_ctx *c, void *s)
{
  if (!c) return CG_EINVAL;
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return CG_OK;
}

extern "C" int cg_sync(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  if (c->ostream) CUDA_TRY(c, cudaStreamSynchronize(c->ostream));
  c->opend[0] = c->opend[1] = c->opend[2] = false;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" long long cg_kernel_launches(const cg_ctx *c) { return c ? c->launches : 0; }

/* ------------------------------------------------------------------------ */
/* stages                                                                   */
/* ------------------------------------------------------------------------ */
extern "C" int cg_create_cartesian_fields(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  cudaSetDevice(c->device);
  cg_field_launch L;
  L.stream = c->stream;
  L.f[0] = reinterpret_cast<float2 *>(c->d_dens);
  L.f[1] = reinterpret_cast<float2 *>(c->d_npot);
  L.f[2] = nullptr;
  L.fill = c->fill;
  L.norm = (float)std::pow(std::sqrt(2 * M_PI) / c->cfg.l_box, 3);
  L.partials = c->d_part;
  L.twN = c->d_twN;
  L.twH = c->d_twH;
  L.src = nullptr;
  L.err = c->d_err;
  L.ev = nullptr;
  {
    const int passes[3] = {CG_PASS_FILL2, CG_PASS_Y, CG_PASS_X}, nfs[3] = {2, 2, 1};
    if (int rc = tune_field_passes(c, &L, passes, nfs, 3)) return rc;
  }
  {
    ProfScope ps(c, "field_fft");
    PassEvents pe(c, "field_fill", "field_y", "field_x");
    L.ev = pe.after();
    CUDA_TRY(c, run_gauss(c->N, &L));
    const double ncell = (double)c->N * c->N * c->N;
    CUDA_TRY(c, cg_moments_final(c->stream, c->d_part, c->npart, 1.0 / ncell, c->d_stats, c->d_s2f));
  }
  c->launches += 5;
  c->have_fields = 1;
  c->have_density = c->have_norm = c->have_srcs = 0;
  c->pending_mode = CG_DMODE_NONE;
  return CG_OK;
}

extern "C" int cg_get_sigma2(cg_ctx *c, double *sigma2, double *mean)
{
  if (!c) return CG_EINVAL;
  if (!c->have_fields) return fail(c, CG_ESTATE, "fields not created");
  double h[4];
  CUDA_TRY(c, cudaMemcpyAsync(h, c->d_stats, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (sigma2) *sigma2 = h[3];
  if (mean) *mean = h[2];
  return CG_OK;
}

extern "C" int cg_compute_physical_density_field(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  if (!c->have_fields) return fail(c, CG_ESTATE, "create_cartesian_fields first");
  cudaSetDevice(c->device);
  if (c->cfg.dens_type == CG_DENS_LGNR) {
    c->pending_mode = CG_DMODE_LGNR; /* applied in the fused bins pass */
  } else if (c->cfg.dens_type == CG_DENS_CLIP) {
    c->pending_mode = CG_DMODE_CLIP;
  } else {
    int rc;
    const bool two = c->cfg.dens_type == CG_DENS_2LPT;
    for (int a = 0; a < 3; a++)
      if (!c->d_disp[a] && (rc = dalloc(c, &c->d_disp[a], c->grid_floats))) return rc;
    if (two)
      for (int a = 0; a < 6; a++)
        if (!c->d_lpt2[a] && (rc = dalloc(c, &c->d_lpt2[a], c->grid_floats))) return rc;
    cg_field_launch L;
    memset(&L, 0, sizeof(L));
    L.stream = c->stream;
    L.fill = c->fill;
    L.norm = 1.0f;
    L.partials = nullptr;
    L.twN = c->d_twN;
    L.twH = c->d_twH;
    L.err = c->d_err;
    {
      for (int a = 0; a < 3; a++) L.f[a] = reinterpret_cast<float2 *>(c->d_disp[a]);
      const int passes[3] = {CG_PASS_FILL3, CG_PASS_Y, CG_PASS_X}, nfs[3] = {3, 3, 3};
      if (int rc = tune_field_passes(c, &L, passes, nfs, 3)) return rc;
    }
    if (two) { /* lpt_2, density.c:646-812 */
      ProfScope ps(c, "lpt2_fft");
      for (int set = 0; set < 2; set++) { /* xx xy xz, then yy yz zz */
        L.fill.lpt_kind = 1 + set;
        for (int a = 0; a < 3; a++) L.f[a] = reinterpret_cast<float2 *>(c->d_lpt2[3 * set + a]);
        CUDA_TRY(c, run_lpt(c->N, &L));
      }
      CUDA_TRY(c, cg_lpt2_source(c->stream, c->d_lpt2[0], c->d_lpt2[1], c->d_lpt2[2], c->d_lpt2[3], c->d_lpt2[4],
                                 c->d_lpt2[5], c->N, c->nsm));
      L.src = reinterpret_cast<float2 *>(c->d_lpt2[5]);
      for (int a = 0; a < 3; a++) L.f[a] = reinterpret_cast<float2 *>(c->d_lpt2[a]);
      CUDA_TRY(c, run_lpt2(c->N, &L));
      c->launches += 2 * 3 + 1 + 5;
    }
    L.fill.lpt_kind = 0;
    for (int a = 0; a < 3; a++) L.f[a] = reinterpret_cast<float2 *>(c->d_disp[a]);
    {
      ProfScope ps(c, "lpt_fft");
      PassEvents pe(c, "lpt_fill", "lpt_y", "lpt_x");
      L.ev = pe.after();
      CUDA_TRY(c, run_lpt(c->N, &L));
      L.ev = nullptr;
    }
    ProfScope ps2(c, "lpt_cic");
    CUDA_TRY(c, cudaMemsetAsync(c->d_dens, 0, c->grid_floats * sizeof(float), c->stream));
    cg_lpt_params lp;
    lp.box = c->box;
    lp.g = c->g;
    lp.d1 = c->d1;
    lp.interp = c->cfg.lpt_interp_type;
    lp.d2x = two ? c->d_lpt2[0] : nullptr;
    lp.d2y = two ? c->d_lpt2[1] : nullptr;
    lp.d2z = two ? c->d_lpt2[2] : nullptr;
    lp.d2 = c->d2;
    CUDA_TRY(c, cg_lpt_cic(c->stream, c->d_dens, c->d_disp[0], c->d_disp[1], c->d_disp[2], &lp, c->nsm));
    c->launches += 4;
    c->pending_mode = CG_DMODE_RHO;
  }
  c->have_density = 1;
  c->have_norm = c->have_srcs = 0;
  return CG_OK;
}

/* Tracers of the normalisation: source populations, then intensity species,
 * then custom maps (collect_density_normalization_from_grid, density.c:1128-1211). */
static int n_imap_block(const cg_ctx *c) { return c->cfg.n_imap + c->cfg.n_cstm; }

static Tab tracer_bias(const cg_ctx *c, int t)
{
  const int nts = c->cfg.n_srcs, nti = c->cfg.n_imap;
  return t < nts ? c->bz[t] : (t < nts + nti ? c->bzi[t - nts] : c->bzc[t - nts - nti]);
}

/* Launch the bins pass over all tracers (one launch carries up to the
 * kernel's maximum number of bias tables). */
static int run_bins(cg_ctx *c, int nz, double idz)
{
  const int nts = c->cfg.n_srcs, nti = n_imap_block(c), nt = nts + nti;
  const int MT = cg_dens_bins_max_tracers();
  if (nt > MT) return fail(c, CG_EINVAL, "%d tracers: at most %d per run are supported", nt, MT);
  int rc;
  if (nz > c->bins_nz_cap || std::max(nt, 1) > c->bins_nt_cap) { /* grow only */
    c->bins_nz_cap = c->bins_nt_cap = 0;
    if ((rc = dalloc(c, &c->d_ncount, (size_t)nz)) || (rc = dalloc(c, &c->d_zsum, (size_t)nz)) ||
        (rc = dalloc(c, &c->d_bsum, (size_t)std::max(nt, 1) * nz)) ||
        (rc = dalloc(c, &c->d_bacc, (size_t)2 * (1 + std::max(nt, 1)) * nz)))
      return rc;
    c->bins_nz_cap = nz;
    c->bins_nt_cap = std::max(nt, 1);
  }
  CUDA_TRY(c, cudaMemsetAsync(c->d_ncount, 0, sizeof(unsigned long long) * nz, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_bacc, 0, sizeof(unsigned long long) * 2 * (1 + nt) * nz, c->stream));
  cg_bins_params p;
  memset(&p, 0, sizeof(p));
  p.box = c->box;
  p.g = c->g;
  p.zt = c->zt;
  p.d1 = c->d1;
  p.mode = c->pending_mode;
  p.err = c->d_err;
  p.sigma2f = c->d_s2f;
  p.nz = nz;
  p.idz = (float)idz;
  p.bias_model = c->cfg.bias_model;
  p.nt = nt;
  for (int t = 0; t < nt; t++) p.bz[t] = tracer_bias(c, t);
  p.ncount = c->d_ncount;
  p.acc = c->d_bacc;
  p.zsum = c->d_zsum;
  p.bsum = c->d_bsum;
  {
    ProfScope ps(c, "dens_bins");
    CUDA_TRY(c, cg_dens_bins(c->stream, c->d_dens, &p, c->nsm));
  }
  c->launches += 2;
  c->pending_mode = CG_DMODE_NONE;
  return CG_OK;
}

extern "C" int cg_collect_density_normalization(cg_ctx *c, int nz, double idz, double *zarr,
                                                unsigned long long *narr, double *norm_srcs, double *norm_imap)
{
  if (!c) return CG_EINVAL;
  if (!c->have_density) return fail(c, CG_ESTATE, "compute_physical_density_field first");
  if (nz < 2 || nz > 4096) return fail(c, CG_EINVAL, "nz=%d out of range", nz);
  cudaSetDevice(c->device);
  if (int rc = run_bins(c, nz, idz)) return rc;
  const int nts = c->cfg.n_srcs, nti = n_imap_block(c);
  std::vector<double> b((size_t)(nts + nti) * nz);
  std::vector<unsigned long long> n(nz);
  std::vector<double> z(nz);
  CUDA_TRY(c, cudaMemcpyAsync(n.data(), c->d_ncount, nz * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(z.data(), c->d_zsum, nz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (!b.empty())
    CUDA_TRY(c, cudaMemcpyAsync(b.data(), c->d_bsum, b.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (narr) memcpy(narr, n.data(), nz * sizeof(unsigned long long));
  if (zarr) memcpy(zarr, z.data(), nz * sizeof(double));
  if (norm_srcs && nts) memcpy(norm_srcs, b.data(), (size_t)nts * nz * sizeof(double));
  if (norm_imap && nti) memcpy(norm_imap, b.data() + (size_t)nts * nz, (size_t)nti * nz * sizeof(double));
  return CG_OK;
}

/* Device address of the static bins scratch, looked up once per device with
 * that device current (cudaGetSymbolAddress may load the module, so the
 * first call on a device must not be inside a stream capture) and kept for
 * the life of the process.  The address belongs to the device's primary
 * context: a host that calls cudaDeviceReset and keeps using the library
 * leaves a stale entry here. */
static std::mutex g_bins_scratch_mu;
static void *g_bins_scratch_ptr[CG_MAX_DEVICES];

static int bins_static_scratch(cg_ctx *c, void **out)
{
  if (c->device < 0 || c->device >= CG_MAX_DEVICES) return fail(c, CG_EINVAL, "device %d out of range", c->device);
  std::lock_guard<std::mutex> lock(g_bins_scratch_mu);
  if (!g_bins_scratch_ptr[c->device]) {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t e = cg_dens_bins_static_scratch(&ptr, &bytes);
    if (e != cudaSuccess || !ptr)
      return fail(c, CG_ECUDA, "cudaGetSymbolAddress(bins scratch): %s", cudaGetErrorString(e));
    g_bins_scratch_ptr[c->device] = ptr;
  }
  *out = g_bins_scratch_ptr[c->device];
  return CG_OK;
}

/* cg_collect_density_normalization without any allocation: the per-bin
 * counts and sums live in a fixed module-scope device array instead of
 * buffers made with cudaMalloc, and the results are copied straight into the
 * caller's arrays.  Calls overlapping on the GPU (two contexts on one device,
 * or two streams) share that array and race. */
extern "C" int cg_collect_density_normalization_static(cg_ctx *c, int nz, double idz, double *zarr,
                                                       unsigned long long *narr, double *norm_srcs,
                                                       double *norm_imap)
{
  if (!c) return CG_EINVAL;
  if (!c->have_density) return fail(c, CG_ESTATE, "compute_physical_density_field first");
  if (nz < 2 || nz > CG_BINS_STATIC_NZ)
    return fail(c, CG_EINVAL, "nz=%d: the static bins scratch holds 2 to %d bins", nz, CG_BINS_STATIC_NZ);
  const int nts = c->cfg.n_srcs, nti = n_imap_block(c), nt = nts + nti;
  if (nt > cg_dens_bins_max_tracers())
    return fail(c, CG_EINVAL, "%d tracers: at most %d per run are supported", nt, cg_dens_bins_max_tracers());
  CUDA_TRY(c, cudaSetDevice(c->device));
  void *scratch = nullptr;
  if (int rc = bins_static_scratch(c, &scratch)) return rc;
  unsigned long long *ncount = static_cast<unsigned long long *>(scratch);
  double *zsum = static_cast<double *>(scratch) + CG_BINS_STATIC_NZ;
  double *bsum = static_cast<double *>(scratch) + 2 * CG_BINS_STATIC_NZ;
  unsigned long long *acc = static_cast<unsigned long long *>(scratch) + (size_t)(2 + cg_dens_bins_max_tracers()) * CG_BINS_STATIC_NZ;
  /* the sums start at zero on every call */
  CUDA_TRY(c, cudaMemsetAsync(ncount, 0, sizeof(unsigned long long) * nz, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 2 * (1 + nt) * nz, c->stream));
  cg_bins_params p;
  memset(&p, 0, sizeof(p));
  p.box = c->box;
  p.g = c->g;
  p.zt = c->zt;
  p.d1 = c->d1;
  p.mode = c->pending_mode;
  p.err = c->d_err;
  p.sigma2f = c->d_s2f;
  p.nz = nz;
  p.idz = (float)idz;
  p.bias_model = c->cfg.bias_model;
  p.nt = nt;
  for (int t = 0; t < nt; t++) p.bz[t] = tracer_bias(c, t);
  p.ncount = ncount;
  p.acc = acc;
  p.zsum = zsum;
  p.bsum = bsum;
  {
    ProfScope ps(c, "dens_bins");
    CUDA_TRY(c, cg_dens_bins(c->stream, c->d_dens, &p, c->nsm));
  }
  c->launches += 2;
  c->pending_mode = CG_DMODE_NONE;
  if (narr)
    CUDA_TRY(c, cudaMemcpyAsync(narr, ncount, nz * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  if (zarr) CUDA_TRY(c, cudaMemcpyAsync(zarr, zsum, nz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (norm_srcs && nts)
    CUDA_TRY(c, cudaMemcpyAsync(norm_srcs, bsum, (size_t)nts * nz * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
  if (norm_imap && nti)
    CUDA_TRY(c, cudaMemcpyAsync(norm_imap, bsum + (size_t)nts * nz, (size_t)nti * nz * sizeof(double),
                                cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return CG_OK;
}

extern "C" int cg_set_norm_tables(cg_ctx *c, const double *srcs_norm, const double *srcs_norm_0f,
                                  const double *imap_norm, const double *imap_norm_0f)
{
  if (!c) return CG_EINVAL;
  const int na = CG_NA, nas = CG_NA + 2, nts = c->cfg.n_srcs, nti = n_imap_block(c), nsp = c->cfg.n_imap;
  if (nts + nti == 0) return CG_OK;
  std::vector<float> h((size_t)(nts + nti) * nas);
  for (int p = 0; p < nts + nti; p++) {
    const double *src = p < nts ? srcs_norm + (size_t)p * na : imap_norm + (size_t)(p - nts) * na;
    const double *e = p < nts ? srcs_norm_0f + 2 * p : imap_norm_0f + 2 * (p - nts);
    for (int i = 0; i < na; i++) h[(size_t)p * nas + i] = (float)src[i];
    h[(size_t)p * nas + na] = (float)e[0];
    h[(size_t)p * nas + na + 1] = (float)e[1];
  }
  CUDA_TRY(c, cudaMemcpyAsync(c->d_norm, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  std::vector<double> hd((size_t)(nts + nti) * nas);
  for (int p = 0; p < nts + nti; p++) {
    const double *src = p < nts ? srcs_norm + (size_t)p * na : imap_norm + (size_t)(p - nts) * na;
    const double *e = p < nts ? srcs_norm_0f + 2 * p : imap_norm_0f + 2 * (p - nts);
    memcpy(hd.data() + (size_t)p * nas, src, na * sizeof(double));
    hd[(size_t)p * nas + na] = e[0];
    hd[(size_t)p * nas + na + 1] = e[1];
  }
  CUDA_TRY(c, cudaMemcpyAsync(c->d_norm64, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* h and hd are local buffers */
  for (int p = 0; p < nts + nti; p++) {
    const Tab t = Tab{c->d_norm + (size_t)p * nas, h[(size_t)p * nas + na], h[(size_t)p * nas + na + 1]};
    if (p < nts) c->norm[p] = t;
    else if (p - nts < nsp) c->normi[p - nts] = t;
    else c->normc[p - nts - nsp] = t;
  }
  c->have_norm = 1;
  return CG_OK;
}

/* compute_density_normalization (density.c:1227-1393): the bin sums of the
 * fused density pass, then the tables built on the device (k_norm_tables,
 * the double-precision steps of density.c:1272-1355), with no host round
 * trip; the edge values travel inside the tables. */
extern "C" int cg_compute_density_normalization(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  if (!c->have_density) return fail(c, CG_ESTATE, "compute_physical_density_field first");
  const int nts = c->cfg.n_srcs, nti = n_imap_block(c), nt = nts + nti, nz = c->norm_nz;
  if (nz < 2 || nz > CG_NORM_NZ_MAX)
    return fail(c, CG_EINVAL, "%d redshift bins: the device tables take 2 to %d", nz, CG_NORM_NZ_MAX);
  cudaSetDevice(c->device);
  if (int rc = run_bins(c, nz, c->norm_idz)) return rc;
  if (nt > 0) {
    ProfScope ps(c, "norm_tables");
    CUDA_TRY(c, cg_norm_tables(c->stream, c->d_ncount, c->d_zsum, c->d_bsum, nz, nt, c->norm_zlast, c->d_zr,
                               c->d_norm, c->d_norm64));
    c->launches++;
  }
  const int nas = CG_NA + 2, nsp = c->cfg.n_imap;
  for (int p = 0; p < nt; p++) { /* edges are read from the tables by the kernels */
    const Tab t = Tab{c->d_norm + (size_t)p * nas, 0.0f, 0.0f};
    if (p < nts) c->norm[p] = t;
    else if (p - nts < nsp) c->normi[p - nts] = t;
    else c->normc[p - nts - nsp] = t;
  }
  c->have_norm = 1;
  c->have_srcs = 0;
  return CG_OK;
}

static void srcs_params(cg_ctx *c, int ipop, cg_srcs_params &p)
{
  memset(&p, 0, sizeof(p));
  p.box = c->box;
  p.g = c->g;
  p.zt = c->zt;
  p.v1 = c->v1;
  p.nz = c->nz[ipop];
  p.bz = c->bz[ipop];
  p.norm = c->norm[ipop];
  p.a_a2r = c->a_a2r;
  p.r_a2r = c->r_a2r;
  p.na = CG_NA;
  p.bias_model = c->cfg.bias_model;
  p.kp0 = (uint32_t)c->cfg.seed;
  p.kp1 = (uint32_t)(c->cfg.seed >> 32) ^ (CG_STREAM_POIS + (uint32_t)ipop);
  p.kq0 = (uint32_t)c->cfg.seed;
  p.kq1 = (uint32_t)(c->cfg.seed >> 32) ^ (CG_STREAM_POS + (uint32_t)ipop);
  p.rlim = (float)(c->cfg.l_box / 2 + 20.);
  const double dx = c->cfg.l_box / c->N;
  p.cell_vol = (float)(dx * dx * dx);
  p.factor_vel = (float)(-c->cfg.fgrowth_0 / (1.5 * c->cfg.hubble_0 * c->cfg.omega_m));
  p.need_beaming = c->cfg.need_beaming;
  p.nside_base = c->cfg.nside_base;
  p.base_r2n = c->d_r2n;
  p.nside_count = c->cfg.nside_count[ipop];
  p.cmap = c->cat[ipop].cmap;
  p.counts = c->d_counts;
  p.block_sums = c->d_bsums;
  p.ovf_cell = c->d_ovf_cell;
  p.ovf_cnt = c->d_ovf_cnt;
  p.ovf_n = c->d_ovf_n;
  p.capacity = c->cat[ipop].cap;
  p.pos = c->cat[ipop].pos;
  p.ipix = c->cat[ipop].ipix;
  p.src = c->cat[ipop].src;
  p.err = c->d_err;
  /* the exact decisions (cg_exact.h) */
  const int na = CG_NA, N = c->N, nas = CG_NA + 2;
  cg_pois_args &a = p.pa;
  a.r = c->g.r;
  a.nz = c->nz[ipop].f;
  a.bz = c->bz[ipop].f;
  a.norm = c->norm[ipop].f;
  a.xc = c->d_corner;
  a.yc = c->d_corner + N;
  a.zc = c->d_corner + 2 * N;
  a.idr = c->g.idr;
  a.r_last = c->g.r_last;
  a.bz0 = (float)c->cfg.srcs_bz_arr[ipop][0];
  a.cell_vol = p.cell_vol;
  a.rlim = p.rlim;
  a.na = na;
  a.bias_model = c->cfg.bias_model;
  cgx_srcs_tabs &x = a.x;
  x.r = c->d_tabs64;
  x.nz = c->d_tabs64 + (size_t)(4 + 2 * ipop) * na;
  x.bz = c->d_tabs64 + (size_t)(5 + 2 * ipop) * na;
  x.norm = c->d_norm64 + (size_t)ipop * nas;
  x.idr = c->cfg.glob_idr;
  x.r_last = c->cfg.r_arr_r2z[na - 1];
  x.bz0 = c->cfg.srcs_bz_arr[ipop][0];
  x.dx = dx;
  x.cell_vol = dx * dx * dx;
  x.rlim = c->cfg.l_box / 2 + 20.;
  for (int k = 0; k < 3; k++) x.p[k] = c->cfg.pos_obs[k];
  x.bias_model = c->cfg.bias_model;
  p.dx64 = dx;
  for (int k = 0; k < 3; k++) p.p64[k] = c->cfg.pos_obs[k];
  for (int k = 0; k < 3; k++) p.cl[k] = c->d_corner + (size_t)(3 + k) * N;
  p.dxh = (float)dx;
  p.dxl = (float)(dx - (double)p.dxh);
  p.force_double = c->force_double;
  p.xstats = c->d_xstats;
}

/* srcs_set_cartesian for every population: count -> scan -> emit.  With
 * readback the total is read after the count to size the catalogue (the
 * public entry point); without it the catalogue keeps its capacity, emit
 * drops what does not fit and flags the overflow, and the totals stay on
 * the device until read (the graph-captured sequence). */
static int srcs_run(cg_ctx *c, long long *nsrc, bool readback)
{
  if (!c->have_density) return fail(c, CG_ESTATE, "density not computed");
  if (!c->have_norm) return fail(c, CG_ESTATE, "compute_density_normalization first");
  cudaSetDevice(c->device);
  const long long ncell = (long long)c->N * c->N * c->N;
  int rc;
  if (c->cfg.n_srcs > 0) {
    if (!c->d_counts && (rc = dalloc(c, &c->d_counts, (size_t)ncell))) return rc;
    if (!c->d_bsums && (rc = dalloc(c, &c->d_bsums, (size_t)(cg_srcs_nblocks(c->N) +
                                                             cg_srcs_scan_room(cg_srcs_nblocks(c->N))))))
      return rc;
    if (!c->d_total && (rc = dalloc(c, &c->d_total, (size_t)CG_NPOP_MAX))) return rc;
    if (!c->d_ovf_n && ((rc = dalloc(c, &c->d_ovf_cell, (size_t)CG_OVF_CAP)) ||
                        (rc = dalloc(c, &c->d_ovf_cnt, (size_t)CG_OVF_CAP)) || (rc = dalloc(c, &c->d_ovf_n, (size_t)1))))
      return rc;
  }
  for (int ip = 0; ip < c->cfg.n_srcs; ip++) {
    Cat &K = c->cat[ip];
    cg_srcs_params p;
    srcs_params(c, ip, p);
    {
      ProfScope ps(c, "srcs_count");
      CUDA_TRY(c, cg_srcs_count(c->stream, c->d_dens, &p, c->d_total + ip));
    }
    if (readback) {
      long long tot = 0;
      CUDA_TRY(c, cudaMemcpyAsync(&tot, c->d_total + ip, sizeof(tot), cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      if ((rc = check_device_errors(c))) return rc;
      if (tot > K.cap) {
        long long cap = tot + tot / 8 + 1024;
        if ((rc = dalloc(c, &K.pos, (size_t)cap)) || (rc = dalloc(c, &K.ipix, (size_t)cap)) ||
            (rc = dalloc(c, &K.src, (size_t)cap * 9)))
          return rc;
        K.cap = cap;
      }
      K.n = tot;
      if (nsrc) nsrc[ip] = tot;
    } else {
      K.n = -1; /* on the device until refresh_counts */
    }
    const int ns = c->cfg.nside_count[ip];
    if (ns > 0) {
      long long np = 12LL * ns * ns;
      if (K.cmap_npix != np) {
        if ((rc = dalloc(c, &K.cmap, (size_t)np))) return rc;
        K.cmap_npix = np;
      }
      CUDA_TRY(c, cudaMemsetAsync(K.cmap, 0, np * sizeof(int), c->stream));
    }
    srcs_params(c, ip, p);
    {
      ProfScope ps(c, "srcs_emit");
      CUDA_TRY(c, cg_srcs_emit(c->stream, c->d_npot, &p));
    }
    c->launches += 5; /* count, three scan passes, emission */
  }
  c->have_srcs = 1;
  return CG_OK;
}

extern "C" int cg_srcs_set_cartesian(cg_ctx *c, long long *nsrc)
{
  if (!c) return CG_EINVAL;
  out_join(c, 0); /* the catalogues are rewritten */
  return srcs_run(c, nsrc, true);
}

/* Source totals left on the device by a graph launch: wait for it, read
 * them and check the catalogues held every source. */
static int refresh_counts(cg_ctx *c)
{
  bool stale = false;
  for (int ip = 0; ip < c->cfg.n_srcs; ip++) stale |= c->cat[ip].n < 0;
  if (!stale) return CG_OK;
  if (c->graph_done) CUDA_TRY(c, cudaEventSynchronize(c->graph_done));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  long long tot[CG_NPOP_MAX];
  CUDA_TRY(c, cudaMemcpy(tot, c->d_total, c->cfg.n_srcs * sizeof(long long), cudaMemcpyDeviceToHost));
  for (int ip = 0; ip < c->cfg.n_srcs; ip++) c->cat[ip].n = tot[ip];
  if (int rc = check_device_errors(c)) return rc;
  for (int ip = 0; ip < c->cfg.n_srcs; ip++)
    if (c->cat[ip].n > c->cat[ip].cap)
      return fail(c, CG_EDEVICE, "population %d: %lld sources, catalogue holds %lld", ip, c->cat[ip].n,
                  c->cat[ip].cap);
  return CG_OK;
}

extern "C" long long cg_num_sources(cg_ctx *c, int ipop)
{
  if (!c || ipop < 0 || ipop >= c->cfg.n_srcs) return -1;
  if (refresh_counts(c)) return -1;
  return c->cat[ipop].n;
}

/* Stage tables are built outside a stream capture only. */
static int not_capturing(cg_ctx *c, const char *what)
{
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CUDA_TRY(c, cudaStreamIsCapturing(c->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return fail(c, CG_ESTATE, "%s: tables not built before the capture", what);
  return CG_OK;
}

/* Tables of intensity species ip (imap_preproc, imap.c:105-133, and the
 * sub-sampling factors, imap.c:153-174): shells sorted by r0 and their edges
 * as intervals, the buckets' slots, the cell list and the queue.  Built
 * once per table generation (or list bound), with host round trips; never
 * inside a stream capture. */
static int imap_prepare(cg_ctx *c, int ip)
{
  Imap &M = c->im[ip];
  if (M.gen == c->tab_gen) return CG_OK;
  int rc;
  if ((rc = not_capturing(c, "intensity maps"))) return rc;
  const int nr = c->cfg.imap_nr[ip];
  const int nside = c->cfg.nside_imap[ip];
  const long long npix = 12LL * nside * nside;
  const double dx = c->cfg.l_box / c->N;
  const int nbk = nr + 2;
  if (nbk > CG_IMAP_BUCKETS_MAX) return fail(c, CG_EINVAL, "intensity species %d: %d shells", ip, nr);
  std::vector<float> r0f(nr), rff(nr), bb(2 * nr), dxs(nr + 2);
  std::vector<int> shell_of(2 * nr + 1), nsub(nr + 2);
  const int nb = cg_imap_shells(c->cfg.imap_r0[ip], c->cfg.imap_rf[ip], nr, dx, npix, r0f.data(), rff.data(),
                                bb.data(), shell_of.data(), nsub.data(), dxs.data());
  for (int i = 0; i < nr + 2; i++)
    if (nsub[i] < 1 || nsub[i] > 1024)
      return fail(c, CG_EINVAL, "intensity species %d: nsub %d outside 1..1024", ip, nsub[i]);
  if (M.nr != nr) {
    if ((rc = dalloc(c, &M.b, (size_t)2 * nr)) || (rc = dalloc(c, &M.shell_of, (size_t)2 * nr + 1)) ||
        (rc = dalloc(c, &M.nsub, (size_t)nr + 2)) || (rc = dalloc(c, &M.dxs, (size_t)nr + 2)) ||
        (rc = dalloc(c, &M.dxsl, (size_t)nr + 2)) ||
        (rc = dalloc(c, &M.base, (size_t)nbk)) || (rc = dalloc(c, &M.cap, (size_t)nbk)) ||
        (rc = dalloc(c, &M.cnt, (size_t)nbk)) || (rc = dalloc(c, &M.chunk_off, (size_t)nbk + 1)))
      return rc;
  }
  if (M.nr != nr || M.npix != npix) {
    if ((rc = dalloc(c, &M.data, (size_t)nr * npix)) || (rc = dalloc(c, &M.nadd, (size_t)nr * npix))) return rc;
  }
  M.nr = nr;
  M.nside = nside;
  M.npix = npix;
  const double rmin = (double)r0f[0] - 20., rmax = (double)rff[nr - 1] + 20.;
  /* slots per bucket: the corners of the cells of bucket j + 1 lie in the
   * radii of the intervals of shell j; each corner's dx-cube lies within
   * sqrt(3)/2 dx of it, so (expanded shell volume) / dx^3 bounds them */
  std::vector<double> want(nbk, 0.0);
  const double h = 0.8660254037844386 * dx, ncell = (double)c->N * c->N * c->N;
  for (int k = -1; k < nb; k++) {
    double lo = k < 0 ? rmin : (double)bb[k], hi = k + 1 < nb ? (double)bb[k + 1] : rmax;
    lo = lo < rmin ? rmin : lo;
    hi = hi > rmax ? rmax : hi;
    if (hi <= lo) continue;
    const double a = lo - h > 0 ? lo - h : 0, z = hi + h;
    want[shell_of[k + 1] + 1] += 4.0 / 3.0 * M_PI * (z * z * z - a * a * a) / (dx * dx * dx);
  }
  double tot = 0;
  for (int i = 0; i < nbk; i++) {
    want[i] = std::min(want[i], ncell) + 64;
    tot += want[i];
  }
  /* room: every cell, within a quarter of the free memory and the
   * caller's bound (cells beyond are painted by the listing kernel) */
  size_t fr = 0, tt = 0;
  CUDA_TRY(c, cudaMemGetInfo(&fr, &tt));
  double room = (double)(fr + (size_t)c->list_cap * CG_IMAP_REC_BYTES) * 0.25 / CG_IMAP_REC_BYTES;
  if (c->list_cap_max > 0 && room > (double)c->list_cap_max) room = (double)c->list_cap_max;
  const double scale = tot > room ? room / tot : 1.0;
  std::vector<long long> base(nbk), capv(nbk);
  long long acc = 0;
  for (int i = 0; i < nbk; i++) {
    base[i] = acc;
    capv[i] = (long long)(want[i] * scale);
    acc += capv[i];
  }
  if (acc > c->list_cap) {
    if ((rc = dalloc(c, &c->d_recs, (size_t)acc))) return rc;
    c->list_cap = acc;
  }
  if (!M.ctr && (rc = dalloc(c, &M.ctr, (size_t)5))) return rc;
  if (!c->d_imap_queue) {
    const long long qc = 1LL << 27;
    if ((rc = dalloc(c, &c->d_imap_queue, (size_t)qc))) return rc;
    c->queue_cap = qc;
  }
  CUDA_TRY(c, cudaMemcpyAsync(M.b, bb.data(), nb * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(M.shell_of, shell_of.data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(M.nsub, nsub.data(), (nr + 2) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(M.dxs, dxs.data(), (nr + 2) * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  std::vector<float> dxsl(nr + 2);
  for (int i = 0; i < nr + 2; i++) dxsl[i] = (float)(dx / nsub[i] - (double)dxs[i]);
  CUDA_TRY(c, cudaMemcpyAsync(M.dxsl, dxsl.data(), (nr + 2) * sizeof(float), cudaMemcpyHostToDevice, c->stream));

  CUDA_TRY(c, cudaMemcpyAsync(M.base, base.data(), nbk * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(M.cap, capv.data(), nbk * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vectors */
  M.nb = nb;
  M.contig = cg_imap_contig(r0f.data(), rff.data(), nr, nb);
  M.rmin = rmin;
  M.rmax = rmax;
  M.gen = c->tab_gen;
  return CG_OK;
}

/* The painting of species ip on the context's stream: no host round trip,
 * so that it can be captured in a graph; the samples drawn are read on
 * demand (cg_imap_samples). */
static int imap_launch(cg_ctx *c, int ip)
{
  Imap &M = c->im[ip];
  const int nr = M.nr, nside = M.nside, nbk = nr + 2;
  const long long npix = M.npix;
  const double dx = c->cfg.l_box / c->N;
  CUDA_TRY(c, cudaMemsetAsync(M.data, 0, (size_t)nr * npix * sizeof(float), c->stream));
  CUDA_TRY(c, cudaMemsetAsync(M.nadd, 0, (size_t)nr * npix * sizeof(int), c->stream));
  cg_imap_params p;
  memset(&p, 0, sizeof(p));
  p.box = c->box;
  cg_imap_args &a = p.a;
  const int na = CG_NA, N = c->N, nt0 = 4 + 2 * c->cfg.n_srcs;
  a.r = c->g.r;
  a.tz = c->tz[ip].f;
  a.bz = c->bzi[ip].f;
  a.norm = c->normi[ip].f;
  a.v1 = c->v1.f;
  a.ih = c->ih.f;
  a.xc = c->d_corner;
  a.yc = c->d_corner + N;
  a.zc = c->d_corner + 2 * N;
  a.xl = c->d_corner + 3 * N;
  a.yl = c->d_corner + 4 * N;
  a.zl = c->d_corner + 5 * N;
  a.idr = c->g.idr;
  a.r_last = c->g.r_last;
  a.rmin = (float)M.rmin;
  a.rmax = (float)M.rmax;
  const double fv = -c->cfg.fgrowth_0 / (1.5 * c->cfg.hubble_0 * c->cfg.omega_m);
  a.fvh = (float)(fv * (0.5 * (c->cfg.n_grid / c->cfg.l_box)));
  a.dx = (float)dx;
  a.na = na;
  a.bias_model = c->cfg.bias_model;
  a.nside = nside;
  a.sh.b = M.b;
  a.sh.shell_of = M.shell_of;
  a.sh.nb = M.nb;
  a.sh.nr = nr;
  a.sh.contig = M.contig;
  a.nsub = M.nsub;
  a.dxs = M.dxs;
  a.dxsl = M.dxsl;
  a.att = c->d_att;
  a.r64 = c->d_tabs64;
  a.v164 = c->d_tabs64 + (size_t)2 * na;
  a.ih64 = c->d_tabs64 + (size_t)3 * na;
  a.tz64 = c->d_tabs64 + (size_t)(nt0 + 2 * ip) * na;
  a.bz64 = c->d_tabs64 + (size_t)(nt0 + 2 * ip + 1) * na;
  a.norm64 = c->d_norm64 + (size_t)(c->cfg.n_srcs + ip) * (na + 2);
  a.idr64 = c->cfg.glob_idr;
  a.r_last64 = c->cfg.r_arr_r2z[na - 1];
  a.dx64 = dx;
  for (int k = 0; k < 3; k++) a.p64[k] = c->cfg.pos_obs[k];
  a.idx64 = c->cfg.n_grid / c->cfg.l_box;
  a.fv64 = fv;
  a.rmin64 = M.rmin;
  a.rmax64 = M.rmax;
  p.nr = nr;
  p.nbk = nbk;
  p.npix = npix;
  p.data = M.data;
  p.nadd = M.nadd;
  p.err = c->d_err;
  p.xstats = c->d_xstats;
  p.force_double = c->force_double;
  p.recs = c->d_recs;
  p.base = M.base;
  p.cap = M.cap;
  p.cnt = M.cnt;
  p.chunk_off = M.chunk_off;
  p.ctr = M.ctr;
  p.queue = c->d_imap_queue;
  p.queue_cap = c->queue_cap;
  {
    ProfScope ps(c, "imap_paint");
    CUDA_TRY(c, cg_imap_paint(c->stream, c->d_dens, c->d_npot, &p, c->nsm));
  }
  M.samples_stale = true;
  c->launches += 4; /* list, chunks, paint, double */
  return CG_OK;
}

/* Every species; with host_out, the final maps go to registered host
 * buffers (not in a captured sequence). */
static int imap_run(cg_ctx *c, bool host_out)
{
  for (int ip = 0; ip < c->cfg.n_imap; ip++) {
    if (int rc = imap_prepare(c, ip)) return rc;
    if (int rc = imap_launch(c, ip)) return rc;
  }
  if (!host_out) return CG_OK;
  /* final maps to registered host buffers (write_imap, io.c:738-741:
   * data/nadd where nadd > 0), overlapping the stages still to run */
  for (int ip = 0; ip < c->cfg.n_imap; ip++) {
    if (!c->h_imap[ip]) continue;
    const Imap &M = c->im[ip];
    const long long m = (long long)M.nr * M.npix;
    if (c->imap_out_n[ip] != m) {
      if (int rc = dalloc(c, &c->d_imap_out[ip], (size_t)m)) return rc;
      c->imap_out_n[ip] = m;
    }
    k_div_nadd<<<(unsigned)std::min<long long>((m + 255) / 256, (long long)c->nsm * 16), 256, 0, c->stream>>>(
        M.data, M.nadd, c->d_imap_out[ip], m);
    CUDA_TRY(c, cudaGetLastError());
    c->launches++;
    if (int rc = out_begin(c)) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->h_imap[ip], c->d_imap_out[ip], m * sizeof(float), cudaMemcpyDeviceToHost,
                                c->ostream));
    if (int rc = out_end(c, 1)) return rc;
  }
  return CG_OK;
}

extern "C" int cg_imap_set_cartesian(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  if (c->cfg.n_imap == 0) return CG_OK;
  if (!c->have_norm) return fail(c, CG_ESTATE, "compute_density_normalization first");
  cudaSetDevice(c->device);
  out_join(c, 1); /* the maps are rewritten */
  return imap_run(c, true);
}


extern "C" int cg_set_imap_list_cap(cg_ctx *c, long long cap)
{
  if (!c || cap < 0) return CG_EINVAL;
  c->list_cap_max = cap;
  for (int ip = 0; ip < CG_NPOP_MAX; ip++) c->im[ip].gen = 0; /* bucket room is recomputed */
  return CG_OK;
}

extern "C" int cg_imap_samples(cg_ctx *c, int ipop, unsigned long long *n)
{
  if (!c || !n || ipop < 0 || ipop >= c->cfg.n_imap) return CG_EINVAL;
  Imap &M = c->im[ipop];
  if (M.samples_stale && M.ctr) {
    if (c->graph_done) CUDA_TRY(c, cudaEventSynchronize(c->graph_done));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    unsigned long long ctr[5];
    CUDA_TRY(c, cudaMemcpy(ctr, M.ctr, sizeof(ctr), cudaMemcpyDeviceToHost));
    M.samples = ctr[2];
    M.samples_stale = false;
  }
  *n = M.samples;
  return CG_OK;
}

static int kappa_run(cg_ctx *c)
{
  const int np = c->cfg.n_kappa;
  const int nside = c->cfg.nside_kappa;
  const long long npix = 12LL * nside * nside;
  const int nr = c->N / 2; /* get_radial_params with NSAMP_RAD = 1 */
  const double dr = c->cfg.r_max / nr, idr = 1. / dr;
  int rc;
  if (c->kgen != c->tab_gen || c->kpl != np || c->knpix != npix || c->knr != nr) {
    if ((rc = not_capturing(c, "convergence"))) return rc;
    /* kappa_beams_preproc: sort planes by distance (stored as flouble) */
    std::vector<float> rp(np);
    for (int i = 0; i < np; i++) rp[i] = (float)c->cfg.kappa_r[i];
    std::stable_sort(rp.begin(), rp.end());
    std::vector<int> ir(2 * np);
    std::vector<float> inv(np), fac(2 * (size_t)nr);
    for (int i = 0; i < np; i++) {
      int irh = (int)((double)rp[i] * idr + 0.5);
      inv[i] = (float)(1. / (irh * dr));
      ir[np + i] = std::min(irh, nr - 1);
    }
    ir[0] = 0;
    for (int i = 1; i < np; i++) ir[i] = ir[np + i - 1] + 1;
    for (int i = 0; i < nr; i++) {
      double rm = (i + 0.5) * dr;
      double pg = host_bg(c, c->h_d1, 1, c->h_d1[CG_NA - 1], rm) * (1 + host_bg(c, c->h_z, 0, c->h_z[CG_NA - 1], rm));
      fac[i] = (float)(rm * pg * dr);
      fac[nr + i] = (float)(rm * rm * pg * dr);
    }
    if (c->kpl != np || c->knpix != npix) {
      if ((rc = dalloc(c, &c->d_kmap, (size_t)np * npix))) return rc;
    }
    if (c->knr != nr || c->kpl != np) {
      if ((rc = dalloc(c, &c->d_kfac, 2 * (size_t)nr)) || (rc = dalloc(c, &c->d_kinv, (size_t)np)) ||
          (rc = dalloc(c, &c->d_kir, 2 * (size_t)np)))
        return rc;
    }
    c->kpl = np;
    c->knpix = npix;
    c->knr = nr;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_kfac, fac.data(), fac.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_kinv, inv.data(), inv.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_kir, ir.data(), ir.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vectors */
    c->kgen = c->tab_gen;
  }
  cg_kappa_params p;
  p.box = c->box;
  p.nside = nside;
  p.npix = npix;
  p.nplanes = np;
  p.ir_min = c->d_kir;
  p.ir_max = c->d_kir + np;
  p.inv_r_max = c->d_kinv;
  p.nr = nr;
  p.dr = (float)dr;
  p.fac1 = c->d_kfac;
  p.fac2 = c->d_kfac + nr;
  p.map = c->d_kmap;
  {
    ProfScope ps(c, "kappa");
    CUDA_TRY(c, cg_kappa_integrate(c->stream, c->d_npot, &p));
  }
  c->launches++;
  return CG_OK;
}

/* isw_beams_preproc + isw_get_beam_properties (isw.c:38-147) */
static int isw_run(cg_ctx *c)
{
  const int np = c->cfg.n_isw;
  const int nside = c->cfg.nside_isw;
  const long long npix = 12LL * nside * nside;
  const int nr = c->N / 2; /* get_radial_params with NSAMP_RAD = 1 */
  const double dr = c->cfg.r_max / nr, idr = 1. / dr;
  int rc;
  if (c->igen != c->tab_gen || c->ipl != np || c->inpix != npix || c->inr != nr) {
    if ((rc = not_capturing(c, "ISW"))) return rc;
    std::vector<float> rp(np); /* plane distances, stored as flouble and sorted */
    for (int i = 0; i < np; i++) rp[i] = (float)c->cfg.isw_r[i];
    std::stable_sort(rp.begin(), rp.end());
    std::vector<int> ir(2 * np);
    for (int i = 0; i < np; i++) ir[np + i] = std::min((int)((double)rp[i] * idr + 0.5), nr - 1);
    ir[0] = 0;
    for (int i = 1; i < np; i++) ir[i] = ir[np + i - 1] + 1;
    std::vector<float> fac(nr);
    for (int i = 0; i < nr; i++) {
      const double rm = (i + 0.5) * dr;
      fac[i] = (float)(2 * host_bg(c, c->h_pd, c->h_pd[0], c->h_pd[CG_NA - 1], rm) * dr);
    }
    if (c->ipl != np || c->inpix != npix)
      if ((rc = dalloc(c, &c->d_imap_isw, (size_t)np * npix))) return rc;
    if (c->inr != nr || c->ipl != np)
      if ((rc = dalloc(c, &c->d_ifac, (size_t)nr)) || (rc = dalloc(c, &c->d_iir, 2 * (size_t)np))) return rc;
    c->ipl = np;
    c->inpix = npix;
    c->inr = nr;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_ifac, fac.data(), fac.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_iir, ir.data(), ir.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vectors */
    c->igen = c->tab_gen;
  }
  cg_kappa_params p;
  memset(&p, 0, sizeof(p));
  p.box = c->box;
  p.nside = nside;
  p.npix = npix;
  p.nplanes = np;
  p.ir_min = c->d_iir;
  p.ir_max = c->d_iir + np;
  p.nr = nr;
  p.dr = (float)dr;
  p.fac1 = c->d_ifac;
  p.map = c->d_imap_isw;
  {
    ProfScope ps(c, "isw");
    CUDA_TRY(c, cg_isw_integrate(c->stream, c->d_npot, &p));
  }
  c->launches++;
  return CG_OK;
}

/* cstm_beams_preproc + cstm_get_beam_properties (cstm.c:39-145): the step
 * tables kz = K(r)/IH(r) and bz on the N/2 radial step centres from the
 * FP64 tables, the integration range where |kz| > 1e-4 max|kz|, then one ray
 * per pixel (the kernel evaluates the FP32 normalisation table itself, as
 * every other tracer kernel does). */
static int cstm_run(cg_ctx *c)
{
  if (!c->have_norm) return fail(c, CG_ESTATE, "custom maps need the density normalisation");
  const int nr = c->N / 2, nc = c->cfg.n_cstm; /* get_radial_params with NSAMP_RAD = 1 */
  const double dr = c->cfg.r_max / nr;
  int rc;
  if (c->cgen != c->tab_gen || c->cnr != nr) {
    if ((rc = not_capturing(c, "custom maps"))) return rc;
    if (c->cnr != nr)
      if ((rc = dalloc(c, &c->d_cfac, 2 * (size_t)nr * CG_NPOP_MAX))) return rc;
    c->cnr = nr;
    std::vector<float> tab(2 * (size_t)nr * nc);
    int *irange = c->cir;
    for (int p = 0; p < nc; p++) {
      float *kz = tab.data() + 2 * (size_t)nr * p, *bz = kz + nr;
      double kmax = -1e100;
      std::vector<double> kzd(nr);
      for (int i = 0; i < nr; i++) {
        const double rm = (i + 0.5) * dr;
        kzd[i] = host_bg(c, c->h_kzc[p], 0, 0, rm) / host_bg(c, c->h_ih, c->h_ih[0], c->h_ih[CG_NA - 1], rm);
        kz[i] = (float)kzd[i];
        bz[i] = (float)host_bg(c, c->h_bzc[p], c->h_bzc[p][0], 1, rm);
        kmax = std::max(kmax, fabs(kzd[i]));
      }
      int lo = 0, hi = nr - 1;
      for (int i = 0; i < nr; i++)
        if (fabs(kzd[i]) > 1e-4 * kmax) {
          lo = i;
          break;
        }
      for (int i = nr - 1; i >= 0; i--)
        if (fabs(kzd[i]) > 1e-4 * kmax) {
          hi = i;
          break;
        }
      if (hi < lo) return fail(c, CG_EINVAL, "Custom kernel %d has no support", p);
      irange[2 * p] = lo;
      irange[2 * p + 1] = hi;
      const long long npix = 12LL * c->cfg.nside_cstm[p] * c->cfg.nside_cstm[p];
      if (c->cnpix[p] != npix) {
        if ((rc = dalloc(c, &c->d_cmap[p], (size_t)npix))) return rc;
        c->cnpix[p] = npix;
      }
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->d_cfac, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vector */
    c->cgen = c->tab_gen;
  }
  const int *irange = c->cir;
  for (int p = 0; p < nc; p++) {
    cg_cstm_params q;
    memset(&q, 0, sizeof(q));
    q.box = c->box;
    q.g = c->g;
    q.norm = c->normc[p];
    q.nside = c->cfg.nside_cstm[p];
    q.npix = c->cnpix[p];
    q.ir_min = irange[2 * p];
    q.ir_max = irange[2 * p + 1];
    q.bias_model = c->cfg.bias_model;
    q.dr = (float)dr;
    q.kz = c->d_cfac + 2 * (size_t)nr * p;
    q.bz = q.kz + nr;
    q.map = c->d_cmap[p];
    ProfScope ps(c, "cstm");
    CUDA_TRY(c, cg_cstm_integrate(c->stream, c->d_dens, &q));
    c->launches++;
  }
  return CG_OK;
}

/* Step tables of srcs_get_beam_properties_single and
 * srcs_beams_postproc_single (srcs.c:465-478, 725-733) on the N/2 steps of
 * the catalogue's radial grid (catalog_alloc, common.c:377-379):
 * 2 pg dr and rm pg dr with pg = D(rm) (1 + z(rm)), then V1(rm) factor_vel. */
static int los_tables(cg_ctx *c)
{
  const int nr = c->N / 2;
  const double dr = c->cfg.r_max / nr;
  if (c->losnr == nr && c->losgen == c->tab_gen) return CG_OK;
  if (int rc = not_capturing(c, "line-of-sight quantities")) return rc;
  if (c->losnr != nr)
    if (int rc = dalloc(c, &c->d_losfac, 3 * (size_t)nr)) return rc;
  const double fv = -c->cfg.fgrowth_0 / (1.5 * c->cfg.hubble_0 * c->cfg.omega_m);
  std::vector<float> t(3 * (size_t)nr);
  for (int i = 0; i < nr; i++) {
    const double rm = (i + 0.5) * dr;
    const double pg = host_bg(c, c->h_d1, 1, c->h_d1[CG_NA - 1], rm) * (1 + host_bg(c, c->h_z, 0, c->h_z[CG_NA - 1], rm));
    t[i] = (float)(2 * pg * dr);
    t[nr + i] = (float)(rm * pg * dr);
    t[2 * nr + i] = (float)(host_bg(c, c->h_v1, c->h_v1[0], c->h_v1[CG_NA - 1], rm) * fv);
  }
  CUDA_TRY(c, cudaMemcpyAsync(c->d_losfac, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream)); /* host staging vector */
  c->losnr = nr;
  c->losgen = c->tab_gen;
  return CG_OK;
}

/* async: inside a captured sequence, the source total read on the device
 * (the catalogue's capacity bounds the launch). */
static int srcs_los_run(cg_ctx *c, int ip, bool async)
{
  Cat &K = c->cat[ip];
  const bool lens = c->cfg.lensing_srcs[ip] != 0, skw = c->cfg.skw_srcs[ip] != 0;
  if (!lens && !skw) return CG_OK;
  int rc;
  if ((rc = los_tables(c))) return rc;
  const int nr = c->losnr;
  cg_los_params q;
  memset(&q, 0, sizeof(q));
  q.box = c->box;
  q.g = c->g;
  q.d1 = c->d1;
  q.pos = K.pos;
  q.src = K.src;
  q.nsrc = async ? K.cap : K.n;
  q.nsrc_dev = async ? c->d_total + ip : nullptr;
  q.nr = nr;
  q.dr = (float)(c->cfg.r_max / nr);
  q.idr = (float)(nr / c->cfg.r_max);
  q.lfac = c->d_losfac;
  q.vfac = c->d_losfac + 2 * (size_t)nr;
  q.skw_gauss = c->cfg.skw_gauss[ip];
  q.sigma2 = c->d_s2f;
  if (lens && q.nsrc > 0) {
    ProfScope ps(c, "srcs_lensing");
    CUDA_TRY(c, cg_srcs_lensing(c->stream, c->d_npot, &q, c->nsm));
    c->launches++;
  }
  if (skw) {
    /* room for the catalogue's capacity, so that a captured sequence fits */
    if (async && K.skw_cap < K.cap) return fail(c, CG_ESTATE, "skewers of population %d not sized before the capture", ip);
    if (K.n > K.skw_cap || K.cap > K.skw_cap) {
      const long long cap = std::max(K.n + K.n / 8 + 64, K.cap);
      if ((rc = dalloc(c, &K.skw_d, (size_t)cap * nr)) || (rc = dalloc(c, &K.skw_v, (size_t)cap * nr))) {
        K.skw_cap = 0;
        return rc;
      }
      K.skw_cap = cap;
    }
    q.skw_d = K.skw_d;
    q.skw_v = K.skw_v;
    if (q.nsrc > 0) {
      ProfScope ps(c, "srcs_skewers");
      CUDA_TRY(c, cg_srcs_skewers(c->stream, c->d_dens, c->d_npot, &q, c->nsm));
      c->launches++;
    }
    K.skw_n = async ? -2 : K.n; /* -2: for the device total */
  }
  return CG_OK;
}

/* Final catalogues to registered host buffers (the counts are current:
 * cg_get_beam_properties reads them first). */
static int out_catalogs(cg_ctx *c)
{
  for (int ip = 0; ip < c->cfg.n_srcs; ip++) {
    if (!c->h_src[ip]) continue;
    const Cat &K = c->cat[ip];
    const long long k = std::min(K.n, c->h_cap[ip]);
    *c->h_n[ip] = K.n;
    if (k <= 0) continue;
    if (int rc = out_begin(c)) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->h_src[ip], K.src, (size_t)k * 9 * sizeof(float), cudaMemcpyDeviceToHost,
                                c->ostream));
    if (int rc = out_end(c, 0)) return rc;
  }
  return CG_OK;
}

/* The beam stage (beaming.c:293-374).  async: inside a captured sequence --
 * source totals stay on the device, no host outputs. */
/* The per-source half of the beam stage (beaming.c:293-374): RSD, lensing
 * and skewers at the sources, then (plain runs) the catalogues to the host.
 * The reference computes the beam quantities last; the passes are
 * independent of the maps, so the mock sequence runs them before the
 * intensity and convergence maps and the catalogues cross the host link
 * while the maps are computed. */
static int beam_srcs(cg_ctx *c, bool async)
{
  if (!async) {
    if (int rc = refresh_counts(c)) return rc;
    if (!c->cfg.need_beaming) return out_catalogs(c); /* beaming.c:296-299 */
  } else if (!c->cfg.need_beaming) {
    return CG_OK;
  }
  if (!c->have_fields) return fail(c, CG_ESTATE, "fields not created");
  cudaSetDevice(c->device);
  if (!async) {
    out_join(c, 0); /* RSD and lensing columns are rewritten */
    out_join(c, 2);
  }
  if (c->cfg.n_srcs > 0) {
    if (!c->have_srcs) return fail(c, CG_ESTATE, "srcs_set_cartesian first");
    for (int ip = 0; ip < c->cfg.n_srcs; ip++) {
      cg_srcs_params p;
      srcs_params(c, ip, p);
      const long long n = async ? c->cat[ip].cap : c->cat[ip].n;
      ProfScope ps(c, "srcs_beam_rsd");
      CUDA_TRY(c, cg_srcs_beam_rsd(c->stream, c->d_npot, &p, n, async ? c->d_total + ip : nullptr, c->nsm));
      if (n > 0) c->launches++;
      if (int rc = srcs_los_run(c, ip, async)) return rc;
    }
    if (!async)
      if (int rc = out_catalogs(c)) return rc;
  }
  return CG_OK;
}

/* The map half of the beam stage: convergence (and its host copy), ISW and
 * custom maps. */
static int beam_maps(cg_ctx *c, bool async)
{
  if (!c->cfg.need_beaming) return CG_OK;
  if (!c->have_fields) return fail(c, CG_ESTATE, "fields not created");
  cudaSetDevice(c->device);
  if (c->cfg.do_kappa) {
    if (int rc = kappa_run(c)) return rc;
    if (!async && c->h_kappa) {
      if (int rc = out_begin(c)) return rc;
      CUDA_TRY(c, cudaMemcpyAsync(c->h_kappa, c->d_kmap, (size_t)c->kpl * c->knpix * sizeof(float),
                                  cudaMemcpyDeviceToHost, c->ostream));
      if (int rc = out_end(c, 2)) return rc;
    }
  }
  if (c->cfg.do_isw)
    if (int rc = isw_run(c)) return rc;
  if (c->cfg.n_cstm > 0)
    if (int rc = cstm_run(c)) return rc;
  return CG_OK;
}

static int beam_run(cg_ctx *c, bool async)
{
  if (int rc = beam_srcs(c, async)) return rc;
  return beam_maps(c, async);
}

extern "C" int cg_get_beam_properties(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  return beam_run(c, false);
}

extern "C" int cg_set_host_catalog(cg_ctx *c, int ipop, float *src9, long long cap, long long *n_out)
{
  if (!c || ipop < 0 || ipop >= c->cfg.n_srcs) return CG_EINVAL;
  cudaSetDevice(c->device);
  out_wait_all(c);
  if (!src9) {
    c->h_src[ipop] = nullptr;
    return CG_OK;
  }
  if (cap < 0 || !n_out) return CG_EINVAL;
  void *a = nullptr;
  if (int rc = host_view(c, src9, &a)) return rc;
  c->h_src[ipop] = src9;
  c->h_n[ipop] = n_out;
  c->h_cap[ipop] = cap;
  return CG_OK;
}

extern "C" int cg_set_host_imap(cg_ctx *c, int ipop, float *map)
{
  if (!c || ipop < 0 || ipop >= c->cfg.n_imap) return CG_EINVAL;
  cudaSetDevice(c->device);
  out_wait_all(c);
  void *a = nullptr;
  if (map)
    if (int rc = host_view(c, map, &a)) return rc;
  c->h_imap[ipop] = map;
  return CG_OK;
}

extern "C" int cg_set_host_kappa(cg_ctx *c, float *map)
{
  if (!c || (map && !c->cfg.do_kappa)) return CG_EINVAL;
  cudaSetDevice(c->device);
  out_wait_all(c);
  void *a = nullptr;
  if (map)
    if (int rc = host_view(c, map, &a)) return rc;
  c->h_kappa = map;
  return CG_OK;
}

extern "C" int cg_run_mock(cg_ctx *c)
{
  int rc;
  if ((rc = cg_create_cartesian_fields(c))) return rc;
  if ((rc = cg_compute_physical_density_field(c))) return rc;
  if ((rc = cg_compute_density_normalization(c))) return rc;
  if ((rc = cg_srcs_set_cartesian(c, nullptr))) return rc;
  /* the sources' beam quantities before the maps (beam_srcs) */
  if ((rc = beam_srcs(c, false))) return rc;
  if ((rc = cg_imap_set_cartesian(c))) return rc;
  return beam_maps(c, false);
}

/* ------------------------------------------------------------------------ */
/* graph-captured sequence and batches of realisations                      */
/* ------------------------------------------------------------------------ */
/* The whole sequence without host round trips: fields, density,
 * normalisation tables, sources (totals left on the device), intensity maps
 * and the beam stage (per-source quantities bounded by the catalogue's
 * capacity and reading the totals on the device; convergence, ISW and custom
 * maps).  Stage tables are built by the plain run that precedes a capture. */
static int run_mock_async(cg_ctx *c)
{
  int rc;
  if ((rc = cg_create_cartesian_fields(c))) return rc;
  if ((rc = cg_compute_physical_density_field(c))) return rc;
  if ((rc = cg_compute_density_normalization(c))) return rc;
  if ((rc = srcs_run(c, nullptr, false))) return rc;
  if ((rc = beam_srcs(c, true))) return rc;
  if (c->cfg.n_imap > 0 && (rc = imap_run(c, false))) return rc;
  return beam_maps(c, true);
}

extern "C" int cg_graph_capture(cg_ctx *c)
{
  if (!c) return CG_EINVAL;
  if (c->profiling) return fail(c, CG_EINVAL, "switch profiling off before capturing");
  cudaSetDevice(c->device);
  graph_free(c);
  /* one plain run sizes every buffer (the catalogue with slack); the
   * captured sequence allocates nothing */
  int rc = cg_run_mock(c);
  if (!rc) rc = cg_sync(c);
  if (rc) return rc;
  const long long l0 = c->launches;
  CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  rc = run_mock_async(c);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    for (int ip = 0; ip < c->cfg.n_srcs; ip++) c->cat[ip].n = -1;
    return rc ? rc : fail(c, CG_ECUDA, "stream capture: %s", cudaGetErrorString(e));
  }
  c->graph_launches = c->launches - l0;
  c->launches = l0;
  c->graph = g;
  CUDA_TRY(c, cudaGraphInstantiate(&c->gexec, g, 0));
  if (!c->graph_done) CUDA_TRY(c, cudaEventCreateWithFlags(&c->graph_done, cudaEventDisableTiming));
  /* nothing ran during the capture: the totals on the device are the plain
   * run's, read again on demand */
  return CG_OK;
}

extern "C" int cg_graph_launch(cg_ctx *c, void *stream)
{
  if (!c) return CG_EINVAL;
  if (!c->gexec) return fail(c, CG_ESTATE, "cg_graph_capture first");
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  CUDA_TRY(c, cudaGraphLaunch(c->gexec, s));
  CUDA_TRY(c, cudaEventRecord(c->graph_done, s));
  if (s != c->stream) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->graph_done, 0));
  c->launches += c->graph_launches;
  for (int ip = 0; ip < c->cfg.n_srcs; ip++) c->cat[ip].n = -1;
  c->have_fields = c->have_density = c->have_norm = c->have_srcs = 1;
  c->pending_mode = CG_DMODE_NONE;
  return CG_OK;
}

struct cg_batch {
  int device = 0, n = 0, nstreams = 0;
  std::vector<cg_ctx *> ctx;
  std::vector<int> order; /* largest grids first */
  std::vector<cudaStream_t> streams;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> joins;
  std::vector<float> tune_ms; /* autotuner: time per stream count tried */
  /* cg_batch_set_host_catalog: per realisation, the population whose Src
   * array each pass copies to pinned host memory (-1: none), the destination,
   * the count slot and the destination's size */
  std::vector<int> out_pop;
  std::vector<float *> out_src;
  std::vector<long long *> out_n;
  std::vector<long long> out_cap;
  char err[1024] = {0};
};

static int batch_fail(cg_batch *b, int code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(b->err, sizeof(b->err), fmt, ap);
  va_end(ap);
  return code;
}

static int batch_set_streams(cg_batch *b, int ns)
{
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  b->streams.assign(ns, nullptr);
  b->joins.assign(ns, nullptr);
  for (int k = 0; k < ns; k++) {
    if (cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming) != cudaSuccess)
      return batch_fail(b, CG_ECUDA, "stream or event creation failed");
  }
  b->nstreams = ns;
  return CG_OK;
}

/* One pass over every realisation: graph launches dealt round-robin, largest
 * grid first, over the batch's streams, joined on the first. */
static int batch_pass(cg_batch *b, float *ms)
{
  cudaStream_t s0 = b->streams[0];
  if (cudaEventRecord(b->t0, s0) != cudaSuccess) return batch_fail(b, CG_ECUDA, "event record");
  for (int k = 1; k < b->nstreams; k++) cudaStreamWaitEvent(b->streams[k], b->t0, 0);
  for (size_t j = 0; j < b->order.size(); j++) {
    const int i = b->order[j];
    cg_ctx *c = b->ctx[i];
    cudaStream_t st = b->streams[j % b->nstreams];
    if (int rc = cg_graph_launch(c, st)) return batch_fail(b, rc, "realisation %d: %s", i, c->err);
    /* the catalogue goes to the host behind the graph on its stream, while
     * the other streams compute */
    const int ip = b->out_pop.empty() ? -1 : b->out_pop[i];
    if (ip >= 0) {
      /* copy-engine transfers (no SM taken from the other graphs): the count,
       * and the catalogue up to the smaller of the two capacities, since the
       * count is only known on the device */
      const Cat &K = c->cat[ip];
      const long long k = std::min(K.cap, b->out_cap[i]);
      if (cudaMemcpyAsync(b->out_n[i], c->d_total + ip, sizeof(long long), cudaMemcpyDeviceToHost, st) !=
              cudaSuccess ||
          (k > 0 && cudaMemcpyAsync(b->out_src[i], K.src, (size_t)k * 9 * sizeof(float), cudaMemcpyDeviceToHost, st) !=
                        cudaSuccess))
        return batch_fail(b, CG_ECUDA, "realisation %d: catalogue copy", i);
    }
  }
  for (int k = 1; k < b->nstreams; k++) {
    cudaEventRecord(b->joins[k], b->streams[k]);
    cudaStreamWaitEvent(s0, b->joins[k], 0);
  }
  cudaEventRecord(b->t1, s0);
  if (cudaEventSynchronize(b->t1) != cudaSuccess) return batch_fail(b, CG_ECUDA, "batch synchronisation");
  if (ms) cudaEventElapsedTime(ms, b->t0, b->t1);
  return CG_OK;
}

extern "C" int cg_batch_create(cg_batch **out, int n, const cg_config *cfgs, int device, int nstreams)
{
  if (!out || n < 1 || !cfgs || nstreams < 0 || nstreams > 64) return CG_EINVAL;
  *out = nullptr;
  cg_batch *b = new cg_batch;
  b->device = device;
  b->n = n;
  *out = b;
  if (cudaSetDevice(device) != cudaSuccess) return batch_fail(b, CG_ECUDA, "cudaSetDevice(%d)", device);
  b->ctx.assign(n, nullptr);
  for (int i = 0; i < n; i++) {
    int rc = cg_create(&b->ctx[i], &cfgs[i], device);
    if (!rc) rc = cg_graph_capture(b->ctx[i]);
    if (rc) return batch_fail(b, rc, "realisation %d: %s", i, b->ctx[i] ? b->ctx[i]->err : "cg_create failed");
  }
  b->order.resize(n);
  for (int i = 0; i < n; i++) b->order[i] = i;
  std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) { return b->ctx[a]->N > b->ctx[c]->N; });
  if (cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess)
    return batch_fail(b, CG_ECUDA, "event creation");
  if (nstreams > 0) return batch_set_streams(b, nstreams);
  /* autotune the stream count: one warm pass, then the best of two timed
   * passes per candidate */
  const int cand[] = {1, 2, 4, 8, 16};
  int best = 1;
  float best_ms = 1e30f;
  for (int ns : cand) {
    if (int rc = batch_set_streams(b, ns)) return rc;
    float t = 0, tmin = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
      if (int rc = batch_pass(b, &t)) return rc;
      if (rep > 0) tmin = std::min(tmin, t);
    }
    b->tune_ms.push_back(tmin);
    if (tmin < best_ms) {
      best_ms = tmin;
      best = ns;
    }
  }
  return batch_set_streams(b, best);
}

extern "C" int cg_batch_run(cg_batch *b, float *ms)
{
  if (!b || b->nstreams < 1) return CG_EINVAL;
  cudaSetDevice(b->device);
  return batch_pass(b, ms);
}

extern "C" int cg_batch_set_host_catalog(cg_batch *b, int i, int ipop, float *src9, long long cap, long long *n_out)
{
  if (!b || i < 0 || i >= b->n) return CG_EINVAL;
  if (b->out_pop.empty()) {
    b->out_pop.assign(b->n, -1);
    b->out_src.assign(b->n, nullptr);
    b->out_n.assign(b->n, nullptr);
    b->out_cap.assign(b->n, 0);
  }
  if (!src9) { /* unregister */
    b->out_pop[i] = -1;
    return CG_OK;
  }
  cg_ctx *c = b->ctx[i];
  if (ipop < 0 || ipop >= c->cfg.n_srcs || cap < 0 || !n_out) return CG_EINVAL;
  if (!c->d_total || !c->gexec)
    return batch_fail(b, CG_ESTATE, "realisation %d: no captured source stage", i);
  cudaSetDevice(b->device);
  /* both ends must be page-locked, or the copies would not be asynchronous */
  const void *hp[2] = {src9, n_out};
  for (int k = 0; k < 2; k++) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, hp[k]) != cudaSuccess || a.type != cudaMemoryTypeHost) {
      cudaGetLastError();
      return batch_fail(b, CG_EINVAL, "realisation %d: host catalogue buffers must be pinned (cudaHostAlloc)", i);
    }
  }
  b->out_pop[i] = ipop;
  b->out_src[i] = src9;
  b->out_n[i] = n_out;
  b->out_cap[i] = cap;
  return CG_OK;
}

extern "C" int cg_batch_streams(const cg_batch *b) { return b ? b->nstreams : -1; }

extern "C" int cg_batch_tuning(const cg_batch *b, float *ms, int cap)
{
  if (!b) return -1;
  const int k = (int)b->tune_ms.size();
  for (int i = 0; i < k && i < cap && ms; i++) ms[i] = b->tune_ms[i];
  return k;
}

extern "C" cg_ctx *cg_batch_context(cg_batch *b, int i) { return (b && i >= 0 && i < b->n) ? b->ctx[i] : nullptr; }

extern "C" const char *cg_batch_last_error(const cg_batch *b) { return b ? b->err : "null batch"; }

extern "C" void cg_batch_destroy(cg_batch *b)
{
  if (!b) return;
  cudaSetDevice(b->device);
  for (cudaStream_t s : b->streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  for (cg_ctx *c : b->ctx) cg_destroy(c);
  delete b;
}

/* ------------------------------------------------------------------------ */
/* host mirrors                                                             */
/* ------------------------------------------------------------------------ */
static int apply_pending(cg_ctx *c)
{
  if (c->pending_mode == CG_DMODE_NONE) return CG_OK;
  /* the density transform on its own: a bins pass with no bins */
  cg_bins_params p;
  memset(&p, 0, sizeof(p));
  p.box = c->box;
  p.g = c->g;
  p.zt = c->zt;
  p.d1 = c->d1;
  p.mode = c->pending_mode;
  p.err = c->d_err;
  p.sigma2f = c->d_s2f;
  p.nz = 0;
  p.nt = 0;
  p.bias_model = c->cfg.bias_model;
  CUDA_TRY(c, cg_dens_bins(c->stream, c->d_dens, &p, c->nsm));
  c->launches++;
  c->pending_mode = CG_DMODE_NONE;
  return CG_OK;
}

extern "C" int cg_download_grid(cg_ctx *c, int which, void *dst)
{
  if (!c || !dst) return CG_EINVAL;
  float *src = nullptr;
  if (which == 0) {
    if (int rc = apply_pending(c)) return rc;
    src = c->d_dens;
  } else if (which == 1) src = c->d_npot;
  else if (which >= 2 && which <= 4) src = c->d_disp[which - 2];
  else if (which >= 5 && which <= 7) src = c->d_lpt2[which - 5];
  if (!src) return fail(c, CG_ESTATE, "grid %d not available", which);
  CUDA_TRY(c, cudaMemcpyAsync(dst, src, c->grid_floats * sizeof(float), cudaMemcpyDefault, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_catalog(cg_ctx *c, int ipop, float *pos4, int *ipix, float *src9)
{
  if (!c || ipop < 0 || ipop >= c->cfg.n_srcs) return CG_EINVAL;
  if (int rc = refresh_counts(c)) return rc;
  const Cat &K = c->cat[ipop];
  if (K.n > 0) {
    if (pos4) CUDA_TRY(c, cudaMemcpyAsync(pos4, K.pos, K.n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    if (ipix) CUDA_TRY(c, cudaMemcpyAsync(ipix, K.ipix, K.n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (src9) CUDA_TRY(c, cudaMemcpyAsync(src9, K.src, K.n * 9 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_skewers(cg_ctx *c, int ipop, float *dens, float *vel)
{
  if (!c || ipop < 0 || ipop >= c->cfg.n_srcs) return CG_EINVAL;
  if (int rc = refresh_counts(c)) return rc;
  const Cat &K = c->cat[ipop];
  if (!c->cfg.skw_srcs[ipop]) return fail(c, CG_ESTATE, "population %d stores no skewers", ipop);
  if (K.skw_n != K.n && K.skw_n != -2) return fail(c, CG_ESTATE, "skewers of population %d not computed", ipop);
  const size_t m = (size_t)K.n * c->losnr;
  if (m) {
    if (dens) CUDA_TRY(c, cudaMemcpyAsync(dens, K.skw_d, m * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (vel) CUDA_TRY(c, cudaMemcpyAsync(vel, K.skw_v, m * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_count_map(cg_ctx *c, int ipop, int *counts)
{
  if (!c || !counts || ipop < 0 || ipop >= c->cfg.n_srcs) return CG_EINVAL;
  if (int rc = refresh_counts(c)) return rc;
  const Cat &K = c->cat[ipop];
  if (!K.cmap) return fail(c, CG_ESTATE, "no count map for population %d", ipop);
  CUDA_TRY(c, cudaMemcpyAsync(counts, K.cmap, K.cmap_npix * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}


extern "C" int cg_download_imap(cg_ctx *c, int ipop, float *map, int *nadd)
{
  if (!c || ipop < 0 || ipop >= c->cfg.n_imap) return CG_EINVAL;
  const Imap &M = c->im[ipop];
  if (!M.data) return fail(c, CG_ESTATE, "intensity map %d not painted", ipop);
  const long long m = (long long)M.nr * M.npix;
  if (map) {
    if (c->tmpmap_n < (size_t)m) {
      if (int rc = dalloc(c, &c->d_tmpmap, (size_t)m)) return rc;
      c->tmpmap_n = m;
    }
    /* write_imap, io.c:738-741: data/nadd where nadd > 0 */
    k_div_nadd<<<(unsigned)std::min<long long>((m + 255) / 256, (long long)c->nsm * 16), 256, 0, c->stream>>>(
        M.data, M.nadd, c->d_tmpmap, m);
    CUDA_TRY(c, cudaGetLastError());
    c->launches++;
    CUDA_TRY(c, cudaMemcpyAsync(map, c->d_tmpmap, m * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  if (nadd) CUDA_TRY(c, cudaMemcpyAsync(nadd, M.nadd, m * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_custom(cg_ctx *c, int ipop, float *map)
{
  if (!c || !map || ipop < 0 || ipop >= c->cfg.n_cstm) return CG_EINVAL;
  if (!c->d_cmap[ipop]) return fail(c, CG_ESTATE, "custom map %d not computed", ipop);
  CUDA_TRY(c, cudaMemcpyAsync(map, c->d_cmap[ipop], (size_t)c->cnpix[ipop] * sizeof(float), cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_isw(cg_ctx *c, float *map)
{
  if (!c || !map) return CG_EINVAL;
  if (!c->d_imap_isw) return fail(c, CG_ESTATE, "ISW maps not computed");
  CUDA_TRY(c, cudaMemcpyAsync(map, c->d_imap_isw, (size_t)c->ipl * c->inpix * sizeof(float), cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_kappa(cg_ctx *c, float *map)
{
  if (!c || !map) return CG_EINVAL;
  if (!c->d_kmap) return fail(c, CG_ESTATE, "kappa not computed");
  CUDA_TRY(c, cudaMemcpyAsync(map, c->d_kmap, (size_t)c->kpl * c->knpix * sizeof(float), cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int cg_download_norm(cg_ctx *c, int kind, int ipop, float *tab, float *edges)
{
  if (!c || !tab || !edges) return CG_EINVAL;
  const Tab *t = nullptr;
  if (kind == 0 && ipop >= 0 && ipop < c->cfg.n_srcs) t = &c->norm[ipop];
  if (kind == 1 && ipop >= 0 && ipop < c->cfg.n_imap) t = &c->normi[ipop];
  if (kind == 2 && ipop >= 0 && ipop < c->cfg.n_cstm) t = &c->normc[ipop];
  if (!t || !t->f) return fail(c, CG_EINVAL, "no normalisation table %d/%d", kind, ipop);
  float e[2];
  CUDA_TRY(c, cudaMemcpyAsync(tab, t->f, CG_NA * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(e, t->f + CG_NA, 2 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  edges[0] = e[0];
  edges[1] = e[1];
  return CG_OK;
}

extern "C" int cg_download_norm64(cg_ctx *c, int kind, int ipop, double *tab, double *edges)
{
  if (!c || !tab || !edges || !c->d_norm64) return CG_EINVAL;
  int t = -1;
  if (kind == 0 && ipop >= 0 && ipop < c->cfg.n_srcs) t = ipop;
  if (kind == 1 && ipop >= 0 && ipop < c->cfg.n_imap) t = c->cfg.n_srcs + ipop;
  if (kind == 2 && ipop >= 0 && ipop < c->cfg.n_cstm) t = c->cfg.n_srcs + c->cfg.n_imap + ipop;
  if (t < 0) return fail(c, CG_EINVAL, "no normalisation table %d/%d", kind, ipop);
  const double *src = c->d_norm64 + (size_t)t * (CG_NA + 2);
  CUDA_TRY(c, cudaMemcpyAsync(tab, src, CG_NA * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(edges, src + CG_NA, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return CG_OK;
}

extern "C" int cg_ring_pixels_checked(int device, int nside, const float *xyz, long long n, float ein,
                                      long long *pix)
{
  if (!xyz || !pix || n < 0 || nside < 1 || nside > 8192 || (nside & (nside - 1))) return CG_EINVAL;
  if (n == 0) return CG_OK;
  if (cudaSetDevice(device) != cudaSuccess) return CG_ECUDA;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  float *dx = nullptr;
  long long *dp = nullptr;
  int rc = CG_OK;
  if (cudaMalloc((void **)&dx, (size_t)n * 3 * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void **)&dp, (size_t)n * sizeof(long long)) != cudaSuccess) {
    rc = CG_ENOMEM;
  } else if (cudaMemcpy(dx, xyz, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
             cg_pix_checked_dev(0, nside, dx, n, ein, dp, nsm) != cudaSuccess ||
             cudaMemcpy(pix, dp, (size_t)n * sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess) {
    rc = CG_ECUDA;
  }
  if (dx) cudaFree(dx);
  if (dp) cudaFree(dp);
  cudaGetLastError();
  return rc;
}

extern "C" int cg_set_decisions_in_double(cg_ctx *c, int all)
{
  if (!c) return CG_EINVAL;
  graph_free(c); /* a captured graph holds the old setting */
  c->force_double = all ? 1 : 0;
  return CG_OK;
}

extern "C" int cg_exact_stats(cg_ctx *c, unsigned long long *out, int reset)
{
  if (!c || !c->d_xstats) return CG_EINVAL;
  if (out) {
    CUDA_TRY(c, cudaMemcpyAsync(out, c->d_xstats, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  if (reset) CUDA_TRY(c, cudaMemsetAsync(c->d_xstats, 0, 4 * sizeof(unsigned long long), c->stream));
  return CG_OK;
}

extern "C" int cg_set_profiling(cg_ctx *c, int on)
{
  if (!c) return CG_EINVAL;
  c->profiling = on;
  return CG_OK;
}

extern "C" int cg_kernel_times(cg_ctx *c, char *names, size_t names_len, float *ms, int cap, int *n)
{
  if (!c || !n) return CG_EINVAL;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  size_t off = 0;
  int k = 0;
  if (names && names_len) names[0] = 0;
  for (auto &e : c->evlog) {
    float t = 0;
    cudaEventElapsedTime(&t, e.a, e.b);
    if (k < cap) {
      if (ms) ms[k] = t;
      if (names) {
        int w = snprintf(names + off, names_len > off ? names_len - off : 0, "%s;", e.name);
        if (w > 0) off += (size_t)w;
      }
    }
    k++;
  }
  /* entries may share a boundary event: destroy once every time is read */
  for (auto &e : c->evlog) {
    if (e.own_a) cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  c->evlog.clear();
  *n = k;
  return CG_OK;
}
