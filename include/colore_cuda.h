/*
 * colore_cuda.h -- C ABI of libcolore_cuda.so, the sm_103a implementation
 * of CoLoRe's mock-generation path (Gaussian field -> lognormal/1LPT density
 * -> bias normalisation -> Poisson sources -> HEALPix sources, intensity and
 * convergence maps).
 *
 * One cg_ctx owns one GPU's grids, tables, catalogs and maps.  Every call is
 * enqueued on the context's CUDA stream and returns 0 on success or a
 * nonzero CG_E* status; cg_last_error() gives the message.  Device work
 * never traps: bounded loops set an error word that the next host
 * synchronisation turns into CG_EDEVICE.
 *
 * The stage entry points map one-to-one onto the reference's hot-path
 * functions (paths relative to the CoLoRe source tree):
 *
 *   cg_create_cartesian_fields        src/fourier.c:361  create_cartesian_fields
 *   cg_compute_physical_density_field src/density.c:1105 compute_physical_density_field
 *   cg_compute_density_normalization  src/density.c:1227 compute_density_normalization
 *   cg_srcs_set_cartesian             src/srcs.c:285     srcs_set_cartesian
 *                                     (+ src/srcs.c:375 srcs_distribute, an identity
 *                                      on one GPU, + src/srcs.c:418
 *                                      srcs_get_local_properties, fused)
 *   cg_imap_set_cartesian             src/imap.c:247     imap_set_cartesian
 *   cg_get_beam_properties            src/beaming.c:293  get_beam_properties
 *                                     (kappa: src/kappa.c:39,78; source RSD:
 *                                      src/srcs.c:445,627,739)
 *   cg_download_*                     host mirrors consumed by src/io.c writers
 *
 * Layouts at the boundary are the reference's: padded real grids
 * index = ix + 2(N/2+1)(iy + N iz) (src/fourier.c:46-51); catalogs as
 * CatalogCartesian (4 floats + 1 int per source, src/common.h:162-167) and
 * Src (9 floats, src/common.h:169-179); maps full-sky RING order.
 */
#ifndef COLORE_CUDA_H
#define COLORE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_OK 0
#define CG_EINVAL 1   /* bad argument or configuration            */
#define CG_ENOMEM 2   /* device or host allocation failed          */
#define CG_ECUDA 3    /* CUDA runtime / library error              */
#define CG_EDEVICE 4  /* a kernel reported an error through its flag */
#define CG_ESTATE 5   /* stage called out of order                 */

#define CG_PREC_F32 0 /* FP32 fields and per-cell math, FP64 reductions */
#define CG_PREC_F64 1 /* plain FP64 path: cuFFT Z2D + unfused FP64 kernels */

#define CG_NPOP_MAX 10      /* NPOP_MAX, src/common.h:133    */
#define CG_NPLANES_MAX 100  /* NPLANES_MAX, src/common.h:134 */
#define CG_NA 5001          /* NA, src/common.h:132          */

/* dens_type values, src/common.h:115-118 */
#define CG_DENS_LGNR 0
#define CG_DENS_1LPT 1
#define CG_DENS_2LPT 2
#define CG_DENS_CLIP 3

/* bias models, src/common.h:414-431 */
#define CG_BIAS_MODEL_POW 1    /* (1+d)^b, built without flags      */
#define CG_BIAS_MODEL_EXPLIN 2 /* -D_BIAS_MODEL_2 (Makefile default) */
#define CG_BIAS_MODEL_LIN 3    /* -D_BIAS_MODEL_3                    */

/*
 * Everything the hot path reads from ParamCoLoRe (src/common.h:220-381).
 * Tables are host arrays in double precision, copied by cg_upload_tables.
 */
typedef struct {
  int precision;           /* CG_PREC_*                                    */
  int n_grid;              /* N                                            */
  double l_box;            /* box side [Mpc/h], src/cosmo.c:544            */
  double pos_obs[3];       /* observer, src/cosmo.c:545-547                */
  uint64_t seed;           /* seed_rng                                     */
  /* cosmology scalars */
  double omega_m, hubble_0, fgrowth_0, prefac_lensing, r_max;
  /* field options */
  double r2_smooth;        /* squared smoothing length (src/io.c:453-458)  */
  int do_smoothing, smooth_potential, dens_type, bias_model;
  /* P(k): uniform in log10 k, already sigma8-normalised (src/cosmo.c:444-495) */
  int numk;
  double logkmin, logkmax, idlogk, n_scal;
  const double *pkarr;
  /* background on the r-uniform grid r_i = i/glob_idr, CG_NA entries
   * (src/cosmo.c:668-717), and the a-uniform r(a) table (src/cosmo.c:669-674) */
  double glob_idr;
  const double *r_arr_r2z, *z_arr_r2z, *growth_d_arr, *growth_d2_arr, *growth_v_arr,
      *growth_pd_arr, *ihub_arr;
  const double *a_arr_a2r, *r_arr_a2r;
  /* galaxy populations */
  int n_srcs;
  const double *srcs_nz_arr[CG_NPOP_MAX];
  const double *srcs_bz_arr[CG_NPOP_MAX];
  int nside_base;                  /* src/io.c:224-244 (2 on one GPU)      */
  int nside_count[CG_NPOP_MAX];    /* source count map resolution, 0 = off */
  /* intensity-mapping species */
  int n_imap;
  const double *imap_tz_arr[CG_NPOP_MAX];
  const double *imap_bz_arr[CG_NPOP_MAX];
  int nside_imap[CG_NPOP_MAX];
  int imap_nr[CG_NPOP_MAX];
  const double *imap_r0[CG_NPOP_MAX]; /* shell edges, any order (sorted here) */
  const double *imap_rf[CG_NPOP_MAX];
  /* convergence */
  int do_kappa, n_kappa, nside_kappa;
  double kappa_r[CG_NPLANES_MAX]; /* source-plane comoving distances */
  /* need_beaming, src/io.c:460-461 */
  int need_beaming;
  /* integrated Sachs-Wolfe maps (isw.c:78-147), planes as kappa's */
  int do_isw, n_isw, nside_isw;
  double isw_r[CG_NPLANES_MAX]; /* plane comoving distances (cosmo.c:839-845) */
  /* mass assignment of the 1LPT particles (density.c:178-187): 0 NGP,
   * 1 CIC (the reference's default, io.c:66), 2 TSC */
  int lpt_interp_type;
  /* custom maps (cstm.c:68-145): kernel K(z) and bias b(z) on the r grid
   * (cosmo.c:631-716), HEALPix resolution */
  int n_cstm;
  const double *cstm_kz_arr[CG_NPOP_MAX];
  const double *cstm_bz_arr[CG_NPOP_MAX];
  int nside_cstm[CG_NPOP_MAX];
  /* per source population: line-of-sight lensing (include_lensing), skewers
   * (store_skewers) and Gaussian rather than density skewers
   * (gaussian_skewers), src/io.c:331-339 */
  int lensing_srcs[CG_NPOP_MAX];
  int skw_srcs[CG_NPOP_MAX];
  int skw_gauss[CG_NPOP_MAX];
} cg_config;

typedef struct cg_ctx cg_ctx;

/* Lifetime ---------------------------------------------------------------- */
int cg_create(cg_ctx **out, const cg_config *cfg, int device);
void cg_destroy(cg_ctx *ctx);
const char *cg_last_error(const cg_ctx *ctx);
int cg_set_stream(cg_ctx *ctx, void *cuda_stream); /* NULL = context's own */
int cg_sync(cg_ctx *ctx);
/* Bytes of device memory the context would hold for cfg (get_max_memory,
 * src/common.c:571-750). */
int cg_memory_estimate(const cg_config *cfg, unsigned long long *bytes);

/* Upload (or re-upload) every table of cfg (same geometry as at create). */
int cg_upload_tables(cg_ctx *ctx, const cg_config *cfg);

/* Stages ------------------------------------------------------------------ */
int cg_create_cartesian_fields(cg_ctx *ctx);
int cg_get_sigma2(cg_ctx *ctx, double *sigma2_gauss, double *mean_gauss);
int cg_compute_physical_density_field(cg_ctx *ctx);
int cg_compute_density_normalization(cg_ctx *ctx);
/* Device half of compute_density_normalization (density.c:1128-1211):
 * per-redshift-bin cell counts, summed redshifts and summed bias_model per
 * tracer.  Arrays have nz entries; norm arrays are [n_srcs][nz] and
 * [n_imap + n_cstm][nz]: the intensity species, then the custom maps
 * (norm_cstm_arr, src/density.c:1178), in one block. */
int cg_collect_density_normalization(cg_ctx *ctx, int nz, double idz, double *zarr,
                                     unsigned long long *narr, double *norm_srcs,
                                     double *norm_imap);
/* Allocation-free variant of cg_collect_density_normalization (no
 * counterpart in the reference): same arguments and results, for callers
 * that may not allocate while the pipeline runs (a fixed memory budget, a
 * pool that must not grow).  Its per-bin scratch is a fixed 224 KiB
 * module-scope device array rather than cudaMalloc'd buffers, so
 *  - nz is limited to 2..1024 bins (CG_EINVAL beyond, with a message);
 *  - the first call on each device looks up that array's address with the
 *    device current; make that first call before any stream capture;
 *  - that address is kept for the life of the process: it belongs to the
 *    device's primary context and goes stale if the host calls
 *    cudaDeviceReset and then keeps using the library;
 *  - calls that overlap on the GPU (two contexts on one device, or the
 *    same context on two streams) share the array and race.
 * The sums are zeroed on the context's stream at every call.  With
 * profiling switched on (cg_set_profiling, off by default) the call logs a
 * CUDA event pair around its kernel, as every stage does. */
int cg_collect_density_normalization_static(cg_ctx *ctx, int nz, double idz, double *zarr,
                                            unsigned long long *narr, double *norm_srcs,
                                            double *norm_imap);
/* Replace the NA-point normalisation tables (src/density.c:1323-1355).
 * srcs_*: [n_srcs] tables; imap_*: [n_imap + n_cstm] tables, the intensity
 * species then the custom maps; *_0f: (below, above) edge pairs. */
int cg_set_norm_tables(cg_ctx *ctx, const double *srcs_norm, const double *srcs_norm_0f,
                       const double *imap_norm, const double *imap_norm_0f);
int cg_srcs_set_cartesian(cg_ctx *ctx, long long *nsrc_per_pop);
int cg_imap_set_cartesian(cg_ctx *ctx);
/* Sub-samples (cells x nsub^3, imap.c:158-231) painted for species ipop by
 * the last cg_imap_set_cartesian. */
int cg_imap_samples(cg_ctx *ctx, int ipop, unsigned long long *n);
/* Upper bound on the intensity-map cell list (no counterpart in the
 * reference, whose loop paints each cell as it goes; 0, the default: every
 * cell inside the shells' outer radius, up to a quarter of the free device
 * memory).  Cells past the bound are painted by the listing kernel itself;
 * the maps are the same either way. */
int cg_set_imap_list_cap(cg_ctx *ctx, long long cap);
int cg_get_beam_properties(cg_ctx *ctx);

/* Host outputs (no counterpart in the reference, whose writers read host
 * arrays the run filled).  Each call registers page-locked host memory
 * (cudaHostAlloc) that the stages fill as the output becomes final, on a
 * copy stream that overlaps the stages still to run: the maps of species
 * ipop (nr x 12 nside^2 floats, RING, data/nadd as cg_download_imap gives)
 * after cg_imap_set_cartesian; the Src array of population ipop (cap
 * sources, 9 floats each; *n_out receives the source count, more than cap
 * when the buffer was short) and the convergence maps (as cg_download_kappa
 * gives) during cg_get_beam_properties.  The data are valid after cg_sync.
 * A registered map costs a device staging buffer of its size (data/nadd is
 * formed there for the copy), beyond cg_memory_estimate.  NULL stops the
 * copies. */
int cg_set_host_catalog(cg_ctx *ctx, int ipop, float *src9, long long cap, long long *n_out);
int cg_set_host_imap(cg_ctx *ctx, int ipop, float *map);
int cg_set_host_kappa(cg_ctx *ctx, float *map);
/* Run the whole driver sequence of src/main.c:66-125 in one call.  The
 * sources' beam quantities (RSD, lensing, skewers) run right after the
 * sources and before the intensity and convergence maps, on which they do
 * not depend, so that a registered host catalogue is copied while the maps
 * are computed; the outputs are those of the reference's order. */
int cg_run_mock(cg_ctx *ctx);

/* Graph-captured sequence (no counterpart in the reference; the batching
 * pattern of the GPU path).  cg_graph_capture runs the sequence once to size
 * every buffer and build the stage tables, then captures the whole sequence
 * -- fields, density, normalisation, sources, intensity maps and the beam
 * stage -- into a CUDA graph.  cg_graph_launch replays it on a stream (NULL:
 * the context's); the source totals and the intensity maps' sample counts
 * stay on the device until a download, cg_num_sources or cg_imap_samples
 * reads them, and a total that outgrew the catalogue is reported there
 * (CG_EDEVICE).  Replays deliver nothing to registered host buffers
 * (cg_set_host_*): download after cg_sync.  Replays repeat the captured
 * realisation: change the seed with cg_upload_tables and capture again. */
int cg_graph_capture(cg_ctx *ctx);
int cg_graph_launch(cg_ctx *ctx, void *cuda_stream);

/* Batches of independent realisations (no counterpart in the reference):
 * one context and captured graph per configuration, the graphs dealt over
 * nstreams streams (largest grids first) so that small grids run side by
 * side.  nstreams = 0 autotunes the stream count (1, 2, 4, 8 or 16) by
 * timing whole passes.  cg_batch_run runs every realisation once and
 * reports the device time of the pass; cg_batch_context gives the context
 * of realisation i for the download calls.  The configurations' tables must
 * outlive the batch. */
typedef struct cg_batch cg_batch;
int cg_batch_create(cg_batch **out, int n, const cg_config *cfgs, int device, int nstreams);
int cg_batch_run(cg_batch *b, float *ms);
int cg_batch_streams(const cg_batch *b);
/* stream-count autotuning: the pass time of each candidate, in order */
int cg_batch_tuning(const cg_batch *b, float *ms, int cap);
cg_ctx *cg_batch_context(cg_batch *b, int i);
/* Have every cg_batch_run copy realisation i's catalogue of population ipop
 * (its Src array, 9 floats per source) into src9 and its source count into
 * *n_out, behind the realisation's graph on the same stream, so the copies
 * overlap the other realisations' work and need no host synchronisation.
 * src9 (cap sources) and n_out must be page-locked host memory
 * (cudaHostAlloc).  The count is only known on the device, so the copy
 * moves min(cap, the catalogue's device capacity) records; those past
 * *n_out are unspecified, and when *n_out > cap only cap sources arrived.
 * src9 = NULL stops the copies for realisation i. */
int cg_batch_set_host_catalog(cg_batch *b, int i, int ipop, float *src9, long long cap, long long *n_out);
const char *cg_batch_last_error(const cg_batch *b);
void cg_batch_destroy(cg_batch *b);

/* Host mirrors -------------------------------------------------------------- */
/* which: 0 = density (grid_dens), 1 = potential (grid_npot), 2..4 = 1LPT
 * (first-order) displacement x,y,z, 5..7 = 2LPT second-order displacement
 * x,y,z.  dst holds N*N*2(N/2+1) values of the context's
 * precision (float or double), padded layout; it may be host or device
 * memory. */
int cg_download_grid(cg_ctx *ctx, int which, void *dst);
long long cg_num_sources(cg_ctx *ctx, int ipop);
/* pos4: 4 floats per source (x,y,z,dz_rsd) as CatalogCartesian.pos;
 * ipix: nside_base NEST id; src9: 9 floats per source as Src.  Any may be NULL. */
int cg_download_catalog(cg_ctx *ctx, int ipop, float *pos4, int *ipix, float *src9);
/* Counts of sources per RING pixel at nside_count[ipop]. */
int cg_download_count_map(cg_ctx *ctx, int ipop, int *counts);
/* Intensity map of species ipop: nr * 12 nside^2 values in RING order,
 * finalised as data/nadd where nadd > 0 (src/io.c:738-741); nadd may be NULL. */
int cg_download_imap(cg_ctx *ctx, int ipop, float *map, int *nadd);
/* Convergence maps: n_kappa * 12 nside^2 values, RING order (src/io.c:826-873). */
int cg_download_kappa(cg_ctx *ctx, float *map);
/* ISW maps: n_isw * 12 nside_isw^2 values, RING order (write_isw, src/io.c:946-1010). */
int cg_download_isw(cg_ctx *ctx, float *map);
/* Custom map ipop: 12 nside_cstm[ipop]^2 values in NEST order, the layout
 * write_cstm (src/io.c:754-800) puts in its file (it copies the shell data,
 * listed in NEST order by hp_shell_alloc, src/common.c:505-552, without
 * the nest-to-ring step of the kappa and ISW writers). */
int cg_download_custom(cg_ctx *ctx, int ipop, float *map);
/* Skewers of source population ipop (store_skewers; srcs.c:509-536 and the
 * velocity scaling of srcs_beams_postproc, srcs.c:725-733): nsrc x nr floats
 * each, catalogue order, nr = n_grid/2 steps of r_max/nr.  dens holds the
 * density contrast, or the Gaussian field with gaussian_skewers; vel the
 * radial velocity in units of redshift.  Steps beyond a source are 0.
 * Either pointer may be NULL. */
int cg_download_skewers(cg_ctx *ctx, int ipop, float *dens, float *vel);

/* FP32 normalisation table the kernels use: kind 0 = source population
 * ipop (srcs_norm_arr, src/common.h:318), 1 = intensity species
 * (imap_norm_arr, src/common.h:336), 2 = custom map (cstm_norm_arr,
 * src/cosmo.c:78-81).  tab: CG_NA floats; edges: the values
 * below and above the table (norm_*_0 / norm_*_f). */
int cg_download_norm(cg_ctx *ctx, int kind, int ipop, float *tab, float *edges);
/* The same table in double, as the double decisions read it
 * (compute_density_normalization keeps both, density.c:1323-1355). */
int cg_download_norm64(cg_ctx *ctx, int kind, int ipop, double *tab, double *edges);

/* Per-kernel timing: when on, every launch group is bracketed by CUDA
 * events on the context's stream; cg_kernel_times synchronises, returns the
 * groups in launch order (names ';'-separated, milliseconds) and clears the
 * log. */
int cg_set_profiling(cg_ctx *ctx, int on);

/* Integer outputs by the reference's double arithmetic (no counterpart in
 * the reference, which computes in double throughout): Poisson counts,
 * base and count-map pixels and intensity-map hits are decided in single
 * precision where a bound on the distance to the double value proves the
 * decision, and in double otherwise (intensity-map samples try float-float
 * arithmetic in between).  With all != 0 every such decision is taken in
 * double (slow; for checking).  cg_exact_stats reads the numbers of
 * decisions taken in double since the last reset: [0] cells' counts,
 * [1] source pixels, [2] intensity-map cells, [3] intensity-map samples. */
int cg_set_decisions_in_double(cg_ctx *ctx, int all);
/* The RING pixel decision of the intensity maps on its own, on device
 * `device`: pix[i] = he_ang2pix(nside, cos theta, phi) of direction
 * xyz[3i..3i+2] (host arrays) as the reference's double arithmetic decides
 * it, or -1 where the single-precision margin does not prove the decision
 * (the kernels then decide in double); ein bounds the coordinates' error
 * relative to |xyz|.  nside a power of two up to 8192. */
int cg_ring_pixels_checked(int device, int nside, const float *xyz, long long n, float ein, long long *pix);
int cg_exact_stats(cg_ctx *ctx, unsigned long long *out4, int reset);
int cg_kernel_times(cg_ctx *ctx, char *names, size_t names_len, float *ms, int cap, int *n);

/* Tile autotuner of the transform passes (no counterpart in the reference;
 * the reference plans with FFTW_ESTIMATE, src/fourier.c:84-91).  The first
 * time a grid size runs on a device, each pass -- pass 0 the fill + z of the
 * Gaussian field and potential, 1 the fill + z of the 1LPT displacements,
 * 2 the y columns, 3 the x rows -- is timed with each valid tile width (the
 * plan's, half, twice) on the context's grids and the fastest is kept for
 * the process.  Tile widths change only the block shape: results are the
 * same bits.  Environment COLORE_GB300_TUNE=0 keeps the plans' widths.
 * cg_set_field_variant forces variant v (0 plan, 1 half, 2 twice; -1 back to
 * the tuner) of one pass for this context; cg_field_plan writes the widths
 * in use and the timings as a JSON object. */
int cg_set_field_variant(cg_ctx *ctx, int pass, int v);
int cg_field_plan(cg_ctx *ctx, char *buf, size_t len);

/* Launch accounting: number of kernels this context has launched. */
long long cg_kernel_launches(const cg_ctx *ctx);

/* FP64 baseline (no counterpart in the reference) -------------------------
 * The same driver sequence (src/main.c:66-125) with plain double-precision
 * kernels, one thread per mode / cell / source / pixel, cuFFT transforms and
 * no fusion: the denominator of the FP32 path's speed-up on the same GPU.
 * Sources are written in an unspecified order. */
typedef struct cg64_ctx cg64_ctx;
int cg64_create(cg64_ctx **out, const cg_config *cfg, int device);
void cg64_destroy(cg64_ctx *ctx);
const char *cg64_last_error(const cg64_ctx *ctx);
/* Whole sequence; *ms (may be NULL) gets its device time from CUDA events. */
int cg64_run_mock(cg64_ctx *ctx, float *ms);
long long cg64_num_sources(const cg64_ctx *ctx, int ipop);
/* Gaussian field and potential only (create_cartesian_fields,
 * fourier.c:361-423); cg64_download 0 and 1 then give delta_G and phi. */
int cg64_create_cartesian_fields(cg64_ctx *ctx);
/* what: 0 density, 1 potential (N^3 doubles, [z][y][x]); 2 intensity-map
 * temperature sums and 3 hit counts (int) of species ipop (nr * npix, RING);
 * 4 convergence (n_kappa * npix doubles, RING); 5 normalisation table of
 * tracer ipop (CG_NA doubles; source populations first, then species);
 * 6 source count map of population ipop (12 nside_count^2 ints, RING).
 * dst of 0 and 1 may be host or device memory. */
int cg64_download(cg64_ctx *ctx, int what, int ipop, void *dst);

#ifdef __cplusplus
}
#endif

#endif /* COLORE_CUDA_H */
