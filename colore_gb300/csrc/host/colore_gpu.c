/*
 * colore_gpu.c -- command-line driver with the stage sequence of CoLoRe's
 * main() (main.c:24-154), running every hot-path stage on the GPU through
 * libcolore_cuda.so:
 *
 *   ./colore_gpu params.cfg            run and write outputs
 *   ./colore_gpu --test-memory params  print the memory plan and exit
 *
 * Outputs follow io.c through the writers of host_io.c: raw density grids
 * (write_density_grid, io.c:565-595), source catalogues in FITS or ASCII
 * (write_catalog, io.c:1069-1236) and HEALPix maps in FITS binary tables
 * (he_write_healpix_map, healpix_extra.c:4-57).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <math.h>

#include "colore_cuda.h"
#include "colore_host.h"

static double now_ms(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static double t_rel;
static void timer0(void) { t_rel = now_ms(); }
static void timer2(void)
{
  double t = now_ms();
  printf(">    Relative time ellapsed %.1lf ms\n", t - t_rel);
  t_rel = t;
}

static void die(cg_ctx *c, int rc, const char *what)
{
  fprintf(stderr, "MPI task 0, Fatal: %s failed (%d): %s\n", what, rc, c ? cg_last_error(c) : "");
  exit(1);
}

static void write_density_grid(cg_ctx *c, const cg_params *p, const char *tag)
{
  const int N = p->n_grid, ngx = 2 * (N / 2 + 1);
  float *g = malloc((size_t)N * N * ngx * sizeof(float));
  if (!g) die(c, CG_ENOMEM, "density grid buffer");
  int rc = cg_download_grid(c, 0, g);
  if (rc) die(c, rc, "download_grid");
  if ((rc = cg_write_density_grid(p->prefix_out, tag, g, N, p->l_box))) die(c, rc, "write_density_grid");
  free(g);
}

static void write_map(cg_ctx *c, const char *fname, const float *m, long nside)
{
  int rc = cg_write_healpix_map(fname, m, nside);
  if (rc) die(c, rc, fname);
}

int main(int argc, char **argv)
{
  if (argc < 2) {
    fprintf(stderr, "Usage: ./colore_gpu file_name\n");
    return 0;
  }
  int test_memory = !strcmp(argv[1], "--test-memory");
  const char *fname = test_memory ? (argc > 2 ? argv[2] : "") : argv[1];
  setbuf(stdout, NULL);
  printf("\n|-------------------------------------------------|\n");
  printf("|                 CoLoRe (GB300)                  |\n");
  printf("|-------------------------------------------------|\n\n");
  double t_abs = now_ms();
  cg_params *p;
  char err[1024];
  int rc = cg_read_run_params(fname, &p, err, sizeof(err));
  if (rc) {
    fprintf(stderr, "MPI task 0, Fatal: %s\n", err);
    return 1;
  }
  cg_config cfg;
  cg_params_to_config(p, &cfg);
  unsigned long long mem = 0;
  cg_memory_estimate(&cfg, &mem);
  printf("Run parameters: \n");
  printf("  %.3lf < z < %.3lf\n", p->z_min, p->z_max);
  printf("  %.3lf < r/(Mpc/h) < %.3lf\n", p->r_min, p->r_max);
  printf("  L_box = %.3lf Mpc/h, N_grid = %d \n", p->l_box, p->n_grid);
  printf("  Real-space resolution: dx = %.3lE Mpc/h\n", p->l_box / p->n_grid);
  printf("  Original sigma8=%lf, Sigma_Gauss should be %lf\n", p->sigma8_input, p->sigma2_gauss_theory > 0 ? sqrt(p->sigma2_gauss_theory) : 0.0);
  printf("  GPU memory plan: %.3f GB\n", mem / 1e9);
  if (test_memory) {
    cg_params_free(p);
    return 0;
  }
  printf("Seed : %llu\n", (unsigned long long)p->seed);
  if (p->write_pred) { /* main.c:61-63 */
    printf("*** Writing predictions\n");
    if ((rc = cg_write_predictions(p))) die(NULL, rc, "write_predictions");
  }
  if (p->just_write_pred) {
    cg_params_free(p);
    return 0;
  }
  cg_ctx *c;
  if ((rc = cg_create(&c, &cfg, 0))) die(NULL, rc, "cg_create");
  printf("*** Creating Gaussian density field \n");
  timer0();
  if ((rc = cg_create_cartesian_fields(c))) die(c, rc, "create_cartesian_fields");
  double s2, mean;
  if ((rc = cg_get_sigma2(c, &s2, &mean))) die(c, rc, "sigma2");
  timer2();
  printf(" <d>=%.3lE, <d^2>=%.3lE\n\n", mean, sqrt(s2));
  if (p->output_density) write_density_grid(c, p, "gaussian");
  printf("*** Creating physical matter density\n");
  if ((rc = cg_compute_physical_density_field(c))) die(c, rc, "compute_physical_density_field");
  if (p->output_density) write_density_grid(c, p, "lightcone");
  printf("*** Computing normalization of density field\n");
  if ((rc = cg_compute_density_normalization(c))) die(c, rc, "compute_density_normalization");
  cg_sync(c);
  timer2();
  long long ns[CG_NPOP_MAX] = {0};
  if (p->n_srcs > 0) {
    printf("*** Getting point sources\n");
    if ((rc = cg_srcs_set_cartesian(c, ns))) die(c, rc, "srcs_set_cartesian");
    for (int i = 0; i < p->n_srcs; i++) printf("   There will be %lld objects in total \n", ns[i]);
    timer2();
  }
  if (p->n_imap > 0) {
    printf("*** Filling up intensity maps\n");
    if ((rc = cg_imap_set_cartesian(c))) die(c, rc, "imap_set_cartesian");
    cg_sync(c);
    timer2();
  }
  printf("*** Getting LOS information\n");
  if ((rc = cg_get_beam_properties(c))) die(c, rc, "get_beam_properties");
  if ((rc = cg_sync(c))) die(c, rc, "sync");
  timer2();
  char out[600];
  if (p->do_kappa) {
    printf("*** Writing kappa source maps\n");
    long npix = 12L * p->nside_kappa * p->nside_kappa;
    float *m = malloc((size_t)p->n_kappa * npix * sizeof(float));
    if ((rc = cg_download_kappa(c, m))) die(c, rc, "download_kappa");
    for (int i = 0; i < p->n_kappa; i++) {
      snprintf(out, sizeof(out), "%s_kappa_z%03d.fits", p->prefix_out, i);
      write_map(c, out, m + (size_t)i * npix, p->nside_kappa);
    }
    free(m);
  }
  /* write_catalog (io.c:1069-1236): FITS or ASCII; HDF5 is not built */
  const int fmt = !strcmp(p->output_format, "FITS") ? CG_OUT_FITS : CG_OUT_ASCII;
  if (p->n_srcs > 0 && !strcmp(p->output_format, "HDF5")) printf("HDF5 not supported\n");
  if (p->do_isw) {
    printf("*** Writing isw source maps\n");
    long npix = 12L * p->nside_isw * p->nside_isw;
    float *m = malloc((size_t)p->n_isw * npix * sizeof(float));
    if (!m) die(c, CG_ENOMEM, "ISW buffer");
    if ((rc = cg_download_isw(c, m))) die(c, rc, "download_isw");
    for (int i = 0; i < p->n_isw; i++) {
      snprintf(out, sizeof(out), "%s_isw_z%03d.fits", p->prefix_out, i);
      write_map(c, out, m + (size_t)i * npix, p->nside_isw);
    }
    free(m);
  }
  for (int ip = 0; ip < p->n_srcs; ip++) {
    printf("*** Writing source catalogs\n %d-th population (%s)\n", ip, fmt == CG_OUT_FITS ? "FITS" : "ASCII");
    float *src = malloc((size_t)(ns[ip] > 0 ? ns[ip] : 1) * 9 * sizeof(float));
    if (!src) die(c, CG_ENOMEM, "catalogue buffer");
    if ((rc = cg_download_catalog(c, ip, NULL, NULL, src))) die(c, rc, "download_catalog");
    cg_skewer_set skw, *pskw = NULL;
    float *skw_buf = NULL;
    if (p->skw_srcs[ip] && fmt == CG_OUT_FITS) { /* io.c:1140-1189 */
      const int nr = p->n_grid / 2;
      const size_t m = (size_t)(ns[ip] > 0 ? ns[ip] : 0) * nr;
      skw_buf = malloc((2 * m + 4 * (size_t)nr) * sizeof(float));
      if (!skw_buf) die(c, CG_ENOMEM, "skewer buffer");
      float *bgr = skw_buf + 2 * m;
      if ((rc = cg_download_skewers(c, ip, skw_buf, skw_buf + m))) die(c, rc, "download_skewers");
      cg_skewer_background(p, nr, bgr, bgr + nr, bgr + 2 * nr, bgr + 3 * nr);
      skw = (cg_skewer_set){nr, p->skw_gauss[ip], skw_buf, skw_buf + m, bgr, bgr + nr, bgr + 2 * nr, bgr + 3 * nr,
                            (float)sqrt(s2)};
      pskw = &skw;
    }
    if ((rc = cg_write_catalog(p->prefix_out, ip, fmt, src, ns[ip], p->lensing_srcs[ip], pskw)))
      die(c, rc, "write_catalog");
    free(skw_buf);
    free(src);
    if (p->nside_count[ip] > 0) {
      long npix = 12L * p->nside_count[ip] * p->nside_count[ip];
      int *cm = malloc(npix * sizeof(int));
      float *fm = malloc(npix * sizeof(float));
      if ((rc = cg_download_count_map(c, ip, cm))) die(c, rc, "download_count_map");
      for (long i = 0; i < npix; i++) fm[i] = (float)cm[i];
      snprintf(out, sizeof(out), "%s_srcs_s%d_counts.fits", p->prefix_out, ip + 1);
      write_map(c, out, fm, p->nside_count[ip]);
      free(cm);
      free(fm);
    }
  }
  for (int ip = 0; ip < p->n_imap; ip++) {
    printf("*** Writing intensity maps\n %d-th species\n", ip);
    long npix = 12L * p->nside_imap[ip] * p->nside_imap[ip];
    float *m = malloc((size_t)p->imap_nr[ip] * npix * sizeof(float));
    if ((rc = cg_download_imap(c, ip, m, NULL))) die(c, rc, "download_imap");
    for (int ir = 0; ir < p->imap_nr[ip]; ir++) {
      snprintf(out, sizeof(out), "%s_imap_s%d_nu%03d.fits", p->prefix_out, ip + 1, ir);
      write_map(c, out, m + (size_t)ir * npix, p->nside_imap[ip]);
    }
    free(m);
  }
  /* write_cstm (io.c:754-800): one map per custom kernel, NEST order */
  if (p->n_cstm > 0) printf("*** Writing custom maps\n");
  for (int ip = 0; ip < p->n_cstm; ip++) {
    long npix = 12L * p->nside_cstm[ip] * p->nside_cstm[ip];
    float *m = malloc(npix * sizeof(float));
    if (!m) die(c, CG_ENOMEM, "custom map buffer");
    if ((rc = cg_download_custom(c, ip, m))) die(c, rc, "download_custom");
    snprintf(out, sizeof(out), "%s_custom_s%d.fits", p->prefix_out, ip + 1);
    write_map(c, out, m, p->nside_cstm[ip]);
    free(m);
  }
  printf("\n|-------------------------------------------------|\n\n");
  cg_destroy(c);
  cg_params_free(p);
  printf(">    Total time ellapsed %.1lf ms\n", now_ms() - t_abs);
  return 0;
}
