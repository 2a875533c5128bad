/*
 * colore_gpu.c -- command-line driver with the stage sequence of CoLoRe's
 * main() (main.c:24-154), running every hot-path stage on the GPU through
 * libcolore_cuda.so:
 *
 *   ./colore_gpu params.cfg            run and write outputs
 *   ./colore_gpu --test-memory params  print the memory plan and exit
 *
 * Outputs follow io.c: raw density grids (write_density_grid, io.c:565-595),
 * source catalogues in ASCII (io.c:1210-1236) and HEALPix maps in FITS
 * binary tables (he_write_healpix_map, healpix_extra.c:4-57), written by a
 * minimal FITS writer of this file since cfitsio is not required.
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

/* ---- minimal FITS writer: primary HDU + one BINTABLE column of 1E ---- */
static void fits_card(FILE *f, const char *key, const char *val, const char *cmt)
{
  char card[81];
  if (val) snprintf(card, sizeof(card), "%-8.8s= %20s / %-47.47s", key, val, cmt ? cmt : "");
  else snprintf(card, sizeof(card), "%-80.80s", key);
  fprintf(f, "%-80.80s", card);
}

static void fits_end(FILE *f, long *nbytes)
{
  fits_card(f, "END", NULL, NULL);
  *nbytes += 80;
  while (*nbytes % 2880) {
    fputc(' ', f);
    (*nbytes)++;
  }
}

static int write_healpix_fits(const char *fname, const float *map, long nside)
{
  FILE *f = fopen(fname, "wb");
  if (!f) return -1;
  long nb = 0;
  char v[32];
  fits_card(f, "SIMPLE", "T", "conforms to FITS standard");
  fits_card(f, "BITPIX", "8", "");
  fits_card(f, "NAXIS", "0", "");
  fits_card(f, "EXTEND", "T", "");
  nb = 4 * 80;
  fits_end(f, &nb);
  long npix = 12 * nside * nside;
  nb = 0;
  fits_card(f, "XTENSION", "'BINTABLE'", "binary table extension");
  fits_card(f, "BITPIX", "8", "");
  fits_card(f, "NAXIS", "2", "");
  fits_card(f, "NAXIS1", "4", "bytes per row");
  snprintf(v, sizeof(v), "%ld", npix);
  fits_card(f, "NAXIS2", v, "rows");
  fits_card(f, "PCOUNT", "0", "");
  fits_card(f, "GCOUNT", "1", "");
  fits_card(f, "TFIELDS", "1", "");
  fits_card(f, "TTYPE1", "'map 1   '", "");
  fits_card(f, "TFORM1", "'1E      '", "");
  fits_card(f, "TUNIT1", "'uK      '", "");
  fits_card(f, "EXTNAME", "'BINTABLE'", "");
  fits_card(f, "PIXTYPE", "'HEALPIX '", "HEALPIX Pixelisation");
  fits_card(f, "ORDERING", "'RING    '", "Pixel ordering scheme, either RING or NESTED");
  snprintf(v, sizeof(v), "%ld", nside);
  fits_card(f, "NSIDE", v, "Resolution parameter for HEALPIX");
  fits_card(f, "COORDSYS", "'G       '", "Pixelisation coordinate system");
  nb = 16 * 80;
  fits_end(f, &nb);
  for (long i = 0; i < npix; i++) { /* big-endian IEEE float */
    uint32_t u;
    memcpy(&u, &map[i], 4);
    unsigned char b[4] = {(unsigned char)(u >> 24), (unsigned char)(u >> 16), (unsigned char)(u >> 8),
                          (unsigned char)u};
    fwrite(b, 1, 4, f);
  }
  long data = npix * 4;
  while (data % 2880) {
    fputc(0, f);
    data++;
  }
  fclose(f);
  return 0;
}

static void write_density_grid(cg_ctx *c, const cg_params *p, const char *tag)
{
  const int N = p->n_grid, ngx = 2 * (N / 2 + 1);
  size_t nf = (size_t)N * N * ngx;
  float *g = malloc(nf * sizeof(float));
  int rc = cg_download_grid(c, 0, g);
  if (rc) die(c, rc, "download_grid");
  char fname[512];
  snprintf(fname, sizeof(fname), "%s_dens_%s_0.dat", p->prefix_out, tag);
  FILE *f = fopen(fname, "wb");
  if (!f) die(c, CG_EINVAL, fname);
  int one = 1, sz = (int)sizeof(float), zero = 0;
  double lb = p->l_box;
  fwrite(&one, sizeof(int), 1, f);
  fwrite(&sz, sizeof(int), 1, f);
  fwrite(&lb, sizeof(double), 1, f);
  fwrite(&N, sizeof(int), 1, f);
  fwrite(&N, sizeof(int), 1, f);
  fwrite(&zero, sizeof(int), 1, f);
  for (int iz = 0; iz < N; iz++)
    for (int iy = 0; iy < N; iy++) fwrite(g + (size_t)ngx * (iy + (size_t)iz * N), sizeof(float), N, f);
  fclose(f);
  free(g);
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
  if (p->n_cstm || p->do_isw || p->do_skewers || p->do_srcs_lensing)
    fprintf(stderr, "Warning: custom maps, ISW, skewers and source lensing are not produced by this build\n");
  if (test_memory) {
    cg_params_free(p);
    return 0;
  }
  printf("Seed : %llu\n", (unsigned long long)p->seed);
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
      write_healpix_fits(out, m + (size_t)i * npix, p->nside_kappa);
    }
    free(m);
  }
  for (int ip = 0; ip < p->n_srcs; ip++) {
    printf("*** Writing source catalogs\n %d-th population (ASCII)\n", ip);
    float *src = malloc((size_t)(ns[ip] > 0 ? ns[ip] : 1) * 9 * sizeof(float));
    if ((rc = cg_download_catalog(c, ip, NULL, NULL, src))) die(c, rc, "download_catalog");
    snprintf(out, sizeof(out), "%s_srcs_s%d_0.txt", p->prefix_out, ip + 1);
    FILE *f = fopen(out, "w");
    if (!f) die(c, CG_EINVAL, out);
    fprintf(f, "#[1]type [2]RA, [3]dec, [4]z0, [5]dz_RSD \n");
    for (long long j = 0; j < ns[ip]; j++)
      fprintf(f, "%d %E %E %E %E \n", ip, src[9 * j], src[9 * j + 1], src[9 * j + 2], src[9 * j + 3]);
    fclose(f);
    free(src);
    if (p->nside_count[ip] > 0) {
      long npix = 12L * p->nside_count[ip] * p->nside_count[ip];
      int *cm = malloc(npix * sizeof(int));
      float *fm = malloc(npix * sizeof(float));
      if ((rc = cg_download_count_map(c, ip, cm))) die(c, rc, "download_count_map");
      for (long i = 0; i < npix; i++) fm[i] = (float)cm[i];
      snprintf(out, sizeof(out), "%s_srcs_s%d_counts.fits", p->prefix_out, ip + 1);
      write_healpix_fits(out, fm, p->nside_count[ip]);
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
      write_healpix_fits(out, m + (size_t)ir * npix, p->nside_imap[ip]);
    }
    free(m);
  }
  printf("\n|-------------------------------------------------|\n\n");
  cg_destroy(c);
  cg_params_free(p);
  printf(">    Total time ellapsed %.1lf ms\n", now_ms() - t_abs);
  return 0;
}
