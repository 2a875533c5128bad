/*
 * host_io.c -- the output writers of io.c for the host side, without
 * cfitsio: HEALPix maps as FITS binary tables (he_write_healpix_map,
 * healpix_extra.c:4-57), source catalogues as FITS binary tables or ASCII
 * (write_catalog, io.c:1069-1236, with the lensing columns and the
 * skewer extensions) and density grids in the native binary format
 * (write_density_grid, io.c:565-595).
 *
 * FITS: 2880-byte blocks of 80-character header cards, big-endian data; an
 * empty primary HDU followed by one BINTABLE extension, as cfitsio's
 * fits_create_tbl writes them.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "colore_host.h"

typedef struct {
  FILE *f;
  long n; /* bytes written in the current header */
} Hdr;

static void card_raw(Hdr *h, const char *text)
{
  char c[81];
  snprintf(c, sizeof(c), "%-80.80s", text);
  fwrite(c, 1, 80, h->f);
  h->n += 80;
}

/* value already formatted (numbers, T/F, quoted strings) right-aligned in
 * columns 11-30 for numbers and logicals, left-aligned for strings */
static void card_val(Hdr *h, const char *key, const char *val, int is_string, const char *cmt)
{
  char c[128];
  if (is_string) snprintf(c, sizeof(c), "%-8.8s= %-20s / %s", key, val, cmt ? cmt : "");
  else snprintf(c, sizeof(c), "%-8.8s= %20s / %s", key, val, cmt ? cmt : "");
  card_raw(h, c);
}

static void card_str(Hdr *h, const char *key, const char *s, const char *cmt)
{
  char q[80];
  snprintf(q, sizeof(q), "'%-8s'", s); /* FITS strings: at least 8 characters inside the quotes */
  card_val(h, key, q, 1, cmt);
}

static void card_long(Hdr *h, const char *key, long v, const char *cmt)
{
  char q[32];
  snprintf(q, sizeof(q), "%ld", v);
  card_val(h, key, q, 0, cmt);
}

static void hdr_end(Hdr *h)
{
  card_raw(h, "END");
  while (h->n % 2880) {
    fputc(' ', h->f);
    h->n++;
  }
}

static void pad_data(FILE *f, long bytes)
{
  while (bytes % 2880) {
    fputc(0, f);
    bytes++;
  }
}

static void put_be32(unsigned char *b, uint32_t u)
{
  b[0] = (unsigned char)(u >> 24);
  b[1] = (unsigned char)(u >> 16);
  b[2] = (unsigned char)(u >> 8);
  b[3] = (unsigned char)u;
}

static void primary_hdu(FILE *f)
{
  Hdr h = {f, 0};
  card_val(&h, "SIMPLE", "T", 0, "file does conform to FITS standard");
  card_long(&h, "BITPIX", 8, "number of bits per data pixel");
  card_long(&h, "NAXIS", 0, "number of data axes");
  card_val(&h, "EXTEND", "T", 0, "FITS dataset may contain extensions");
  hdr_end(&h);
}

static void table_head(Hdr *h, long rowbytes, long nrows, int nf, const char **ttype, const char **tform,
                       const char **tunit, const char *extname)
{
  char k[16];
  card_str(h, "XTENSION", "BINTABLE", "binary table extension");
  card_long(h, "BITPIX", 8, "8-bit bytes");
  card_long(h, "NAXIS", 2, "2-dimensional binary table");
  card_long(h, "NAXIS1", rowbytes, "width of table in bytes");
  card_long(h, "NAXIS2", nrows, "number of rows in table");
  card_long(h, "PCOUNT", 0, "size of special data area");
  card_long(h, "GCOUNT", 1, "one data group (required keyword)");
  card_long(h, "TFIELDS", nf, "number of fields in each row");
  for (int i = 0; i < nf; i++) {
    snprintf(k, sizeof(k), "TTYPE%d", i + 1);
    card_str(h, k, ttype[i], "label for field");
    snprintf(k, sizeof(k), "TFORM%d", i + 1);
    card_str(h, k, tform[i], "data format of field");
    snprintf(k, sizeof(k), "TUNIT%d", i + 1);
    card_str(h, k, tunit[i], "physical unit of field");
  }
  if (extname) card_str(h, "EXTNAME", extname, "name of this binary table extension");
}

int cg_write_healpix_map(const char *fname, const float *map, long nside)
{
  FILE *f = fopen(fname, "wb");
  if (!f) return CG_EINVAL;
  primary_hdu(f);
  const long npix = 12 * nside * nside;
  const char *tt[1] = {"map 1"}, *tf[1] = {"1E"}, *tu[1] = {"uK"};
  Hdr h = {f, 0};
  table_head(&h, 4, npix, 1, tt, tf, tu, "BINTABLE");
  card_str(&h, "PIXTYPE", "HEALPIX", "HEALPIX Pixelisation");
  card_str(&h, "ORDERING", "RING", "Pixel ordering scheme, either RING or NESTED");
  card_long(&h, "NSIDE", nside, "Resolution parameter for HEALPIX");
  card_str(&h, "COORDSYS", "G", "Pixelisation coordinate system");
  card_raw(&h, "COMMENT G = Galactic, E = ecliptic, C = celestial = equatorial");
  hdr_end(&h);
  unsigned char buf[4096];
  long k = 0;
  for (long i = 0; i < npix; i++) {
    uint32_t u;
    memcpy(&u, &map[i], 4);
    put_be32(buf + k, u);
    k += 4;
    if (k == (long)sizeof(buf)) {
      fwrite(buf, 1, k, f);
      k = 0;
    }
  }
  if (k) fwrite(buf, 1, k, f);
  pad_data(f, npix * 4);
  return fclose(f) ? CG_EINVAL : CG_OK;
}

static void card_float(Hdr *h, const char *key, double v, const char *cmt)
{
  char q[32];
  snprintf(q, sizeof(q), "%.8E", v);
  card_val(h, key, q, 0, cmt);
}

static void write_be32_array(FILE *f, const float *a, long long n)
{
  unsigned char buf[4096];
  long k = 0;
  for (long long i = 0; i < n; i++) {
    uint32_t u;
    memcpy(&u, &a[i], 4);
    put_be32(buf + k, u);
    k += 4;
    if (k == (long)sizeof(buf)) {
      fwrite(buf, 1, k, f);
      k = 0;
    }
  }
  if (k) fwrite(buf, 1, k, f);
}

/* 2-D float image extension (fits_create_img FLOAT_IMG + fits_write_img) */
static void image_hdu(FILE *f, long nx, long ny, const float *data, const char *contents)
{
  Hdr h = {f, 0};
  card_str(&h, "XTENSION", "IMAGE", "IMAGE extension");
  card_long(&h, "BITPIX", -32, "number of bits per data pixel");
  card_long(&h, "NAXIS", 2, "number of data axes");
  card_long(&h, "NAXIS1", nx, "length of data axis 1");
  card_long(&h, "NAXIS2", ny, "length of data axis 2");
  card_long(&h, "PCOUNT", 0, "required keyword; must = 0");
  card_long(&h, "GCOUNT", 1, "required keyword; must = 1");
  card_str(&h, "CONTENTS", contents, "");
  hdr_end(&h);
  write_be32_array(f, data, (long long)nx * ny);
  pad_data(f, nx * ny * 4);
}

int cg_write_catalog(const char *prefix, int ipop, int format, const float *src9, long long n, int has_lensing,
                     const cg_skewer_set *skw)
{
  char fname[1024];
  if (format == CG_OUT_FITS) {
    snprintf(fname, sizeof(fname), "%s_srcs_s%d_0.fits", prefix, ipop + 1);
    FILE *f = fopen(fname, "wb");
    if (!f) return CG_EINVAL;
    primary_hdu(f);
    /* the reference's TFORM of DRA reads "1E!"; the column is a plain 1E */
    const char *tt[10] = {"TYPE", "RA", "DEC", "Z_COSMO", "DZ_RSD", "E1", "E2", "KAPPA", "DRA", "DDEC"};
    const char *tf[10] = {"1J", "1E", "1E", "1E", "1E", "1E", "1E", "1E", "1E", "1E"};
    const char *tu[10] = {"NA", "DEG", "DEG", "NA", "NA", "NA", "NA", "NA", "DEG", "DEG"};
    const int nf = has_lensing ? 10 : 5;
    Hdr h = {f, 0};
    table_head(&h, 4L * nf, (long)n, nf, tt, tf, tu, NULL);
    card_str(&h, "CONTENTS", "Source catalog", "");
    hdr_end(&h);
    unsigned char row[40];
    for (long long j = 0; j < n; j++) {
      put_be32(row, (uint32_t)ipop);
      for (int c = 1; c < nf; c++) {
        uint32_t u; /* ra, dec, z0, dz_rsd, e1, e2, kappa, dra, ddec */
        memcpy(&u, &src9[9 * j + c - 1], 4);
        put_be32(row + 4 * c, u);
      }
      fwrite(row, 1, 4 * nf, f);
    }
    pad_data(f, (long)n * 4 * nf);
    if (skw && skw->nr > 0) {
      image_hdu(f, skw->nr, (long)n, skw->dens, skw->gauss ? "gaussian skewers" : "density skewers");
      image_hdu(f, skw->nr, (long)n, skw->vel, "velocity skewers");
      const char *bt[4] = {"R", "Z", "D", "V"}, *bf[4] = {"1E", "1E", "1E", "1E"},
                 *bu[4] = {"MPC_H", "NA", "NA", "NA"};
      Hdr b = {f, 0};
      table_head(&b, 16, skw->nr, 4, bt, bf, bu, NULL);
      card_str(&b, "CONTENTS", "Background cosmology", "");
      card_float(&b, "SIGMA_G", skw->sigma_g, "");
      hdr_end(&b);
      for (int i = 0; i < skw->nr; i++) {
        const float v[4] = {skw->r[i], skw->z[i], skw->d1[i], skw->v1[i]};
        for (int c = 0; c < 4; c++) {
          uint32_t u;
          memcpy(&u, &v[c], 4);
          put_be32(row + 4 * c, u);
        }
        fwrite(row, 1, 16, f);
      }
      pad_data(f, 16L * skw->nr);
    }
    return fclose(f) ? CG_EINVAL : CG_OK;
  }
  snprintf(fname, sizeof(fname), "%s_srcs_s%d_0.txt", prefix, ipop + 1);
  FILE *f = fopen(fname, "w");
  if (!f) return CG_EINVAL;
  fprintf(f, "#[1]type [2]RA, [3]dec, [4]z0, [5]dz_RSD ");
  fprintf(f, has_lensing ? "#[6]e1, [7]e2 [8]kappa [9]d_ra [10]d_dec\n" : "\n");
  for (long long j = 0; j < n; j++) {
    const float *q = src9 + 9 * j;
    fprintf(f, "%d %E %E %E %E ", ipop, q[0], q[1], q[2], q[3]);
    if (has_lensing) fprintf(f, "%E %E %E %E %E \n", q[4], q[5], q[6], q[7], q[8]);
    else fprintf(f, "\n");
  }
  return fclose(f) ? CG_EINVAL : CG_OK;
}

/* f_of_r_linear (cosmo.c:30-38) on the tables of p */
static double bg_lin(const cg_params *p, const double *f, double f0, double ff, double r)
{
  if (r <= 0) return f0;
  if (r >= p->r_arr_r2z[CG_NA - 1]) return ff;
  int ir = (int)(r * p->glob_idr);
  return f[ir] + (f[ir + 1] - f[ir]) * (r - p->r_arr_r2z[ir]) * p->glob_idr;
}

int cg_skewer_background(const cg_params *p, int nr, float *r, float *z, float *d1, float *v1)
{
  if (!p || nr < 1 || !r || !z || !d1 || !v1) return CG_EINVAL;
  const double dr = p->r_max / nr;
  for (int i = 0; i < nr; i++) {
    const double rr = dr * (i + 0.5);
    r[i] = (float)rr;
    z[i] = (float)bg_lin(p, p->z_arr_r2z, 0, p->z_arr_r2z[CG_NA - 1], rr);
    d1[i] = (float)bg_lin(p, p->growth_d_arr, 1, p->growth_d_arr[CG_NA - 1], rr);
    v1[i] = (float)bg_lin(p, p->growth_v_arr, p->growth_v_arr[0], p->growth_v_arr[CG_NA - 1], rr);
  }
  return CG_OK;
}

int cg_write_density_grid(const char *prefix, const char *tag, const float *grid, int n_grid, double l_box)
{
  char fname[1024];
  snprintf(fname, sizeof(fname), "%s_dens_%s_0.dat", prefix, tag);
  FILE *f = fopen(fname, "wb");
  if (!f) return CG_EINVAL;
  const int nnodes = 1, sz = (int)sizeof(float), iz0 = 0, N = n_grid, ngx = 2 * (n_grid / 2 + 1);
  fwrite(&nnodes, sizeof(int), 1, f);
  fwrite(&sz, sizeof(int), 1, f);
  fwrite(&l_box, sizeof(double), 1, f);
  fwrite(&N, sizeof(int), 1, f);
  fwrite(&N, sizeof(int), 1, f); /* nz_here: the whole grid on one node */
  fwrite(&iz0, sizeof(int), 1, f);
  for (int iz = 0; iz < N; iz++)
    for (int iy = 0; iy < N; iy++) fwrite(grid + (size_t)ngx * (iy + (size_t)iz * N), sizeof(float), N, f);
  return fclose(f) ? CG_EINVAL : CG_OK;
}
