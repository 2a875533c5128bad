/*
 * host_params.c -- the param-file API of CoLoRe without libconfig.
 *
 * A recursive-descent reader for the libconfig grammar used by CoLoRe's
 * param files (settings "name = value;" or "name: value", groups { },
 * arrays [ ], lists ( ), strings with adjacent-literal concatenation, ints,
 * floats, booleans, and #, // and C comments), and read_run_params
 * (io.c:246-563) on top of it, with the same required keys, defaults and
 * error messages.  Numbers convert between int and float on lookup, as with
 * CONFIG_OPTION_AUTOCONVERT (io.c:261).
 *
 * Two optional keys extend the reference's format: global.bias_model
 * (1: (1+d)^b, 2: the Makefile's default _BIAS_MODEL_2, 3: _BIAS_MODEL_3;
 * default 2) and srcsN.nside_count (resolution of a source count map,
 * default 0 = none).
 */
#include <ctype.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "colore_host.h"

int cg_host_cosmo_set(cg_params *p, char *err, size_t el);

enum { T_GROUP, T_ARRAY, T_LIST, T_INT, T_FLOAT, T_BOOL, T_STRING };

typedef struct node {
  char name[128];
  int type;
  double num;
  int bval;
  char *str;
  struct node **kid;
  int nkid, cap;
} node;

typedef struct {
  const char *s;
  size_t i, n;
  int line;
  char err[256];
} lexer;

static void node_free(node *x)
{
  if (!x) return;
  for (int i = 0; i < x->nkid; i++) node_free(x->kid[i]);
  free(x->kid);
  free(x->str);
  free(x);
}

static node *node_new(int type)
{
  node *x = calloc(1, sizeof(node));
  if (x) x->type = type;
  return x;
}

static int node_add(node *p, node *k)
{
  if (p->nkid == p->cap) {
    int nc = p->cap ? 2 * p->cap : 8;
    node **nk = realloc(p->kid, nc * sizeof(node *));
    if (!nk) return -1;
    p->kid = nk;
    p->cap = nc;
  }
  p->kid[p->nkid++] = k;
  return 0;
}

static void skip_ws(lexer *L)
{
  for (;;) {
    while (L->i < L->n && isspace((unsigned char)L->s[L->i])) {
      if (L->s[L->i] == '\n') L->line++;
      L->i++;
    }
    if (L->i < L->n && L->s[L->i] == '#') {
      while (L->i < L->n && L->s[L->i] != '\n') L->i++;
      continue;
    }
    if (L->i + 1 < L->n && L->s[L->i] == '/' && L->s[L->i + 1] == '/') {
      while (L->i < L->n && L->s[L->i] != '\n') L->i++;
      continue;
    }
    if (L->i + 1 < L->n && L->s[L->i] == '/' && L->s[L->i + 1] == '*') {
      L->i += 2;
      while (L->i + 1 < L->n && !(L->s[L->i] == '*' && L->s[L->i + 1] == '/')) {
        if (L->s[L->i] == '\n') L->line++;
        L->i++;
      }
      L->i += 2;
      continue;
    }
    break;
  }
}

static int perr(lexer *L, const char *msg)
{
  snprintf(L->err, sizeof(L->err), "line %d: %s", L->line, msg);
  return -1;
}

static int parse_settings(lexer *L, node *grp, char close);

static node *parse_value(lexer *L)
{
  skip_ws(L);
  if (L->i >= L->n) return perr(L, "unexpected end of file"), NULL;
  char ch = L->s[L->i];
  if (ch == '{') {
    L->i++;
    node *g = node_new(T_GROUP);
    if (!g || parse_settings(L, g, '}')) return node_free(g), NULL;
    return g;
  }
  if (ch == '[' || ch == '(') {
    char close = ch == '[' ? ']' : ')';
    node *a = node_new(ch == '[' ? T_ARRAY : T_LIST);
    L->i++;
    skip_ws(L);
    if (L->i < L->n && L->s[L->i] == close) {
      L->i++;
      return a;
    }
    for (;;) {
      node *v = parse_value(L);
      if (!v) return node_free(a), NULL;
      node_add(a, v);
      skip_ws(L);
      if (L->i < L->n && L->s[L->i] == ',') {
        L->i++;
        continue;
      }
      if (L->i < L->n && L->s[L->i] == close) {
        L->i++;
        return a;
      }
      return perr(L, "expected ',' or closing bracket"), node_free(a), NULL;
    }
  }
  if (ch == '"') {
    node *v = node_new(T_STRING);
    size_t cap = 64, len = 0;
    v->str = malloc(cap);
    while (L->i < L->n && L->s[L->i] == '"') { /* adjacent literals concatenate */
      L->i++;
      while (L->i < L->n && L->s[L->i] != '"') {
        char c = L->s[L->i++];
        if (c == '\\' && L->i < L->n) {
          char e = L->s[L->i++];
          c = e == 'n' ? '\n' : e == 't' ? '\t' : e;
        }
        if (len + 2 > cap) v->str = realloc(v->str, cap *= 2);
        v->str[len++] = c;
      }
      if (L->i >= L->n) return perr(L, "unterminated string"), node_free(v), NULL;
      L->i++;
      skip_ws(L);
    }
    v->str[len] = 0;
    return v;
  }
  /* bool or number */
  size_t j = L->i;
  while (j < L->n && (isalnum((unsigned char)L->s[j]) || strchr("+-._", L->s[j]))) j++;
  char tok[128];
  size_t len = j - L->i;
  if (len == 0 || len >= sizeof(tok)) return perr(L, "bad value"), NULL;
  memcpy(tok, L->s + L->i, len);
  tok[len] = 0;
  L->i = j;
  char low[128];
  for (size_t k = 0; k <= len; k++) low[k] = (char)tolower((unsigned char)tok[k]);
  if (!strcmp(low, "true") || !strcmp(low, "false")) {
    node *v = node_new(T_BOOL);
    v->bval = low[0] == 't';
    return v;
  }
  char *end;
  int is_float = strpbrk(tok, ".eE") != NULL && !(tok[0] == '0' && (tok[1] == 'x' || tok[1] == 'X'));
  node *v = node_new(is_float ? T_FLOAT : T_INT);
  if (is_float) v->num = strtod(tok, &end);
  else {
    long long iv = strtoll(tok, &end, 0);
    if (*end == 'L' || *end == 'l') end++;
    v->num = (double)iv;
  }
  if (*end) return perr(L, "bad number"), node_free(v), NULL;
  return v;
}

static int parse_settings(lexer *L, node *grp, char close)
{
  for (;;) {
    skip_ws(L);
    if (L->i >= L->n) {
      if (close) return perr(L, "missing '}'");
      return 0;
    }
    if (close && L->s[L->i] == close) {
      L->i++;
      return 0;
    }
    size_t j = L->i;
    if (!(isalpha((unsigned char)L->s[j]) || L->s[j] == '*')) return perr(L, "expected a setting name");
    while (j < L->n && (isalnum((unsigned char)L->s[j]) || strchr("-_*", L->s[j]))) j++;
    char name[128];
    size_t len = j - L->i;
    if (len >= sizeof(name)) return perr(L, "name too long");
    memcpy(name, L->s + L->i, len);
    name[len] = 0;
    L->i = j;
    skip_ws(L);
    if (L->i >= L->n || (L->s[L->i] != '=' && L->s[L->i] != ':')) return perr(L, "expected '=' or ':'");
    L->i++;
    node *v = parse_value(L);
    if (!v) return -1;
    snprintf(v->name, sizeof(v->name), "%s", name);
    node_add(grp, v);
    skip_ws(L);
    if (L->i < L->n && (L->s[L->i] == ';' || L->s[L->i] == ',')) L->i++;
  }
}

static node *lookup(node *root, const char *path)
{
  char buf[256];
  snprintf(buf, sizeof(buf), "%s", path);
  node *cur = root;
  for (char *tok = strtok(buf, "."); tok; tok = strtok(NULL, ".")) {
    if (!cur || cur->type != T_GROUP) return NULL;
    node *nx = NULL;
    for (int i = 0; i < cur->nkid; i++)
      if (!strcmp(cur->kid[i]->name, tok)) nx = cur->kid[i];
    cur = nx;
  }
  return cur;
}

typedef struct {
  node *root;
  char *err;
  size_t el;
  int rc;
} reader;

static void rfail(reader *r, const char *fmt, ...)
{
  if (r->rc) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(r->err, r->el, fmt, ap);
  va_end(ap);
  r->rc = CG_EINVAL;
}

static void rd_string(reader *r, const char *sec, const char *var, char *out, size_t len)
{
  char path[256];
  snprintf(path, sizeof(path), "%s.%s", sec, var);
  node *n = lookup(r->root, path);
  if (!n || n->type != T_STRING) return rfail(r, "Couldn't read variable %s", path);
  snprintf(out, len, "%s", n->str);
}

static void rd_double(reader *r, const char *sec, const char *var, double *out)
{
  char path[256];
  snprintf(path, sizeof(path), "%s.%s", sec, var);
  node *n = lookup(r->root, path);
  if (!n || (n->type != T_FLOAT && n->type != T_INT)) return rfail(r, "Couldn't read variable %s", path);
  *out = n->num;
}

static void rd_int(reader *r, const char *sec, const char *var, int *out)
{
  char path[256];
  snprintf(path, sizeof(path), "%s.%s", sec, var);
  node *n = lookup(r->root, path);
  if (!n || (n->type != T_FLOAT && n->type != T_INT)) return rfail(r, "Couldn't read variable %s", path);
  *out = (int)n->num;
}

static void rd_bool(reader *r, const char *sec, const char *var, int *out)
{
  char path[256];
  snprintf(path, sizeof(path), "%s.%s", sec, var);
  node *n = lookup(r->root, path);
  if (!n || n->type != T_BOOL) return rfail(r, "Couldn't read variable %s", path);
  *out = n->bval;
}

static int opt_bool(reader *r, const char *path, int def)
{
  node *n = lookup(r->root, path);
  return (n && n->type == T_BOOL) ? n->bval : def;
}

static int opt_int(reader *r, const char *path, int def)
{
  node *n = lookup(r->root, path);
  return (n && (n->type == T_INT || n->type == T_FLOAT)) ? (int)n->num : def;
}

static void rd_double_array(reader *r, const char *sec, const char *var, double *out, int *nel, int nmax)
{
  char path[256];
  snprintf(path, sizeof(path), "%s.%s", sec, var);
  node *n = lookup(r->root, path);
  if (!n || (n->type != T_ARRAY && n->type != T_LIST) || n->nkid == 0)
    return rfail(r, "Couldn't read variable %s", path);
  if (n->nkid > nmax) return rfail(r, "Too many elements in %s (%d > %d)", path, n->nkid, nmax);
  for (int i = 0; i < n->nkid; i++) out[i] = n->kid[i]->num;
  *nel = n->nkid;
}

static int count_sections(node *root, const char *prefix)
{
  int n = 0;
  char name[64];
  for (;;) {
    snprintf(name, sizeof(name), "%s%d", prefix, n + 1);
    if (!lookup(root, name)) return n;
    n++;
  }
}

void cg_params_free(cg_params *p)
{
  if (!p) return;
  free(p->logkarr);
  free(p->pkarr);
  for (int i = 0; i < CG_NPOP_MAX; i++) {
    free(p->srcs_nz_arr[i]);
    free(p->srcs_bz_arr[i]);
    free(p->imap_tz_arr[i]);
    free(p->imap_bz_arr[i]);
    free(p->cstm_kz_arr[i]);
    free(p->cstm_bz_arr[i]);
    free(p->imap_r0[i]);
    free(p->imap_rf[i]);
  }
  free(p);
}

int cg_read_run_params(const char *fname, cg_params **out, char *err, size_t el)
{
  *out = NULL;
  FILE *f = fopen(fname, "rb");
  if (!f) return snprintf(err, el, "Couldn't open file %s", fname), CG_EINVAL;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *txt = malloc(sz + 1);
  if (!txt || fread(txt, 1, sz, f) != (size_t)sz) {
    fclose(f);
    free(txt);
    return snprintf(err, el, "Couldn't read file %s", fname), CG_EINVAL;
  }
  txt[sz] = 0;
  fclose(f);
  lexer L = {txt, 0, (size_t)sz, 1, {0}};
  node *root = node_new(T_GROUP);
  if (parse_settings(&L, root, 0)) {
    snprintf(err, el, "%s: %s", fname, L.err);
    free(txt);
    node_free(root);
    return CG_EINVAL;
  }
  free(txt);
  cg_params *p = calloc(1, sizeof(cg_params));
  reader r = {root, err, el, 0};
  /* defaults of param_colore_new, io.c:24-158 */
  p->dens_type = CG_DENS_LGNR;
  p->lpt_interp_type = 1; /* INTERP_CIC, io.c:66 */
  p->nside_base = 2; /* choose_nside_base with one task, io.c:224-244 */
  rd_string(&r, "global", "prefix_out", p->prefix_out, sizeof(p->prefix_out));
  rd_string(&r, "global", "pk_filename", p->pk_filename, sizeof(p->pk_filename));
  rd_double(&r, "global", "z_min", &p->z_min);
  rd_double(&r, "global", "z_max", &p->z_max);
  rd_bool(&r, "global", "output_density", &p->output_density);
  int seed = 0;
  rd_int(&r, "global", "seed", &seed);
  p->seed = (unsigned int)seed;
  rd_bool(&r, "global", "write_pred", &p->write_pred);
  if (p->write_pred) { /* io.c:273-276 */
    rd_bool(&r, "global", "just_write_pred", &p->just_write_pred);
    rd_double(&r, "global", "pred_dz", &p->pred_dz);
  }
  rd_double(&r, "field_par", "r_smooth", &p->r_smooth);
  rd_bool(&r, "field_par", "smooth_potential", &p->smooth_potential);
  rd_int(&r, "field_par", "n_grid", &p->n_grid);
  rd_int(&r, "field_par", "dens_type", &p->dens_type);
  rd_double(&r, "field_par", "lpt_buffer_fraction", &p->lpt_buffer_fraction);
  rd_int(&r, "field_par", "lpt_interp_type", &p->lpt_interp_type);
  rd_int(&r, "field_par", "output_lpt", &p->output_lpt);
  rd_string(&r, "global", "output_format", p->output_format, sizeof(p->output_format));
  rd_double(&r, "cosmo_par", "omega_M", &p->omega_m);
  rd_double(&r, "cosmo_par", "omega_L", &p->omega_l);
  rd_double(&r, "cosmo_par", "omega_B", &p->omega_b);
  rd_double(&r, "cosmo_par", "h", &p->h);
  rd_double(&r, "cosmo_par", "w", &p->w);
  rd_double(&r, "cosmo_par", "ns", &p->ns);
  rd_double(&r, "cosmo_par", "sigma_8", &p->sigma8);
  p->bias_model = opt_int(&r, "global.bias_model", CG_BIAS_MODEL_EXPLIN);
  if (!r.rc && strcmp(p->output_format, "ASCII") && strcmp(p->output_format, "FITS") &&
      strcmp(p->output_format, "HDF5"))
    rfail(&r, "Unrecognized format %s", p->output_format);
  p->n_srcs = count_sections(root, "srcs");
  if (p->n_srcs > CG_NPOP_MAX) rfail(&r, "You're asking for too many populations %d! Enlarge NPOP_MAX", p->n_srcs);
  for (int i = 0; i < p->n_srcs && !r.rc; i++) {
    char sec[32];
    snprintf(sec, sizeof(sec), "srcs%d", i + 1);
    rd_string(&r, sec, "nz_filename", p->fname_nz_srcs[i], 256);
    rd_string(&r, sec, "bias_filename", p->fname_bz_srcs[i], 256);
    rd_bool(&r, sec, "include_lensing", &p->lensing_srcs[i]);
    if (p->lensing_srcs[i]) p->do_srcs_lensing = 1;
    rd_bool(&r, sec, "store_skewers", &p->skw_srcs[i]);
    if (p->skw_srcs[i]) {
      p->do_skewers = 1;
      char gpath[64];
      snprintf(gpath, sizeof(gpath), "%s.gaussian_skewers", sec);
      p->skw_gauss[i] = opt_bool(&r, gpath, 0);
    }
    char path[64];
    snprintf(path, sizeof(path), "%s.nside_count", sec);
    p->nside_count[i] = opt_int(&r, path, 0);
  }
  p->n_cstm = count_sections(root, "custom");
  if (p->n_cstm > CG_NPOP_MAX) rfail(&r, "You're asking for too many populations %d! Enlarge NPOP_MAX", p->n_cstm);
  for (int i = 0; i < p->n_cstm && !r.rc; i++) {
    char sec[32];
    snprintf(sec, sizeof(sec), "custom%d", i + 1);
    rd_string(&r, sec, "kz_filename", p->fname_kz_cstm[i], 256);
    rd_string(&r, sec, "bias_filename", p->fname_bz_cstm[i], 256);
    rd_int(&r, sec, "nside", &p->nside_cstm[i]);
  }
  p->n_imap = count_sections(root, "imap");
  if (p->n_imap > CG_NPOP_MAX) rfail(&r, "You're asking for too many populations %d! Enlarge NPOP_MAX", p->n_imap);
  for (int i = 0; i < p->n_imap && !r.rc; i++) {
    char sec[32];
    snprintf(sec, sizeof(sec), "imap%d", i + 1);
    rd_string(&r, sec, "tbak_filename", p->fname_tz_imap[i], 256);
    rd_string(&r, sec, "bias_filename", p->fname_bz_imap[i], 256);
    rd_string(&r, sec, "freq_list", p->fname_nu_imap[i], 256);
    rd_double(&r, sec, "freq_rest", &p->nu0_imap[i]);
    rd_int(&r, sec, "nside", &p->nside_imap[i]);
  }
  if (lookup(root, "kappa")) {
    p->do_kappa = 1;
    rd_double_array(&r, "kappa", "z_out", p->z_kappa_out, &p->n_kappa, CG_NPLANES_MAX);
    rd_int(&r, "kappa", "nside", &p->nside_kappa);
  }
  if (lookup(root, "isw")) {
    p->do_isw = 1;
    rd_double_array(&r, "isw", "z_out", p->z_isw_out, &p->n_isw, CG_NPLANES_MAX);
    rd_int(&r, "isw", "nside", &p->nside_isw);
  }
  node_free(root);
  if (r.rc) {
    free(p);
    return r.rc;
  }
  if (p->r_smooth > 0) { /* io.c:453-458 */
    p->r2_smooth = p->r_smooth * p->r_smooth;
    p->do_smoothing = 1;
  } else {
    p->r2_smooth = p->r_smooth;
    p->do_smoothing = 0;
  }
  p->need_beaming = p->do_srcs_lensing + p->do_kappa + p->do_isw + p->do_skewers + (p->n_cstm > 0);
  if (p->n_grid <= 0) {
    free(p);
    return snprintf(err, el, "n_grid must be positive"), CG_EINVAL;
  }
  int rc = cg_host_cosmo_set(p, err, el);
  if (rc) {
    cg_params_free(p);
    return rc;
  }
  *out = p;
  return CG_OK;
}

int cg_params_to_config(const cg_params *p, cg_config *c)
{
  if (!p || !c) return CG_EINVAL;
  memset(c, 0, sizeof(*c));
  c->precision = CG_PREC_F32;
  c->n_grid = p->n_grid;
  c->l_box = p->l_box;
  for (int i = 0; i < 3; i++) c->pos_obs[i] = p->pos_obs[i];
  c->seed = p->seed;
  c->omega_m = p->omega_m;
  c->hubble_0 = p->hubble_0;
  c->fgrowth_0 = p->fgrowth_0;
  c->prefac_lensing = p->prefac_lensing;
  c->r_max = p->r_max;
  c->r2_smooth = p->r2_smooth;
  c->do_smoothing = p->do_smoothing;
  c->smooth_potential = p->smooth_potential;
  c->dens_type = p->dens_type;
  c->lpt_interp_type = p->lpt_interp_type;
  c->n_cstm = p->n_cstm;
  for (int i = 0; i < p->n_cstm; i++) {
    c->cstm_kz_arr[i] = p->cstm_kz_arr[i];
    c->cstm_bz_arr[i] = p->cstm_bz_arr[i];
    c->nside_cstm[i] = p->nside_cstm[i];
  }
  c->bias_model = p->bias_model;
  c->numk = p->numk;
  c->logkmin = p->logkmin;
  c->logkmax = p->logkmax;
  c->idlogk = p->idlogk;
  c->n_scal = p->ns;
  c->pkarr = p->pkarr;
  c->glob_idr = p->glob_idr;
  c->r_arr_r2z = p->r_arr_r2z;
  c->z_arr_r2z = p->z_arr_r2z;
  c->growth_d_arr = p->growth_d_arr;
  c->growth_d2_arr = p->growth_d2_arr;
  c->growth_v_arr = p->growth_v_arr;
  c->growth_pd_arr = p->growth_pd_arr;
  c->ihub_arr = p->ihub_arr;
  c->a_arr_a2r = p->a_arr_a2r;
  c->r_arr_a2r = p->r_arr_a2r;
  c->n_srcs = p->n_srcs;
  for (int i = 0; i < p->n_srcs; i++) {
    c->srcs_nz_arr[i] = p->srcs_nz_arr[i];
    c->srcs_bz_arr[i] = p->srcs_bz_arr[i];
    c->nside_count[i] = p->nside_count[i];
    c->lensing_srcs[i] = p->lensing_srcs[i];
    c->skw_srcs[i] = p->skw_srcs[i];
    c->skw_gauss[i] = p->skw_gauss[i];
  }
  c->nside_base = p->nside_base;
  c->n_imap = p->n_imap;
  for (int i = 0; i < p->n_imap; i++) {
    c->imap_tz_arr[i] = p->imap_tz_arr[i];
    c->imap_bz_arr[i] = p->imap_bz_arr[i];
    c->nside_imap[i] = p->nside_imap[i];
    c->imap_nr[i] = p->imap_nr[i];
    c->imap_r0[i] = p->imap_r0[i];
    c->imap_rf[i] = p->imap_rf[i];
  }
  c->do_kappa = p->do_kappa;
  c->n_kappa = p->n_kappa;
  c->nside_kappa = p->nside_kappa;
  for (int i = 0; i < p->n_kappa; i++) c->kappa_r[i] = p->kappa_r[i];
  c->need_beaming = p->need_beaming;
  c->do_isw = p->do_isw;
  c->n_isw = p->n_isw;
  c->nside_isw = p->nside_isw;
  for (int i = 0; i < p->n_isw; i++) c->isw_r[i] = p->isw_r[i];
  return CG_OK;
}
