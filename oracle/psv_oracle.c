/*
 * psv_oracle.c -- CPU restatement of psvWave's solver (larsgeb/psvWave,
 * src/fdModel.cpp). TEST INFRASTRUCTURE ONLY: the checker of the GPU library
 * and the CPU baseline of bench.py; see psv_oracle.h.
 *
 * Every floating-point expression keeps the reference's operation order so
 * that, compiled with -ffp-contract=off (no fused multiply-add), results are
 * bit-identical to the reference's own double-precision code.
 */
#include "psv_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The reference's own constant for degrees->radians (src/fdModel.cpp:14). */
#define PO_PI 3.14159265
/* M_PI as the reference's Ricker wavelet uses it (src/fdModel.cpp:227). */
#define PO_M_PI 3.14159265358979323846

struct po_model {
  /* configuration (src/fdModel.h:262-302) */
  int nt, nx_inner, nz_inner, nx_inner_boundary, nz_inner_boundary;
  double dx, dz, dt;
  int np_boundary;
  double np_factor, scalar_rho, scalar_vp, scalar_vs;
  int npx, npz;
  double peak_frequency, t0, delay_cycles_per_shot, alpha;
  int n_sources, n_shots, nr, snapshot_interval, snapshots;
  int nx, nz, nx_free, nz_free, free_parameters;
  int *ix_sources, *iz_sources, *ix_receivers, *iz_receivers;
  double *moment_angles;
  int *shot_offsets, *shot_sources;
  double misfit;
  /* arrays (src/fdModel.h:209-252) */
  double *vx, *vz, *txx, *tzz, *txz;
  double *lm, *la, *mu, *b_vx, *b_vz, *rho, *vp, *vs;
  double *lambda_kernel, *mu_kernel, *density_l_kernel;
  double *vp_kernel, *vs_kernel, *density_v_kernel;
  double *taper, *t, *stf, *moment;
  double *rtf_ux, *rtf_uz, *rtf_ux_true, *rtf_uz_true, *a_stf_ux, *a_stf_uz;
  double *accu_vx, *accu_vz, *accu_txx, *accu_tzz, *accu_txz;
};

static const double C1 = 9.0 / 8.0;  /* src/fdModel.h:201 */
static const double C2 = 1.0 / 24.0; /* src/fdModel.h:202 */

static void set_err(char *err, int errlen, const char *msg) {
  if (err && errlen > 0) {
    strncpy(err, msg, (size_t)errlen - 1);
    err[errlen - 1] = 0;
  }
}

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* ---------------------------------------------------------------- setup -- */

/* allocate_memory + initialize_arrays (src/fdModel.cpp:139-299). */
static void po_setup(po_model *m) {
  size_t g = (size_t)m->nx * m->nz;
  size_t rec = (size_t)m->n_shots * m->nr * m->nt;
  size_t accu = (size_t)m->n_shots * m->snapshots * g;
  double **grid[] = {&m->vx, &m->vz, &m->txx, &m->tzz, &m->txz, &m->lm, &m->la,
                     &m->mu, &m->b_vx, &m->b_vz, &m->rho, &m->vp, &m->vs,
                     &m->lambda_kernel, &m->mu_kernel, &m->density_l_kernel,
                     &m->vp_kernel, &m->vs_kernel, &m->density_v_kernel, &m->taper};
  for (size_t i = 0; i < sizeof(grid) / sizeof(grid[0]); ++i) *grid[i] = zalloc(g);
  m->t = zalloc((size_t)m->nt);
  m->stf = zalloc((size_t)m->n_sources * m->nt);
  m->moment = zalloc((size_t)m->n_sources * 4);
  double **recs[] = {&m->rtf_ux, &m->rtf_uz, &m->rtf_ux_true, &m->rtf_uz_true,
                     &m->a_stf_ux, &m->a_stf_uz};
  for (size_t i = 0; i < 6; ++i) *recs[i] = zalloc(rec);
  double **acc[] = {&m->accu_vx, &m->accu_vz, &m->accu_txx, &m->accu_tzz, &m->accu_txz};
  for (size_t i = 0; i < 5; ++i) *acc[i] = zalloc(accu);
}

static void po_initialize(po_model *m) {
  int nx = m->nx, nz = m->nz;
  /* Shift sources/receivers into the padded grid (src/fdModel.cpp:197-212). */
  for (int ir = 0; ir < m->nr; ++ir) {
    m->ix_receivers[ir] += m->np_boundary;
    m->iz_receivers[ir] += m->np_boundary;
  }
  for (int is = 0; is < m->n_sources; ++is) {
    m->ix_sources[is] += m->np_boundary;
    m->iz_sources[is] += m->np_boundary;
  }
  /* Ricker wavelet per source, delayed by its position in the shot
   * (src/fdModel.cpp:215-231). */
  for (int shot = 0; shot < m->n_shots; ++shot) {
    for (int k = m->shot_offsets[shot]; k < m->shot_offsets[shot + 1]; ++k) {
      int pos = k - m->shot_offsets[shot];
      int src = m->shot_sources[k];
      for (int it = 0; it < m->nt; ++it) {
        m->t[it] = (double)(unsigned)it * m->dt;
        double f = 1.0 / m->alpha;
        double shifted = m->t[it] - 1.4 / f - m->delay_cycles_per_shot * pos / f;
        double a = PO_M_PI * f * shifted;
        m->stf[(size_t)src * m->nt + it] = (1 - 2 * (a * a)) * exp(-(a * a));
      }
    }
  }
  /* Moment tensors of dip-rotated reverse faults (src/fdModel.cpp:234-246). */
  for (int is = 0; is < m->n_sources; ++is) {
    double r = m->moment_angles[is] * PO_PI / 180.0;
    m->moment[is * 4 + 0] = cos(r) * 1e15;
    m->moment[is * 4 + 1] = -sin(r) * 1e15;
    m->moment[is * 4 + 2] = -sin(r) * 1e15;
    m->moment[is * 4 + 3] = -cos(r) * 1e15;
  }
  /* Homogeneous background medium (src/fdModel.cpp:249-261). */
  for (size_t i = 0; i < (size_t)nx * nz; ++i) {
    m->vp[i] = m->scalar_vp;
    m->vs[i] = m->scalar_vs;
    m->rho[i] = m->scalar_rho;
  }
  po_update_from_velocity(m);
  /* Cerjan taper: count the nested frames that contain each point, then
   * exp(-(factor*(np-count))^2) (src/fdModel.cpp:264-298). */
  for (int id = 0; id < m->np_boundary; ++id)
    for (int ix = id; ix < nx - id; ++ix)
      for (int iz = id; iz < nz - id; ++iz) m->taper[(size_t)ix * nz + iz] += 1.0;
  for (size_t i = 0; i < (size_t)nx * nz; ++i) {
    double a = m->np_factor * (m->np_boundary - m->taper[i]);
    m->taper[i] = exp(-(a * a));
  }
}

/* parse_parameters (src/fdModel.cpp:390-468). */
static po_model *po_build(const po_params *p, char *err, int errlen) {
  if (p->nt <= 0 || p->snapshot_interval <= 0 || p->npx <= 0 || p->npz <= 0) {
    set_err(err, errlen, "nt, snapshot_interval, npx and npz must be positive");
    return NULL;
  }
  po_model *m = (po_model *)calloc(1, sizeof(po_model));
  m->nt = p->nt;
  m->nx_inner = p->nx_inner;
  m->nz_inner = p->nz_inner;
  m->nx_inner_boundary = p->nx_inner_boundary;
  m->nz_inner_boundary = p->nz_inner_boundary;
  m->dx = p->dx;
  m->dz = p->dz;
  m->dt = p->dt;
  m->np_boundary = p->np_boundary;
  m->np_factor = p->np_factor;
  m->scalar_rho = p->scalar_rho;
  m->scalar_vp = p->scalar_vp;
  m->scalar_vs = p->scalar_vs;
  m->npx = p->npx;
  m->npz = p->npz;
  m->peak_frequency = p->peak_frequency;
  m->t0 = p->source_timeshift;
  m->delay_cycles_per_shot = p->delay_cycles_per_shot;
  m->n_sources = p->n_sources;
  m->n_shots = p->n_shots;
  m->nr = p->nr;
  m->snapshot_interval = p->snapshot_interval;
  m->nx = m->nx_inner + 2 * m->np_boundary;
  m->nz = m->nz_inner + 2 * m->np_boundary;
  m->nx_free = m->nx_inner - 2 * m->nx_inner_boundary;
  m->nz_free = m->nz_inner - 2 * m->nz_inner_boundary;
  if (m->nx_free % m->npx || m->nz_free % m->npz) {
    set_err(err, errlen, "free-parameter region is not divisible by the basis size");
    free(m);
    return NULL;
  }
  m->free_parameters = 3 * m->nx_free * m->nz_free / (m->npx * m->npz);
  int total = p->shot_offsets[p->n_shots];
  if (total != m->n_sources) {
    set_err(err, errlen, "Mismatch between n_sources and sources.which_source_to_fire_in_which_shot.");
    free(m);
    return NULL;
  }
  m->ix_sources = (int *)malloc(sizeof(int) * (m->n_sources + 1));
  m->iz_sources = (int *)malloc(sizeof(int) * (m->n_sources + 1));
  m->moment_angles = (double *)malloc(sizeof(double) * (m->n_sources + 1));
  memcpy(m->ix_sources, p->ix_sources, sizeof(int) * m->n_sources);
  memcpy(m->iz_sources, p->iz_sources, sizeof(int) * m->n_sources);
  memcpy(m->moment_angles, p->moment_angles, sizeof(double) * m->n_sources);
  m->shot_offsets = (int *)malloc(sizeof(int) * (m->n_shots + 1));
  memcpy(m->shot_offsets, p->shot_offsets, sizeof(int) * (m->n_shots + 1));
  m->shot_sources = (int *)malloc(sizeof(int) * (total + 1));
  memcpy(m->shot_sources, p->shot_sources, sizeof(int) * total);
  m->ix_receivers = (int *)malloc(sizeof(int) * (m->nr + 1));
  m->iz_receivers = (int *)malloc(sizeof(int) * (m->nr + 1));
  memcpy(m->ix_receivers, p->ix_receivers, sizeof(int) * m->nr);
  memcpy(m->iz_receivers, p->iz_receivers, sizeof(int) * m->nr);
  m->alpha = 1.0 / m->peak_frequency;
  m->snapshots = m->nt / m->snapshot_interval;
  if (m->nt % m->snapshot_interval) {
    set_err(err, errlen, "Snapshot interval and size of accumulator don't match!");
    po_destroy(m);
    return NULL;
  }
  po_setup(m);
  po_initialize(m);
  return m;
}

po_model *po_create(const po_params *p, char *err, int errlen) {
  return po_build(p, err, errlen);
}

/* ------------------------------------------------------- INI parsing ---- */
/* inih-compatible reading of the keys src/fdModel.cpp:482-518 asks for:
 * '[section]' headers, 'name = value' pairs, ';'/'#' comment lines and ';'
 * inline comments that follow whitespace; case-insensitive names. */

typedef struct {
  char key[128];
  char value[2048];
} po_kv;

static void strip(char *s) {
  size_t n = strlen(s), a = 0;
  while (n && isspace((unsigned char)s[n - 1])) s[--n] = 0;
  while (s[a] && isspace((unsigned char)s[a])) ++a;
  if (a) memmove(s, s + a, n - a + 1);
}

static char *scan_stop(char *s, const char *stops) {
  int was_space = 0;
  for (; *s; ++s) {
    if (stops && strchr(stops, *s)) return s;
    if (was_space && *s == ';') return s;
    was_space = isspace((unsigned char)*s) != 0;
  }
  return s;
}

static int ini_read(const char *path, po_kv **out, int *n_out) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char line[4096], section[128] = "";
  int cap = 64, n = 0, lineno = 0, error = 0;
  po_kv *kv = (po_kv *)calloc((size_t)cap, sizeof(po_kv));
  while (fgets(line, sizeof line, f)) {
    ++lineno;
    strip(line);
    if (!line[0] || line[0] == ';' || line[0] == '#') continue;
    if (line[0] == '[') {
      char *e = scan_stop(line + 1, "]");
      if (*e == ']') {
        *e = 0;
        snprintf(section, sizeof section, "%s", line + 1);
        strip(section);
      } else if (!error) {
        error = lineno;
      }
      continue;
    }
    char *e = scan_stop(line, "=:");
    if (*e != '=' && *e != ':') {
      if (!error) error = lineno;
      continue;
    }
    *e = 0;
    char *name = line, *value = e + 1;
    strip(name);
    strip(value);
    *scan_stop(value, NULL) = 0;
    strip(value);
    if (n == cap) {
      cap *= 2;
      kv = (po_kv *)realloc(kv, sizeof(po_kv) * (size_t)cap);
    }
    snprintf(kv[n].key, sizeof kv[n].key, "%s=%s", section, name);
    for (char *c = kv[n].key; *c; ++c) *c = (char)tolower((unsigned char)*c);
    snprintf(kv[n].value, sizeof kv[n].value, "%s", value);
    ++n;
  }
  fclose(f);
  *out = kv;
  *n_out = n;
  return error;
}

static const char *ini_get(po_kv *kv, int n, const char *sec, const char *name) {
  char key[128];
  snprintf(key, sizeof key, "%s=%s", sec, name);
  for (char *c = key; *c; ++c) *c = (char)tolower((unsigned char)*c);
  for (int i = 0; i < n; ++i)
    if (!strcmp(kv[i].key, key)) return kv[i].value;
  return "";
}

static long ini_int(po_kv *kv, int n, const char *sec, const char *name) {
  const char *v = ini_get(kv, n, sec, name);
  char *end;
  long x = strtol(v, &end, 0);
  return end > v ? x : 0;
}

static double ini_real(po_kv *kv, int n, const char *sec, const char *name) {
  const char *v = ini_get(kv, n, sec, name);
  char *end;
  double x = strtod(v, &end);
  return end > v ? x : 0.0;
}

/* parse_string_to_vector (src/fdModel.cpp:1574-1599): drop whitespace, keep
 * what lies between the first character and the first '}', split on ','
 * and read each token with atof. */
static int parse_list(const char *s, double *out, int cap) {
  char buf[2048];
  int k = 0;
  for (const char *c = s; *c && k < (int)sizeof buf - 1; ++c)
    if (!isspace((unsigned char)*c)) buf[k++] = *c;
  buf[k] = 0;
  char *close = strchr(buf, '}');
  if (close) *close = 0;
  char *p = buf[0] ? buf + 1 : buf;
  int n = 0;
  for (;;) {
    char *comma = strchr(p, ',');
    if (comma) *comma = 0;
    if (n < cap) out[n] = atof(p);
    ++n;
    if (!comma) break;
    p = comma + 1;
  }
  return n;
}

/* parse_string_to_nested_int_vector (src/fdModel.cpp:1601-1659): drop
 * whitespace and the leading "{{", split groups on "},{", the last group
 * ends at "}};" (or runs to the end), items are read with atof. */
static int parse_nested(const char *s, int *offsets, int *items, int cap_groups, int cap_items) {
  char buf[2048];
  int k = 0;
  for (const char *c = s; *c && k < (int)sizeof buf - 1; ++c)
    if (!isspace((unsigned char)*c)) buf[k++] = *c;
  buf[k] = 0;
  char *p = strlen(buf) >= 2 ? buf + 2 : buf + strlen(buf);
  int groups = 0, n = 0;
  offsets[0] = 0;
  for (;;) {
    char *sep = strstr(p, "},{");
    char *end = sep;
    if (!sep) {
      end = strstr(p, "}};");
      if (!end) end = p + strlen(p);
    }
    char save = *end;
    *end = 0;
    char *q = p;
    for (;;) {
      char *comma = strchr(q, ',');
      if (comma) *comma = 0;
      if (n < cap_items) items[n] = (int)atof(q);
      ++n;
      if (!comma) break;
      q = comma + 1;
    }
    *end = save;
    ++groups;
    if (groups <= cap_groups) offsets[groups] = n;
    if (!sep) break;
    p = sep + 3;
  }
  return groups;
}

po_model *po_create_from_ini(const char *path, char *err, int errlen) {
  po_kv *kv = NULL;
  int n = 0;
  if (ini_read(path, &kv, &n) < 0) {
    set_err(err, errlen, "Can't load .ini file.");
    return NULL;
  }
  po_params p;
  memset(&p, 0, sizeof p);
  p.nt = (int)ini_int(kv, n, "domain", "nt");
  p.nx_inner = (int)ini_int(kv, n, "domain", "nx_inner");
  p.nz_inner = (int)ini_int(kv, n, "domain", "nz_inner");
  p.nx_inner_boundary = (int)ini_int(kv, n, "domain", "nx_inner_boundary");
  p.nz_inner_boundary = (int)ini_int(kv, n, "domain", "nz_inner_boundary");
  p.dx = ini_real(kv, n, "domain", "dx");
  p.dz = ini_real(kv, n, "domain", "dz");
  p.dt = ini_real(kv, n, "domain", "dt");
  p.np_boundary = (int)ini_int(kv, n, "boundary", "np_boundary");
  p.np_factor = ini_real(kv, n, "boundary", "np_factor");
  p.scalar_rho = ini_real(kv, n, "medium", "scalar_rho");
  p.scalar_vp = ini_real(kv, n, "medium", "scalar_vp");
  p.scalar_vs = ini_real(kv, n, "medium", "scalar_vs");
  p.npx = (int)ini_int(kv, n, "basis", "npx");
  p.npz = (int)ini_int(kv, n, "basis", "npz");
  p.peak_frequency = ini_real(kv, n, "sources", "peak_frequency");
  p.source_timeshift = ini_real(kv, n, "sources", "source_timeshift");
  p.delay_cycles_per_shot = ini_real(kv, n, "sources", "delay_cycles_per_shot");
  p.n_sources = (int)ini_int(kv, n, "sources", "n_sources");
  p.n_shots = (int)ini_int(kv, n, "sources", "n_shots");
  p.nr = (int)ini_int(kv, n, "receivers", "nr");
  p.snapshot_interval = (int)ini_int(kv, n, "inversion", "snapshot_interval");

  enum { CAP = 4096 };
  static double tmp[CAP];
  int *ixs = (int *)calloc(CAP, sizeof(int)), *izs = (int *)calloc(CAP, sizeof(int));
  int *ixr = (int *)calloc(CAP, sizeof(int)), *izr = (int *)calloc(CAP, sizeof(int));
  double *ang = (double *)calloc(CAP, sizeof(double));
  int *offs = (int *)calloc(CAP + 1, sizeof(int)), *items = (int *)calloc(CAP, sizeof(int));
  int nixs = parse_list(ini_get(kv, n, "sources", "ix_sources"), tmp, CAP);
  for (int i = 0; i < nixs && i < CAP; ++i) ixs[i] = (int)tmp[i];
  int nizs = parse_list(ini_get(kv, n, "sources", "iz_sources"), tmp, CAP);
  for (int i = 0; i < nizs && i < CAP; ++i) izs[i] = (int)tmp[i];
  int nang = parse_list(ini_get(kv, n, "sources", "moment_angles"), ang, CAP);
  int ngroups = parse_nested(ini_get(kv, n, "sources", "which_source_to_fire_in_which_shot"),
                             offs, items, CAP, CAP);
  int nixr = parse_list(ini_get(kv, n, "receivers", "ix_receivers"), tmp, CAP);
  for (int i = 0; i < nixr && i < CAP; ++i) ixr[i] = (int)tmp[i];
  int nizr = parse_list(ini_get(kv, n, "receivers", "iz_receivers"), tmp, CAP);
  for (int i = 0; i < nizr && i < CAP; ++i) izr[i] = (int)tmp[i];
  free(kv);

  po_model *m = NULL;
  if (nixs != p.n_sources || nizs != p.n_sources || nang != p.n_sources) {
    set_err(err, errlen,
            "Dimension mismatch between n_sources and sources.ix_sources, "
            "sources.iz_sources or sources.moment_angles");
  } else if (ngroups != p.n_shots) {
    set_err(err, errlen, "Mismatch between n_shots and sources.which_source_to_fire_in_which_shot");
  } else if (nixr != p.nr || nizr != p.nr) {
    set_err(err, errlen, "Mismatch between nr and receivers.ix_receivers or receivers.iz_receivers");
  } else {
    p.ix_sources = ixs;
    p.iz_sources = izs;
    p.moment_angles = ang;
    p.shot_offsets = offs;
    p.shot_sources = items;
    p.ix_receivers = ixr;
    p.iz_receivers = izr;
    m = po_build(&p, err, errlen);
  }
  free(ixs);
  free(izs);
  free(ixr);
  free(izr);
  free(ang);
  free(offs);
  free(items);
  return m;
}

po_model *po_copy(const po_model *s) {
  po_params p;
  memset(&p, 0, sizeof p);
  p.nt = s->nt;
  p.nx_inner = s->nx_inner;
  p.nz_inner = s->nz_inner;
  p.nx_inner_boundary = s->nx_inner_boundary;
  p.nz_inner_boundary = s->nz_inner_boundary;
  p.dx = s->dx;
  p.dz = s->dz;
  p.dt = s->dt;
  p.np_boundary = s->np_boundary;
  p.np_factor = s->np_factor;
  p.scalar_rho = s->scalar_rho;
  p.scalar_vp = s->scalar_vp;
  p.scalar_vs = s->scalar_vs;
  p.npx = s->npx;
  p.npz = s->npz;
  p.peak_frequency = s->peak_frequency;
  p.source_timeshift = s->t0;
  p.delay_cycles_per_shot = s->delay_cycles_per_shot;
  p.n_sources = s->n_sources;
  p.n_shots = s->n_shots;
  p.nr = s->nr;
  p.snapshot_interval = s->snapshot_interval;
  /* Undo the np shift; po_initialize re-applies it. */
  int *ixs = (int *)malloc(sizeof(int) * (s->n_sources + 1));
  int *izs = (int *)malloc(sizeof(int) * (s->n_sources + 1));
  int *ixr = (int *)malloc(sizeof(int) * (s->nr + 1));
  int *izr = (int *)malloc(sizeof(int) * (s->nr + 1));
  for (int i = 0; i < s->n_sources; ++i) {
    ixs[i] = s->ix_sources[i] - s->np_boundary;
    izs[i] = s->iz_sources[i] - s->np_boundary;
  }
  for (int i = 0; i < s->nr; ++i) {
    ixr[i] = s->ix_receivers[i] - s->np_boundary;
    izr[i] = s->iz_receivers[i] - s->np_boundary;
  }
  p.ix_sources = ixs;
  p.iz_sources = izs;
  p.moment_angles = s->moment_angles;
  p.shot_offsets = s->shot_offsets;
  p.shot_sources = s->shot_sources;
  p.ix_receivers = ixr;
  p.iz_receivers = izr;
  po_model *m = po_build(&p, NULL, 0);
  free(ixs);
  free(izs);
  free(ixr);
  free(izr);
  if (!m) return NULL;
  /* copy_arrays (src/fdModel.cpp:301-388): every array follows the source. */
  size_t g = (size_t)m->nx * m->nz, rec = (size_t)m->n_shots * m->nr * m->nt;
  size_t accu = (size_t)m->n_shots * m->snapshots * g;
  const char *gn[] = {"vx", "vz", "txx", "tzz", "txz", "lm", "la", "mu", "b_vx", "b_vz",
                      "rho", "vp", "vs", "lambda_kernel", "mu_kernel", "density_l_kernel",
                      "vp_kernel", "vs_kernel", "density_v_kernel", "taper"};
  for (size_t i = 0; i < sizeof(gn) / sizeof(gn[0]); ++i)
    memcpy(po_array(m, gn[i]), po_array((po_model *)s, gn[i]), g * sizeof(double));
  const char *rn[] = {"rtf_ux", "rtf_uz", "rtf_ux_true", "rtf_uz_true", "a_stf_ux", "a_stf_uz"};
  for (size_t i = 0; i < 6; ++i)
    memcpy(po_array(m, rn[i]), po_array((po_model *)s, rn[i]), rec * sizeof(double));
  const char *an[] = {"accu_vx", "accu_vz", "accu_txx", "accu_tzz", "accu_txz"};
  for (size_t i = 0; i < 5; ++i)
    memcpy(po_array(m, an[i]), po_array((po_model *)s, an[i]), accu * sizeof(double));
  memcpy(m->stf, s->stf, sizeof(double) * (size_t)m->n_sources * m->nt);
  memcpy(m->moment, s->moment, sizeof(double) * (size_t)m->n_sources * 4);
  m->misfit = s->misfit;
  return m;
}

void po_destroy(po_model *m) {
  if (!m) return;
  void *ptrs[] = {m->vx, m->vz, m->txx, m->tzz, m->txz, m->lm, m->la, m->mu, m->b_vx,
                  m->b_vz, m->rho, m->vp, m->vs, m->lambda_kernel, m->mu_kernel,
                  m->density_l_kernel, m->vp_kernel, m->vs_kernel, m->density_v_kernel,
                  m->taper, m->t, m->stf, m->moment, m->rtf_ux, m->rtf_uz, m->rtf_ux_true,
                  m->rtf_uz_true, m->a_stf_ux, m->a_stf_uz, m->accu_vx, m->accu_vz,
                  m->accu_txx, m->accu_tzz, m->accu_txz, m->ix_sources, m->iz_sources,
                  m->ix_receivers, m->iz_receivers, m->moment_angles, m->shot_offsets,
                  m->shot_sources};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  free(m);
}

void po_info(const po_model *m, int *o) {
  int v[18] = {m->nt, m->nx, m->nz, m->nx_inner, m->nz_inner, m->nx_inner_boundary,
               m->nz_inner_boundary, m->np_boundary, m->n_shots, m->n_sources, m->nr,
               m->snapshot_interval, m->snapshots, m->nx_free, m->nz_free,
               m->free_parameters, m->npx, m->npz};
  memcpy(o, v, sizeof v);
}

void po_scalars(const po_model *m, double *o) {
  double v[8] = {m->dt, m->dx, m->dz, m->np_factor, m->peak_frequency, m->alpha,
                 m->delay_cycles_per_shot, m->misfit};
  memcpy(o, v, sizeof v);
}

double *po_array(po_model *m, const char *n) {
#define PO_NAMED(x) if (!strcmp(n, #x)) return m->x;
  PO_NAMED(vx) PO_NAMED(vz) PO_NAMED(txx) PO_NAMED(tzz) PO_NAMED(txz)
  PO_NAMED(lm) PO_NAMED(la) PO_NAMED(mu) PO_NAMED(b_vx) PO_NAMED(b_vz)
  PO_NAMED(rho) PO_NAMED(vp) PO_NAMED(vs) PO_NAMED(taper) PO_NAMED(stf)
  PO_NAMED(moment) PO_NAMED(rtf_ux) PO_NAMED(rtf_uz) PO_NAMED(rtf_ux_true)
  PO_NAMED(rtf_uz_true) PO_NAMED(a_stf_ux) PO_NAMED(a_stf_uz)
  PO_NAMED(lambda_kernel) PO_NAMED(mu_kernel) PO_NAMED(density_l_kernel)
  PO_NAMED(vp_kernel) PO_NAMED(vs_kernel) PO_NAMED(density_v_kernel)
  PO_NAMED(accu_vx) PO_NAMED(accu_vz) PO_NAMED(accu_txx) PO_NAMED(accu_tzz)
  PO_NAMED(accu_txz)
#undef PO_NAMED
  return NULL;
}

int *po_int_array(po_model *m, const char *n) {
  if (!strcmp(n, "ix_sources")) return m->ix_sources;
  if (!strcmp(n, "iz_sources")) return m->iz_sources;
  if (!strcmp(n, "ix_receivers")) return m->ix_receivers;
  if (!strcmp(n, "iz_receivers")) return m->iz_receivers;
  return NULL;
}

/* ------------------------------------------------------------- solver -- */

/* update_from_velocity (src/fdModel.cpp:1034-1051). */
void po_update_from_velocity(po_model *m) {
  long n = (long)m->nx * m->nz;
#pragma omp parallel for
  for (long i = 0; i < n; ++i) {
    m->mu[i] = (m->vs[i] * m->vs[i]) * m->rho[i];
    m->lm[i] = (m->vp[i] * m->vp[i]) * m->rho[i];
    m->la[i] = m->lm[i] - 2 * m->mu[i];
    m->b_vx[i] = 1.0 / m->rho[i];
    m->b_vz[i] = m->b_vx[i];
  }
}

/* One stress half-step over ix,iz in [2, n-2) (src/fdModel.cpp:599-644, and
 * with sgn = -1 the reverse-time form of src/fdModel.cpp:864-911). */
static void stress_step(po_model *m, double sgn) {
  const int nx = m->nx, nz = m->nz;
  const double dx = m->dx, dz = m->dz, dt = m->dt;
  double *vx = m->vx, *vz = m->vz, *txx = m->txx, *tzz = m->tzz, *txz = m->txz;
  const double *lm = m->lm, *la = m->la, *mu = m->mu, *tp = m->taper;
#pragma omp parallel for collapse(2)
  for (int ix = 2; ix < nx - 2; ++ix) {
    for (int iz = 2; iz < nz - 2; ++iz) {
      long i = (long)ix * nz + iz;
      long xp1 = i + nz, xp2 = i + 2 * nz, xm1 = i - nz, xm2 = i - 2 * nz;
      long zp1 = i + 1, zp2 = i + 2, zm1 = i - 1, zm2 = i - 2;
      double dvx = C1 * (vx[xp1] - vx[i]) + C2 * (vx[xm1] - vx[xp2]);
      double dvz = C1 * (vz[i] - vz[zm1]) + C2 * (vz[zm2] - vz[zp1]);
      double sxx = lm[i] * dvx / dx + la[i] * dvz / dz;
      double szz = la[i] * dvx / dx + lm[i] * dvz / dz;
      double sxz = (C1 * (vx[zp1] - vx[i]) + C2 * (vx[zm1] - vx[zp2])) / dz +
                   (C1 * (vz[i] - vz[xm1]) + C2 * (vz[xm2] - vz[xp1])) / dx;
      if (sgn > 0) {
        txx[i] = tp[i] * (txx[i] + dt * sxx);
        tzz[i] = tp[i] * (tzz[i] + dt * szz);
        txz[i] = tp[i] * (txz[i] + dt * mu[i] * sxz);
      } else {
        txx[i] = tp[i] * (txx[i] - dt * sxx);
        tzz[i] = tp[i] * (tzz[i] - dt * szz);
        txz[i] = tp[i] * (txz[i] - dt * mu[i] * sxz);
      }
    }
  }
}

/* One velocity half-step (src/fdModel.cpp:646-678; reverse time :913-948). */
static void velocity_step(po_model *m, double sgn) {
  const int nx = m->nx, nz = m->nz;
  const double dx = m->dx, dz = m->dz, dt = m->dt;
  double *vx = m->vx, *vz = m->vz, *txx = m->txx, *tzz = m->tzz, *txz = m->txz;
  const double *bx = m->b_vx, *bz = m->b_vz, *tp = m->taper;
#pragma omp parallel for collapse(2)
  for (int ix = 2; ix < nx - 2; ++ix) {
    for (int iz = 2; iz < nz - 2; ++iz) {
      long i = (long)ix * nz + iz;
      long xp1 = i + nz, xp2 = i + 2 * nz, xm1 = i - nz, xm2 = i - 2 * nz;
      long zp1 = i + 1, zp2 = i + 2, zm1 = i - 1, zm2 = i - 2;
      double ax = (C1 * (txx[i] - txx[xm1]) + C2 * (txx[xm2] - txx[xp1])) / dx +
                  (C1 * (txz[i] - txz[zm1]) + C2 * (txz[zm2] - txz[zp1])) / dz;
      double az = (C1 * (txz[xp1] - txz[i]) + C2 * (txz[xm1] - txz[xp2])) / dx +
                  (C1 * (tzz[zp1] - tzz[i]) + C2 * (tzz[zm1] - tzz[zp2])) / dz;
      if (sgn > 0) {
        vx[i] = tp[i] * (vx[i] + bx[i] * dt * ax);
        vz[i] = tp[i] * (vz[i] + bz[i] * dt * az);
      } else {
        vx[i] = tp[i] * (vx[i] - bx[i] * dt * ax);
        vz[i] = tp[i] * (vz[i] - bz[i] * dt * az);
      }
    }
  }
}

/* Moment-tensor injection of every source of the shot, serially and in the
 * reference's order (src/fdModel.cpp:681-751). */
static void inject_sources(po_model *m, int shot, int it) {
  const int nz = m->nz, nt = m->nt;
  const double dx = m->dx, dz = m->dz, dt = m->dt;
  const double dx4 = dx * dx * dx * dx, dz4 = dz * dz * dz * dz;
  double *vx = m->vx, *vz = m->vz;
  const double *b = m->b_vz;
  for (int k = m->shot_offsets[shot]; k < m->shot_offsets[shot + 1]; ++k) {
    int s = m->shot_sources[k];
    double stf = m->stf[(long)s * nt + it];
    const double *M = m->moment + 4 * s;
    long c = (long)m->ix_sources[s] * nz + m->iz_sources[s];
    long xm1 = c - nz, xp1 = c + nz, zm1 = c - 1, zp1 = c + 1;
    long xp1zm1 = c + nz - 1, xm1zp1 = c - nz + 1, xm1zm1 = c - nz - 1;
    vx[xm1] -= M[0] * stf * dt * b[xm1] / dx4;
    vx[c] += M[0] * stf * dt * b[c] / dx4;
    vz[zm1] -= M[3] * stf * dt * b[zm1] / dz4;
    vz[c] += M[3] * stf * dt * b[c] / dz4;
    vx[xm1zp1] += 0.25 * M[1] * stf * dt * b[xm1zp1] / dx4;
    vx[zp1] += 0.25 * M[1] * stf * dt * b[zp1] / dx4;
    vx[xm1zm1] -= 0.25 * M[1] * stf * dt * b[xm1zm1] / dx4;
    vx[zm1] -= 0.25 * M[1] * stf * dt * b[zm1] / dx4;
    vz[xp1zm1] += 0.25 * M[2] * stf * dt * b[xp1zm1] / dz4;
    vz[xp1] += 0.25 * M[2] * stf * dt * b[xp1] / dz4;
    vz[xm1zm1] -= 0.25 * M[2] * stf * dt * b[xm1zm1] / dz4;
    vz[xm1] -= 0.25 * M[2] * stf * dt * b[xm1] / dz4;
  }
}

void po_forward_steps(po_model *m, int shot, int store, int n_steps) {
  const long g = (long)m->nx * m->nz;
  const int nt = m->nt, nr = m->nr, si = m->snapshot_interval;
  /* Zero the wavefields (src/fdModel.cpp:530-542). */
  memset(m->vx, 0, g * sizeof(double));
  memset(m->vz, 0, g * sizeof(double));
  memset(m->txx, 0, g * sizeof(double));
  memset(m->tzz, 0, g * sizeof(double));
  memset(m->txz, 0, g * sizeof(double));
  for (int it = 0; it < n_steps; ++it) {
    /* Snapshot of the pre-step state (src/fdModel.cpp:555-572). */
    if (it % si == 0 && store) {
      long off = ((long)shot * m->snapshots + it / si) * g;
      memcpy(m->accu_vx + off, m->vx, g * sizeof(double));
      memcpy(m->accu_vz + off, m->vz, g * sizeof(double));
      memcpy(m->accu_txx + off, m->txx, g * sizeof(double));
      memcpy(m->accu_txz + off, m->txz, g * sizeof(double));
      memcpy(m->accu_tzz + off, m->tzz, g * sizeof(double));
    }
    /* Displacement seismograms from the pre-step velocities
     * (src/fdModel.cpp:576-596). */
    for (int r = 0; r < nr; ++r) {
      long ir = ((long)shot * nr + r) * nt + it;
      long loc = (long)m->ix_receivers[r] * m->nz + m->iz_receivers[r];
      if (it == 0) {
        m->rtf_ux[ir] = m->dt * m->vx[loc] / (m->dx * m->dz);
        m->rtf_uz[ir] = m->dt * m->vz[loc] / (m->dx * m->dz);
      } else {
        m->rtf_ux[ir] = m->rtf_ux[ir - 1] + m->dt * m->vx[loc] / (m->dx * m->dz);
        m->rtf_uz[ir] = m->rtf_uz[ir - 1] + m->dt * m->vz[loc] / (m->dx * m->dz);
      }
    }
    stress_step(m, 1.0);
    velocity_step(m, 1.0);
    inject_sources(m, shot, it);
  }
}

void po_forward(po_model *m, int shot, int store) { po_forward_steps(m, shot, store, m->nt); }

/* Snapshot correlation for the Lame/density kernels over the free region
 * (src/fdModel.cpp:817-861); the a* values are the stored forward state. */
static void correlate(po_model *m, int shot, int it) {
  const int nz = m->nz, si = m->snapshot_interval;
  const long g = (long)m->nx * nz;
  const long off = ((long)shot * m->snapshots + it / si) * g;
  const double dt = m->dt;
  const int x0 = m->np_boundary + m->nx_inner_boundary;
  const int x1 = m->np_boundary + m->nx_inner - m->nx_inner_boundary;
  const int z0 = m->np_boundary + m->nz_inner_boundary;
  const int z1 = m->np_boundary + m->nz_inner - m->nz_inner_boundary;
#pragma omp parallel for collapse(2)
  for (int ix = x0; ix < x1; ++ix) {
    for (int iz = z0; iz < z1; ++iz) {
      long i = (long)ix * nz + iz, a = off + i;
      double lm = m->lm[i], la = m->la[i], mu = m->mu[i];
      double atxx = m->accu_txx[a], atzz = m->accu_tzz[a], atxz = m->accu_txz[a];
      double txx = m->txx[i], tzz = m->tzz[i], txz = m->txz[i];
      double den = (lm - ((la * la) / (lm))) * (lm - ((la * la) / (lm)));
      m->density_l_kernel[i] -=
          si * dt * (m->accu_vx[a] * m->vx[i] + m->accu_vz[a] * m->vz[i]);
      m->lambda_kernel[i] +=
          si * dt *
          (((atxx - (atzz * la) / lm) + (atzz - (atxx * la) / lm)) *
           ((txx - (tzz * la) / lm) + (tzz - (txx * la) / lm))) /
          den;
      m->mu_kernel[i] +=
          si * dt * 2 *
          ((((txx - (tzz * la) / lm) * (atxx - (atzz * la) / lm)) +
            ((tzz - (txx * la) / lm) * (atzz - (atxx * la) / lm))) /
               den +
           2 * (txz * atxz / (4 * mu * mu)));
    }
  }
}

void po_adjoint(po_model *m, int shot) {
  const long g = (long)m->nx * m->nz;
  const int nt = m->nt, nr = m->nr, nz = m->nz;
  memset(m->vx, 0, g * sizeof(double));
  memset(m->vz, 0, g * sizeof(double));
  memset(m->txx, 0, g * sizeof(double));
  memset(m->tzz, 0, g * sizeof(double));
  memset(m->txz, 0, g * sizeof(double));
  for (int it = nt - 1; it >= 0; --it) {
    if (it % m->snapshot_interval == 0) correlate(m, shot, it);
    stress_step(m, -1.0);
    velocity_step(m, -1.0);
    /* Adjoint sources at the receivers (src/fdModel.cpp:951-958). */
    for (int r = 0; r < nr; ++r) {
      long loc = (long)m->ix_receivers[r] * nz + m->iz_receivers[r];
      long ir = ((long)shot * nr + r) * nt + it;
      m->vx[loc] += m->dt * m->b_vx[loc] * m->a_stf_ux[ir] / (m->dx * m->dz);
      m->vz[loc] += m->dt * m->b_vz[loc] * m->a_stf_uz[ir] / (m->dx * m->dz);
    }
  }
}

/* Serial L2 misfit (src/fdModel.cpp:1128-1145). */
double po_misfit(po_model *m) {
  long n = (long)m->n_shots * m->nr * m->nt;
  double misfit = 0;
  for (long i = 0; i < n; ++i) {
    double dx_ = m->rtf_ux_true[i] - m->rtf_ux[i];
    double dz_ = m->rtf_uz_true[i] - m->rtf_uz[i];
    misfit += 0.5 * m->dt * (dx_ * dx_);
    misfit += 0.5 * m->dt * (dz_ * dz_);
  }
  m->misfit = misfit;
  return misfit;
}

/* src/fdModel.cpp:1147-1162. */
void po_adjoint_sources(po_model *m) {
  long n = (long)m->n_shots * m->nr * m->nt;
#pragma omp parallel for
  for (long i = 0; i < n; ++i) {
    m->a_stf_ux[i] = m->rtf_ux[i] - m->rtf_ux_true[i];
    m->a_stf_uz[i] = m->rtf_uz[i] - m->rtf_uz_true[i];
  }
}

void po_reset_kernels(po_model *m) {
  size_t g = (size_t)m->nx * m->nz * sizeof(double);
  memset(m->lambda_kernel, 0, g);
  memset(m->mu_kernel, 0, g);
  memset(m->density_l_kernel, 0, g);
}

/* Lame -> velocity kernels (src/fdModel.cpp:1164-1183). */
void po_map_kernels(po_model *m) {
  long n = (long)m->nx * m->nz;
#pragma omp parallel for
  for (long i = 0; i < n; ++i) {
    double vp = m->vp[i], vs = m->vs[i], lk = m->lambda_kernel[i], mk = m->mu_kernel[i];
    m->vp_kernel[i] = 2 * vp * lk / m->b_vx[i];
    m->vs_kernel[i] = (2 * vs * mk - 4 * vs * lk) / m->b_vx[i];
    m->density_v_kernel[i] = m->density_l_kernel[i] + (vp * vp - 2 * vs * vs) * lk + vs * vs * mk;
  }
}

/* src/fdModel.cpp:1291-1308. */
void po_run_model(po_model *m, int adjoint) {
  for (int s = 0; s < m->n_shots; ++s) po_forward(m, s, 1);
  po_misfit(m);
  if (adjoint) {
    po_adjoint_sources(m);
    po_reset_kernels(m);
    for (int s = 0; s < m->n_shots; ++s) po_adjoint(m, s);
    po_map_kernels(m);
  }
}

/* Block basis over the free region; parameter index ix + iz*(nxf/npx)
 * (src/fdModel.cpp:1358-1515). */
void po_get_model_vector(const po_model *m, double *out) {
  int bx = m->nx_free / m->npx, bz = m->nz_free / m->npz, per = bx * bz;
  for (int ix = 0; ix < bx; ++ix)
    for (int iz = 0; iz < bz; ++iz) {
      int p = ix + iz * m->nx_free / m->npx;
      int gx = ix * m->npx + m->nx_inner_boundary + m->np_boundary;
      int gz = iz * m->npz + m->nz_inner_boundary + m->np_boundary;
      out[p] = out[p + per] = out[p + 2 * per] = 0;
      for (int sx = 0; sx < m->npx; ++sx)
        for (int sz = 0; sz < m->npz; ++sz) {
          long i = (long)(gx + sx) * m->nz + gz + sz;
          out[p] += m->vp[i] / (m->npx * m->npz);
          out[p + per] += m->vs[i] / (m->npx * m->npz);
          out[p + 2 * per] += m->rho[i] / (m->npx * m->npz);
        }
    }
}

void po_set_model_vector(po_model *m, const double *in) {
  int bx = m->nx_free / m->npx, bz = m->nz_free / m->npz, per = bx * bz;
  for (int ix = 0; ix < bx; ++ix)
    for (int iz = 0; iz < bz; ++iz) {
      int p = ix + iz * m->nx_free / m->npx;
      int gx = ix * m->npx + m->nx_inner_boundary + m->np_boundary;
      int gz = iz * m->npz + m->nz_inner_boundary + m->np_boundary;
      for (int sx = 0; sx < m->npx; ++sx)
        for (int sz = 0; sz < m->npz; ++sz) {
          long i = (long)(gx + sx) * m->nz + gz + sz;
          m->vp[i] = in[p];
          m->vs[i] = in[p + per];
          m->rho[i] = in[p + 2 * per];
        }
    }
  po_update_from_velocity(m);
}

void po_get_gradient_vector(const po_model *m, double *out) {
  int bx = m->nx_free / m->npx, bz = m->nz_free / m->npz, per = bx * bz;
  for (int ix = 0; ix < bx; ++ix)
    for (int iz = 0; iz < bz; ++iz) {
      int p = ix + iz * m->nx_free / m->npx;
      int gx = ix * m->npx + m->nx_inner_boundary + m->np_boundary;
      int gz = iz * m->npz + m->nz_inner_boundary + m->np_boundary;
      out[p] = out[p + per] = out[p + 2 * per] = 0;
      for (int sx = 0; sx < m->npx; ++sx)
        for (int sz = 0; sz < m->npz; ++sz) {
          long i = (long)(gx + sx) * m->nz + gz + sz;
          out[p] += m->vp_kernel[i];
          out[p + per] += m->vs_kernel[i];
          out[p + 2 * per] += m->density_v_kernel[i];
        }
    }
}
