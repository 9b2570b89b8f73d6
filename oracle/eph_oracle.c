/*
 * CPU restatement of the USER-EPH `fix eph` hot path.  TEST INFRASTRUCTURE
 * ONLY (parity checker and timed CPU baseline); see eph_oracle.h for the map
 * from functions to reference lines.  Compiled with -ffp-contract=off: every
 * expression below is written in the reference's evaluation order so that the
 * rounding is the reference's rounding on any host.
 */
#define _POSIX_C_SOURCE 200809L
#include "eph_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ spline */

/* eph_spline.h:31-132: Akima weights |d_{i+1}-d_i|, |d_{i-1}-d_{i-2}| with two
 * extrapolated slopes at each end, then the cubic of each interval rewritten
 * in absolute x. */
int orc_spline_build(orc_spline *s, double dx, const double *y, long points) {
  if (!(dx > 0) || points <= 3) return 1;
  s->inv_dx = 1. / dx;
  s->n = points;
  /* one zero knot past the end: the derivative loop of the reference reads
   * the slope of knot `points` (one past its table) at i = points-1; a zero
   * slope there reproduces its result unless that stray value equals z2 */
  s->c = (double *)calloc((size_t)(points + 1) * 4, sizeof(double));
  if (!s->c) return 1;
  double *c = s->c;
#define A(i) c[4 * (i) + 0]
#define B(i) c[4 * (i) + 1]
#define C(i) c[4 * (i) + 2]
#define D(i) c[4 * (i) + 3]
  double z0, z1, z2, z3;
  for (long i = 0; i < points - 1; ++i) B(i) = (y[i + 1] - y[i]) / dx;
  z1 = 2.0 * B(0) - B(1);
  z0 = 2.0 * z1 - B(0);
  z2 = 2.0 * B(points - 2) - B(points - 1);
  z3 = 2.0 * z2 - B(points - 1);
  B(points - 1) = z2;
  for (long i = 2; i < points - 2; ++i) {
    C(i) = fabs(B(i + 1) - B(i));
    D(i) = fabs(B(i - 1) - B(i - 2));
  }
  C(0) = fabs(B(1) - B(0));
  D(0) = fabs(z1 - z0);
  C(1) = fabs(B(2) - B(1));
  D(1) = fabs(B(0) - z1);
  C(points - 2) = fabs(z2 - B(points - 2));
  D(points - 2) = fabs(B(points - 3) - B(points - 4));
  C(points - 1) = fabs(z3 - z2);
  D(points - 1) = fabs(B(points - 2) - B(points - 3));
  for (long i = 0; i < points; ++i) {
    double w0, w1, d_2, d_1, d0, d1;
    if (i == 0) {
      d_2 = z0; d_1 = z1; d1 = B(i + 1);
    } else if (i == 1) {
      d_2 = z1; d_1 = B(i - 1); d1 = B(i + 1);
    } else {
      d_2 = B(i - 2); d_1 = B(i - 1); d1 = B(i + 1);
    }
    d0 = B(i); w1 = C(i); w0 = D(i);
    if (d_2 == d_1 && d0 != d1)
      A(i) = d_1;
    else if (d0 == d1 && d_2 == d_1)
      A(i) = d0;
    else if (d_1 == d0)
      A(i) = d0;
    else if (d_2 == d_1 && d0 == d1 && d0 != d_1)
      A(i) = 0.5 * (d_1 + d0);
    else
      A(i) = (d_1 * w1 + d0 * w0) / (w1 + w0);
  }
  for (long i = 0; i < points - 1; ++i) {
    /* size_t arithmetic promoted to double, as in the reference */
    double fi = (double)(size_t)i, fi1 = (double)(size_t)(i + 1);
    double dx3 = dx * dx * dx;
    double x0_1 = fi * dx;
    double x0_2 = fi * dx * x0_1;
    double x0_3 = fi * dx * x0_2;
    double x1_1 = fi1 * dx;
    double x1_2 = fi1 * dx * x1_1;
    double x1_3 = fi1 * dx * x1_2;
    D(i) = (-A(i) * x0_1 - A(i + 1) * x0_1 + A(i) * x1_1 + A(i + 1) * x1_1 + 2.0 * y[i] - 2.0 * y[i + 1]) / dx3;
    C(i) = (-A(i) + A(i + 1) + 3.0 * D(i) * x0_2 - 3.0 * D(i) * x1_2) / 2.0 / dx;
    B(i) = (C(i) * x0_2 + D(i) * x0_3 - C(i) * x1_2 - D(i) * x1_3 - y[i] + y[i + 1]) / dx;
    A(i) = y[i] - B(i) * x0_1 - C(i) * x0_2 - D(i) * x0_3;
  }
  A(points - 1) = y[points - 1];
  B(points - 1) = 0.0;
  C(points - 1) = 0.0;
  D(points - 1) = 0.0;
#undef A
#undef B
#undef C
#undef D
  return 0;
}

/* eph_spline.h:134-142 (no clamp: callers keep x inside the table) */
double orc_spline_eval(const orc_spline *s, double x) {
  size_t index = (size_t)(x * s->inv_dx);
  if (x < 0.0 || index >= (size_t)s->n) {
    fprintf(stderr, "orc_spline_eval: x=%g outside the table\n", x);
    abort();
  }
  const double *c = s->c + 4 * index;
  return c[0] + x * (c[1] + x * (c[2] + x * c[3]));
}

void orc_spline_free(orc_spline *s) {
  free(s->c);
  s->c = NULL;
}

/* -------------------------------------------------------------------- beta */

#define ORC_MAX_ELEM 16
struct orc_beta {
  int n_elements;
  char name[ORC_MAX_ELEM][32];
  int number[ORC_MAX_ELEM];
  double r_cutoff, r_cutoff_sq, rho_cutoff;
  orc_spline rho[ORC_MAX_ELEM], rho_r_sq[ORC_MAX_ELEM], beta[ORC_MAX_ELEM], alpha[ORC_MAX_ELEM];
  int warned;
};

/* eph_beta.h:39-128: three comment lines; "N name..." ; "Nrho dr Nbeta drho
 * rcut"; per element: Z, Nrho rho(r) knots, Nbeta beta(rho) knots. */
orc_beta *orc_beta_load(const char *path) {
  FILE *fd = fopen(path, "r");
  if (!fd) return NULL;
  orc_beta *b = (orc_beta *)calloc(1, sizeof(orc_beta));
  char line[1024];
  for (int k = 0; k < 3; ++k)
    if (!fgets(line, sizeof line, fd)) goto fail;
  if (!fgets(line, sizeof line, fd)) goto fail;
  {
    char *p = line;
    int used = 0;
    if (sscanf(p, "%d%n", &b->n_elements, &used) != 1 || b->n_elements < 1 || b->n_elements > ORC_MAX_ELEM)
      goto fail;
    p += used;
    for (int i = 0; i < b->n_elements; ++i) {
      if (sscanf(p, "%31s%n", b->name[i], &used) != 1) goto fail;
      p += used;
    }
  }
  long n_rho, n_beta;
  double dr, drho;
  if (fscanf(fd, "%ld %lf %ld %lf %lf", &n_rho, &dr, &n_beta, &drho, &b->r_cutoff) != 5) goto fail;
  b->r_cutoff_sq = b->r_cutoff * b->r_cutoff;
  b->rho_cutoff = drho * (double)(size_t)(n_beta - 1);
  double dr_sq = b->r_cutoff_sq / (double)(size_t)(n_rho - 1);
  double *buf = (double *)malloc(sizeof(double) * (size_t)(n_rho > n_beta ? n_rho : n_beta));
  for (int e = 0; e < b->n_elements; ++e) {
    unsigned short z;
    if (fscanf(fd, "%hu", &z) != 1) goto fail_buf;
    b->number[e] = (unsigned char)z;
    for (long j = 0; j < n_rho; ++j)
      if (fscanf(fd, "%lf", &buf[j]) != 1) goto fail_buf;
    if (orc_spline_build(&b->rho[e], dr, buf, n_rho)) goto fail_buf;
    for (long j = 0; j < n_rho; ++j) buf[j] = orc_spline_eval(&b->rho[e], sqrt((double)(size_t)j * dr_sq));
    if (orc_spline_build(&b->rho_r_sq[e], dr_sq, buf, n_rho)) goto fail_buf;
    for (long j = 0; j < n_beta; ++j)
      if (fscanf(fd, "%lf", &buf[j]) != 1) goto fail_buf;
    if (orc_spline_build(&b->beta[e], drho, buf, n_beta)) goto fail_buf;
    for (long j = 0; j < n_beta; ++j) buf[j] = sqrt(buf[j]);
    if (orc_spline_build(&b->alpha[e], drho, buf, n_beta)) goto fail_buf;
  }
  free(buf);
  fclose(fd);
  return b;
fail_buf:
  free(buf);
fail:
  fclose(fd);
  orc_beta_free(b);
  return NULL;
}

void orc_beta_free(orc_beta *b) {
  if (!b) return;
  for (int e = 0; e < ORC_MAX_ELEM; ++e) {
    orc_spline_free(&b->rho[e]);
    orc_spline_free(&b->rho_r_sq[e]);
    orc_spline_free(&b->beta[e]);
    orc_spline_free(&b->alpha[e]);
  }
  free(b);
}

int orc_beta_n_elements(const orc_beta *b) { return b->n_elements; }
const char *orc_beta_element_name(const orc_beta *b, int i) { return b->name[i]; }
double orc_beta_r_cutoff(const orc_beta *b) { return b->r_cutoff; }
double orc_beta_rho_cutoff(const orc_beta *b) { return b->rho_cutoff; }

static const orc_spline *beta_spline(const orc_beta *b, int which, int elem) {
  switch (which) {
    case 0: return &b->rho[elem];
    case 1: return &b->rho_r_sq[elem];
    case 2: return &b->beta[elem];
    default: return &b->alpha[elem];
  }
}

double orc_beta_eval(const orc_beta *b, int which, int elem, double x) {
  return orc_spline_eval(beta_spline(b, which, elem), x);
}

long orc_beta_table(const orc_beta *b, int which, int elem, double *out) {
  const orc_spline *s = beta_spline(b, which, elem);
  if (out) memcpy(out, s->c, sizeof(double) * 4 * (size_t)s->n);
  return s->n;
}

/* eph_beta.h:174-197: zero above rho_cutoff (one warning) */
double orc_beta_get_beta(orc_beta *b, int elem, double rho) {
  if (rho > b->rho_cutoff) {
    b->warned = 1;
    return 0.;
  }
  return orc_spline_eval(&b->beta[elem], rho);
}

double orc_beta_get_alpha(orc_beta *b, int elem, double rho) {
  if (rho > b->rho_cutoff) {
    b->warned = 1;
    return 0.;
  }
  return orc_spline_eval(&b->alpha[elem], rho);
}

static inline double beta_rho_r_sq(const orc_beta *b, int elem, double r_sq) {
  return orc_spline_eval(&b->rho_r_sq[elem], r_sq);
}

/* --------------------------------------------------------------------- fdm */

enum { FDM_CONSTANT = 0, FDM_DYNAMIC = 1, FDM_ZERO_DERIVATIVE = 2 };

/* eph_linear.h: piecewise-linear table with reverse lookup */
typedef struct {
  double dx;
  long n;
  double *y, *dy; /* dy[n-1] = 0: the reference reads one past its slopes there */
} orc_linear;

struct orc_fdm {
  int has_tdyn;
  orc_spline C_T, K_T;
  orc_linear E_T;
  long nx, ny, nz, ntotal;
  double x0, x1, y0, y1, z0, z1, dx, dy, dz, dV;
  double *T, *dT, *ddT, *C, *rho, *kappa, *S;
  short *flag;
  unsigned short *Tdyn;
  char parameter_filename[1024];
  long steps;
  double dt;
};

static orc_fdm *fdm_alloc(long nx, long ny, long nz) {
  orc_fdm *g = (orc_fdm *)calloc(1, sizeof(orc_fdm));
  g->nx = nx;
  g->ny = ny;
  g->nz = nz;
  g->ntotal = nx * ny * nz;
  size_t n = (size_t)g->ntotal;
  g->T = (double *)calloc(n, sizeof(double));
  g->dT = (double *)calloc(n, sizeof(double));
  g->ddT = (double *)calloc(n, sizeof(double));
  g->C = (double *)calloc(n, sizeof(double));
  g->rho = (double *)calloc(n, sizeof(double));
  g->kappa = (double *)calloc(n, sizeof(double));
  g->S = (double *)calloc(n, sizeof(double));
  g->flag = (short *)malloc(n * sizeof(short));
  g->Tdyn = (unsigned short *)calloc(n, sizeof(unsigned short));
  for (size_t i = 0; i < n; ++i) g->flag[i] = 1;
  return g;
}

/* eph_fdm.h:127-146 */
static void fdm_set_box(orc_fdm *g, double x0, double x1, double y0, double y1, double z0, double z1) {
  g->x0 = x0; g->x1 = x1; g->y0 = y0; g->y1 = y1; g->z0 = z0; g->z1 = z1;
  g->dx = (x1 - x0) / (double)(size_t)g->nx;
  g->dy = (y1 - y0) / (double)(size_t)g->ny;
  g->dz = (z1 - z0) / (double)(size_t)g->nz;
  g->dV = g->dx * g->dy * g->dz;
}

/* eph_fdm.h:28-46 */
orc_fdm *orc_fdm_create(long nx, long ny, long nz, double x0, double x1, double y0, double y1, double z0,
                        double z1, double T_e, double C_e, double rho_e, double kappa_e) {
  orc_fdm *g = fdm_alloc(nx, ny, nz);
  fdm_set_box(g, x0, x1, y0, y1, z0, z1);
  for (long i = 0; i < g->ntotal; ++i) {
    g->T[i] = T_e;
    g->rho[i] = rho_e;
    g->C[i] = C_e;
    g->kappa[i] = kappa_e;
    g->flag[i] = 1;
    g->Tdyn[i] = 0;
  }
  g->steps = 1;
  g->dt = 1;
  strcpy(g->parameter_filename, "NULL");
  return g;
}

/* eph_fdm.h:48-119 (files whose parameter line is NULL) */
orc_fdm *orc_fdm_load(const char *path) {
  FILE *fd = fopen(path, "r");
  if (!fd) return NULL;
  char line[1024];
  for (int k = 0; k < 3; ++k)
    if (!fgets(line, sizeof line, fd) || line[0] != '#') {
      fclose(fd);
      return NULL;
    }
  long nx, ny, nz, steps;
  if (fscanf(fd, "%ld %ld %ld %ld", &nx, &ny, &nz, &steps) != 4 || nx < 1 || ny < 1 || nz < 1) {
    fclose(fd);
    return NULL;
  }
  orc_fdm *g = fdm_alloc(nx, ny, nz);
  g->steps = steps;
  double b[6];
  if (fscanf(fd, "%lf %lf %lf %lf %lf %lf", &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]) != 6) goto fail;
  fdm_set_box(g, b[0], b[1], b[2], b[3], b[4], b[5]);
  if (fscanf(fd, "%1023s", g->parameter_filename) != 1) goto fail;
  if (strcmp(g->parameter_filename, "NULL") != 0) {
    /* eph_fdm.h:73-104: C_e(T), kappa_e(T) splines and E_e(T) = sum C_e dT */
    FILE *pf = fopen(g->parameter_filename, "r");
    if (!pf) goto fail;
    char ln[1024];
    long n = 0;
    double dT = 0;
    int ok = 1;
    for (int k = 0; k < 3 && ok; ++k) ok = fgets(ln, sizeof ln, pf) && ln[0] == '#';
    if (ok) ok = fscanf(pf, "%ld %lf", &n, &dT) == 2 && n > 4;
    double *c = ok ? (double *)malloc(sizeof(double) * (size_t)n) : NULL;
    double *kk = ok ? (double *)malloc(sizeof(double) * (size_t)n) : NULL;
    for (long i = 0; ok && i < n; ++i) ok = fscanf(pf, "%lf %lf", &c[i], &kk[i]) == 2;
    fclose(pf);
    if (ok) {
      orc_spline_build(&g->C_T, dT, c, n);
      orc_spline_build(&g->K_T, dT, kk, n);
      c[0] = 0.;
      for (long i = 1; i < n; ++i) c[i] = c[i - 1] + c[i] * dT;
      g->E_T.dx = dT;
      g->E_T.n = n;
      g->E_T.y = c;
      g->E_T.dy = (double *)calloc((size_t)n, sizeof(double));
      for (long i = 0; i < n - 1; ++i) g->E_T.dy[i] = (c[i + 1] - c[i]) / dT;
      g->has_tdyn = 1;
      free(kk);
    } else {
      free(c);
      free(kk);
      goto fail;
    }
  }
  for (long c = 0; c < g->ntotal; ++c) {
    int lx, ly, lz, fl, td;
    double T, S, rho, Ce, kap;
    if (fscanf(fd, "%d %d %d %lf %lf %lf %lf %lf %d %d", &lx, &ly, &lz, &T, &S, &rho, &Ce, &kap, &fl, &td) != 10)
      goto fail;
    size_t index = (size_t)lx + (size_t)ly * (size_t)nx + (size_t)lz * (size_t)nx * (size_t)ny;
    if (index >= (size_t)g->ntotal) goto fail;
    g->T[index] = T;
    g->S[index] = S;
    g->rho[index] = rho;
    g->C[index] = Ce;
    g->kappa[index] = kap;
    g->flag[index] = (short)fl;
    g->Tdyn[index] = (unsigned short)td;
  }
  g->dt = 1;
  fclose(fd);
  return g;
fail:
  fclose(fd);
  orc_fdm_free(g);
  return NULL;
}

void orc_fdm_free(orc_fdm *g) {
  if (!g) return;
  if (g->has_tdyn) {
    orc_spline_free(&g->C_T);
    orc_spline_free(&g->K_T);
    free(g->E_T.y);
    free(g->E_T.dy);
  }
  free(g->T); free(g->dT); free(g->ddT); free(g->C); free(g->rho); free(g->kappa); free(g->S);
  free(g->flag); free(g->Tdyn);
  free(g);
}

void orc_fdm_set_dt(orc_fdm *g, double dt) { g->dt = dt; }
long orc_fdm_ncells(const orc_fdm *g) { return g->ntotal; }

/* eph_fdm.h:494-509: floor of the cell coordinate, wrapped periodically */
long orc_fdm_get_index(const orc_fdm *g, double x, double y, double z) {
  int lx = (int)floor((x - g->x0) / g->dx);
  int px = (int)floor(((double)lx) / (double)(size_t)g->nx);
  lx -= px * (int)g->nx;
  int ly = (int)floor((y - g->y0) / g->dy);
  int py = (int)floor(((double)ly) / (double)(size_t)g->ny);
  ly -= py * (int)g->ny;
  int lz = (int)floor((z - g->z0) / g->dz);
  int pz = (int)floor(((double)lz) / (double)(size_t)g->nz);
  lz -= pz * (int)g->nz;
  return (long)((size_t)lx + (size_t)ly * (size_t)g->nx + (size_t)lz * (size_t)g->nx * (size_t)g->ny);
}

/* eph_fdm.h:172-179 */
void orc_fdm_insert_energy(orc_fdm *g, double x, double y, double z, double E) {
  unsigned int index = (unsigned int)orc_fdm_get_index(g, x, y, z);
  double prescale = g->dV * g->dt;
  g->dT[index] += E / prescale;
}

/* eph_fdm.h:182-187 */
double orc_fdm_get_T(const orc_fdm *g, double x, double y, double z) {
  unsigned int index = (unsigned int)orc_fdm_get_index(g, x, y, z);
  return g->T[index];
}

/* eph_fdm.h:189-196 */
double orc_fdm_get_T_total(const orc_fdm *g) {
  double result = 0.;
  for (long i = 0; i < g->ntotal; ++i) result = result + g->T[i];
  result /= (double)(size_t)g->ntotal;
  return result;
}

/* eph_linear.h:41-48 */
static double linear_eval(const orc_linear *l, double x) {
  size_t idx = (size_t)(x / l->dx);
  if (idx < (size_t)l->n) {
    double delta = x - idx * l->dx;
    return l->y[idx] + l->dy[idx] * delta;
  }
  return 0.;
}

/* eph_linear.h:51-60 (first knot above v) */
static double linear_reverse(const orc_linear *l, double v) {
  size_t lo = 0, hi = (size_t)l->n;
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (!(v < l->y[mid]))
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo != (size_t)l->n && lo > 0) {
    size_t idx = lo - 1;
    return idx * l->dx + 1. / l->dy[idx] * (v - l->y[idx]);
  }
  return 0.;
}

/* eph_fdm.h:267-400 */
unsigned orc_fdm_solve(orc_fdm *g) {
  const size_t nx = (size_t)g->nx, ny = (size_t)g->ny, nz = (size_t)g->nz, ntotal = (size_t)g->ntotal;
  if (g->has_tdyn) /* eph_fdm.h:280-287 */
    for (size_t i = 0; i < ntotal; ++i)
      if (g->Tdyn[i]) {
        g->C[i] = orc_spline_eval(&g->C_T, g->T[i]);
        g->kappa[i] = orc_spline_eval(&g->K_T, g->T[i]);
      }
  double inner_dt = g->dt / (double)(size_t)g->steps;
  double dtdxdydz = inner_dt * (1.0 / g->dx / g->dx + 1.0 / g->dy / g->dy + 1.0 / g->dz / g->dz);
  double c_min = g->C[0], rho_min = g->rho[0], kappa_max = g->kappa[0];
  for (size_t i = 1; i < ntotal; ++i)
    if (g->flag[i] != FDM_CONSTANT) {
      if (g->C[i] < c_min) c_min = g->C[i];
      if (g->rho[i] < rho_min) rho_min = g->rho[i];
      if (g->kappa[i] > kappa_max) kappa_max = g->kappa[i];
    }
  double r = dtdxdydz / c_min / rho_min * kappa_max;
  unsigned int new_steps = (unsigned int)g->steps;
  if (r > 0.4) {
    inner_dt = 0.4 * inner_dt / r;
    unsigned int s = (unsigned int)(g->dt / inner_dt);
    new_steps = s > 1u ? s : 1u;
    inner_dt = g->dt / new_steps;
  }
  const double dx = g->dx, dy = g->dy, dz = g->dz;
  double *T = g->T, *K = g->kappa, *ddT = g->ddT;
  const short *fl = g->flag;
  for (unsigned n = 0; n < new_steps; ++n) {
#pragma omp parallel for schedule(static)
    for (long kk = 0; kk < (long)nz; ++kk) {
      const size_t k = (size_t)kk;
      for (size_t j = 0; j < ny; ++j)
        for (size_t i = 0; i < nx; ++i) {
          size_t q, p, rr = i + j * nx + k * nx * ny;
          ddT[rr] = 0.0;
          if (fl[rr] == FDM_ZERO_DERIVATIVE) continue;
          p = (i > 0) ? (i - 1) + j * nx + k * nx * ny : (nx - 1) + j * nx + k * nx * ny;
          q = (i < nx - 1) ? (i + 1) + j * nx + k * nx * ny : j * nx + k * nx * ny;
          if (fl[q] == FDM_ZERO_DERIVATIVE) q = rr;
          else if (fl[p] == FDM_ZERO_DERIVATIVE) p = rr;
          ddT[rr] += (K[q] - K[p]) * (T[q] - T[p]) / dx / dx / 4.0;
          ddT[rr] += K[rr] * ((T[q] + T[p] - 2.0 * T[rr]) / dx / dx);
          p = (j > 0) ? i + (j - 1) * nx + k * nx * ny : i + (ny - 1) * nx + k * nx * ny;
          q = (j < ny - 1) ? i + (j + 1) * nx + k * nx * ny : i + k * nx * ny;
          if (fl[q] == FDM_ZERO_DERIVATIVE) q = rr;
          else if (fl[p] == FDM_ZERO_DERIVATIVE) p = rr;
          ddT[rr] += (K[q] - K[p]) * (T[q] - T[p]) / dy / dy / 4.0;
          ddT[rr] += K[rr] * ((T[q] + T[p] - 2.0 * T[rr]) / dy / dy);
          p = (k > 0) ? i + j * nx + (k - 1) * nx * ny : i + j * nx + (nz - 1) * nx * ny;
          q = (k < nz - 1) ? i + j * nx + (k + 1) * nx * ny : i + j * nx;
          if (fl[q] == FDM_ZERO_DERIVATIVE) q = rr;
          else if (fl[p] == FDM_ZERO_DERIVATIVE) p = rr;
          ddT[rr] += (K[q] - K[p]) * (T[q] - T[p]) / dz / dz / 4.0;
          ddT[rr] += K[rr] * ((T[q] + T[p] - 2.0 * T[rr]) / dz / dz);
        }
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)ntotal; i++) {
      double prescaler = g->rho[i] * g->C[i];
      if (fl[i] == FDM_DYNAMIC) {
        if (g->Tdyn[i] == 1) { /* eph_fdm.h:378-382 */
          double E_e = linear_eval(&g->E_T, T[i]);
          E_e += (ddT[i] + g->dT[i] + g->S[i]) / g->rho[i] * inner_dt;
          T[i] = linear_reverse(&g->E_T, E_e);
        } else {
          T[i] += (ddT[i] + g->dT[i] + g->S[i]) / prescaler * inner_dt;
        }
      }
      if (T[i] < 0.0) T[i] = 0.0;
    }
  }
  memset(g->dT, 0, sizeof(double) * ntotal);
  return new_steps;
}

/* eph_fdm.h:226-265 */
int orc_fdm_save_state(const orc_fdm *g, const char *path) {
  FILE *fd = fopen(path, "w");
  if (!fd) return 1;
  fprintf(fd, "# A comment\n#\n#\n");
  fprintf(fd, "%ld %ld %ld %ld\n", g->nx, g->ny, g->nz, g->steps);
  fprintf(fd, "%.6e %.6e\n", g->x0, g->x1);
  fprintf(fd, "%.6e %.6e\n", g->y0, g->y1);
  fprintf(fd, "%.6e %.6e\n", g->z0, g->z1);
  fprintf(fd, "%s\n", g->parameter_filename);
  for (int k = 0; k < g->nz; ++k)
    for (int j = 0; j < g->ny; ++j)
      for (int i = 0; i < g->nx; ++i) {
        unsigned int index = (unsigned)(i + j * g->nx + k * g->nx * g->ny);
        fprintf(fd, "%d %d %d %.6e %.6e %.6e %.6e %.6e %d %d\n", i, j, k, g->T[index], g->S[index], g->rho[index],
                g->C[index], g->kappa[index], g->flag[index], g->Tdyn[index]);
      }
  fclose(fd);
  return 0;
}

/* eph_fdm.h:198-224 */
int orc_fdm_save_temperature(const orc_fdm *g, const char *path, int n) {
  char fn[1100];
  snprintf(fn, sizeof fn, "%s_%06d", path, n);
  FILE *fd = fopen(fn, "w");
  if (!fd) return 1;
  fprintf(fd, "x y z Te\n");
  for (int k = 0; k < g->nz; ++k)
    for (int j = 0; j < g->ny; ++j)
      for (int i = 0; i < g->nx; ++i) {
        unsigned int index = (unsigned)(i + j * g->nx + k * g->nx * g->ny);
        double x = g->x0 + i * g->dx, y = g->y0 + j * g->dy, z = g->z0 + k * g->dz;
        fprintf(fd, "%.6e %.6e %.6e %.6e\n", x, y, z, g->T[index]);
      }
  fclose(fd);
  return 0;
}

int orc_fdm_get(const orc_fdm *g, int field, double *out) {
  const double *src[] = {g->T, g->dT, g->S, g->rho, g->C, g->kappa};
  if (field < 0 || field > 5) return 1;
  memcpy(out, src[field], sizeof(double) * (size_t)g->ntotal);
  return 0;
}

int orc_fdm_set(orc_fdm *g, int field, const double *in) {
  double *dst[] = {g->T, g->dT, g->S, g->rho, g->C, g->kappa};
  if (field < 0 || field > 5) return 1;
  memcpy(dst[field], in, sizeof(double) * (size_t)g->ntotal);
  return 0;
}

/* ----------------------------------------------------------------- ranmars */

/* Marsaglia, Zaman & Tsang (1990) RANMAR: lagged Fibonacci (97, 33) on
 * 24-bit fractions combined with an arithmetic sequence; the initial table
 * is filled from a 3-lag Fibonacci and a congruential generator. */
void orc_ranmars_init_ijkl(orc_ranmars *r, int ij, int kl) {
  int i = (ij / 177) % 177 + 2, j = ij % 177 + 2, k = (kl / 169) % 178 + 1, l = kl % 169;
  for (int ii = 1; ii <= 97; ++ii) {
    double s = 0.0, t = 0.5;
    for (int jj = 1; jj <= 24; ++jj) {
      int m = ((i * j) % 179) * k % 179;
      i = j;
      j = k;
      k = m;
      l = (53 * l + 1) % 169;
      if ((l * m) % 64 >= 32) s = s + t;
      t = 0.5 * t;
    }
    r->u[ii] = s;
  }
  r->c = 362436.0 / 16777216.0;
  r->cd = 7654321.0 / 16777216.0;
  r->cm = 16777213.0 / 16777216.0;
  r->i97 = 97;
  r->j97 = 33;
  r->save = 0;
}

/* a single seed split into the algorithm's two seeds */
int orc_ranmars_init(orc_ranmars *r, int seed) {
  if (seed <= 0 || seed > 900000000) return 1;
  int ij = (seed - 1) / 30082, kl = (seed - 1) - 30082 * ij;
  orc_ranmars_init_ijkl(r, ij, kl);
  return 0;
}

double orc_ranmars_uniform(orc_ranmars *r) {
  double uni = r->u[r->i97] - r->u[r->j97];
  if (uni < 0.0) uni += 1.0;
  r->u[r->i97] = uni;
  if (--r->i97 == 0) r->i97 = 97;
  if (--r->j97 == 0) r->j97 = 97;
  r->c -= r->cd;
  if (r->c < 0.0) r->c += r->cm;
  uni -= r->c;
  if (uni < 0.0) uni += 1.0;
  return uni;
}

/* Marsaglia polar method; the second deviate of each pair is kept */
double orc_ranmars_gaussian(orc_ranmars *r) {
  if (r->save) {
    r->save = 0;
    return r->second;
  }
  double v1, v2, rsq;
  do {
    v1 = 2.0 * orc_ranmars_uniform(r) - 1.0;
    v2 = 2.0 * orc_ranmars_uniform(r) - 1.0;
    rsq = v1 * v1 + v2 * v2;
  } while (rsq >= 1.0 || rsq == 0.0);
  double fac = sqrt(-2.0 * log(rsq) / rsq);
  r->second = v1 * fac;
  r->save = 1;
  return v2 * fac;
}

/* --------------------------------------------------------------------- fix */

enum { F_FRICTION = 0x01, F_RANDOM = 0x02, F_FDM = 0x04, F_NOINT = 0x08, F_NOFRICTION = 0x10, F_NORANDOM = 0x20 };

struct orc_fix {
  int eph_flag, eph_model, seed, types;
  int coloured;       /* style eph/coloured/exp: arg[5] is tau0, model 4 */
  double tau0, zeta;  /* zeta = 1 - exp(-dt/tau0) (fix_eph_coloured_exp.cpp:190) */
  double *f_dis, *f_sto;
  int type_map[64];
  orc_beta *beta;
  orc_fdm *fdm;
  double dtv, dtf, dt, r_cutoff, r_cutoff_sq, rho_cutoff, eta_factor, Ee;
  int T_freq;
  char T_out[1024], T_state[1100];
  double mass[65];
  double lo[3], hi[3], prd[3];
  double skin;
  long ntimestep;
  orc_ranmars rng;
  int nthreads;
  /* atoms */
  int n, groupbit;
  double *x, *v, *f, *fext;
  int *type, *mask;
  /* fix arrays */
  double *rho, *alpha, *f_eph, *f_rng, *w, *xi, *array;
  /* neighbour list (cutoff rc + skin), ascending owner index */
  int *numneigh, *neigh, maxneigh;
  signed char *shift; /* 3 per entry: -1, 0, +1 periodic image */
  double *xhold;
  long nbuild;
  double t_fix, t_neigh;
};

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void seterr(char *err, int errlen, const char *msg) {
  if (err && errlen > 0) {
    strncpy(err, msg, (size_t)errlen - 1);
    err[errlen - 1] = 0;
  }
}

/* fix_eph.cpp:61-241 */
orc_fix *orc_fix_create(int narg, const char **arg, int ntypes, const double *mass, const double *boxlo,
                        const double *boxhi, double dt, double boltz, double ftm2v, double skin, char *err,
                        int errlen) {
  if (narg < 18) {
    seterr(err, errlen, "Illegal fix eph command: too few arguments");
    return NULL;
  }
  if (ntypes < 1 || ntypes > 64) {
    seterr(err, errlen, "fix_eph oracle: bad number of types");
    return NULL;
  }
  orc_fix *f = (orc_fix *)calloc(1, sizeof(orc_fix));
  f->nthreads = 1;
  f->seed = atoi(arg[3]);
  orc_ranmars_init(&f->rng, f->seed + 0);
  f->eph_flag = (int)strtol(arg[4], NULL, 0);
  f->coloured = strcmp(arg[2], "eph/coloured/exp") == 0;
  if (f->coloured) {
    f->tau0 = atof(arg[5]);
    f->eph_model = 4;
  } else {
    f->eph_model = atoi(arg[5]);
  }
  double v_rho = atof(arg[6]), v_Ce = atof(arg[7]), v_kappa = atof(arg[8]), v_Te = atof(arg[9]);
  int nx = atoi(arg[10]), ny = atoi(arg[11]), nz = atoi(arg[12]);
  for (int k = 0; k < 3; ++k) {
    f->lo[k] = boxlo[k];
    f->hi[k] = boxhi[k];
    f->prd[k] = boxhi[k] - boxlo[k];
  }
  if (strcmp("NULL", arg[13]) == 0) {
    if (nx < 1 || ny < 1 || nz < 1) {
      seterr(err, errlen, "FixEPH: non-positive grid values");
      free(f);
      return NULL;
    }
    f->fdm = orc_fdm_create(nx, ny, nz, boxlo[0], boxhi[0], boxlo[1], boxhi[1], boxlo[2], boxhi[2], v_Te, v_Ce,
                            v_rho, v_kappa);
    strcpy(f->T_state, "T.restart");
  } else {
    f->fdm = orc_fdm_load(arg[13]);
    if (!f->fdm) {
      seterr(err, errlen, "FixEPH: cannot read the T_e grid file");
      free(f);
      return NULL;
    }
    snprintf(f->T_state, sizeof f->T_state, "%s.restart", arg[13]);
  }
  f->T_freq = atoi(arg[14]);
  if (f->T_freq > 0) snprintf(f->T_out, sizeof f->T_out, "%s", arg[15]);
  orc_fdm_set_dt(f->fdm, dt);
  f->types = ntypes;
  if (f->types > narg - 17) {
    seterr(err, errlen, "Fix eph: number of types larger than provided in fix");
    orc_fix_free(f);
    return NULL;
  }
  f->beta = orc_beta_load(arg[16]);
  if (!f->beta || orc_beta_n_elements(f->beta) < 1) {
    seterr(err, errlen, "Fix eph: no elements found in input file");
    orc_fix_free(f);
    return NULL;
  }
  f->r_cutoff = f->beta->r_cutoff;
  f->r_cutoff_sq = f->beta->r_cutoff_sq;
  f->rho_cutoff = f->beta->rho_cutoff;
  for (int i = 0; i < f->types; ++i) {
    f->type_map[i] = INT_MAX;
    for (int j = 0; j < f->beta->n_elements; ++j)
      if (strcmp(f->beta->name[j], arg[17 + i]) == 0) f->type_map[i] = j;
    if (f->type_map[i] > f->types) {
      seterr(err, errlen, "Fix eph: elements not found in input file");
      orc_fix_free(f);
      return NULL;
    }
  }
  f->eta_factor = sqrt(2.0 * boltz / dt);
  if (f->coloured) f->zeta = 1.0 - exp(-dt / f->tau0);
  f->dt = dt;
  f->dtv = dt;
  f->dtf = 0.5 * dt * ftm2v;
  for (int t = 0; t <= ntypes; ++t) f->mass[t] = mass[t];
  f->skin = skin;
  return f;
}

void orc_fix_free(orc_fix *f) {
  if (!f) return;
  orc_beta_free(f->beta);
  orc_fdm_free(f->fdm);
  free(f->x); free(f->v); free(f->f); free(f->fext); free(f->type); free(f->mask);
  free(f->rho); free(f->alpha); free(f->f_eph); free(f->f_rng); free(f->w); free(f->xi); free(f->array);
  free(f->numneigh); free(f->neigh); free(f->shift); free(f->xhold);
  free(f->f_dis); free(f->f_sto);
  free(f);
}

void orc_fix_set_threads(orc_fix *f, int nthreads) { f->nthreads = nthreads > 0 ? nthreads : 1; }

/* wrap into [lo, hi) as the engine does before a rebuild */
static void fix_pbc(orc_fix *f) {
  for (int i = 0; i < f->n; ++i)
    for (int k = 0; k < 3; ++k) {
      double c = f->x[3 * (size_t)i + k];
      if (c < f->lo[k]) c += f->prd[k];
      if (c >= f->hi[k]) {
        c -= f->prd[k];
        c = c > f->lo[k] ? c : f->lo[k];
      }
      f->x[3 * (size_t)i + k] = c;
    }
}

/* image coordinate of atom j as its ghost holds it: x_j + s*prd (one add) */
static inline double image_coord(const orc_fix *f, int j, int k, int s) {
  const double c = f->x[3 * (size_t)j + k];
  if (s > 0) return c + f->prd[k];
  if (s < 0) return c + (-f->prd[k]);
  return c;
}

/* Full list with cutoff rc + skin for every atom, neighbours in ascending
 * index, each with the periodic image nearest to atom i. */
static int fix_build_list(orc_fix *f) {
  double t0 = now_s();
  fix_pbc(f);
  const int n = f->n;
  const double cut = f->r_cutoff + f->skin, cutsq = cut * cut;
  for (int k = 0; k < 3; ++k)
    if (f->prd[k] < 2.0 * cut) return 1;
  int nb[3];
  double w[3];
  for (int k = 0; k < 3; ++k) {
    nb[k] = (int)(f->prd[k] / cut);
    if (nb[k] < 1) nb[k] = 1;
    w[k] = f->prd[k] / nb[k];
  }
  const int use_bins = nb[0] >= 3 && nb[1] >= 3 && nb[2] >= 3;
  long nbins = use_bins ? (long)nb[0] * nb[1] * nb[2] : 1;
  int *bin_of = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int *head = (int *)malloc(sizeof(int) * (size_t)nbins), *next = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (long b = 0; b < nbins; ++b) head[b] = -1;
  for (int i = n - 1; i >= 0; --i) {
    long b = 0;
    if (use_bins) {
      int c[3];
      for (int k = 0; k < 3; ++k) {
        c[k] = (int)floor((f->x[3 * (size_t)i + k] - f->lo[k]) / w[k]);
        if (c[k] < 0) c[k] = 0;
        if (c[k] >= nb[k]) c[k] = nb[k] - 1;
      }
      b = c[0] + (long)nb[0] * (c[1] + (long)nb[1] * c[2]);
    }
    bin_of[i] = (int)b;
    next[i] = head[b];
    head[b] = i;
  }
  int cap = 64;
  int *tmp_j = NULL;
  signed char *tmp_s = NULL;
  int maxn = 0;
  int *counts = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  /* two passes: count, then fill at the final capacity */
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      cap = maxn > 0 ? maxn : 1;
      free(f->neigh);
      free(f->shift);
      f->neigh = (int *)malloc(sizeof(int) * (size_t)n * (size_t)cap + 1);
      f->shift = (signed char *)malloc((size_t)n * (size_t)cap * 3 + 1);
      f->maxneigh = cap;
    }
#pragma omp parallel num_threads(f->nthreads)
    {
      int lcap = 256;
      int *lj = (int *)malloc(sizeof(int) * (size_t)lcap);
      signed char *ls = (signed char *)malloc((size_t)lcap * 3);
#pragma omp for schedule(static) reduction(max : maxn)
      for (int i = 0; i < n; ++i) {
        int cnt = 0;
        int bc[3] = {0, 0, 0};
        if (use_bins) {
          int b = bin_of[i];
          bc[0] = b % nb[0];
          bc[1] = (b / nb[0]) % nb[1];
          bc[2] = b / (nb[0] * nb[1]);
        }
        int nst = use_bins ? 27 : 1;
        for (int st = 0; st < nst; ++st) {
          long b = 0;
          if (use_bins) {
            int c0 = (bc[0] + st % 3 - 1 + nb[0]) % nb[0];
            int c1 = (bc[1] + (st / 3) % 3 - 1 + nb[1]) % nb[1];
            int c2 = (bc[2] + st / 9 - 1 + nb[2]) % nb[2];
            b = c0 + (long)nb[0] * (c1 + (long)nb[1] * c2);
          }
          for (int j = head[b]; j >= 0; j = next[j]) {
            if (j == i) continue;
            int s[3];
            double e[3];
            for (int k = 0; k < 3; ++k) {
              double d = f->x[3 * (size_t)j + k] - f->x[3 * (size_t)i + k];
              s[k] = d > 0.5 * f->prd[k] ? -1 : (d < -0.5 * f->prd[k] ? 1 : 0);
              e[k] = image_coord(f, j, k, s[k]) - f->x[3 * (size_t)i + k];
            }
            double rsq = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
            if (rsq < cutsq) {
              if (cnt >= lcap) {
                lcap *= 2;
                lj = (int *)realloc(lj, sizeof(int) * (size_t)lcap);
                ls = (signed char *)realloc(ls, (size_t)lcap * 3);
              }
              /* insertion in ascending j */
              int pos = cnt;
              while (pos > 0 && lj[pos - 1] > j) {
                lj[pos] = lj[pos - 1];
                memcpy(ls + 3 * pos, ls + 3 * (pos - 1), 3);
                --pos;
              }
              lj[pos] = j;
              for (int k = 0; k < 3; ++k) ls[3 * pos + k] = (signed char)s[k];
              ++cnt;
            }
          }
        }
        if (cnt > maxn) maxn = cnt;
        if (pass == 1) {
          counts[i] = cnt;
          memcpy(f->neigh + (size_t)i * cap, lj, sizeof(int) * (size_t)cnt);
          memcpy(f->shift + (size_t)i * cap * 3, ls, (size_t)cnt * 3);
        }
      }
      free(lj);
      free(ls);
    }
  }
  free(f->numneigh);
  f->numneigh = counts;
  free(bin_of);
  free(head);
  free(next);
  (void)tmp_j;
  (void)tmp_s;
  if (!f->xhold) f->xhold = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  memcpy(f->xhold, f->x, sizeof(double) * 3 * (size_t)n);
  ++f->nbuild;
  f->t_neigh += now_s() - t0;
  return 0;
}

int orc_fix_set_atoms(orc_fix *f, int n, const double *x, const double *v, const int *type, const int *mask,
                      int groupbit) {
  if (n < 1) return 1; /* fix_eph.cpp:65 */
  f->n = n;
  f->groupbit = groupbit;
  size_t n3 = 3 * (size_t)n;
#define REALLOC(p, cnt, T) p = (T *)realloc(p, sizeof(T) * (cnt))
  REALLOC(f->x, n3, double);
  REALLOC(f->v, n3, double);
  REALLOC(f->f, n3, double);
  REALLOC(f->type, (size_t)n, int);
  REALLOC(f->mask, (size_t)n, int);
  REALLOC(f->rho, (size_t)n, double);
  REALLOC(f->alpha, (size_t)n, double);
  REALLOC(f->f_eph, n3, double);
  REALLOC(f->f_rng, n3, double);
  REALLOC(f->w, n3, double);
  REALLOC(f->xi, n3, double);
  REALLOC(f->array, 8 * (size_t)n, double);
  REALLOC(f->f_dis, n3, double);
  REALLOC(f->f_sto, n3, double);
  free(f->xhold);
  f->xhold = NULL;
#undef REALLOC
  memcpy(f->x, x, sizeof(double) * n3);
  memcpy(f->v, v, sizeof(double) * n3);
  memcpy(f->type, type, sizeof(int) * (size_t)n);
  for (int i = 0; i < n; ++i) f->mask[i] = mask ? mask[i] : 1;
  memset(f->f, 0, sizeof(double) * n3);
  memset(f->rho, 0, sizeof(double) * (size_t)n);
  memset(f->alpha, 0, sizeof(double) * (size_t)n);
  memset(f->f_eph, 0, sizeof(double) * n3);
  memset(f->f_rng, 0, sizeof(double) * n3);
  memset(f->w, 0, sizeof(double) * n3);
  memset(f->xi, 0, sizeof(double) * n3);
  memset(f->array, 0, sizeof(double) * 8 * (size_t)n);
  memset(f->f_dis, 0, sizeof(double) * n3);
  memset(f->f_sto, 0, sizeof(double) * n3);
  free(f->fext);
  f->fext = NULL;
  /* engine setup: wrap, list, force clear */
  if (fix_build_list(f)) return 2;
  orc_fix_clear_forces(f);
  return 0;
}

int orc_fix_set_fext(orc_fix *f, const double *fext) {
  free(f->fext);
  f->fext = NULL;
  if (fext) {
    f->fext = (double *)malloc(sizeof(double) * 3 * (size_t)f->n);
    memcpy(f->fext, fext, sizeof(double) * 3 * (size_t)f->n);
  }
  orc_fix_clear_forces(f);
  return 0;
}

void orc_fix_clear_forces(orc_fix *f) {
  size_t n3 = 3 * (size_t)f->n;
  if (f->fext)
    memcpy(f->f, f->fext, sizeof(double) * n3);
  else
    memset(f->f, 0, sizeof(double) * n3);
}

/* fix_eph.cpp:305-328 */
void orc_fix_initial_integrate(orc_fix *f) {
  if (f->eph_flag & F_NOINT) return;
  double t0 = now_s();
#pragma omp parallel for schedule(static) num_threads(f->nthreads)
  for (int i = 0; i < f->n; ++i)
    if (f->mask[i] & f->groupbit) {
      double dtfm = f->dtf / f->mass[f->type[i]];
      double *v = f->v + 3 * (size_t)i, *x = f->x + 3 * (size_t)i;
      const double *fo = f->f + 3 * (size_t)i;
      v[0] += dtfm * fo[0];
      v[1] += dtfm * fo[1];
      v[2] += dtfm * fo[2];
      x[0] += f->dtv * v[0];
      x[1] += f->dtv * v[1];
      x[2] += f->dtv * v[2];
    }
  f->t_fix += now_s() - t0;
}

/* rebuild when an atom moved more than skin/2 since the last build */
void orc_fix_neighbor_decide(orc_fix *f) {
  const double triggersq = 0.25 * f->skin * f->skin;
  int flag = 0;
  for (int i = 0; i < f->n && !flag; ++i) {
    const double dx = f->x[3 * (size_t)i + 0] - f->xhold[3 * (size_t)i + 0];
    const double dy = f->x[3 * (size_t)i + 1] - f->xhold[3 * (size_t)i + 1];
    const double dz = f->x[3 * (size_t)i + 2] - f->xhold[3 * (size_t)i + 2];
    if (dx * dx + dy * dy + dz * dz > triggersq) flag = 1;
  }
  if (flag) fix_build_list(f);
}

/* fix_eph.cpp:431-466 */
static void fix_density(orc_fix *f) {
  const int n = f->n;
#pragma omp parallel for schedule(static) num_threads(f->nthreads)
  for (int i = 0; i < n; ++i) {
    f->rho[i] = 0;
    if (!(f->mask[i] & f->groupbit)) continue;
    const int *jl = f->neigh + (size_t)i * f->maxneigh;
    const signed char *sl = f->shift + (size_t)i * f->maxneigh * 3;
    const double *xi = f->x + 3 * (size_t)i;
    double rho = 0;
    for (int jn = 0; jn < f->numneigh[i]; ++jn) {
      const int jj = jl[jn];
      double d[3];
      for (int k = 0; k < 3; ++k) d[k] = image_coord(f, jj, k, sl[3 * jn + k]) - xi[k];
      double r_sq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      if (r_sq < f->r_cutoff_sq) rho += beta_rho_r_sq(f->beta, f->type_map[f->type[jj] - 1], r_sq);
    }
    f->rho[i] = rho;
  }
}

static inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* fix_eph.cpp:687-837 */
static void fix_force_prl(orc_fix *f) {
  const int n = f->n;
  const double rcsq = f->r_cutoff_sq;
  /* alpha of every atom with rho > 0, once (the reference evaluates the same
   * value inside every loop) */
  for (int i = 0; i < n; ++i)
    f->alpha[i] = (f->rho[i] > 0) ? orc_beta_get_alpha(f->beta, f->type_map[f->type[i] - 1], f->rho[i]) : 0.0;
  if (f->eph_flag & F_FRICTION) {
#pragma omp parallel for schedule(static) num_threads(f->nthreads)
    for (int i = 0; i < n; ++i) {
      if (!(f->mask[i] & f->groupbit)) continue;
      if (!(f->rho[i] > 0)) continue;
      const double alpha_i = f->alpha[i];
      const int *jl = f->neigh + (size_t)i * f->maxneigh;
      const signed char *sl = f->shift + (size_t)i * f->maxneigh * 3;
      const double *xi = f->x + 3 * (size_t)i, *vi = f->v + 3 * (size_t)i;
      double *wi = f->w + 3 * (size_t)i;
      for (int jn = 0; jn < f->numneigh[i]; ++jn) {
        const int jj = jl[jn];
        double e[3];
        for (int k = 0; k < 3; ++k) e[k] = image_coord(f, jj, k, sl[3 * jn + k]) - xi[k];
        double e_r_sq = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        if (e_r_sq >= rcsq) continue;
        double v_rho_ji = beta_rho_r_sq(f->beta, f->type_map[f->type[jj] - 1], e_r_sq);
        double prescaler = alpha_i * v_rho_ji / (f->rho[i] * e_r_sq);
        double var1 = prescaler * dot3(e, vi);
        double var2 = prescaler * dot3(e, f->v + 3 * (size_t)jj);
        double dvar = var1 - var2;
        wi[0] += dvar * e[0];
        wi[1] += dvar * e[1];
        wi[2] += dvar * e[2];
      }
    }
#pragma omp parallel for schedule(static) num_threads(f->nthreads)
    for (int i = 0; i < n; ++i) {
      if (!(f->mask[i] & f->groupbit)) continue;
      if (!(f->rho[i] > 0)) continue;
      const int itype = f->type[i];
      const double alpha_i = f->alpha[i];
      const int *jl = f->neigh + (size_t)i * f->maxneigh;
      const signed char *sl = f->shift + (size_t)i * f->maxneigh * 3;
      const double *xi = f->x + 3 * (size_t)i, *wi = f->w + 3 * (size_t)i;
      double *fe = f->f_eph + 3 * (size_t)i;
      for (int jn = 0; jn < f->numneigh[i]; ++jn) {
        const int jj = jl[jn];
        double e[3];
        for (int k = 0; k < 3; ++k) e[k] = image_coord(f, jj, k, sl[3 * jn + k]) - xi[k];
        double e_r_sq = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        if (e_r_sq >= rcsq || !(f->rho[jj] > 0)) continue;
        double alpha_j = f->alpha[jj];
        double v_rho_ji = beta_rho_r_sq(f->beta, f->type_map[f->type[jj] - 1], e_r_sq);
        double var1 = alpha_i * v_rho_ji * dot3(e, wi) / (f->rho[i] * e_r_sq);
        double v_rho_ij = beta_rho_r_sq(f->beta, f->type_map[itype - 1], e_r_sq);
        double var2 = alpha_j * v_rho_ij * dot3(e, f->w + 3 * (size_t)jj) / (f->rho[jj] * e_r_sq);
        double dvar = var1 - var2;
        fe[0] -= dvar * e[0];
        fe[1] -= dvar * e[1];
        fe[2] -= dvar * e[2];
      }
      if (f->coloured) { /* fix_eph_coloured_exp.cpp:562-568 */
        double *fd = f->f_dis + 3 * (size_t)i;
        for (int k = 0; k < 3; ++k) {
          fd[k] = fd[k] * (1. - f->zeta) + f->zeta * fe[k];
          fe[k] = fd[k];
        }
      }
    }
  }
  if (f->eph_flag & F_RANDOM) {
#pragma omp parallel for schedule(static) num_threads(f->nthreads)
    for (int i = 0; i < n; ++i) {
      if (!(f->mask[i] & f->groupbit)) continue;
      if (!(f->rho[i] > 0)) continue;
      const int itype = f->type[i];
      const double alpha_i = f->alpha[i];
      const int *jl = f->neigh + (size_t)i * f->maxneigh;
      const signed char *sl = f->shift + (size_t)i * f->maxneigh * 3;
      const double *xi = f->x + 3 * (size_t)i, *xii = f->xi + 3 * (size_t)i;
      double *fr = f->f_rng + 3 * (size_t)i;
      for (int jn = 0; jn < f->numneigh[i]; ++jn) {
        const int jj = jl[jn];
        double e[3];
        for (int k = 0; k < 3; ++k) e[k] = image_coord(f, jj, k, sl[3 * jn + k]) - xi[k];
        double e_r_sq = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        if (e_r_sq >= rcsq || !(f->rho[jj] > 0)) continue;
        double alpha_j = f->alpha[jj];
        double v_rho_ji = beta_rho_r_sq(f->beta, f->type_map[f->type[jj] - 1], e_r_sq);
        double var1 = alpha_i * v_rho_ji * dot3(e, xii) / (f->rho[i] * e_r_sq);
        double v_rho_ij = beta_rho_r_sq(f->beta, f->type_map[itype - 1], e_r_sq);
        double var2 = alpha_j * v_rho_ij * dot3(e, f->xi + 3 * (size_t)jj) / (f->rho[jj] * e_r_sq);
        double dvar = var1 - var2;
        fr[0] += dvar * e[0];
        fr[1] += dvar * e[1];
        fr[2] += dvar * e[2];
      }
      double v_Te = orc_fdm_get_T(f->fdm, xi[0], xi[1], xi[2]);
      double var = f->eta_factor * sqrt(v_Te);
      fr[0] *= var;
      fr[1] *= var;
      fr[2] *= var;
      if (f->coloured) { /* fix_eph_coloured_exp.cpp:619-625 */
        double *fs = f->f_sto + 3 * (size_t)i;
        for (int k = 0; k < 3; ++k) {
          fs[k] = fs[k] * (1. - f->zeta) + f->zeta * fr[k];
          fr[k] = fs[k];
        }
      }
    }
  }
}

/* fix_eph.cpp:468-503: model 1, local Langevin with beta(rho_i) */
static void fix_force_ttm(orc_fix *f) {
  const int n = f->n;
  if (f->eph_flag & F_FRICTION)
    for (int i = 0; i < n; ++i)
      if (f->mask[i] & f->groupbit) {
        double var = -orc_beta_get_beta(f->beta, f->type_map[f->type[i] - 1], f->rho[i]);
        for (int k = 0; k < 3; ++k) f->f_eph[3 * (size_t)i + k] = var * f->v[3 * (size_t)i + k];
      }
  if (f->eph_flag & F_RANDOM)
    for (int i = 0; i < n; ++i)
      if (f->mask[i] & f->groupbit) {
        const double *x = f->x + 3 * (size_t)i;
        double v_Te = orc_fdm_get_T(f->fdm, x[0], x[1], x[2]);
        double var = f->eta_factor * orc_beta_get_alpha(f->beta, f->type_map[f->type[i] - 1], f->rho[i]) * sqrt(v_Te);
        for (int k = 0; k < 3; ++k) f->f_rng[3 * (size_t)i + k] = var * f->xi[3 * (size_t)i + k];
      }
}

/* fix_eph.cpp:841-907 (models 1 and 4) */
int orc_fix_post_force(orc_fix *f, const double *xi) {
  if (f->eph_model != 4 && f->eph_model != 1) return 3;
  double t0 = now_s();
  const int n = f->n;
  size_t n3 = 3 * (size_t)n;
  memset(f->w, 0, sizeof(double) * n3);
  memset(f->xi, 0, sizeof(double) * n3);
  memset(f->f_eph, 0, sizeof(double) * n3);
  memset(f->f_rng, 0, sizeof(double) * n3);
  if (f->eph_flag & F_RANDOM) {
    long m = 0;
    for (int i = 0; i < n; ++i)
      if (f->mask[i] & f->groupbit)
        for (int k = 0; k < 3; ++k) f->xi[3 * (size_t)i + k] = xi ? xi[m++] : orc_ranmars_gaussian(&f->rng);
  }
  fix_density(f);
  if (f->eph_model == 1)
    fix_force_ttm(f);
  else
    fix_force_prl(f);
  if ((f->eph_flag & F_FRICTION) && !(f->eph_flag & F_NOFRICTION))
    for (size_t k = 0; k < n3; ++k) f->f[k] += f->f_eph[k];
  if ((f->eph_flag & F_RANDOM) && !(f->eph_flag & F_NORANDOM))
    for (size_t k = 0; k < n3; ++k) f->f[k] += f->f_rng[k];
  f->t_fix += now_s() - t0;
  return 0;
}

/* fix_eph.cpp:330-348 */
void orc_fix_final_integrate(orc_fix *f) {
  if (f->eph_flag & F_NOINT) return;
  double t0 = now_s();
#pragma omp parallel for schedule(static) num_threads(f->nthreads)
  for (int i = 0; i < f->n; ++i)
    if (f->mask[i] & f->groupbit) {
      double dtfm = f->dtf / f->mass[f->type[i]];
      double *v = f->v + 3 * (size_t)i;
      const double *fo = f->f + 3 * (size_t)i;
      v[0] += dtfm * fo[0];
      v[1] += dtfm * fo[1];
      v[2] += dtfm * fo[2];
    }
  f->t_fix += now_s() - t0;
}

/* fix_eph.cpp:350-429 */
void orc_fix_end_of_step(orc_fix *f) {
  double t0 = now_s();
  const int n = f->n;
  double E_local = 0.0;
  const double dt = f->dt;
  if (f->eph_flag & F_FRICTION)
    for (int i = 0; i < n; ++i)
      if (f->mask[i] & f->groupbit) {
        const double *fe = f->f_eph + 3 * (size_t)i, *v = f->v + 3 * (size_t)i, *x = f->x + 3 * (size_t)i;
        double dE_i = 0.0;
        dE_i -= fe[0] * v[0] * dt;
        dE_i -= fe[1] * v[1] * dt;
        dE_i -= fe[2] * v[2] * dt;
        orc_fdm_insert_energy(f->fdm, x[0], x[1], x[2], dE_i);
        E_local += dE_i;
      }
  if (f->eph_flag & F_RANDOM)
    for (int i = 0; i < n; ++i)
      if (f->mask[i] & f->groupbit) {
        const double *fr = f->f_rng + 3 * (size_t)i, *v = f->v + 3 * (size_t)i, *x = f->x + 3 * (size_t)i;
        double dE_i = 0.0;
        dE_i -= fr[0] * v[0] * dt;
        dE_i -= fr[1] * v[1] * dt;
        dE_i -= fr[2] * v[2] * dt;
        orc_fdm_insert_energy(f->fdm, x[0], x[1], x[2], dE_i);
        E_local += dE_i;
      }
  if (f->eph_flag & F_FDM) orc_fdm_solve(f->fdm);
  if (f->T_freq > 0 && (f->ntimestep % f->T_freq) == 0)
    orc_fdm_save_temperature(f->fdm, f->T_out, (int)(f->ntimestep / f->T_freq));
  f->Ee += E_local;
  for (int i = 0; i < n; ++i) {
    double *a = f->array + 8 * (size_t)i;
    if (f->mask[i] & f->groupbit) {
      a[0] = f->rho[i];
      a[1] = orc_beta_get_beta(f->beta, f->type_map[f->type[i] - 1], f->rho[i]);
      for (int k = 0; k < 3; ++k) {
        a[2 + k] = f->f_eph[3 * (size_t)i + k];
        a[5 + k] = f->f_rng[3 * (size_t)i + k];
      }
    } else
      memset(a, 0, 8 * sizeof(double));
  }
  f->t_fix += now_s() - t0;
}

int orc_fix_step(orc_fix *f, const double *xi) {
  f->ntimestep += 1;
  orc_fix_initial_integrate(f);
  orc_fix_neighbor_decide(f);
  orc_fix_clear_forces(f);
  int rc = orc_fix_post_force(f, xi);
  if (rc) return rc;
  orc_fix_final_integrate(f);
  orc_fix_end_of_step(f);
  return 0;
}

int orc_fix_get(orc_fix *f, const char *what, double *out) {
  size_t n = (size_t)f->n, n3 = 3 * n;
  if (!strcmp(what, "x")) memcpy(out, f->x, n3 * sizeof(double));
  else if (!strcmp(what, "v")) memcpy(out, f->v, n3 * sizeof(double));
  else if (!strcmp(what, "f")) memcpy(out, f->f, n3 * sizeof(double));
  else if (!strcmp(what, "f_eph")) memcpy(out, f->f_eph, n3 * sizeof(double));
  else if (!strcmp(what, "f_rng")) memcpy(out, f->f_rng, n3 * sizeof(double));
  else if (!strcmp(what, "w")) memcpy(out, f->w, n3 * sizeof(double));
  else if (!strcmp(what, "xi")) memcpy(out, f->xi, n3 * sizeof(double));
  else if (!strcmp(what, "rho")) memcpy(out, f->rho, n * sizeof(double));
  else if (!strcmp(what, "alpha")) memcpy(out, f->alpha, n * sizeof(double));
  else if (!strcmp(what, "array")) memcpy(out, f->array, 8 * n * sizeof(double));
  else if (!strcmp(what, "vector")) {
    out[0] = f->Ee;
    out[1] = orc_fdm_get_T_total(f->fdm);
  } else if (!strcmp(what, "T")) memcpy(out, f->fdm->T, (size_t)f->fdm->ntotal * sizeof(double));
  else return 1;
  return 0;
}

int orc_fix_set(orc_fix *f, const char *what, const double *in) {
  size_t n3 = 3 * (size_t)f->n;
  if (!strcmp(what, "x")) memcpy(f->x, in, n3 * sizeof(double));
  else if (!strcmp(what, "v")) memcpy(f->v, in, n3 * sizeof(double));
  else if (!strcmp(what, "f")) memcpy(f->f, in, n3 * sizeof(double));
  else if (!strcmp(what, "T")) memcpy(f->fdm->T, in, (size_t)f->fdm->ntotal * sizeof(double));
  else return 1;
  return 0;
}

orc_fdm *orc_fix_fdm(orc_fix *f) { return f->fdm; }
orc_beta *orc_fix_beta(orc_fix *f) { return f->beta; }
long orc_fix_nbuild(const orc_fix *f) { return f->nbuild; }
double orc_fix_seconds(const orc_fix *f, int which) { return which == 0 ? f->t_fix : f->t_neigh; }

int orc_fix_neigh(const orc_fix *f, int *numneigh, int *owners, int maxn) {
  int mx = 0;
  for (int i = 0; i < f->n; ++i) {
    int c = f->numneigh[i];
    if (c > mx) mx = c;
    numneigh[i] = c;
    for (int k = 0; k < c && k < maxn; ++k) owners[(size_t)i * maxn + k] = f->neigh[(size_t)i * f->maxneigh + k];
  }
  return mx;
}
