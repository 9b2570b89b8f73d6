/*
 * CPU restatement of the USER-EPH `fix eph` hot path (model 4, PRL 120,
 * 185501).  TEST INFRASTRUCTURE ONLY: the parity checker of the CUDA path and
 * the timed CPU baseline.  The product never links it.
 *
 * Every function follows a reference function and keeps its floating-point
 * expression order (the file is compiled with -ffp-contract=off):
 *   orc_spline_*   eph_spline.h:31-142
 *   orc_beta_*     eph_beta.h:39-198
 *   orc_fdm_*      eph_fdm.h:28-400, :494-509
 *   orc_fix_*      fix_eph.cpp:61-241 (construction), :305-348 (integrator),
 *                  :350-429 (end_of_step), :431-466 (density),
 *                  :687-837 (force_prl), :841-907 (post_force)
 *   orc_ranmars_*  Marsaglia-Zaman RANMAR uniform generator and the
 *                  Marsaglia polar Gaussian, the generator the engine's
 *                  RanMars uses (LAMMPS random_mars.cpp is not part of the
 *                  reference tree; restated from the published algorithm)
 * The engine around the fix (ghost images, neighbour list with skin, the
 * rebuild schedule, position wrapping) follows the LAMMPS behaviour the fix
 * relies on; the neighbour order is ascending atom index.
 */
#ifndef EPH_ORACLE_H
#define EPH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_beta orc_beta;
typedef struct orc_fdm orc_fdm;
typedef struct orc_fix orc_fix;

/* Akima-type spline of eph_spline.h on knots y[0..n-1] spaced dx from 0. */
typedef struct {
  double inv_dx;
  long n;
  double *c; /* 4 per knot: a, b, c, d (absolute-x polynomial) */
} orc_spline;
int orc_spline_build(orc_spline *s, double dx, const double *y, long n);
double orc_spline_eval(const orc_spline *s, double x);
void orc_spline_free(orc_spline *s);

orc_beta *orc_beta_load(const char *path);
void orc_beta_free(orc_beta *b);
int orc_beta_n_elements(const orc_beta *b);
const char *orc_beta_element_name(const orc_beta *b, int i);
double orc_beta_r_cutoff(const orc_beta *b);
double orc_beta_rho_cutoff(const orc_beta *b);
/* which: 0 rho(r), 1 rho(r^2), 2 beta(rho), 3 alpha(rho) -- raw spline value */
double orc_beta_eval(const orc_beta *b, int which, int elem, double x);
double orc_beta_get_beta(orc_beta *b, int elem, double rho);
double orc_beta_get_alpha(orc_beta *b, int elem, double rho);
/* copy the coefficient table (4 doubles per knot) of one spline; returns knots */
long orc_beta_table(const orc_beta *b, int which, int elem, double *out);

orc_fdm *orc_fdm_create(long nx, long ny, long nz, double x0, double x1, double y0, double y1, double z0,
                        double z1, double T_e, double C_e, double rho_e, double kappa_e);
orc_fdm *orc_fdm_load(const char *path);
void orc_fdm_free(orc_fdm *g);
void orc_fdm_set_dt(orc_fdm *g, double dt);
void orc_fdm_insert_energy(orc_fdm *g, double x, double y, double z, double E);
double orc_fdm_get_T(const orc_fdm *g, double x, double y, double z);
double orc_fdm_get_T_total(const orc_fdm *g);
long orc_fdm_get_index(const orc_fdm *g, double x, double y, double z);
/* returns the number of substeps taken */
unsigned orc_fdm_solve(orc_fdm *g);
int orc_fdm_save_state(const orc_fdm *g, const char *path);
int orc_fdm_save_temperature(const orc_fdm *g, const char *path, int n);
long orc_fdm_ncells(const orc_fdm *g);
/* field: 0 T_e, 1 dT_e, 2 S_e, 3 rho_e, 4 C_e, 5 kappa_e */
int orc_fdm_get(const orc_fdm *g, int field, double *out);
int orc_fdm_set(orc_fdm *g, int field, const double *in);

/* The fix, constructed from the words of the fix command exactly as the
 * reference parses them (arg[0] fix ID, arg[1] group, arg[2] style name,
 * arg[3..] positional arguments).  mass[1..ntypes]; boxlo/boxhi the periodic
 * box; skin the neighbour skin of the engine.  Returns NULL and fills err. */
orc_fix *orc_fix_create(int narg, const char **arg, int ntypes, const double *mass, const double *boxlo,
                        const double *boxhi, double dt, double boltz, double ftm2v, double skin, char *err,
                        int errlen);
void orc_fix_free(orc_fix *f);
int orc_fix_set_atoms(orc_fix *f, int n, const double *x, const double *v, const int *type, const int *mask,
                      int groupbit);
int orc_fix_set_fext(orc_fix *f, const double *fext);
/* number of OpenMP threads used by the per-atom loops (1 = serial) */
void orc_fix_set_threads(orc_fix *f, int nthreads);
/* One engine step (initial_integrate, neighbour decision, force clear,
 * post_force, final_integrate, end_of_step).  xi: 3 deviates per in-group atom
 * in atom order when the random term is on; NULL draws them from the
 * restated RanMars seeded like the reference (seed + rank 0). */
int orc_fix_step(orc_fix *f, const double *xi);
/* the four hooks, for callers that drive the step themselves */
void orc_fix_initial_integrate(orc_fix *f);
void orc_fix_neighbor_decide(orc_fix *f);
void orc_fix_clear_forces(orc_fix *f);
int orc_fix_post_force(orc_fix *f, const double *xi);
void orc_fix_final_integrate(orc_fix *f);
void orc_fix_end_of_step(orc_fix *f);
/* "x","v","f","f_eph","f_rng","w","xi" (3/atom), "rho","alpha" (1/atom),
 * "array" (8/atom), "vector" (2), "T" (grid) */
int orc_fix_get(orc_fix *f, const char *what, double *out);
int orc_fix_set(orc_fix *f, const char *what, const double *in);
orc_fdm *orc_fix_fdm(orc_fix *f);
orc_beta *orc_fix_beta(orc_fix *f);
long orc_fix_nbuild(const orc_fix *f);
/* per-atom neighbour list in ascending owner order (cutoff rc + skin):
 * returns the largest row; row i holds numneigh[i] owners at i*maxn */
int orc_fix_neigh(const orc_fix *f, int *numneigh, int *owners, int maxn);
/* the seconds spent in the fix's own hooks (integrator, post_force,
 * end_of_step) since creation, and in neighbour-list builds */
double orc_fix_seconds(const orc_fix *f, int which);

/* RANMAR uniform + polar Gaussian (restated published algorithm) */
typedef struct {
  double u[98];
  double c, cd, cm;
  int i97, j97;
  int save;
  double second;
} orc_ranmars;
int orc_ranmars_init(orc_ranmars *r, int seed);
double orc_ranmars_uniform(orc_ranmars *r);
double orc_ranmars_gaussian(orc_ranmars *r);
/* Marsaglia-Zaman two-seed initialisation (ij in [0,31328], kl in [0,30081]) */
void orc_ranmars_init_ijkl(orc_ranmars *r, int ij, int kl);

#ifdef __cplusplus
}
#endif
#endif
