// Host side of the GB300 fix-eph path: the beta(rho) parametrisation, the
// electronic-temperature grid and the fix argument parser.  Everything here
// runs on the CPU once per set-up (or per file write); the per-step work is in
// eph_kernels.cuh.  Compiled without floating-point contraction so that the
// spline tables and grid constants are the reference's to the last bit.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ephgb {

// Cubic spline of eph_spline.h (Akima-type slopes, coefficients in absolute x,
// evaluated as a + x(b + x(c + x d)) with index floor(x / dx)).
struct Spline {
  double inv_dx = 0.0;
  std::vector<double> c;  // a, b, c, d per knot
  long n = 0;
  // eph_spline.h:31-132
  void build(double dx, const std::vector<double> &y);
  // eph_spline.h:134-142
  double operator()(double x) const;
};

// beta(rho) file of eph_beta.h:39-128: per element rho(r), rho(r^2) (re-spline
// of rho(r) sampled at sqrt(j dr^2)), beta(rho) and alpha(rho) = spline of
// sqrt(beta) knots.
struct Beta {
  int n_elements = 0;
  std::vector<std::string> names;
  std::vector<int> numbers;
  double r_cutoff = 0, r_cutoff_sq = 0, rho_cutoff = 0;
  long n_rho = 0, n_beta = 0;
  double dr = 0, dr_sq = 0, drho = 0;
  std::vector<Spline> rho, rho_r_sq, beta, alpha;
  // the file's knot columns per element: rho(r) (n_rho values), beta(rho) (n_beta)
  std::vector<std::vector<double>> rho_knots, beta_knots;
  // returns an empty string on success, else the reason
  std::string load(const char *path);
  // replace element e's knot columns and rebuild its four tables as load() does
  std::string set_knots(int e, const double *rho_col, long nr, const double *beta_col, long nb);
  // Chain rule through the table construction: from dL/d(coefficients) of the
  // rho(r^2) table (n_rho x 4) and of the alpha table (n_beta x 4) of element
  // e to dL/d(knot columns), written to g_rho (n_rho) and g_beta (n_beta).
  void knot_gradient(int e, const double *g_rho_r_sq, const double *g_alpha, double *g_rho, double *g_beta) const;
  const Spline &table(int which, int elem) const;
  // eph_beta.h:174-197 (zero above rho_cutoff)
  double get_beta(int elem, double r) const;
  double get_alpha(int elem, double r) const;
};

// Reverse-mode product of Spline::build: given cbar = dL/d(coefficients)
// (4 per knot) of the table built from knots y with spacing dx, adds
// dL/dy to ybar.  The construction is local (the coefficients of interval i
// depend on y[i-2 .. i+3]), so 16 forward-mode passes with interleaved seeds
// give the exact Jacobian-transpose product for any number of knots.
void spline_build_vjp(double dx, const std::vector<double> &y, const double *cbar, double *ybar);

enum : int { GRID_CONSTANT = 0, GRID_DYNAMIC = 1, GRID_ZERO_DERIVATIVE = 2 };

// Piecewise-linear table with a reverse lookup (eph_linear.h:21-75), used for
// the electronic energy E_e(T) = integral of C_e(T) dT.
struct Linear {
  double dx = 1;
  std::vector<double> y, dy;  // dy[i] = (y[i+1] - y[i]) / dx; dy[n-1] = 0
  void build(double dx, const std::vector<double> &y);
  double operator()(double x) const;        // eph_linear.h:41-48
  double reverse_lookup(double v) const;    // eph_linear.h:51-60
};

// Electronic grid of eph_fdm.h: uniform (constructor :28-46) or read from a
// grid file (:48-119); index i + j nx + k nx ny.
struct Grid {
  long nx = 1, ny = 1, nz = 1, ntotal = 1;
  double x0 = 0, x1 = 1, y0 = 0, y1 = 1, z0 = 0, z1 = 1, dx = 1, dy = 1, dz = 1, dV = 1;
  std::vector<double> T, S, rho, C, kappa;
  std::vector<int16_t> flag;
  std::vector<uint16_t> T_dynamic;
  std::string parameter_filename = "NULL";
  long steps = 1;
  double dt = 1;
  // temperature-dependent cells (T_dynamic != 0): C_e(T), kappa_e(T) splines
  // and E_e(T), read from the parameter file (eph_fdm.h:73-104)
  bool has_tdyn = false;
  Spline C_T, kappa_T;
  Linear E_T;
  std::string load_parameters(const char *path);
  // substeps from given bounds (c_min, rho_min, kappa_max over the grid)
  unsigned substeps_from(double c_min, double rho_min, double kappa_max, double *inner_dt) const;

  void create(long nx, long ny, long nz, double x0, double x1, double y0, double y1, double z0, double z1,
              double T_e, double C_e, double rho_e, double kappa_e);
  std::string load(const char *path);
  void set_box(double x0, double x1, double y0, double y1, double z0, double z1);
  // eph_fdm.h:275-313: number and length of the stability substeps of solve()
  unsigned substeps(double *inner_dt) const;
  // eph_fdm.h:226-265 and :198-224, same text format
  int save_state(const char *path) const;
  int save_temperature(const char *path, int n) const;
};

// Cubic Hermite table of knots y (spacing h): per interval m the coefficients
// {c0, c1, c2, c3} of y(p) = c0 + p (c1 + p (c2 + p c3)) in the local
// coordinate p = x/h - m in [0, 1]; knot slopes from the five-point central
// difference (one-sided at the ends); the last entry continues the last knot
// linearly.  dy/dx = (c1 + p (2 c2 + 3 p c3)) / h.
void hermite_table(const std::vector<double> &y, std::vector<double> &coef);

// eam/alloy potential read from a setfl file (the LAMMPS format: 3 comment
// lines; "N el1 el2 ..."; "Nrho drho Nr dr cutoff"; per element "Z mass a
// lattice", Nrho values of F(rho), Nr values of f(r); then r*phi(r) for every
// pair a >= b, Nr values each).
struct Eam {
  int nel = 0;
  std::vector<std::string> names;
  std::vector<double> mass;
  long nrho = 0, nr = 0;
  double drho = 0, dr = 0, rc = 0;
  std::vector<std::vector<double>> F, f;  // knots per element
  std::vector<std::vector<double>> z2r;   // r*phi knots per pair a*(a+1)/2 + b, a >= b
  std::string load(const char *path);
};

// Parsed `fix ID group eph seed flags model rho_e C_e kappa_e T_e NX NY NZ
// T_infile freq T_out beta_file A B ...` (fix_eph.cpp:36-58, :61-241).
struct FixArgs {
  std::string style;        // arg[2]: "eph", or "eph/coloured/exp" (arg[5] is then tau0)
  bool coloured = false;
  double tau0 = 0;
  int seed = 0, flags = 0, model = 0;
  double rho_e = 0, C_e = 0, kappa_e = 0, T_e = 0;
  int nx = 0, ny = 0, nz = 0;
  std::string T_infile, T_out, beta_file, T_state;
  int T_freq = 0;
  std::vector<std::string> elements;
};

enum : int {
  FLAG_FRICTION = 0x01,
  FLAG_RANDOM = 0x02,
  FLAG_FDM = 0x04,
  FLAG_NOINT = 0x08,
  FLAG_NOFRICTION = 0x10,
  FLAG_NORANDOM = 0x20
};

// Returns 0 or an EPH_ERR_* code with `why` filled.
int parse_fix_args(int narg, const char *const *arg, FixArgs *out, std::string *why);

}  // namespace ephgb
