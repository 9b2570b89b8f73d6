// Host side of the GB300 fix-eph path (see eph_host.hpp).  Compiled with
// -ffp-contract=off: the spline construction and the grid constants follow
// the reference's expressions term by term, so the device tables are the
// reference's tables bit for bit.
#include "eph_host.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "eph_gb.h"

namespace ephgb {

void Spline::build(double dx, const std::vector<double> &y) {
  const size_t points = y.size();
  inv_dx = 1. / dx;
  n = (long)points;
  // One zero knot past the end: at i = points-1 the slope loop below reads the
  // slope of knot `points`, one past the table (eph_spline.h:79-81 reads
  // c[i+1].b there); a zero slope reproduces the reference's choice in every
  // case except when that stray value equals z2 exactly.
  c.assign((points + 1) * 4, 0.0);
  auto A = [&](size_t i) -> double & { return c[4 * i + 0]; };
  auto B = [&](size_t i) -> double & { return c[4 * i + 1]; };
  auto C = [&](size_t i) -> double & { return c[4 * i + 2]; };
  auto D = [&](size_t i) -> double & { return c[4 * i + 3]; };
  double z0, z1, z2, z3;
  for (size_t i = 0; i < points - 1; ++i) B(i) = (y[i + 1] - y[i]) / dx;
  z1 = 2.0 * B(0) - B(1);
  z0 = 2.0 * z1 - B(0);
  z2 = 2.0 * B(points - 2) - B(points - 1);
  z3 = 2.0 * z2 - B(points - 1);
  B(points - 1) = z2;
  for (size_t i = 2; i < points - 2; ++i) {
    C(i) = std::fabs(B(i + 1) - B(i));
    D(i) = std::fabs(B(i - 1) - B(i - 2));
  }
  C(0) = std::fabs(B(1) - B(0));
  D(0) = std::fabs(z1 - z0);
  C(1) = std::fabs(B(2) - B(1));
  D(1) = std::fabs(B(0) - z1);
  C(points - 2) = std::fabs(z2 - B(points - 2));
  D(points - 2) = std::fabs(B(points - 3) - B(points - 4));
  C(points - 1) = std::fabs(z3 - z2);
  D(points - 1) = std::fabs(B(points - 2) - B(points - 3));
  for (size_t i = 0; i < points; ++i) {
    double d_2, d_1, d0, d1;
    if (i == 0) {
      d_2 = z0;
      d_1 = z1;
    } else if (i == 1) {
      d_2 = z1;
      d_1 = B(i - 1);
    } else {
      d_2 = B(i - 2);
      d_1 = B(i - 1);
    }
    d1 = B(i + 1);
    d0 = B(i);
    const double w1 = C(i), w0 = D(i);
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
  for (size_t i = 0; i < points - 1; ++i) {
    const double fi = (double)i, fi1 = (double)(i + 1);
    const double dx3 = dx * dx * dx;
    const double x0_1 = fi * dx, x0_2 = fi * dx * x0_1, x0_3 = fi * dx * x0_2;
    const double x1_1 = fi1 * dx, x1_2 = fi1 * dx * x1_1, x1_3 = fi1 * dx * x1_2;
    D(i) = (-A(i) * x0_1 - A(i + 1) * x0_1 + A(i) * x1_1 + A(i + 1) * x1_1 + 2.0 * y[i] - 2.0 * y[i + 1]) / dx3;
    C(i) = (-A(i) + A(i + 1) + 3.0 * D(i) * x0_2 - 3.0 * D(i) * x1_2) / 2.0 / dx;
    B(i) = (C(i) * x0_2 + D(i) * x0_3 - C(i) * x1_2 - D(i) * x1_3 - y[i] + y[i + 1]) / dx;
    A(i) = y[i] - B(i) * x0_1 - C(i) * x0_2 - D(i) * x0_3;
  }
  A(points - 1) = y[points - 1];
  B(points - 1) = 0.0;
  C(points - 1) = 0.0;
  D(points - 1) = 0.0;
  c.resize(points * 4);
}

double Spline::operator()(double x) const {
  size_t index = (size_t)(x * inv_dx);
  if (!(x >= 0.0) || index >= (size_t)n) return NAN;
  const double *k = &c[4 * index];
  return k[0] + x * (k[1] + x * (k[2] + x * k[3]));
}

std::string Beta::load(const char *path) {
  std::ifstream fd(path);
  if (!fd.is_open()) return std::string("cannot open beta file ") + path;
  std::string line;
  for (int k = 0; k < 3; ++k)
    if (!std::getline(fd, line)) return "beta file: missing comment lines";
  if (!std::getline(fd, line)) return "beta file: missing element line";
  {
    std::istringstream ss(line);
    if (!(ss >> n_elements) || n_elements < 1) return "beta file: no elements found";
    names.resize(n_elements);
    for (int i = 0; i < n_elements; ++i)
      if (!(ss >> names[i])) return "beta file: fewer element names than elements";
  }
  if (!(fd >> n_rho >> dr >> n_beta >> drho >> r_cutoff)) return "beta file: bad spline header";
  if (n_rho < 5 || n_beta < 5 || !(dr > 0) || !(drho > 0) || !(r_cutoff > 0)) return "beta file: bad spline header";
  r_cutoff_sq = r_cutoff * r_cutoff;
  rho_cutoff = drho * (double)(size_t)(n_beta - 1);
  dr_sq = r_cutoff_sq / (double)(size_t)(n_rho - 1);
  numbers.resize(n_elements);
  rho.resize(n_elements);
  rho_r_sq.resize(n_elements);
  beta.resize(n_elements);
  alpha.resize(n_elements);
  rho_knots.resize(n_elements);
  beta_knots.resize(n_elements);
  for (int e = 0; e < n_elements; ++e) {
    unsigned short z;
    if (!(fd >> z)) return "beta file: missing element number";
    numbers[e] = (uint8_t)z;
    std::vector<double> rk(n_rho, 0.0), bk(n_beta, 0.0);
    for (long j = 0; j < n_rho; ++j)
      if (!(fd >> rk[j])) return "beta file: too few rho(r) knots";
    for (long j = 0; j < n_beta; ++j)
      if (!(fd >> bk[j])) return "beta file: too few beta(rho) knots";
    std::string err = set_knots(e, rk.data(), n_rho, bk.data(), n_beta);
    if (!err.empty()) return err;
  }
  return "";
}

std::string Beta::set_knots(int e, const double *rho_col, long nr, const double *beta_col, long nb) {
  if (e < 0 || e >= n_elements) return "element index outside the beta file";
  if (nr != n_rho || nb != n_beta) return "knot counts differ from the beta file's";
  // eph_beta.h:103-124
  rho_knots[e].assign(rho_col, rho_col + nr);
  beta_knots[e].assign(beta_col, beta_col + nb);
  rho[e].build(dr, rho_knots[e]);
  std::vector<double> buf(n_rho);
  for (long j = 0; j < n_rho; ++j) buf[j] = rho[e](std::sqrt((double)(size_t)j * dr_sq));
  rho_r_sq[e].build(dr_sq, buf);
  beta[e].build(drho, beta_knots[e]);
  buf.assign(n_beta, 0.0);
  for (long j = 0; j < n_beta; ++j) buf[j] = std::sqrt(beta_knots[e][j]);
  alpha[e].build(drho, buf);
  return "";
}

void Beta::knot_gradient(int e, const double *g_rho_r_sq, const double *g_alpha, double *g_rho,
                         double *g_beta) const {
  // rho(r^2) table <- samples z_j = rho(r_j), r_j = sqrt(j dr^2)
  std::vector<double> z(n_rho), zbar(n_rho, 0.0);
  for (long j = 0; j < n_rho; ++j) z[j] = rho[e](std::sqrt((double)(size_t)j * dr_sq));
  spline_build_vjp(dr_sq, z, g_rho_r_sq, zbar.data());
  // z_j = a + r (b + r (c + r d)) of the rho(r) interval holding r_j
  std::vector<double> cbar((size_t)n_rho * 4, 0.0);
  for (long j = 0; j < n_rho; ++j) {
    const double r = std::sqrt((double)(size_t)j * dr_sq);
    const size_t idx = (size_t)(r * rho[e].inv_dx);
    if (!(r >= 0.0) || idx >= (size_t)n_rho) continue;  // outside the table: the value is NaN there
    cbar[4 * idx + 0] += zbar[j];
    cbar[4 * idx + 1] += zbar[j] * r;
    cbar[4 * idx + 2] += zbar[j] * r * r;
    cbar[4 * idx + 3] += zbar[j] * r * r * r;
  }
  for (long j = 0; j < n_rho; ++j) g_rho[j] = 0.0;
  spline_build_vjp(dr, rho_knots[e], cbar.data(), g_rho);
  // alpha knots are sqrt(beta knots)
  std::vector<double> a(n_beta), abar(n_beta, 0.0);
  for (long j = 0; j < n_beta; ++j) a[j] = std::sqrt(beta_knots[e][j]);
  spline_build_vjp(drho, a, g_alpha, abar.data());
  for (long j = 0; j < n_beta; ++j) g_beta[j] = a[j] > 0.0 ? 0.5 * abar[j] / a[j] : 0.0;
}

namespace {

// Forward-mode number: value and one directional derivative.
struct Dual {
  double v = 0.0, d = 0.0;
  Dual() = default;
  Dual(double a) : v(a) {}
  Dual(double a, double b) : v(a), d(b) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline bool operator==(Dual a, Dual b) { return a.v == b.v; }
inline bool operator!=(Dual a, Dual b) { return a.v != b.v; }
inline Dual dabs(Dual a) { return a.v < 0.0 ? -a : (a.v > 0.0 ? a : Dual(0.0, 0.0)); }

// Spline::build (eph_spline.h:31-132) on forward-mode numbers, same steps.
void build_dual(double dx, const std::vector<Dual> &y, std::vector<Dual> &c) {
  const size_t points = y.size();
  c.assign((points + 1) * 4, Dual(0.0));
  auto A = [&](size_t i) -> Dual & { return c[4 * i + 0]; };
  auto B = [&](size_t i) -> Dual & { return c[4 * i + 1]; };
  auto C = [&](size_t i) -> Dual & { return c[4 * i + 2]; };
  auto D = [&](size_t i) -> Dual & { return c[4 * i + 3]; };
  const Dual h(dx);
  for (size_t i = 0; i < points - 1; ++i) B(i) = (y[i + 1] - y[i]) / h;
  const Dual z1 = Dual(2.0) * B(0) - B(1);
  const Dual z0 = Dual(2.0) * z1 - B(0);
  const Dual z2 = Dual(2.0) * B(points - 2) - B(points - 1);
  const Dual z3 = Dual(2.0) * z2 - B(points - 1);
  B(points - 1) = z2;
  for (size_t i = 2; i < points - 2; ++i) {
    C(i) = dabs(B(i + 1) - B(i));
    D(i) = dabs(B(i - 1) - B(i - 2));
  }
  C(0) = dabs(B(1) - B(0));
  D(0) = dabs(z1 - z0);
  C(1) = dabs(B(2) - B(1));
  D(1) = dabs(B(0) - z1);
  C(points - 2) = dabs(z2 - B(points - 2));
  D(points - 2) = dabs(B(points - 3) - B(points - 4));
  C(points - 1) = dabs(z3 - z2);
  D(points - 1) = dabs(B(points - 2) - B(points - 3));
  for (size_t i = 0; i < points; ++i) {
    Dual d_2, d_1;
    if (i == 0) {
      d_2 = z0;
      d_1 = z1;
    } else if (i == 1) {
      d_2 = z1;
      d_1 = B(i - 1);
    } else {
      d_2 = B(i - 2);
      d_1 = B(i - 1);
    }
    const Dual d1 = B(i + 1), d0 = B(i);
    const Dual w1 = C(i), w0 = D(i);
    if (d_2 == d_1 && d0 != d1)
      A(i) = d_1;
    else if (d0 == d1 && d_2 == d_1)
      A(i) = d0;
    else if (d_1 == d0)
      A(i) = d0;
    else if (d_2 == d_1 && d0 == d1 && d0 != d_1)
      A(i) = Dual(0.5) * (d_1 + d0);
    else
      A(i) = (d_1 * w1 + d0 * w0) / (w1 + w0);
  }
  for (size_t i = 0; i < points - 1; ++i) {
    const double fi = (double)i, fi1 = (double)(i + 1);
    const Dual dx3(dx * dx * dx);
    const Dual x0_1(fi * dx), x0_2(fi * dx * (fi * dx)), x0_3(fi * dx * (fi * dx * (fi * dx)));
    const Dual x1_1(fi1 * dx), x1_2(fi1 * dx * (fi1 * dx)), x1_3(fi1 * dx * (fi1 * dx * (fi1 * dx)));
    const Dual two(2.0), three(3.0);
    D(i) = (-A(i) * x0_1 - A(i + 1) * x0_1 + A(i) * x1_1 + A(i + 1) * x1_1 + two * y[i] - two * y[i + 1]) / dx3;
    C(i) = (-A(i) + A(i + 1) + three * D(i) * x0_2 - three * D(i) * x1_2) / two / h;
    B(i) = (C(i) * x0_2 + D(i) * x0_3 - C(i) * x1_2 - D(i) * x1_3 - y[i] + y[i + 1]) / h;
    A(i) = y[i] - B(i) * x0_1 - C(i) * x0_2 - D(i) * x0_3;
  }
  A(points - 1) = y[points - 1];
  B(points - 1) = Dual(0.0);
  C(points - 1) = Dual(0.0);
  D(points - 1) = Dual(0.0);
  c.resize(points * 4);
}

}  // namespace

void spline_build_vjp(double dx, const std::vector<double> &y, const double *cbar, double *ybar) {
  const size_t n = y.size();
  constexpr size_t PERIOD = 16;  // > the width (6) of the window of knots an interval depends on
  std::vector<Dual> yd(n), c;
  for (size_t m = 0; m < PERIOD && m < n; ++m) {
    for (size_t k = 0; k < n; ++k) yd[k] = Dual(y[k], (k % PERIOD == m) ? 1.0 : 0.0);
    build_dual(dx, yd, c);
    // coefficients of interval i depend on knots i-2..i+3 (the two boundary
    // extrapolations z0..z3 stay inside that window): at most one seeded knot
    for (size_t i = 0; i < n; ++i) {
      const long lo = (long)i - 2 > 0 ? (long)i - 2 : 0;
      long k = lo + (long)((m + PERIOD - (size_t)lo % PERIOD) % PERIOD);
      if (k > (long)i + 3 || k >= (long)n) continue;
      double s = 0.0;
      for (int q = 0; q < 4; ++q) s += c[4 * i + q].d * cbar[4 * i + q];
      ybar[k] += s;
    }
  }
}

void Linear::build(double in_dx, const std::vector<double> &in_y) {
  dx = in_dx;
  y = in_y;
  dy.assign(y.size(), 0.0);
  for (size_t i = 0; i + 1 < y.size(); ++i) dy[i] = (y[i + 1] - y[i]) / dx;
  // dy has one entry per interval in the reference; at idx = n-1 it reads one
  // past its end (eph_linear.h:44-45) -- a zero slope there here
}

double Linear::operator()(double x) const {
  const size_t idx = (size_t)(x / dx);
  if (idx < y.size()) {
    const double delta = x - idx * dx;
    return y[idx] + dy[idx] * delta;
  }
  return 0.;
}

double Linear::reverse_lookup(double v) const {
  size_t lo = 0, hi = y.size();  // first element > v (std::upper_bound)
  while (lo < hi) {
    const size_t mid = (lo + hi) / 2;
    if (!(v < y[mid]))
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo != y.size() && lo > 0) {
    const size_t idx = lo - 1;
    return idx * dx + 1. / dy[idx] * (v - y[idx]);
  }
  return 0.;
}

const Spline &Beta::table(int which, int elem) const {
  switch (which) {
    case EPH_SPLINE_RHO_R: return rho[elem];
    case EPH_SPLINE_RHO_R_SQ: return rho_r_sq[elem];
    case EPH_SPLINE_BETA: return beta[elem];
    default: return alpha[elem];
  }
}

double Beta::get_beta(int elem, double r) const { return r > rho_cutoff ? 0. : beta[elem](r); }
double Beta::get_alpha(int elem, double r) const { return r > rho_cutoff ? 0. : alpha[elem](r); }

void Grid::set_box(double a0, double a1, double b0, double b1, double c0, double c1) {
  x0 = a0; x1 = a1; y0 = b0; y1 = b1; z0 = c0; z1 = c1;
  dx = (x1 - x0) / (double)(size_t)nx;
  dy = (y1 - y0) / (double)(size_t)ny;
  dz = (z1 - z0) / (double)(size_t)nz;
  dV = dx * dy * dz;
}

void Grid::create(long inx, long iny, long inz, double a0, double a1, double b0, double b1, double c0, double c1,
                  double T_e, double C_e, double rho_e, double kappa_e) {
  nx = inx; ny = iny; nz = inz;
  ntotal = nx * ny * nz;
  T.assign(ntotal, T_e);
  S.assign(ntotal, 0.0);
  rho.assign(ntotal, rho_e);
  C.assign(ntotal, C_e);
  kappa.assign(ntotal, kappa_e);
  flag.assign(ntotal, GRID_DYNAMIC);
  T_dynamic.assign(ntotal, 0);
  set_box(a0, a1, b0, b1, c0, c1);
  steps = 1;
  dt = 1;
  parameter_filename = "NULL";
}

std::string Grid::load(const char *path) {
  std::ifstream fd(path);
  if (!fd) return std::string("cannot open grid file ") + path;
  std::string line;
  for (int k = 0; k < 3; ++k)
    if (!std::getline(fd, line) || line.empty() || line[0] != '#') return "grid file: three '#' comment lines expected";
  if (!(fd >> nx >> ny >> nz >> steps) || nx < 1 || ny < 1 || nz < 1) return "grid file: bad size line";
  ntotal = nx * ny * nz;
  double b[6];
  for (double &v : b)
    if (!(fd >> v)) return "grid file: bad box lines";
  if (!(fd >> parameter_filename)) return "grid file: missing parameter-file line";
  if (parameter_filename != "NULL") {
    std::string e = load_parameters(parameter_filename.c_str());
    if (!e.empty()) return e;
  }
  T.assign(ntotal, 0.0);
  S.assign(ntotal, 0.0);
  rho.assign(ntotal, 0.0);
  C.assign(ntotal, 0.0);
  kappa.assign(ntotal, 0.0);
  flag.assign(ntotal, GRID_DYNAMIC);
  T_dynamic.assign(ntotal, 0);
  set_box(b[0], b[1], b[2], b[3], b[4], b[5]);
  for (long c = 0; c < ntotal; ++c) {
    long lx, ly, lz;
    int fl, td;
    double t, s, r, ce, k;
    if (!(fd >> lx >> ly >> lz >> t >> s >> r >> ce >> k >> fl >> td)) return "grid file: too few cell lines";
    const long index = lx + ly * nx + lz * nx * ny;
    if (lx < 0 || ly < 0 || lz < 0 || index >= ntotal) return "grid file: cell index outside the grid";
    if (td != 0 && !has_tdyn) return "grid file: temperature-dependent cells need a parameter file";
    T[index] = t;
    S[index] = s;
    rho[index] = r;
    C[index] = ce;
    kappa[index] = k;
    flag[index] = (int16_t)fl;
    T_dynamic[index] = (uint16_t)td;
  }
  dt = 1;
  return "";
}

std::string Grid::load_parameters(const char *path) {
  // eph_fdm.h:73-104: three comment lines, "n dT", then n lines "C_e kappa_e"
  std::ifstream fd(path);
  if (!fd) return std::string("cannot open grid parameter file ") + path;
  std::string line;
  for (int k = 0; k < 3; ++k)
    if (!std::getline(fd, line) || line.empty() || line[0] != '#')
      return "grid parameter file: three '#' comment lines expected";
  size_t n;
  double dT;
  if (!(fd >> n >> dT) || n < 5 || !(dT > 0)) return "grid parameter file: bad size line";
  std::vector<double> c(n), k(n);
  for (size_t i = 0; i < n; ++i)
    if (!(fd >> c[i] >> k[i])) return "grid parameter file: too few lines";
  C_T.build(dT, c);
  kappa_T.build(dT, k);
  c[0] = 0.;
  for (size_t i = 1; i < c.size(); ++i) c[i] = c[i - 1] + c[i] * dT;
  E_T.build(dT, c);
  has_tdyn = true;
  return "";
}

unsigned Grid::substeps(double *inner_dt_out) const {
  double c_min = C[0], rho_min = rho[0], kappa_max = kappa[0];
  for (long i = 1; i < ntotal; ++i)
    if (flag[i] != GRID_CONSTANT) {
      if (C[i] < c_min) c_min = C[i];
      if (rho[i] < rho_min) rho_min = rho[i];
      if (kappa[i] > kappa_max) kappa_max = kappa[i];
    }
  return substeps_from(c_min, rho_min, kappa_max, inner_dt_out);
}

unsigned Grid::substeps_from(double c_min, double rho_min, double kappa_max, double *inner_dt_out) const {
  double inner_dt = dt / (double)(size_t)steps;
  const double dtdxdydz = inner_dt * (1.0 / dx / dx + 1.0 / dy / dy + 1.0 / dz / dz);
  const double r = dtdxdydz / c_min / rho_min * kappa_max;
  unsigned new_steps = (unsigned)steps;
  if (r > 0.4) {
    inner_dt = 0.4 * inner_dt / r;
    const unsigned s = (unsigned)(dt / inner_dt);
    new_steps = s > 1u ? s : 1u;
    inner_dt = dt / new_steps;
  }
  *inner_dt_out = inner_dt;
  return new_steps;
}

int Grid::save_state(const char *path) const {
  FILE *fd = std::fopen(path, "w");
  if (!fd) return 1;
  std::fprintf(fd, "# A comment\n#\n#\n");
  std::fprintf(fd, "%ld %ld %ld %ld\n", nx, ny, nz, steps);
  std::fprintf(fd, "%.6e %.6e\n", x0, x1);
  std::fprintf(fd, "%.6e %.6e\n", y0, y1);
  std::fprintf(fd, "%.6e %.6e\n", z0, z1);
  std::fprintf(fd, "%s\n", parameter_filename.c_str());
  for (long k = 0; k < nz; ++k)
    for (long j = 0; j < ny; ++j)
      for (long i = 0; i < nx; ++i) {
        const long index = i + j * nx + k * nx * ny;
        std::fprintf(fd, "%d %d %d %.6e %.6e %.6e %.6e %.6e %d %d\n", (int)i, (int)j, (int)k, T[index], S[index],
                     rho[index], C[index], kappa[index], (int)flag[index], (int)T_dynamic[index]);
      }
  std::fclose(fd);
  return 0;
}

int Grid::save_temperature(const char *path, int n) const {
  char fn[4096];
  std::snprintf(fn, sizeof fn, "%s_%06d", path, n);
  FILE *fd = std::fopen(fn, "w");
  if (!fd) return 1;
  std::fprintf(fd, "x y z Te\n");
  for (long k = 0; k < nz; ++k)
    for (long j = 0; j < ny; ++j)
      for (long i = 0; i < nx; ++i) {
        const long index = i + j * nx + k * nx * ny;
        const double x = x0 + (int)i * dx, y = y0 + (int)j * dy, z = z0 + (int)k * dz;
        std::fprintf(fd, "%.6e %.6e %.6e %.6e\n", x, y, z, T[index]);
      }
  std::fclose(fd);
  return 0;
}

int parse_fix_args(int narg, const char *const *arg, FixArgs *a, std::string *why) {
  if (narg < 18) {
    *why = "Illegal fix eph command: too few arguments";
    return EPH_ERR_ARG;
  }
  a->style = arg[2];
  // the coloured-noise fix (fix_eph_coloured_exp.cpp:113) reads tau0 where
  // the plain fix reads the model, and always runs the PRL model
  a->coloured = a->style.find("coloured/exp") != std::string::npos;
  a->seed = std::atoi(arg[3]);
  a->flags = (int)std::strtol(arg[4], nullptr, 0);
  if (a->coloured) {
    a->tau0 = std::atof(arg[5]);
    a->model = 4;
  } else {
    a->model = std::atoi(arg[5]);
  }
  a->rho_e = std::atof(arg[6]);
  a->C_e = std::atof(arg[7]);
  a->kappa_e = std::atof(arg[8]);
  a->T_e = std::atof(arg[9]);
  a->nx = std::atoi(arg[10]);
  a->ny = std::atoi(arg[11]);
  a->nz = std::atoi(arg[12]);
  a->T_infile = arg[13];
  if (a->T_infile == "NULL") {
    if (a->nx < 1 || a->ny < 1 || a->nz < 1) {
      *why = "FixEPH: non-positive grid values";
      return EPH_ERR_ARG;
    }
    a->T_state = "T.restart";
  } else {
    a->T_state = a->T_infile + ".restart";
  }
  a->T_freq = std::atoi(arg[14]);
  if (a->T_freq > 0) a->T_out = arg[15];
  a->beta_file = arg[16];
  a->elements.clear();
  for (int i = 17; i < narg; ++i) a->elements.emplace_back(arg[i]);
  return EPH_OK;
}

void hermite_table(const std::vector<double> &y, std::vector<double> &coef) {
  const size_t n = y.size();
  coef.assign(4 * n, 0.0);
  if (n == 0) return;
  if (n == 1) {
    coef[0] = y[0];
    return;
  }
  std::vector<double> s(n);
  s[0] = y[1] - y[0];
  s[n - 1] = y[n - 1] - y[n - 2];
  if (n > 2) {
    s[1] = 0.5 * (y[2] - y[0]);
    s[n - 2] = 0.5 * (y[n - 1] - y[n - 3]);
  }
  for (size_t m = 2; m + 2 < n; ++m) s[m] = ((y[m - 2] - y[m + 2]) + 8.0 * (y[m + 1] - y[m - 1])) / 12.0;
  for (size_t m = 0; m + 1 < n; ++m) {
    const double d = y[m + 1] - y[m];
    coef[4 * m + 0] = y[m];
    coef[4 * m + 1] = s[m];
    coef[4 * m + 2] = 3.0 * d - 2.0 * s[m] - s[m + 1];
    coef[4 * m + 3] = s[m] + s[m + 1] - 2.0 * d;
  }
  coef[4 * (n - 1) + 0] = y[n - 1];
  coef[4 * (n - 1) + 1] = s[n - 1];
}

std::string Eam::load(const char *path) {
  std::ifstream fd(path);
  if (!fd) return std::string("cannot open setfl file ") + path;
  std::string line;
  for (int k = 0; k < 3; ++k)
    if (!std::getline(fd, line)) return "setfl file: missing comment lines";
  if (!std::getline(fd, line)) return "setfl file: missing element line";
  {
    std::istringstream ss(line);
    if (!(ss >> nel) || nel < 1 || nel > 16) return "setfl file: bad element count";
    names.resize(nel);
    for (auto &nm : names)
      if (!(ss >> nm)) return "setfl file: fewer element names than elements";
  }
  if (!(fd >> nrho >> drho >> nr >> dr >> rc) || nrho < 5 || nr < 5 || !(drho > 0) || !(dr > 0) || !(rc > 0))
    return "setfl file: bad table header";
  mass.assign(nel, 0.0);
  F.assign(nel, {});
  f.assign(nel, {});
  for (int e = 0; e < nel; ++e) {
    double z, a;
    std::string lat;
    if (!(fd >> z >> mass[e] >> a >> lat)) return "setfl file: bad element header";
    F[e].resize(nrho);
    for (auto &v : F[e])
      if (!(fd >> v)) return "setfl file: too few F(rho) values";
    f[e].resize(nr);
    for (auto &v : f[e])
      if (!(fd >> v)) return "setfl file: too few f(r) values";
  }
  z2r.assign(nel * (nel + 1) / 2, {});
  for (int a = 0; a < nel; ++a)
    for (int b = 0; b <= a; ++b) {
      auto &t = z2r[a * (a + 1) / 2 + b];
      t.resize(nr);
      for (auto &v : t)
        if (!(fd >> v)) return "setfl file: too few r*phi(r) values";
    }
  return "";
}

}  // namespace ephgb

