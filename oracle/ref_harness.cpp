/*
 * Parity harness around the reference `fix eph` (USER-EPH fix_eph.cpp,
 * fix_eph.h, eph_beta.h, eph_spline.h, eph_fdm.h, eph_linear.h compiled
 * UNCHANGED from the reference tree) running inside the engine stand-in of
 * lammps_mock/.  TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into
 * oracle/_ref/ when the reference sources are present, loaded by tests to pin
 * the CPU restatement (eph_oracle.c) and to write the golden fixtures.
 *
 * Engine behaviour reproduced here (LAMMPS Verlet::run order, see
 * fix_eph.cpp:293-302 for the hooks the fix registers):
 *   setup : wrap positions, make ghosts, build the full list, f = f_ext
 *   step  : ntimestep += 1; initial_integrate (fix_eph.cpp:305-328);
 *           rebuild if any atom moved > skin/2 (wrap, ghosts, list) else
 *           copy owner x, v to ghosts; f = f_ext; post_force (:841-907);
 *           final_integrate (:330-348); end_of_step (:350-429)
 * The Gaussian deviates the fix draws with RanMars::gaussian() are injected.
 */
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "atom.h"
#include "comm.h"
#include "domain.h"
#include "error.h"
#include "fix.h"
#include "force.h"
#include "memory.h"
#include "neigh_list.h"
#include "neighbor.h"
#include "random_mars.h"
#include "update.h"
#include "engine.hpp"

#include "fix_eph.h"
#include "fix_eph_coloured_exp.h"

using namespace LAMMPS_NS;

namespace {

// Read access to the per-atom arrays of a reference fix (`eph` and
// `eph/coloured/exp` name them alike).
struct Access {
  virtual ~Access() = default;
  virtual double *rho() = 0;
  virtual double **feph() = 0;
  virtual double **frng() = 0;
  virtual double **w() = 0;
  virtual double **xi() = 0;
  virtual double **arr() = 0;
  virtual RanMars *rng() = 0;
  virtual double T_at(double x, double y, double z) const = 0;
  virtual void save_T(const char *path, int n) const = 0;
  virtual void save_state(const char *path) const = 0;
};

template <class F>
class Probe : public F, public Access {
 public:
  Probe(LAMMPS *l, int narg, char **arg) : F(l, narg, arg) {}
  double *rho() override { return this->rho_i; }
  double **feph() override { return this->f_EPH; }
  double **frng() override { return this->f_RNG; }
  double **w() override { return this->w_i; }
  double **xi() override { return this->xi_i; }
  double **arr() override { return this->array; }
  RanMars *rng() override { return this->random; }
  double T_at(double x, double y, double z) const override { return this->fdm.get_T(x, y, z); }
  void save_T(const char *path, int n) const override { this->fdm.save_temperature(path, n); }
  void save_state(const char *path) const override { this->fdm.save_state(path); }
};

struct Sim : Engine {
  Access *acc = nullptr;
  Access *probe() { return acc; }
};

void copy_err(const char *msg, char *errbuf, int errlen) {
  if (errbuf && errlen > 0) {
    std::strncpy(errbuf, msg, (size_t)errlen - 1);
    errbuf[errlen - 1] = 0;
  }
}

}  // namespace

extern "C" {

/* Build the engine with `nlocal` atoms and construct the reference fix from
 * the fix command's words (arg[0] = fix ID, arg[1] = group, arg[2] = "eph",
 * then the reference's positional arguments, fix_eph.cpp:36-58).
 * mass[1..ntypes] are per-type masses.  Returns NULL on error. */
void *ref_create(int narg, const char **arg, int nlocal, const double *x, const double *v, const int *type,
                 const int *mask, int ntypes, const double *mass, const double *lo, const double *hi, double dt,
                 double boltz, double ftm2v, double skin, char *errbuf, int errlen) {
  Sim *s = new Sim();
  try {
    s->load(nlocal, x, v, type, mask, ntypes, mass, lo, hi, dt, boltz, ftm2v, skin);
    std::vector<std::string> words(arg, arg + narg);
    std::vector<char *> argv;
    for (auto &w : words) argv.push_back(&w[0]);
    Fix *f;
    if (narg > 2 && std::string(arg[2]) == "eph/coloured/exp") {
      auto *p = new Probe<FixEPHColouredExp>(&s->lmp, narg, argv.data());
      f = p;
      s->acc = p;
    } else {
      auto *p = new Probe<FixEPH>(&s->lmp, narg, argv.data());
      f = p;
      s->acc = p;
    }
    s->fix = f;
    s->rng = s->acc->rng();
    f->init();
    if (s->neighbor.nrequest != 1) throw std::runtime_error("fix did not request a neighbour list");
    s->cutneigh = s->neighbor.request.cutoff + skin;
    f->init_list(0, &s->list);
    s->setup();
  } catch (std::exception &e) {
    copy_err(e.what(), errbuf, errlen);
    delete s;
    return nullptr;
  }
  return s;
}

void ref_destroy(void *h) { delete static_cast<Sim *>(h); }

/* Per-atom constant external force (stands in for the pair style); NULL = 0. */
int ref_set_fext(void *h, const double *fext) {
  Sim *s = static_cast<Sim *>(h);
  if (fext)
    s->fext.assign(fext, fext + 3 * (size_t)s->atom.nlocal);
  else
    s->fext.clear();
  s->clear_forces();
  return 0;
}

/* One Verlet step.  `xi` holds the deviates RanMars::gaussian() returns this
 * step, in draw order (nxi values); pass NULL when the fix draws none. */
int ref_step(void *h, const double *xi, long nxi, char *errbuf, int errlen) {
  Sim *s = static_cast<Sim *>(h);
  try {
    s->step(xi, nxi);
  } catch (std::exception &e) {
    copy_err(e.what(), errbuf, errlen);
    return 1;
  }
  return 0;
}

/* Copy a per-atom quantity of the locals into out:
 * "x","v","f","f_eph","f_rng","w","xi" (3 per atom), "rho" (1 per atom),
 * "array" (8 per atom), "vector" (2 values: compute_vector(0), (1)). */
int ref_get(void *h, const char *what, double *out) {
  Sim *s = static_cast<Sim *>(h);
  const int n = s->atom.nlocal;
  auto rows3 = [&](double **a) {
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) out[3 * (size_t)i + k] = a[i][k];
  };
  const std::string w(what);
  if (w == "x") rows3(s->atom.x);
  else if (w == "v") rows3(s->atom.v);
  else if (w == "f") rows3(s->atom.f);
  else if (w == "f_eph") rows3(s->probe()->feph());
  else if (w == "f_rng") rows3(s->probe()->frng());
  else if (w == "w") rows3(s->probe()->w());
  else if (w == "xi") rows3(s->probe()->xi());
  else if (w == "rho") {
    for (int i = 0; i < n; ++i) out[i] = s->probe()->rho()[i];
  } else if (w == "array") {
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 8; ++k) out[8 * (size_t)i + k] = s->probe()->arr()[i][k];
  } else if (w == "vector") {
    out[0] = s->fix->compute_vector(0);
    out[1] = s->fix->compute_vector(1);
  } else
    return 1;
  return 0;
}

/* Electronic temperature of every grid cell, read at the cell centres of an
 * nx*ny*nz grid spanning [lo, hi); index i + j*nx + k*nx*ny. */
int ref_get_T(void *h, int nx, int ny, int nz, const double *lo, const double *hi, double *out) {
  Sim *s = static_cast<Sim *>(h);
  const double dx = (hi[0] - lo[0]) / nx, dy = (hi[1] - lo[1]) / ny, dz = (hi[2] - lo[2]) / nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        out[i + (size_t)nx * (j + (size_t)ny * k)] =
            s->probe()->T_at(lo[0] + (i + 0.5) * dx, lo[1] + (j + 0.5) * dy, lo[2] + (k + 0.5) * dz);
  return 0;
}

/* The current full list: numneigh[i] and the owner index of each neighbour,
 * row i at neigh[i*maxn ...].  Returns the largest count (fills nothing
 * beyond maxn). */
int ref_get_neigh(void *h, int *numneigh, int *owners, int maxn) {
  Sim *s = static_cast<Sim *>(h);
  int mx = 0;
  for (int i = 0; i < s->atom.nlocal; ++i) {
    const int c = s->numneigh[i];
    mx = std::max(mx, c);
    numneigh[i] = c;
    for (int k = 0; k < c && k < maxn; ++k) owners[(size_t)i * maxn + k] = s->owner(s->neigh[i][k]);
  }
  return mx;
}

long ref_nbuild(void *h) { return static_cast<Sim *>(h)->nbuild; }

int ref_save_temperature(void *h, const char *path, int n) {
  static_cast<Sim *>(h)->probe()->save_T(path, n);
  return 0;
}

int ref_save_state(void *h, const char *path) {
  static_cast<Sim *>(h)->probe()->save_state(path);
  return 0;
}

}  // extern "C"

/* ----------------------------------------------------------------------
 * The reference parametrisation and grid classes on their own
 * (eph_beta.h, eph_spline.h, eph_fdm.h), for table-level comparisons.
 * ---------------------------------------------------------------------- */
namespace {
// Read access to the protected coefficient tables (layout-identical views).
struct SplineView : Spline {
  static const std::vector<Coefficients> &coeffs(const Spline &s) { return static_cast<const SplineView &>(s).c; }
  static size_t coeff_size() { return sizeof(Coefficients); }
};
struct BetaView : Beta {
  static const Spline &table(const Beta &b, int which, int e) {
    const BetaView &v = static_cast<const BetaView &>(b);
    switch (which) {
      case 0: return v.rho[e];
      case 1: return v.rho_r_sq[e];
      case 2: return v.beta[e];
      default: return v.alpha[e];
    }
  }
};
}  // namespace

extern "C" {

void *refb_load(const char *path) { return new Beta(path); }
void refb_free(void *b) { delete static_cast<Beta *>(b); }
int refb_n_elements(void *b) { return (int)static_cast<Beta *>(b)->get_n_elements(); }
double refb_r_cutoff(void *b) { return static_cast<Beta *>(b)->get_r_cutoff(); }
double refb_rho_cutoff(void *b) { return static_cast<Beta *>(b)->get_rho_cutoff(); }

/* which: 0 rho(r), 1 rho(r^2), 2 beta(rho) via get_beta, 3 alpha(rho) via get_alpha */
double refb_eval(void *h, int which, int elem, double x) {
  Beta *b = static_cast<Beta *>(h);
  switch (which) {
    case 0: return b->get_rho(elem, x);
    case 1: return b->get_rho_r_sq(elem, x);
    case 2: return b->get_beta(elem, x);
    default: return b->get_alpha(elem, x);
  }
}

long refb_table(void *h, int which, int elem, double *out) {
  const Spline &s = BetaView::table(*static_cast<Beta *>(h), which, elem);
  const auto &c = SplineView::coeffs(s);
  if (out) std::memcpy(out, c.data(), c.size() * SplineView::coeff_size());
  return (long)c.size();
}

void *refg_create(long nx, long ny, long nz, const double *lo, const double *hi, double T, double Ce, double rho,
                  double kappa) {
  EPH_FDM *g = new EPH_FDM(nx, ny, nz, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], T, Ce, rho, kappa);
  g->set_comm(0, 0, 1);
  return g;
}
void *refg_load(const char *path) {
  EPH_FDM *g = new EPH_FDM(path);
  g->set_comm(0, 0, 1);
  return g;
}
void refg_free(void *g) { delete static_cast<EPH_FDM *>(g); }
void refg_set_dt(void *g, double dt) { static_cast<EPH_FDM *>(g)->set_dt(dt); }
void refg_insert_energy(void *g, double x, double y, double z, double E) {
  static_cast<EPH_FDM *>(g)->insert_energy(x, y, z, E);
}
double refg_get_T(void *g, double x, double y, double z) { return static_cast<EPH_FDM *>(g)->get_T(x, y, z); }
double refg_get_T_total(void *g) { return static_cast<EPH_FDM *>(g)->get_T_total(); }
void refg_solve(void *g) { static_cast<EPH_FDM *>(g)->solve(); }
void refg_save_state(void *g, const char *path) { static_cast<EPH_FDM *>(g)->save_state(path); }
void refg_save_temperature(void *g, const char *path, int n) {
  static_cast<EPH_FDM *>(g)->save_temperature(path, n);
}

}  // extern "C"
