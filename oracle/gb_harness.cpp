/*
 * The GB300 fix eph/gb (user-eph_gb300/lammps/fix_eph_gb.cpp) running inside
 * the same engine stand-in as the reference fix (lammps_mock/engine.hpp).
 * TEST INFRASTRUCTURE ONLY: it shows the fix is a drop-in (same words, same
 * hooks, same RanMars draws) and lets tests compare its outputs with the
 * reference's.  Built by oracle/Makefile against libephgb.so.
 */
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.hpp"
#include "fix_eph_gb.h"

using namespace LAMMPS_NS;

namespace {

class FixGBProbe : public FixEPHGB {
 public:
  FixGBProbe(LAMMPS *l, int narg, char **arg) : FixEPHGB(l, narg, arg) {}
  RanMars *rng() { return random; }
  double **arr() { return array; }
};

struct GbSim : Engine {
  FixGBProbe *probe() { return static_cast<FixGBProbe *>(fix); }
};

void copy_err(const char *msg, char *errbuf, int errlen) {
  if (errbuf && errlen > 0) {
    std::strncpy(errbuf, msg, (size_t)errlen - 1);
    errbuf[errlen - 1] = 0;
  }
}

}  // namespace

extern "C" {

/* The engine with the fix eph/gb built from the fix words; rc is the density
 * cutoff (the engine's ghost/list cutoff is rc + skin, as for the reference
 * fix); mode 0 exact / 1 fast; xi_host 1 draws the deviates from the
 * engine's RanMars stream. */
void *gbh_create(int narg, const char **arg, int nlocal, const double *x, const double *v, const int *type,
                 const int *mask, int ntypes, const double *mass, const double *lo, const double *hi, double dt,
                 double boltz, double ftm2v, double skin, double rc, int mode, int xi_host, char *errbuf,
                 int errlen) {
  GbSim *s = new GbSim();
  try {
    s->load(nlocal, x, v, type, mask, ntypes, mass, lo, hi, dt, boltz, ftm2v, skin);
    std::vector<std::string> words(arg, arg + narg);
    std::vector<char *> argv;
    for (auto &w : words) argv.push_back(&w[0]);
    FixGBProbe *f = new FixGBProbe(&s->lmp, narg, argv.data());
    s->fix = f;
    s->rng = f->rng();
    std::string m0 = "mode", m1 = mode ? "fast" : "exact", x0 = "xi", x1 = xi_host ? "host" : "device";
    char *a1[2] = {&m0[0], &m1[0]}, *a2[2] = {&x0[0], &x1[0]};
    f->modify_param(2, a1);
    f->modify_param(2, a2);
    f->init();
    s->cutneigh = rc + skin;
    s->setup();
  } catch (std::exception &e) {
    copy_err(e.what(), errbuf, errlen);
    delete s;
    return nullptr;
  }
  return s;
}

void gbh_destroy(void *h) { delete static_cast<GbSim *>(h); }

int gbh_step(void *h, const double *xi, long nxi, char *errbuf, int errlen) {
  GbSim *s = static_cast<GbSim *>(h);
  try {
    s->step(xi, nxi);
  } catch (std::exception &e) {
    copy_err(e.what(), errbuf, errlen);
    return 1;
  }
  return 0;
}

/* "x","v","f" (3 per atom, the engine's arrays), "array" (8 per atom),
 * "vector" (2) */
int gbh_get(void *h, const char *what, double *out) {
  GbSim *s = static_cast<GbSim *>(h);
  const int n = s->atom.nlocal;
  const std::string w(what);
  auto rows = [&](double **a, int k) {
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < k; ++c) out[(size_t)k * i + c] = a[i][c];
  };
  try {
    if (w == "x") rows(s->atom.x, 3);
    else if (w == "v") rows(s->atom.v, 3);
    else if (w == "f") rows(s->atom.f, 3);
    else if (w == "array") rows(s->probe()->arr(), 8);
    else if (w == "vector") {
      out[0] = s->fix->compute_vector(0);
      out[1] = s->fix->compute_vector(1);
    } else
      return 1;
  } catch (std::exception &) {
    return 2;
  }
  return 0;
}

/* fix_modify ID key value (e.g. "peratom" "3", "list_skin" "0.3") */
int gbh_modify(void *h, const char *key, const char *value, char *errbuf, int errlen) {
  GbSim *s = static_cast<GbSim *>(h);
  std::string k(key), v(value);
  char *a[2] = {&k[0], &v[0]};
  try {
    return s->fix->modify_param(2, a) == 2 ? 0 : 1;
  } catch (std::exception &e) {
    copy_err(e.what(), errbuf, errlen);
    return 2;
  }
}

int gbh_post_run(void *h) {
  static_cast<GbSim *>(h)->fix->post_run();
  return 0;
}

}  // extern "C"
