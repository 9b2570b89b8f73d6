/*
 * The engine stand-in's driver (TEST INFRASTRUCTURE ONLY): atoms, ghosts,
 * the full neighbour list, the rebuild schedule and the Verlet step order of
 * LAMMPS around one fix.  Used by ref_harness.cpp (the reference fix) and
 * gb_harness.cpp (the GB300 fix eph/gb), so both run in the same engine.
 */
#ifndef EPH_MOCK_ENGINE_HPP
#define EPH_MOCK_ENGINE_HPP

#include <algorithm>
#include <cmath>
#include <stdexcept>
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

namespace LAMMPS_NS {

struct Engine {
  LAMMPS lmp;
  Atom atom;
  Domain domain;
  Neighbor neighbor;
  Memory memory;
  Force force;
  Update update;
  Comm comm;
  Error error;
  NeighList list;
  Fix *fix = nullptr;
  RanMars *rng = nullptr;  // the fix's Gaussian source (injected deviates)

  double skin = 1.0, cutneigh = 0.0;
  std::vector<int> ghost_owner;
  std::vector<int> ghost_shift;  // 3 per ghost, values -1, 0, +1
  std::vector<double> xhold;
  std::vector<double> fext;
  std::vector<int> numneigh;
  std::vector<int *> firstneigh;
  std::vector<std::vector<int>> neigh;
  std::vector<double> commbuf;
  long nbuild = 0;

  Engine() {
    lmp.atom = &atom;
    lmp.domain = &domain;
    lmp.neighbor = &neighbor;
    lmp.memory = &memory;
    lmp.force = &force;
    lmp.update = &update;
    lmp.comm = &comm;
    lmp.error = &error;
  }
  ~Engine() {
    delete fix;
    memory.destroy(atom.x);
    memory.destroy(atom.v);
    memory.destroy(atom.f);
    memory.destroy(atom.type);
    memory.destroy(atom.mask);
    memory.destroy(atom.mass);
  }

  void grow_atoms(int n) {
    if (n <= atom.nmax) return;
    atom.nmax = n;
    memory.grow(atom.x, n, 3, "x");
    memory.grow(atom.v, n, 3, "v");
    memory.grow(atom.f, n, 3, "f");
    memory.grow(atom.type, n, "type");
    memory.grow(atom.mask, n, "mask");
    commbuf.resize((size_t)3 * n);
    comm.buf = commbuf.data();
    if (fix) fix->grow_arrays(n);
  }

  // Domain::pbc for an orthogonal periodic box.
  void pbc() {
    for (int i = 0; i < atom.nlocal; ++i)
      for (int k = 0; k < 3; ++k) {
        double &c = atom.x[i][k];
        if (c < domain.boxlo[k]) c += domain.prd[k];
        if (c >= domain.boxhi[k]) {
          c -= domain.prd[k];
          c = std::max(c, domain.boxlo[k]);
        }
      }
  }

  // Ghosts: every periodic image of a local atom that falls inside the box
  // grown by the neighbour cutoff on each side.
  void borders() {
    const int nlocal = atom.nlocal;
    ghost_owner.clear();
    ghost_shift.clear();
    std::vector<double> gx;
    for (int i = 0; i < nlocal; ++i)
      for (int sz = -1; sz <= 1; ++sz)
        for (int sy = -1; sy <= 1; ++sy)
          for (int sx = -1; sx <= 1; ++sx) {
            if (!sx && !sy && !sz) continue;
            const int s[3] = {sx, sy, sz};
            double c[3];
            bool inside = true;
            for (int k = 0; k < 3; ++k) {
              c[k] = atom.x[i][k];
              if (s[k] > 0) c[k] = atom.x[i][k] + domain.prd[k];
              if (s[k] < 0) c[k] = atom.x[i][k] + (-domain.prd[k]);
              if (!(c[k] >= domain.boxlo[k] - cutneigh && c[k] < domain.boxhi[k] + cutneigh)) inside = false;
            }
            if (!inside) continue;
            ghost_owner.push_back(i);
            ghost_shift.insert(ghost_shift.end(), s, s + 3);
            gx.insert(gx.end(), c, c + 3);
          }
    const int ng = (int)ghost_owner.size();
    grow_atoms(nlocal + ng + 1);
    atom.nghost = ng;
    for (int g = 0; g < ng; ++g) {
      const int j = nlocal + g, o = ghost_owner[g];
      for (int k = 0; k < 3; ++k) {
        atom.x[j][k] = gx[3 * g + k];
        atom.v[j][k] = atom.v[o][k];
      }
      atom.type[j] = atom.type[o];
      atom.mask[j] = atom.mask[o];
    }
    comm.ghost_owner = ghost_owner.data();
    comm.nghost = ng;
    comm.nlocal = nlocal;
  }

  // Owner x, v to ghosts (forward communication with ghost_velocity = 1).
  void forward_xv() {
    const int nlocal = atom.nlocal;
    for (int g = 0; g < atom.nghost; ++g) {
      const int j = nlocal + g, o = ghost_owner[g];
      for (int k = 0; k < 3; ++k) {
        const int s = ghost_shift[3 * g + k];
        double c = atom.x[o][k];
        if (s > 0) c = atom.x[o][k] + domain.prd[k];
        if (s < 0) c = atom.x[o][k] + (-domain.prd[k]);
        atom.x[j][k] = c;
        atom.v[j][k] = atom.v[o][k];
      }
    }
  }

  int owner(int j) const { return j < atom.nlocal ? j : ghost_owner[j - atom.nlocal]; }

  // Full list of every local atom, neighbours ordered by owner index.
  void build_list() {
    const int nlocal = atom.nlocal, ntot = nlocal + atom.nghost;
    const double cutsq = cutneigh * cutneigh;
    // bin all atoms (local + ghost) on a grid of cells of edge >= cutneigh
    double lo[3], w[3];
    int nb[3];
    for (int k = 0; k < 3; ++k) {
      lo[k] = domain.boxlo[k] - cutneigh;
      const double ext = domain.prd[k] + 2.0 * cutneigh;
      nb[k] = std::max(1, (int)(ext / cutneigh));
      w[k] = ext / nb[k];
    }
    auto bin_of = [&](const double *c, int *b) {
      for (int k = 0; k < 3; ++k) {
        int v = (int)std::floor((c[k] - lo[k]) / w[k]);
        b[k] = std::min(std::max(v, 0), nb[k] - 1);
      }
    };
    std::vector<std::vector<int>> bins((size_t)nb[0] * nb[1] * nb[2]);
    for (int j = 0; j < ntot; ++j) {
      int b[3];
      bin_of(atom.x[j], b);
      bins[(size_t)b[0] + (size_t)nb[0] * (b[1] + (size_t)nb[1] * b[2])].push_back(j);
    }
    neigh.assign(nlocal, {});
    numneigh.assign(nlocal, 0);
    firstneigh.assign(nlocal, nullptr);
    for (int i = 0; i < nlocal; ++i) {
      int b[3];
      bin_of(atom.x[i], b);
      std::vector<std::pair<int, int>> cand;
      for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            const int c0 = b[0] + dx, c1 = b[1] + dy, c2 = b[2] + dz;
            if (c0 < 0 || c1 < 0 || c2 < 0 || c0 >= nb[0] || c1 >= nb[1] || c2 >= nb[2]) continue;
            for (int j : bins[(size_t)c0 + (size_t)nb[0] * (c1 + (size_t)nb[1] * c2)]) {
              if (j == i) continue;
              const double ex = atom.x[j][0] - atom.x[i][0];
              const double ey = atom.x[j][1] - atom.x[i][1];
              const double ez = atom.x[j][2] - atom.x[i][2];
              const double rsq = ex * ex + ey * ey + ez * ez;
              if (rsq < cutsq) cand.emplace_back(owner(j), j);
            }
          }
      std::sort(cand.begin(), cand.end());
      for (size_t c = 1; c < cand.size(); ++c)
        if (cand[c].first == cand[c - 1].first)
          throw std::runtime_error("two images of one atom in a list: box narrower than 2*(rc+skin)");
      for (auto &p : cand) neigh[i].push_back(p.second);
      numneigh[i] = (int)neigh[i].size();
      firstneigh[i] = neigh[i].data();
    }
    list.inum = nlocal;
    list.numneigh = numneigh.data();
    list.firstneigh = firstneigh.data();
    xhold.assign((size_t)3 * nlocal, 0.0);
    for (int i = 0; i < nlocal; ++i)
      for (int k = 0; k < 3; ++k) xhold[3 * (size_t)i + k] = atom.x[i][k];
    ++nbuild;
  }

  // The atoms, box and unit constants of a run.
  void load(int nlocal, const double *x, const double *v, const int *type, const int *mask, int ntypes,
            const double *mass, const double *lo, const double *hi, double dt, double boltz, double ftm2v,
            double skin_in) {
    domain.set_box(lo, hi);
    update.dt = dt;
    force.boltz = boltz;
    force.ftm2v = ftm2v;
    skin = skin_in;
    neighbor.skin = skin_in;
    atom.ntypes = ntypes;
    atom.natoms = nlocal;
    atom.nlocal = nlocal;
    memory.grow(atom.mass, ntypes + 1, "mass");
    for (int t = 0; t <= ntypes; ++t) atom.mass[t] = mass[t];
    grow_atoms(std::max(nlocal, 1));
    for (int i = 0; i < nlocal; ++i) {
      for (int k = 0; k < 3; ++k) {
        atom.x[i][k] = x[3 * (size_t)i + k];
        atom.v[i][k] = v[3 * (size_t)i + k];
        atom.f[i][k] = 0.0;
      }
      atom.type[i] = type[i];
      atom.mask[i] = mask ? mask[i] : 1;
    }
  }

  // Verlet::setup: wrap, ghosts, list, forces, then Fix::setup
  void setup() {
    reneighbor();
    fix->grow_arrays(atom.nmax);
    clear_forces();
    fix->setup(0);
  }

  // One Verlet step with `xi` the deviates the fix's RanMars hands out.
  void step(const double *xi, long nxi) {
    update.ntimestep += 1;
    neighbor.ago += 1;
    fix->initial_integrate(0);
    if (decide())
      reneighbor();
    else
      forward_xv();
    clear_forces();
    if (rng) {
      rng->stream = xi;
      rng->count = xi ? nxi : 0;
      rng->pos = 0;
    }
    fix->post_force(0);
    if (rng && xi && rng->pos != nxi) throw std::runtime_error("fix drew a different number of deviates than injected");
    fix->final_integrate();
    fix->end_of_step();
  }

  bool decide() const {
    const double triggersq = 0.25 * skin * skin;
    for (int i = 0; i < atom.nlocal; ++i) {
      const double dx = atom.x[i][0] - xhold[3 * (size_t)i + 0];
      const double dy = atom.x[i][1] - xhold[3 * (size_t)i + 1];
      const double dz = atom.x[i][2] - xhold[3 * (size_t)i + 2];
      if (dx * dx + dy * dy + dz * dz > triggersq) return true;
    }
    return false;
  }

  void reneighbor() {
    pbc();
    borders();
    build_list();
    neighbor.ago = 0;
  }

  void clear_forces() {
    const int ntot = atom.nlocal + atom.nghost;
    for (int i = 0; i < ntot; ++i)
      for (int k = 0; k < 3; ++k) atom.f[i][k] = 0.0;
    if (!fext.empty())
      for (int i = 0; i < atom.nlocal; ++i)
        for (int k = 0; k < 3; ++k) atom.f[i][k] = fext[3 * (size_t)i + k];
  }
};


}  // namespace LAMMPS_NS

#endif
