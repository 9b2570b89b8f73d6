/*
 * Minimal stand-in for the parts of the LAMMPS engine that the reference
 * `fix eph` (fix_eph.cpp / fix_eph.h of USER-EPH) touches.  TEST
 * INFRASTRUCTURE ONLY: it lets the reference fix compile unchanged so that its
 * own code can serve as the parity oracle.  It is not shipped and nothing in
 * the product links it.
 *
 * Engine semantics reproduced (LAMMPS, version 31 Mar 2017 as in the
 * reference's Tests/MD_Run/Reference/log.lammps):
 *   - orthogonal periodic box, ghost atoms = periodic images within the
 *     neighbour cutoff, ghost coordinate = owner coordinate + (+-1)*prd
 *     (one addition, as LAMMPS's pbc forward communication does);
 *   - full neighbour list (REQ_FULL | REQ_GHOST) with cutoff rc + skin;
 *   - rebuild when any atom moved more than skin/2 since the last build,
 *     wrapping positions into [lo, hi) first;
 *   - Verlet step order: initial_integrate, neighbour decision, force
 *     clear (+ optional external force), post_force, final_integrate,
 *     end_of_step.
 * The neighbour list of every atom is ordered by the owner index of each
 * neighbour (ascending); that is the canonical order the CUDA path uses.
 */
#ifndef EPH_MOCK_LAMMPS_H
#define EPH_MOCK_LAMMPS_H

#include <mpi.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <stdexcept>
#include <string>

#define FLERR __FILE__, __LINE__

namespace LAMMPS_NS {

typedef int64_t bigint;
typedef int tagint;

static constexpr int NEIGHMASK = 0x1FFFFFFF;

class Atom;
class Domain;
class Neighbor;
class Memory;
class Force;
class Update;
class Comm;
class Error;

class LAMMPS {
 public:
  Atom *atom = nullptr;
  Domain *domain = nullptr;
  Neighbor *neighbor = nullptr;
  Memory *memory = nullptr;
  Force *force = nullptr;
  Update *update = nullptr;
  Comm *comm = nullptr;
  Error *error = nullptr;
  MPI_Comm world = 0;
};

// Base class giving every engine object the same named pointers LAMMPS gives.
class Pointers {
 public:
  explicit Pointers(LAMMPS *ptr)
      : lmp(ptr), atom(ptr->atom), domain(ptr->domain), neighbor(ptr->neighbor),
        memory(ptr->memory), force(ptr->force), update(ptr->update), comm(ptr->comm),
        error(ptr->error), world(ptr->world) {}
  virtual ~Pointers() = default;

 protected:
  LAMMPS *lmp;
  Atom *&atom;
  Domain *&domain;
  Neighbor *&neighbor;
  Memory *&memory;
  Force *&force;
  Update *&update;
  Comm *&comm;
  Error *&error;
  MPI_Comm &world;
};

class Error {
 public:
  [[noreturn]] void all(const char *file, int line, const std::string &msg) {
    throw std::runtime_error(std::string(file) + ":" + std::to_string(line) + ": " + msg);
  }
  [[noreturn]] void one(const char *file, int line, const std::string &msg) { all(file, line, msg); }
};

}  // namespace LAMMPS_NS

#endif
