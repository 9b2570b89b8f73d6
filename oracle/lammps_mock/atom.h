#ifndef EPH_MOCK_ATOM_H
#define EPH_MOCK_ATOM_H
#include "lammps.h"
namespace LAMMPS_NS {
class Fix;
/* Per-atom storage of the engine: locals first, ghosts after them. */
class Atom {
 public:
  double **x = nullptr, **v = nullptr, **f = nullptr;
  double *mass = nullptr;  // indexed by type 1..ntypes
  int *type = nullptr, *mask = nullptr;
  int nlocal = 0, nghost = 0, nmax = 0, ntypes = 0;
  bigint natoms = 0;
  Fix *grow_client = nullptr;  // the fix registered through add_callback(0)
  void add_callback(int) {}
  void delete_callback(const char *, int) {}
};
}  // namespace LAMMPS_NS
#endif
