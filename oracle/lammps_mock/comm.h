#ifndef EPH_MOCK_COMM_H
#define EPH_MOCK_COMM_H
#include "lammps.h"
#include "atom.h"
namespace LAMMPS_NS {
class Fix;
/* Forward communication on one rank: ghost i (index nlocal + i) receives the
 * fix's packed values of its owner ghost_owner[i]. */
class Comm {
 public:
  int ghost_velocity = 0;
  int me = 0, nprocs = 1;
  int *ghost_owner = nullptr;
  int nghost = 0, nlocal = 0;
  double *buf = nullptr;
  void forward_comm(Fix *fix);
};
}  // namespace LAMMPS_NS
#endif
