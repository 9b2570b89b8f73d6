#ifndef EPH_MOCK_NEIGH_LIST_H
#define EPH_MOCK_NEIGH_LIST_H
#include "lammps.h"
namespace LAMMPS_NS {
class NeighList {
 public:
  int inum = 0;
  int *numneigh = nullptr;
  int **firstneigh = nullptr;
};
}  // namespace LAMMPS_NS
#endif
