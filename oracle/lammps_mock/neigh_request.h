#ifndef EPH_MOCK_NEIGH_REQUEST_H
#define EPH_MOCK_NEIGH_REQUEST_H
#include "lammps.h"
namespace LAMMPS_NS {
namespace NeighConst {
static constexpr int REQ_FULL = 1 << 0;
static constexpr int REQ_GHOST = 1 << 1;
}  // namespace NeighConst
class NeighRequest {
 public:
  int style = 0;
  double cutoff = 0.0;
  void set_cutoff(double c) { cutoff = c; }
};
}  // namespace LAMMPS_NS
#endif
