#ifndef EPH_MOCK_NEIGHBOR_H
#define EPH_MOCK_NEIGHBOR_H
#include "lammps.h"
#include "neigh_request.h"
namespace LAMMPS_NS {
class Fix;
class Neighbor {
 public:
  NeighRequest request;
  Fix *requestor = nullptr;
  int nrequest = 0;
  double skin = 1.0;  // neighbor skin distance
  bigint ago = 0;     // steps since the last re-neighbouring
  NeighRequest *add_request(Fix *f, int style) {
    requestor = f;
    request.style = style;
    ++nrequest;
    return &request;
  }
};
}  // namespace LAMMPS_NS
#endif
