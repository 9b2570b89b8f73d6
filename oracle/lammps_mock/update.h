#ifndef EPH_MOCK_UPDATE_H
#define EPH_MOCK_UPDATE_H
#include "lammps.h"
namespace LAMMPS_NS {
class Update {
 public:
  double dt = 0.001;
  bigint ntimestep = 0;
};
}  // namespace LAMMPS_NS
#endif
