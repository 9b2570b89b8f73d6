#ifndef EPH_MOCK_DOMAIN_H
#define EPH_MOCK_DOMAIN_H
#include "lammps.h"
namespace LAMMPS_NS {
class Domain {
 public:
  double boxlo[3] = {0, 0, 0}, boxhi[3] = {1, 1, 1};
  double prd[3] = {1, 1, 1};  // boxhi - boxlo
  int dimension = 3, nonperiodic = 0, triclinic = 0;
  void set_box(const double *lo, const double *hi) {
    for (int k = 0; k < 3; ++k) {
      boxlo[k] = lo[k];
      boxhi[k] = hi[k];
      prd[k] = hi[k] - lo[k];
    }
  }
};
}  // namespace LAMMPS_NS
#endif
