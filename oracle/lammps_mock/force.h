#ifndef EPH_MOCK_FORCE_H
#define EPH_MOCK_FORCE_H
#include "lammps.h"
namespace LAMMPS_NS {
/* Unit constants; metal units: boltz in eV/K, ftm2v converts eV/A/amu to A/ps^2. */
class Force {
 public:
  double boltz = 8.617343e-5;
  double ftm2v = 1.0 / 1.0364269e-4;
};
}  // namespace LAMMPS_NS
#endif
