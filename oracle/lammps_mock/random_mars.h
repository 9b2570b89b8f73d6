#ifndef EPH_MOCK_RANDOM_MARS_H
#define EPH_MOCK_RANDOM_MARS_H
#include "lammps.h"
namespace LAMMPS_NS {
/* Gaussian source of the engine.  In the oracle the deviates are injected:
 * the harness points `stream` at the values the reference fix must draw, in
 * the order it draws them (three per in-group atom, atoms in index order),
 * so that the CUDA path can be fed the identical deviates. */
class RanMars {
 public:
  RanMars(LAMMPS *, int s) : seed(s) {}
  double gaussian() {
    if (!stream || pos >= count) throw std::runtime_error("RanMars stand-in: injected deviates exhausted");
    return stream[pos++];
  }
  double uniform() { throw std::runtime_error("RanMars stand-in: uniform() not injected"); }
  int seed;
  const double *stream = nullptr;
  long pos = 0, count = 0;
};
}  // namespace LAMMPS_NS
#endif
