#ifndef EPH_MOCK_FIX_H
#define EPH_MOCK_FIX_H
#include "lammps.h"
#include "comm.h"
namespace LAMMPS_NS {
class NeighList;

namespace FixConst {
static constexpr int INITIAL_INTEGRATE = 1 << 0;
static constexpr int POST_FORCE = 1 << 7;
static constexpr int FINAL_INTEGRATE = 1 << 8;
static constexpr int END_OF_STEP = 1 << 9;
}  // namespace FixConst

/* The subset of LAMMPS's Fix base class that the reference fix uses. */
class Fix : protected Pointers {
 public:
  Fix(LAMMPS *lmp, int narg, char **arg) : Pointers(lmp) {
    if (narg < 3) error->all(FLERR, "Illegal fix command");
    id = strdup(arg[0]);
    groupbit = 1;  // group "all"
  }
  ~Fix() override { std::free(id); }

  char *id = nullptr;
  int groupbit = 1;
  int vector_flag = 0, size_vector = 0, global_freq = 0, extvector = 0;
  int nevery = 1, peratom_flag = 0, size_peratom_cols = 0, peratom_freq = 0;
  int comm_forward = 0, time_integrate = 0, maxexchange = 0;
  double **array_atom = nullptr;

  virtual void init() {}
  virtual void setup(int) {}
  virtual int modify_param(int, char **) { return 0; }
  virtual void init_list(int, NeighList *) {}
  virtual int setmask() = 0;
  virtual void post_force(int) {}
  virtual void end_of_step() {}
  virtual void reset_dt() {}
  virtual void grow_arrays(int) {}
  virtual double compute_vector(int) { return 0.0; }
  virtual double memory_usage() { return 0.0; }
  virtual void post_run() {}
  virtual void initial_integrate(int) {}
  virtual void final_integrate() {}
  virtual int pack_forward_comm(int, int *, double *, int, int *) { return 0; }
  virtual int pack_exchange(int, double *) { return 0; }
  virtual int unpack_exchange(int, double *) { return 0; }
  virtual void copy_arrays(int, int, int) {}
  virtual void unpack_forward_comm(int, int, double *) {}
};

inline void Comm::forward_comm(Fix *fix) {
  if (nghost == 0) return;
  fix->pack_forward_comm(nghost, ghost_owner, buf, 0, nullptr);
  fix->unpack_forward_comm(nghost, nlocal, buf);
}
}  // namespace LAMMPS_NS
#endif
