/*
 * LAMMPS fix `eph/gb`: the USER-EPH fix `eph` (fix_eph.h, FixStyle(eph,FixEPH))
 * with its per-step work on one GB300 through the C ABI of eph_gb.h.
 *
 * Same command words as `fix eph` (README.md:186-214) -- or, as
 * `eph/coloured/exp/gb`, those of `fix eph/coloured/exp` (arg[5] = tau0):
 *   fix ID group eph/gb seed flags model rho_e C_e kappa_e T_e NX NY NZ
 *       T_infile freq T_out beta_file A B ...
 * Same hooks (INITIAL_INTEGRATE, POST_FORCE, FINAL_INTEGRATE, END_OF_STEP),
 * global vector (2: energy transferred, mean T_e), per-atom array (8 columns:
 * rho, beta(rho), f_EPH, f_RNG) and restart file on post_run.  Registering it
 * as `eph` instead (FixStyle(eph,FixEPHGB)) makes it a drop-in for the
 * reference fix.
 *
 * fix_modify options: `mode exact|fast` (EPH_MODE_*), `xi host|device`
 * (deviates from the engine's RanMars stream on the host, or the device
 * Philox generator), `device N`, `list_skin S` (skin of the kept candidate
 * lists in distance units, 0: search the bins every step, `auto`: timed
 * trial windows after the next post_force, eph_autotune_list_skin), `pairs df64|fp64`
 * (arithmetic of the FAST-mode pair sums, eph_set_pair_arithmetic; default
 * df64), `peratom N` (copy
 * the per-atom array back only on steps that are multiples of N and declare
 * peratom_freq = N, so that the engine lets computes, dumps and variables
 * read it only then; default 1, every step, as the reference).
 * One MPI rank per GPU holding every atom of the box (the device builds its
 * own periodic minimum-image neighbour pairs, so no ghost communication).
 */
#ifdef FIX_CLASS
// clang-format off
FixStyle(eph/gb,FixEPHGB)
FixStyle(eph/coloured/exp/gb,FixEPHGB)
// clang-format on
#else

#ifndef LMP_FIX_EPH_GB_H
#define LMP_FIX_EPH_GB_H

#include <vector>

#include "eph_gb.h"
#include "fix.h"

namespace LAMMPS_NS {

class FixEPHGB : public Fix {
 public:
  FixEPHGB(class LAMMPS *, int, char **);
  ~FixEPHGB() override;

  int setmask() override;
  void init() override;
  void setup(int) override;
  void initial_integrate(int) override;
  void post_force(int) override;
  void final_integrate() override;
  void end_of_step() override;
  void reset_dt() override;
  void grow_arrays(int) override;
  void copy_arrays(int, int, int) override;
  double compute_vector(int) override;
  void post_run() override;
  int modify_param(int, char **) override;
  double memory_usage() override;

 protected:
  eph_ctx *ctx = nullptr;
  std::vector<char *> words;  // the fix command words, kept for eph_create
  int eph_flag = 0;
  int mode = EPH_MODE_FAST;
  int xi_on_host = 0;
  int device = 0;
  int nlocal_dev = -1;            // atom count the device holds
  double list_skin = -1.0;        // fix_modify list_skin (negative: the library's default)
  bool tune_skin = false;         // fix_modify list_skin auto: autotune after the next post_force
  int pair_arith = -1;            // fix_modify pairs (negative: the library's default, df64)
  bool reordered = false;         // the engine moved atoms between slots since the last upload
  bigint last_upload_step = -1;   // step of the last full atom upload
  class RanMars *random = nullptr;
  std::vector<double> xi;  // deviates drawn on the host (xi host)
  double **array = nullptr;

  void *pinned[4] = {nullptr, nullptr, nullptr, nullptr};  // x, v, f, the per-atom array
  size_t pinned_bytes[4] = {0, 0, 0, 0};

  void create_context();
  void pin_engine_arrays();
  void check(int status, const char *where);
  void upload_atoms();  // x, v, type, mask when the engine re-neighboured
};

}  // namespace LAMMPS_NS

#endif
#endif
