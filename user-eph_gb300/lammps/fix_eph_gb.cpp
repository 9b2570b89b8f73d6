/*
 * LAMMPS fix `eph/gb` (see fix_eph_gb.h): the hooks of the reference fix
 * (fix_eph.cpp:293-302) calling the GB300 C ABI.  Atom data stays owned by
 * the engine on the host; each hook copies in what it reads and copies back
 * what it writes:
 *   initial_integrate  x, v in      -> device integrate -> x, v out
 *   post_force         f in         -> bins, density, force_prl -> f out
 *   final_integrate    f in         -> device integrate -> v out
 *   end_of_step        (device)     -> deposition, FDM, T output; per-atom array
 *                                      out on steps that are multiples of
 *                                      peratom_freq (`fix_modify ID peratom N`,
 *                                      default 1: every step, as the reference)
 * initial_integrate needs no f: the engine changes f only in its force
 * computation and in post_force, and final_integrate sent the device the f
 * left after every fix's post_force (setup() uploads it for the first step).
 * post_force needs no v: initial_integrate copied it back and the engine
 * leaves it alone until post_force.  x changes only when the engine
 * re-neighbours: it wraps atoms into the box (then x goes up again) and may
 * re-sort or migrate them, which it reports through copy_arrays (then the
 * whole atom set goes up again: x, v, type, mask, f).
 */
#include "fix_eph_gb.h"

#include <cstdlib>
#include <cstring>
#include <string>

#include "atom.h"
#include "comm.h"
#include "domain.h"
#include "error.h"
#include "force.h"
#include "memory.h"
#include "neighbor.h"
#include "random_mars.h"
#include "update.h"

using namespace LAMMPS_NS;
using namespace FixConst;

static char *dup_word(const char *s) {
  const size_t n = std::strlen(s) + 1;
  char *p = static_cast<char *>(malloc(n));
  std::memcpy(p, s, n);
  return p;
}

FixEPHGB::FixEPHGB(LAMMPS *lmp, int narg, char **arg) : Fix(lmp, narg, arg) {
  if (narg < 18) error->all(FLERR, "Illegal fix eph/gb command: too few arguments");
  if (atom->natoms < 1) error->all(FLERR, "fix_eph: error no atoms in simulation");
  if (comm->nprocs != 1) error->all(FLERR, "fix eph/gb runs on one MPI rank per GPU holding the whole box");
  vector_flag = 1;
  size_vector = 2;
  global_freq = 1;
  extvector = 1;
  nevery = 1;
  peratom_flag = 1;
  size_peratom_cols = 8;
  peratom_freq = 1;
  eph_flag = (int)strtol(arg[4], nullptr, 0);
  time_integrate = (eph_flag & 0x08) ? 0 : 1;
  for (int i = 0; i < narg; ++i) words.push_back(dup_word(arg[i]));
  random = new RanMars(lmp, atoi(arg[3]) + comm->me);
  grow_arrays(atom->nmax);
  atom->add_callback(0);
  create_context();
}

FixEPHGB::~FixEPHGB() {
  if (ctx) eph_destroy(ctx);
  for (void *p : pinned)
    if (p) eph_unpin(p);
  for (char *w : words) free(w);
  delete random;
  atom->delete_callback(id, 0);
  memory->destroy(array);
}

void FixEPHGB::check(int status, const char *where) {
  if (status != EPH_OK)
    error->all(FLERR, std::string("fix eph/gb: ") + where + ": " + eph_status_string(status) + ": " +
                          eph_last_error(ctx));
}

void FixEPHGB::create_context() {
  if (ctx) eph_destroy(ctx);
  ctx = nullptr;
  eph_md md;
  md.ntypes = atom->ntypes;
  md.mass = atom->mass;
  for (int k = 0; k < 3; ++k) {
    md.boxlo[k] = domain->boxlo[k];
    md.boxhi[k] = domain->boxhi[k];
  }
  md.dt = update->dt;
  md.boltz = force->boltz;
  md.ftm2v = force->ftm2v;
  md.skin = neighbor->skin;
  md.groupbit = groupbit;
  md.device = device;
  md.mode = mode;
  check(eph_create((int)words.size(), words.data(), &md, &ctx), "create");
  // a list skin or pair arithmetic set by fix_modify outlives contexts made
  // by later fix_modify words
  if (list_skin >= 0.0) check(eph_set_list_skin(ctx, list_skin), "list skin");
  if (pair_arith >= 0) check(eph_set_pair_arithmetic(ctx, pair_arith), "pair arithmetic");
  nlocal_dev = -1;
}

int FixEPHGB::setmask() {
  return INITIAL_INTEGRATE | POST_FORCE | FINAL_INTEGRATE | END_OF_STEP;
}

void FixEPHGB::init() {
  if (domain->dimension == 2) error->all(FLERR, "Cannot use fix eph with 2d simulation");
  if (domain->nonperiodic != 0) error->all(FLERR, "Cannot use nonperiodic boundares with fix eph");
  if (domain->triclinic) error->all(FLERR, "Cannot use fix eph with triclinic box");
  reset_dt();
}

int FixEPHGB::modify_param(int narg, char **arg) {
  if (narg < 2) error->all(FLERR, "Illegal fix_modify command");
  if (strcmp(arg[0], "mode") == 0) {
    mode = strcmp(arg[1], "exact") == 0 ? EPH_MODE_EXACT : EPH_MODE_FAST;
  } else if (strcmp(arg[0], "xi") == 0) {
    xi_on_host = strcmp(arg[1], "host") == 0;
    return 2;
  } else if (strcmp(arg[0], "device") == 0) {
    device = atoi(arg[1]);
  } else if (strcmp(arg[0], "list_skin") == 0) {
    // a skin in distance units, or `auto`: eph_autotune_list_skin picks one
    // after the first post_force (trial windows from the device state,
    // restored afterwards)
    if (strcmp(arg[1], "auto") == 0) {
      tune_skin = true;
      return 2;
    }
    list_skin = atof(arg[1]);
    tune_skin = false;
    check(eph_set_list_skin(ctx, list_skin), "list skin");
    return 2;
  } else if (strcmp(arg[0], "pairs") == 0) {
    // arithmetic of the FAST pair sums: df64 (double-float on the FP32 pipe,
    // the default) or fp64
    if (strcmp(arg[1], "df64") == 0)
      pair_arith = EPH_PAIRS_DF64;
    else if (strcmp(arg[1], "fp64") == 0)
      pair_arith = EPH_PAIRS_FP64;
    else
      error->all(FLERR, "fix_modify eph/gb pairs: df64 or fp64");
    check(eph_set_pair_arithmetic(ctx, pair_arith), "pair arithmetic");
    return 2;
  } else if (strcmp(arg[0], "peratom") == 0) {
    // computes, dumps and variables read the per-atom array only on steps
    // that are multiples of peratom_freq (the engine checks), so it is
    // copied back only then
    const int every = atoi(arg[1]);
    if (every < 1) error->all(FLERR, "fix_modify eph/gb peratom: N must be >= 1");
    peratom_freq = every;
    return 2;
  } else {
    return 0;
  }
  create_context();
  return 2;
}

void FixEPHGB::upload_atoms() {
  const int n = atom->nlocal;
  reordered = false;
  check(eph_set_atoms(ctx, n, &atom->x[0][0], &atom->v[0][0], atom->type, atom->mask), "set atoms");
  check(eph_put(ctx, EPH_FIELD_F, &atom->f[0][0], EPH_HOST), "put f");
  nlocal_dev = n;
  last_upload_step = update->ntimestep;
}

void FixEPHGB::setup(int) { upload_atoms(); }

void FixEPHGB::initial_integrate(int) {
  if (eph_flag & 0x08) return;
  if (nlocal_dev != atom->nlocal || reordered) upload_atoms();
  pin_engine_arrays();
  // x, v in (the device keeps the f final_integrate sent), the half kick
  // and drift, x, v out: the copies of chunks of atoms overlap both ways
  check(eph_initial_integrate_host(ctx, &atom->x[0][0], &atom->v[0][0]), "initial_integrate");
}

void FixEPHGB::post_force(int) {
  // the engine re-neighboured this step: atoms may be re-sorted or wrapped,
  // so all of them go up again (x, v, type, mask and f); otherwise the device
  // holds this step's x and v since initial_integrate, and x goes up again
  // only on re-neighbouring steps (the engine wrapped it)
  const bool full = nlocal_dev != atom->nlocal || reordered;
  if (full) upload_atoms();
  pin_engine_arrays();
  int source = EPH_XI_DEVICE_RNG;
  if (xi_on_host && (eph_flag & 0x02)) {
    // the engine's own Gaussian stream, three per in-group atom in atom
    // order, as the reference draws it (fix_eph.cpp:854-860)
    const int n = atom->nlocal;
    xi.assign(3 * (size_t)n, 0.0);
    for (int i = 0; i < n; ++i)
      if (atom->mask[i] & groupbit)
        for (int k = 0; k < 3; ++k) xi[3 * (size_t)i + k] = random->gaussian();
    check(eph_put(ctx, EPH_FIELD_XI, xi.data(), EPH_HOST), "put xi");
    source = EPH_XI_GIVEN;
  }
  // the engine's force in, f_EPH + f_RNG added, f out; the per-atom array
  // (final here, fix_eph.cpp:406-428) leaves on its own stream on the steps
  // the engine reads it and is in place when end_of_step returns
  const double *x = (!full && neighbor->ago == 0) ? &atom->x[0][0] : nullptr;
  double *arr = (update->ntimestep % peratom_freq == 0) ? &array[0][0] : nullptr;
  check(eph_post_force_host(ctx, x, &atom->f[0][0], &atom->f[0][0], arr, source), "post_force");
  if (tune_skin) {
    static const double candidates[] = {0.0, 0.15, 0.2, 0.3, 0.4, 0.6};
    check(eph_autotune_list_skin(ctx, candidates, (int)(sizeof(candidates) / sizeof(candidates[0])), 20,
                                 &list_skin),
          "list skin autotune");
    tune_skin = false;
  }
}

void FixEPHGB::final_integrate() {
  if (eph_flag & 0x08) return;
  pin_engine_arrays();
  check(eph_final_integrate_host(ctx, &atom->f[0][0], &atom->v[0][0]), "final_integrate");
}

void FixEPHGB::end_of_step() {
  check(eph_set_timestep(ctx, (long)update->ntimestep), "set timestep");
  if (eph_flag & 0x08) check(eph_put(ctx, EPH_FIELD_V, &atom->v[0][0], EPH_HOST), "put v");
  check(eph_end_of_step(ctx), "end_of_step");
}

// The engine's x, v, f and the per-atom array page-locked for the hooks'
// copies; pinned again when the engine reallocates them (a range the engine
// has already freed is unpinned as well as the runtime allows).  Pinning
// that fails leaves the copies on pageable memory: slower, not wrong.
void FixEPHGB::pin_engine_arrays() {
  const size_t nmax = atom->nmax > 0 ? (size_t)atom->nmax : 0;
  struct Want {
    void *p;
    size_t bytes;
  } want[4] = {{atom->x ? &atom->x[0][0] : nullptr, 3 * sizeof(double) * nmax},
               {atom->v ? &atom->v[0][0] : nullptr, 3 * sizeof(double) * nmax},
               {atom->f ? &atom->f[0][0] : nullptr, 3 * sizeof(double) * nmax},
               {array ? &array[0][0] : nullptr, 8 * sizeof(double) * nmax}};
  for (int k = 0; k < 4; ++k) {
    if (want[k].p == pinned[k] && want[k].bytes == pinned_bytes[k]) continue;
    if (pinned[k]) eph_unpin(pinned[k]);
    pinned[k] = nullptr;
    pinned_bytes[k] = 0;
    if (want[k].p && want[k].bytes && eph_pin(want[k].p, want[k].bytes) == EPH_OK) {
      pinned[k] = want[k].p;
      pinned_bytes[k] = want[k].bytes;
    }
  }
}

void FixEPHGB::reset_dt() {
  if (ctx) check(eph_reset_dt(ctx, update->dt), "reset_dt");
}

// The engine moves atom i's data to slot j (sorting, deleting, migrating
// atoms): the device's copy is out of order until the next upload.
void FixEPHGB::copy_arrays(int i, int j, int) {
  for (int k = 0; k < 8; ++k) array[j][k] = array[i][k];
  reordered = true;
}

void FixEPHGB::grow_arrays(int ngrow) {
  if (pinned[3]) {  // unpinned before the reallocation frees it
    eph_unpin(pinned[3]);
    pinned[3] = nullptr;
    pinned_bytes[3] = 0;
  }
  memory->grow(array, ngrow, 8, "eph/gb:array");
  array_atom = array;
}

double FixEPHGB::compute_vector(int i) {
  double v = 0.0;
  check(eph_compute_vector(ctx, i == 1 ? 1 : 0, &v), "compute_vector");
  return v;
}

void FixEPHGB::post_run() { check(eph_post_run(ctx), "post_run"); }

double FixEPHGB::memory_usage() { return 8.0 * 8.0 * atom->nmax; }
