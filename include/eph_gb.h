/*
 * eph_gb.h -- C ABI of the GB300 electron-phonon (`fix eph`) hot path.
 *
 * Drop-in boundary for the LAMMPS fix `eph` of USER-EPH (fix_eph.h:11-12,
 * `FixStyle(eph,FixEPH)`): a context is built from the fix command's own words
 * and then driven through the four hooks the reference fix registers
 * (fix_eph.cpp:293-302: INITIAL_INTEGRATE, POST_FORCE, FINAL_INTEGRATE,
 * END_OF_STEP).  All per-step work runs as sm_103a CUDA kernels on one GPU in
 * FP64; there is no CPU fallback.  Plain C types only; every call returns an
 * EPH_OK / EPH_ERR_* status and never throws.
 *
 * Ownership: the context owns all device memory; the caller owns every buffer
 * it passes.  Host buffers use the engine's layout (x[n][3] etc.).  All device
 * work is ordered on the context's CUDA stream; calls that hand data back to
 * the host synchronise that stream.
 */
#ifndef EPH_GB_H
#define EPH_GB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define EPH_OK 0
#define EPH_ERR_ARG 1               /* bad argument (fix_eph.cpp:64, :140, :182, :196 error->all) */
#define EPH_ERR_FILE 2              /* beta or grid file unreadable (eph_beta.h:42, eph_fdm.h:50 asserts) */
#define EPH_ERR_UNSUPPORTED_MODEL 3 /* model other than 1 or 4 (fix_eph.cpp:888 throws on unknown ones) */
#define EPH_ERR_CAPACITY 4          /* a bin or pair list overflowed its capacity */
#define EPH_ERR_TIMEOUT 5           /* a bounded device wait gave up */
#define EPH_ERR_CUDA 6              /* CUDA runtime error (no device, launch failure) */
#define EPH_ERR_STATE 7             /* call out of order (e.g. hooks before eph_set_atoms) */
#define EPH_ERR_RANGE 8             /* an input outside the tables / box the kernels index */

/* arithmetic of the per-pair sweeps */
#define EPH_MODE_EXACT 0 /* the reference's expression order, no FMA: bit-identical forces */
#define EPH_MODE_FAST 1  /* per-atom alpha/rho and per-pair rho(r^2)/r^2 factored out, FMA */

/* where a buffer lives */
#define EPH_HOST 0
#define EPH_DEVICE 1
/* host pointer, copy queued on the context's stream only: the host buffer
 * must stay valid and unchanged (put) or unread (get) until the next call that
 * synchronises (eph_get with EPH_HOST, eph_synchronize, eph_compute_vector);
 * use pinned memory for it to overlap anything */
#define EPH_HOST_ASYNC 2

/* source of the Gaussian deviates xi of the random force */
#define EPH_XI_DEVICE_RNG 0 /* counter-based Philox4x32-10 on the device, seeded by the fix seed */
#define EPH_XI_GIVEN 1      /* the deviates last passed with eph_put(EPH_FIELD_XI) */

/* per-atom and grid fields for eph_put / eph_get */
#define EPH_FIELD_X 0       /* positions, n x 3 (put/get) */
#define EPH_FIELD_V 1       /* velocities, n x 3 (put/get) */
#define EPH_FIELD_F 2       /* total force, n x 3 (put/get) */
#define EPH_FIELD_XI 3      /* Gaussian deviates: put = for the next post_force; get = those the last used, n x 3 */
#define EPH_FIELD_F_EPH 4   /* friction force of the last post_force, n x 3 (get) */
#define EPH_FIELD_F_RNG 5   /* random force of the last post_force, n x 3 (get) */
#define EPH_FIELD_RHO 6     /* site density rho_i, n (get) */
#define EPH_FIELD_W 7       /* friction pre-vector w_i, n x 3 (get) */
#define EPH_FIELD_PERATOM 8 /* the fix's per-atom array, n x 8: rho, beta(rho), f_EPH, f_RNG (get) */
#define EPH_FIELD_T_E 9     /* electronic temperature grid, ncells (put/get) */
#define EPH_FIELD_F_EXT 10  /* external force applied by eph_step as the pair force, n x 3 (put) */

/* splines of a beta file, for eph_beta_eval / eph_beta_table */
#define EPH_SPLINE_RHO_R 0    /* rho(r) */
#define EPH_SPLINE_RHO_R_SQ 1 /* rho(r^2) */
#define EPH_SPLINE_BETA 2     /* beta(rho) */
#define EPH_SPLINE_ALPHA 3    /* alpha(rho), spline of sqrt(beta) knots */

typedef struct eph_ctx eph_ctx;

/* What the fix reads from the engine besides its own words. */
typedef struct eph_md {
  int ntypes;         /* atom->ntypes */
  const double *mass; /* atom->mass, ntypes + 1 entries, index 1..ntypes */
  double boxlo[3];    /* domain->boxlo (orthogonal, periodic, 3-D: fix_eph.cpp:263-271) */
  double boxhi[3];    /* domain->boxhi */
  double dt;          /* update->dt */
  double boltz;       /* force->boltz */
  double ftm2v;       /* force->ftm2v */
  double skin;        /* neighbor->skin: eph_step wraps positions when an atom moved > skin/2 */
  int groupbit;       /* the fix group's bit */
  int device;         /* CUDA device ordinal */
  int mode;           /* EPH_MODE_EXACT or EPH_MODE_FAST */
} eph_md;

/* Build a context from the words of the fix command: arg[0] fix ID, arg[1]
 * group, arg[2] style ("eph"), then seed flags model rho_e C_e kappa_e T_e NX
 * NY NZ T_infile freq T_out beta_file and one element name per atom type.
 * Replaces FixEPH::FixEPH (fix_eph.cpp:61-241) and FixEPH::init
 * (fix_eph.cpp:263-287).  Models 4 (PRL, force_prl) and 1 (TTM, force_ttm)
 * run; with arg[2] = "eph/coloured/exp" the words are those of the
 * coloured-noise fix (fix_eph_coloured_exp.cpp: arg[5] is tau0, model 4 with
 * an exponential memory on both forces). */
int eph_create(int narg, const char *const *arg, const eph_md *md, eph_ctx **out);
void eph_destroy(eph_ctx *ctx);
const char *eph_last_error(const eph_ctx *ctx);
const char *eph_status_string(int status);

/* Set (or reset) the atoms: n locals with positions, velocities, types
 * 1..ntypes and group masks (mask may be NULL: all in the group).  Host
 * buffers.  Replaces FixEPH::grow_arrays (fix_eph.cpp:918-938) plus the
 * engine's atom storage. */
int eph_set_atoms(eph_ctx *ctx, int n, const double *x, const double *v, const int *type, const int *mask);

/* Copy a field in or out (where = EPH_HOST, EPH_HOST_ASYNC or EPH_DEVICE pointer). */
int eph_put(eph_ctx *ctx, int field, const double *src, int where);
int eph_get(eph_ctx *ctx, int field, double *dst, int where);

/* The hooks.  FixEPH::initial_integrate (fix_eph.cpp:305-328). */
int eph_initial_integrate(eph_ctx *ctx);
/* FixEPH::post_force (fix_eph.cpp:841-907) with force_prl
 * (fix_eph.cpp:687-837) and calculate_environment (fix_eph.cpp:431-466):
 * adds f_EPH and f_RNG to the force held by the context. */
int eph_post_force(eph_ctx *ctx, int xi_source);
/* FixEPH::final_integrate (fix_eph.cpp:330-348). */
int eph_final_integrate(eph_ctx *ctx);
/* FixEPH::end_of_step (fix_eph.cpp:350-429): energy deposition onto the
 * grid, EPH_FDM::solve (eph_fdm.h:267-400), temperature output every freq
 * steps, Ee accumulation. */
int eph_end_of_step(eph_ctx *ctx);

/* The hooks with the engine's own host arrays (n x 3 doubles, atom order;
 * pinned or registered with eph_pin for the copies to run at the host
 * link's rate), each equal to the eph_put / hook / eph_get sequence it
 * replaces, with the copies overlapped: the atoms go in chunks whose
 * host->device and device->host copies run at once on two copy streams, and
 * the context's stream runs one fused kernel per chunk.  Each returns when
 * the arrays it writes hold the results (the per-atom array of
 * eph_post_force_host: when eph_end_of_step or eph_synchronize returns).
 * initial_integrate: x, v in; the half kick and drift; x, v out (in place). */
int eph_initial_integrate_host(eph_ctx *ctx, double *x, double *v);
/* post_force: x in when not NULL (a re-neighbouring step: the engine wrapped
 * it; otherwise the device keeps the x of initial_integrate), f_in in (the
 * engine's force; its copy overlaps the binning and the density sweep),
 * f_EPH + f_RNG added, the total out into f_out (which may be f_in: the
 * engine's own f array); with array not NULL the fix's per-atom array
 * (n x 8: rho, beta, f_EPH, f_RNG, fix_eph.cpp:406-428) is copied into it on
 * a third stream while the next hooks run. */
int eph_post_force_host(eph_ctx *ctx, const double *x, const double *f_in, double *f_out, double *array,
                        int xi_source);
/* final_integrate: f in; the half kick; v out. */
int eph_final_integrate_host(eph_ctx *ctx, const double *f, double *v);
/* Page-lock (and unlock) a host range for the copies above (the engine's
 * atom arrays, which it allocates itself); a range may be pinned once. */
int eph_pin(void *p, size_t bytes);
int eph_unpin(void *p);

/* nsteps engine steps on the device (Verlet::run order): initial_integrate,
 * position wrap when an atom moved > skin/2, force = external force,
 * post_force, final_integrate, end_of_step.  Device-resident; with
 * EPH_XI_GIVEN every step reuses the deviates last put. */
int eph_step(eph_ctx *ctx, int nsteps, int xi_source);

/* Replay eph_step from a CUDA graph of one captured step (on != 0): one
 * launch per step instead of one per kernel.  No reference counterpart.
 * Re-captured after eph_set_atoms, eph_reset_dt, eph_set_capacity or a
 * change of deviate source; bypassed while profiling is on. */
int eph_set_graph(eph_ctx *ctx, int on);

/* FixEPH::compute_vector (fix_eph.cpp:940-948): 0 -> cumulative energy
 * transferred to the electrons, 1 -> mean electronic temperature
 * (eph_fdm.h:189-196). */
int eph_compute_vector(eph_ctx *ctx, int i, double *out);
/* FixEPH::reset_dt (fix_eph.cpp:909-916). */
int eph_reset_dt(eph_ctx *ctx, double dt);
/* EPH_FDM::save_state (eph_fdm.h:226-265) and save_temperature
 * (eph_fdm.h:198-224) of the current grid. */
int eph_save_state(eph_ctx *ctx, const char *path);
int eph_save_temperature(eph_ctx *ctx, const char *path, int n);
/* FixEPH::post_run (fix_eph.cpp:1019-1021): writes T.restart or
 * <T_infile>.restart. */
int eph_post_run(eph_ctx *ctx);
/* The current engine step number (update->ntimestep as the context counts it). */
int eph_set_timestep(eph_ctx *ctx, long ntimestep);
/* Order the context's work on a caller's CUDA stream (cudaStream_t), or 0. */
int eph_set_stream(eph_ctx *ctx, void *stream);
/* Wait for the context's work and report any device-side error. */
int eph_synchronize(eph_ctx *ctx);
/* Device-side counters: 0 atoms with rho > rho_cutoff (the reference warns
 * once, eph_beta.h:174-180), 1 grid cells clamped at T = 0 (eph_fdm.h:391-394),
 * 2 neighbour-list builds, 3 position wraps. */
int eph_get_counter(eph_ctx *ctx, int which, long *out);
/* Capacity of a spatial bin and of a per-atom pair list (0 keeps a value). */
int eph_set_capacity(eph_ctx *ctx, int bin_capacity, int pair_capacity);

/* Pair force of the standalone engine (eph_step, batches): eam/alloy from a
 * setfl file, elements[t-1] the file's element for LAMMPS type t (as
 * `pair_coeff * * file E1 E2 ...`).  Evaluated each step on the GPU between
 * initial_integrate and post_force, added to EPH_FIELD_F_EXT if one is set.
 * Call before eph_set_atoms.  No reference counterpart: the reference fix gets
 * the pair force from LAMMPS (Tests/MD_Run/run.lmp: pair_style eam/alloy);
 * the hook functions are unaffected. */
int eph_set_pair_eam(eph_ctx *ctx, const char *path, int ntypes, const char *const *elements);
/* embedding + pair energy of the last step's pair force (0 without one) */
int eph_pair_energy(eph_ctx *ctx, double *E);

/* Lanes per atom of the FAST-mode friction and force sweeps (no reference
 * counterpart): 0 = chosen from the atom count (the default), or 1, 2, 4, 8.
 * More lanes keep small systems (tens of thousands of atoms) from waiting on
 * their loads; the sums' order, and so the last bits, depend on it (EXACT
 * mode always uses one lane). */
int eph_set_threads_per_atom(eph_ctx *ctx, int tpa);
int eph_get_threads_per_atom(eph_ctx *ctx, int *tpa);
/* Time the sweeps with 1, 2, 4 and 8 lanes per atom on the current pairs
 * (after at least one step; forces and memories are restored) and keep the
 * fastest; *chosen gets it (may be NULL). */
int eph_autotune(eph_ctx *ctx, int *chosen);
/* Time a window of `steps` engine steps (eph_step with device deviates,
 * direct launches) from the current state with each list skin of
 * skins[0..nskins-1] (0 = the bin search every step), each window starting
 * with a list build as a run does after eph_set_list_skin (one untimed
 * window first), then restore the state -- positions, velocities, forces,
 * memories, deviates, per-atom records, the atoms' grid cells and T_e there,
 * the grid, the vector, counters and step counters; no T_out file is
 * written, so it may also run between post_force and end_of_step -- and keep the skin of the fastest
 * window; *chosen gets it (may be NULL).  The bins' edge is r_cutoff + skin
 * (their 27-bin stencil), so this chooses the bin size too.  A window that
 * overflows the bins or pair rows rules its skin out.  The trajectory from
 * here is the one eph_set_list_skin(ctx, *chosen) would give at this point:
 * the order of the sums, and so the last bits, depend on the skin.  Where no
 * skin turns the lists on (EXACT mode, model 1, several lanes per atom below
 * 16,384 atoms, the EAM engine, an adjoint, a box narrower than three list
 * radii) nothing runs and *chosen gets the current skin.  Needs one step (or
 * post_force) first and ~0.4 KB of device memory per atom for the saved
 * state.  No reference counterpart (the reference takes its pairs from the
 * engine's Verlet list, whose skin the user sets, fix_eph.cpp:273-275). */
int eph_autotune_list_skin(eph_ctx *ctx, const double *skins, int nskins, int steps, double *chosen);

/* Arithmetic of the FAST-mode per-pair work where the density sweep runs
 * one lane per atom with stage 1 folded (by default from 16,384 atoms on,
 * with the bin search or the kept candidate lists; model 4):
 * EPH_PAIRS_DF64 (the default) forms every pair term and its sums in
 * double-float -- pairs of FP32 numbers carrying 48 significand bits, on the
 * FP32 pipe, which GB300 issues at 64 times its FP64 rate -- and keeps the
 * per-atom work (beta, alpha, the integrator, the grid) in FP64;
 * EPH_PAIRS_FP64 keeps the pair terms in FP64 as well.  Results agree with
 * the reference within the FAST bar (1e-12 relative per atom) either way;
 * the last bits differ.  No reference counterpart. */
#define EPH_PAIRS_FP64 0
#define EPH_PAIRS_DF64 1
int eph_set_pair_arithmetic(eph_ctx *ctx, int which);

/* Skin s of the kept candidate lists (Angstrom; default 0.3, used from 2^15
 * atoms on with the df64 pair sums and from 2^15 to 2^20 atoms with FP64
 * ones, where it pays; a skin set here applies at any size, 0 turns
 * the lists off).  The reference takes its pairs from the engine's Verlet list
 * (fix_eph.cpp:273-275: a full list with cutoff r_cutoff, padded by the
 * engine's skin and rebuilt when an atom moved half of it); here the list is
 * the context's own.  In FAST mode (model 4, the one-lane density sweep) the
 * candidates within r_cutoff + s are found by a bin search on build steps
 * only; in between, up to 32 atoms that moved more than s/2 (and the atoms
 * near them) search afresh every step, and more of them make the step a
 * build step (counter 2 counts the builds).  Pairs and results are those of
 * a search every step, up to the order of the sums.  *active reports whether
 * the context uses it (either pointer may be NULL). */
int eph_set_list_skin(eph_ctx *ctx, double skin);
int eph_get_list_skin(eph_ctx *ctx, double *skin, int *active);

/* Timing of the step's phases with CUDA events on the context's stream
 * (no reference counterpart; the reference relies on gprof, lib/Makefile:25-28).
 * Phases: */
#define EPH_PHASE_INTEGRATE 0  /* initial + final integrate */
#define EPH_PHASE_BIN 1        /* spatial binning */
#define EPH_PHASE_DENSITY 2    /* neighbour pairs + rho_i (calculate_environment) */
#define EPH_PHASE_FRICTION_W 3 /* force_prl stage 1 */
#define EPH_PHASE_FORCES 4     /* force_prl stages 2 + 3 and the force update */
#define EPH_PHASE_DEPOSIT 5    /* energy deposition + energy total */
#define EPH_PHASE_FDM 6        /* EPH_FDM::solve substeps */
#define EPH_PHASE_PAIR 7       /* the engine's pair force (eph_set_pair_eam) */
#define EPH_NPHASES 8
/* on != 0 starts recording (and zeroes the totals); off stops. */
int eph_set_profiling(eph_ctx *ctx, int on);
/* milliseconds and kernel launches per phase since profiling was switched on
 * (arrays of EPH_NPHASES; either may be NULL). */
int eph_phase_times(eph_ctx *ctx, double *ms, long *launches);
/* kernels this context launched since profiling was last switched */
int eph_launch_count(eph_ctx *ctx, long *out);
/* in-cutoff pairs (directed) of the last post_force */
int eph_pair_count(eph_ctx *ctx, long *out);

/* Batched replicas: many independent fix instances (each its own words,
 * box, atoms, grid and seed) on one GPU, stepped together: one step of every
 * replica is captured as parallel branches of one CUDA graph and each
 * eph_batch_step step is one graph launch.  Each replica's results are those
 * of the same replica run alone with eph_step (device deviates).  No
 * reference counterpart (the reference runs one system per LAMMPS run). */
typedef struct eph_batch eph_batch;
int eph_batch_create(int nrep, const int *narg, const char *const *const *arg, const eph_md *md, eph_batch **out);
void eph_batch_destroy(eph_batch *batch);
const char *eph_batch_last_error(const eph_batch *batch);
int eph_batch_set_atoms(eph_batch *batch, int rep, int n, const double *x, const double *v, const int *type,
                        const int *mask);
int eph_batch_step(eph_batch *batch, int nsteps);
int eph_batch_synchronize(eph_batch *batch);
/* the context of replica rep (for eph_get, eph_compute_vector, ...) */
eph_ctx *eph_batch_context(eph_batch *batch, int rep);
/* kernels one batched step launches (inside its graph) */
int eph_batch_launch_count(eph_batch *batch, long *per_step);

/* Electronic-grid solve that allocates nothing.  No counterpart in the
 * reference.  For callers that own all device memory and may not call
 * cudaMalloc/cudaFree while they run (an engine with its own device pool, a
 * time-step loop that must not synchronise the device): one EPH_FDM::solve
 * (eph_fdm.h:267-400, constant C_e and kappa) on caller-owned device arrays of
 * an nx*ny*nz grid spanning [lo, hi): T is updated in place, dT, S, rho_e,
 * C_e, kappa and flag are read (dT is not cleared).  The only other memory is
 * a static scratch array of EPH_NOALLOC_MAX_CELLS + 8 doubles that every GPU
 * loading this library holds until exit; larger grids return
 * EPH_ERR_CAPACITY.  The first call on a device looks up that array's device
 * address, so make it before any stream capture.  All calls share the
 * scratch: calls that overlap on the GPU race.  lo and hi are HOST arrays of
 * 3 doubles (the grid box); every other array is a device pointer.  Work is
 * ordered on `stream` (a cudaStream_t, 0 for the default stream); the call
 * synchronises that stream twice (it reads the stability bounds back to pick
 * the substep count) and has finished on return.  The number of substeps
 * taken goes to *nsub_out (may be NULL).  EPH_ERR_ARG, before any launch:
 * C_e or rho_e of cell 0 or of a non-CONSTANT cell <= 0, or more than
 * EPH_NOALLOC_MAX_SUBSTEPS substeps (given or required by the stability
 * rule). */
#define EPH_NOALLOC_MAX_CELLS 262144 /* 64^3 */
#define EPH_NOALLOC_MAX_SUBSTEPS 1000000
int eph_fdm_solve_noalloc(long nx, long ny, long nz, const double *lo, const double *hi, double dt, long steps,
                          double *T, const double *dT, const double *S, const double *rho_e, const double *C_e,
                          const double *kappa, const signed char *flag, void *stream, unsigned *nsub_out);

/* Host-side parametrisation (no GPU needed): the beta file reader and the
 * splines it builds (eph_beta.h:39-128, eph_spline.h:31-142). */
typedef struct eph_beta eph_beta;
int eph_beta_load(const char *path, eph_beta **out);
void eph_beta_free(eph_beta *b);
int eph_beta_info(const eph_beta *b, int *n_elements, double *r_cutoff, double *rho_cutoff);
/* value of one spline (which = EPH_SPLINE_*) of element elem at x */
double eph_beta_eval(const eph_beta *b, int which, int elem, double x);
/* copy the coefficient table (a, b, c, d per knot) into out (may be NULL);
 * returns the number of knots */
long eph_beta_table(const eph_beta *b, int which, int elem, double *out);

/* Replace element elem's knot columns (the file's rho(r) and beta(rho)
 * columns, n_rho and n_beta values) and rebuild its tables as the reader does
 * (eph_beta.h:103-124).  No reference counterpart: lets a fitting loop change
 * the parametrisation without writing files. */
int eph_beta_set_knots(eph_beta *b, int elem, const double *rho_knots, long n_rho, const double *beta_knots,
                       long n_beta);
/* Chain rule through the table construction of element elem: from dL/d(table
 * coefficients) of the rho(r^2) table (n_rho x 4) and of the alpha table
 * (n_beta x 4) to dL/d(knot columns): g_rho (n_rho), g_beta (n_beta). */
int eph_beta_knot_gradient(const eph_beta *b, int elem, const double *g_rho_r_sq, const double *g_alpha,
                           double *g_rho, double *g_beta);

/* Host-side grid (no GPU needed): uniform grid or grid file
 * (eph_fdm.h:28-119), stability substeps (eph_fdm.h:275-313), writers. */
typedef struct eph_grid eph_grid;
int eph_grid_create(long nx, long ny, long nz, const double *lo, const double *hi, double T_e, double C_e,
                    double rho_e, double kappa_e, eph_grid **out);
int eph_grid_load(const char *path, eph_grid **out);
void eph_grid_free(eph_grid *g);
long eph_grid_ncells(const eph_grid *g);
/* number of substeps solve() takes for time step dt, and their length */
unsigned eph_grid_substeps(const eph_grid *g, double dt, double *inner_dt);
int eph_grid_save_state(const eph_grid *g, const char *path);
int eph_grid_save_temperature(const eph_grid *g, const char *path, int n);

/* ---------------------------------------------------------------- adjoint
 * Reverse-mode gradients of a trajectory loss through the whole fix step
 * (force_prl model 4: density, friction pre-vector, friction and random
 * forces, integrator, deposition, grid solve).  No reference counterpart:
 * the reference computes no derivatives.
 *
 * Parameters a fitting loop changes between trajectories: */
/* element elem's knot columns on a context (see eph_beta_set_knots) */
int eph_set_beta_knots(eph_ctx *ctx, int elem, const double *rho_knots, long n_rho, const double *beta_knots,
                       long n_beta);
/* C_e and kappa_e of every cell of a grid made from the fix's words
 * (T_infile NULL); the substep count follows (eph_fdm.h:275-313). */
int eph_set_grid_constants(eph_ctx *ctx, double C_e, double kappa_e);

/* An adjoint object records the context's state at creation (positions,
 * velocities, forces, T_e grid, random-number counter): every trajectory it
 * runs starts there.  Deviates come from the device generator (EPH_XI_DEVICE_RNG),
 * so a trajectory is a fixed function of the parameters (pathwise gradients).
 * The backward pass recomputes each segment of checkpoint_every steps from a
 * checkpoint taken by the forward pass and records that segment's
 * intermediates on the device.  Supported: model 4, fix eph (not the
 * coloured form), grids without temperature-dependent cells. */
typedef struct eph_adjoint eph_adjoint;
int eph_adjoint_create(eph_ctx *ctx, int checkpoint_every, eph_adjoint **out);
void eph_adjoint_destroy(eph_adjoint *adj);
const char *eph_adjoint_last_error(const eph_adjoint *adj);
/* Run nsteps engine steps from the recorded start.  E[t] = energy the ions
 * gave the electrons in step t (the reference's E_local, fix_eph.cpp:364-404),
 * T_mean[t] = mean T_e of the grid after step t (get_T_total, eph_fdm.h:189-196);
 * either pointer may be NULL.  The context is left at the last step. */
int eph_adjoint_forward(eph_adjoint *adj, long nsteps, double *E, double *T_mean);
/* Reverse sweep over the last forward trajectory for L with dL/dE[t] and
 * dL/dT_mean[t] (host arrays of nsteps values; NULL means zero). */
int eph_adjoint_backward(eph_adjoint *adj, const double *dL_dE, const double *dL_dT_mean);
/* Gradient of L after eph_adjoint_backward: */
#define EPH_GRAD_RHO_KNOTS 0  /* element elem's rho(r) knot column, n_rho values */
#define EPH_GRAD_BETA_KNOTS 1 /* element elem's beta(rho) knot column, n_beta values */
#define EPH_GRAD_C_E 2        /* 1 value: every cell's C_e changed together */
#define EPH_GRAD_KAPPA 3      /* 1 value: every cell's kappa_e changed together */
int eph_adjoint_gradient(eph_adjoint *adj, int which, int elem, double *out, long n);
/* on (the default): each pass is captured once as a CUDA graph and replayed
 * while the number of steps, the step constants and the buffers stay; off:
 * every kernel is launched from the host */
int eph_adjoint_set_graph(eph_adjoint *adj, int on);
/* milliseconds of the last forward and backward passes (CUDA events on the
 * context's stream) and the kernels each launched; any pointer may be NULL */
int eph_adjoint_timing(eph_adjoint *adj, double *forward_ms, double *backward_ms, long *forward_launches,
                       long *backward_launches);

/* Several adjoints (of contexts on one device) run together: each pass of
 * every adjoint is a parallel branch of one CUDA graph, so many small
 * replicas fill the GPU (batched fitting).  The batch does not own the
 * adjoints.  E, T_mean, dL_dE, dL_dT_mean: nadj x nsteps, row per adjoint
 * (NULL allowed); the gradients are read per adjoint with eph_adjoint_gradient. */
typedef struct eph_adjoint_batch eph_adjoint_batch;
int eph_adjoint_batch_create(int nadj, eph_adjoint *const *adj, eph_adjoint_batch **out);
void eph_adjoint_batch_destroy(eph_adjoint_batch *batch);
const char *eph_adjoint_batch_last_error(const eph_adjoint_batch *batch);
int eph_adjoint_batch_forward(eph_adjoint_batch *batch, long nsteps, double *E, double *T_mean);
int eph_adjoint_batch_backward(eph_adjoint_batch *batch, const double *dL_dE, const double *dL_dT_mean);
int eph_adjoint_batch_timing(eph_adjoint_batch *batch, double *forward_ms, double *backward_ms,
                             long *forward_launches, long *backward_launches);

#ifdef __cplusplus
}
#endif
#endif
