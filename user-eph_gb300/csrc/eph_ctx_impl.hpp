// Internal: the context of one fix instance and the launch sequence of one
// engine step, shared by eph_ctx.cu (the plain path and the C ABI) and
// eph_adjoint.cu (the reverse-mode gradient).  Not part of the public ABI.
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "eph_gb.h"
#include "eph_device.cuh"
#include "eph_host.hpp"

namespace ephgb {


template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, sizeof(T) * count);
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { free(); }
};

constexpr int BLOCK = 128;
inline int nblocks(long n, int b = BLOCK) { return (int)((n + b - 1) / b); }

}  // namespace ephgb

using namespace ephgb;

struct EamDevice;  // the engine's eam/alloy pair force (eph_eam.cu)

struct eph_ctx {
  std::string err;
  int device = 0;
  cudaStream_t stream = 0;
  bool own_stream = false;

  FixArgs args;
  Beta beta;
  Grid grid;  // host copy: geometry and parameters (T lives on the device)
  int ntypes = 0;
  std::vector<double> mass;
  std::vector<int> type_map;  // by LAMMPS type 1..ntypes
  double boxlo[3], boxhi[3], prd[3];
  double dt = 0, boltz = 0, ftm2v = 0, skin = 0;
  int groupbit = 1, mode = EPH_MODE_FAST;
  long ntimestep = 0;

  StepParams P{};
  bool multi = false;
  // lanes per atom of the FAST-mode friction and force sweeps (1, 2, 4, 8)
  // and whether it follows the atom count (eph_set_threads_per_atom)
  int tpa = 1;
  bool tpa_auto = true;
  // FAST mode, one lane per atom: stage 1 folded into the density sweep
  bool fuse_w = true;
  // small grids run all their substeps as one thread-block cluster launch
  bool fdm_cluster = false;

  int n = 0;
  DevBuf<D4> x, v, f, xhold, f_eph, f_rng, xi, fext, A, Bw;
  DevBuf<D4> f_dis, f_sto;  // coloured-noise memory (eph/coloured/exp)
  // FAST mode, one lane per atom: M_i (2 x n: {xx,xy,xz,yy}, {yz,zz}) and the
  // gathered records G_i ({a w, a xi_x}, {a xi_y, a xi_z, rho}, interleaved)
  DevBuf<D4> Mm, G;
  bool have_fext = false, have_xi = false;
  DevBuf<int> type, mask, nshort, cell, tmap;
  DevBuf<double> rho, beta_i, Te_i, stage;
  // the hooks with the engine's host arrays (eph_*_host): two copy streams
  // (host->device, device->host) and one for the per-atom array, events of
  // the chunks, staging rows (20 n doubles: 12 n for the hooks' rows, 8 n
  // for the per-atom array, which may still be on its way out while the
  // next hook runs)
  cudaStream_t s_in = nullptr, s_out = nullptr, s_arr = nullptr;
  std::vector<cudaEvent_t> xev;
  DevBuf<double> hstage;
  cudaEvent_t f_ready = nullptr, arr_done = nullptr;
  bool f_pending = false, arr_pending = false;
  DevBuf<int> bin_count;
  DevBuf<BinEntry> bins;
  DevBuf<int4> atom_bin;
  DevBuf<float4> atom_off;
  DevBuf<unsigned> pj;
  DevBuf<D4> pe;
  DevBuf<double2> pg;
  int nbins = 0, bcap = 0, kcap = 0;
  bool bcap_user = false;  // bin capacity set by eph_set_capacity
  // candidate-list reuse (FAST mode, one lane per atom, model 4 with
  // friction): the list skin s (0: search the bins every step), whether it is
  // on, and whether an adjoint keeps it off (its recomputed segments must
  // repeat the recorded ones bit for bit)
  double lskin = 0.3;
  bool lskin_user = false;  // set by eph_set_list_skin: applies at any size
  bool reuse = false, list_block = false;
  int lcap = 0;
  DevBuf<unsigned> cl;  // [lcap][n] candidates
  DevBuf<int> cl_n, state, rb, flist;
  DevBuf<D4> xref;  // positions at the last build

  DevBuf<D4> tab_rho_r_sq, tab_beta, tab_alpha;
  // FAST pair sums in df64 (eph_set_pair_arithmetic, on by default): the
  // rho(r^2) tables in local form (two float4 per knot) and the per-atom
  // records k_bin writes for them (bin offset and bin, velocity: two float4
  // each per atom)
  int pair_arith = EPH_PAIRS_DF64;
  DevBuf<float4> tab_rho_df, dfrec, dfvrec;

  DevBuf<double> T0, T1, kappa, rhoC, irhoC, S, dT;
  // temperature-dependent cells: per-cell C_e and rho_e, the parameter tables
  DevBuf<double> gC, grho, E_y, E_dy, bounds;
  DevBuf<D4> C_T, K_T;
  DevBuf<unsigned char> tdyn;
  TdynTables td{};
  double *h_bounds = nullptr;  // pinned
  DevBuf<signed char> gflag;
  DevBuf<U128> acc, part, gsum;
  unsigned nsub = 1;
  double inner_dt = 0;
  // eam/alloy pair force of the standalone engine (eph_set_pair_eam), or none
  EamDevice *eam = nullptr;
  bool eam_list_fresh = false;  // the EAM pair list is this step's (launch_eam ran since the last density sweep)
  // set by the adjoint while it records a step: substep k of the grid solve
  // writes its output to fdm_rec + k * ncells instead of the ping-pong buffer
  double *fdm_rec = nullptr;

  // per-phase CUDA-event timing (eph_set_profiling) and launch counts
  bool profiling = false;
  struct Mark {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> event_pool;
  double phase_ms[EPH_NPHASES] = {0};
  long phase_launches[EPH_NPHASES] = {0};
  long launches = 0;
  // bumped whenever a device buffer is (re)allocated: graphs captured by
  // others (the adjoint) hold the old addresses and must be captured again
  unsigned long long buf_gen = 0;

  // one captured engine step replayed by eph_step (eph_set_graph)
  bool use_graph = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_xi = -1;
  long graph_launches = 0;  // kernels in one replay

  DevBuf<double> scal;  // 0 Ee, 1 E_local, 2 T_total
  DevBuf<unsigned> d_err;
  DevBuf<unsigned long long> counters;
  DevBuf<int> wrapflag;
  DevBuf<unsigned long long> step_ctr;  // post_force calls so far (the Philox counter)
  unsigned *h_err = nullptr;  // pinned
};

namespace ephgb {
namespace ctxi {

int fail(eph_ctx *c, int code, const std::string &msg);
cudaError_t alloc_pg(eph_ctx *c);
int check_device(eph_ctx *c);
int require_atoms(eph_ctx *c);
int upload_tables(eph_ctx *c);
int upload_grid(eph_ctx *c);
void set_time_params(eph_ctx *c);
void drop_graph(eph_ctx *c);
// the four phases of one engine step on the context's stream
int launch_initial(eph_ctx *c, int check_wrap);
int launch_post_force(eph_ctx *c, int xi_mode);
int launch_final(eph_ctx *c);
int launch_end_of_step(eph_ctx *c);
// post_force in two parts: spatial binning (and the wrap), then the sweeps
int launch_bin(eph_ctx *c);
// candidate-list reuse on or off as the context's settings allow (bins,
// list buffers), and a build requested for the next step; drop_list turns it off
int configure_list(eph_ctx *c);
void drop_list(eph_ctx *c);
int launch_pair_sweeps(eph_ctx *c, int xi_mode);
// the engine's pair force for this step into f (plus the external force)
// bins of edge >= r (1 + 5e-5), at least three per axis (all of P's bin geometry)
int set_bin_geometry(eph_ctx *c, double r);
// the df64 pair sums run (and k_bin writes the atoms' df64 records)
bool df_active(const eph_ctx *c);
int launch_eam(eph_ctx *c);
// the EAM pair list of the step (rows k * n + i, counts) if it holds every
// candidate of the fix's density sweep
bool eam_pair_list(const eph_ctx *c, const unsigned **pj, const int **ns);
int eam_resize(eph_ctx *c);  // per-atom buffers of the pair force for c->n atoms
void eam_free(eph_ctx *c);

inline cudaEvent_t take_event(eph_ctx *c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets the launches of one phase with CUDA events on the context's
// stream when profiling is on; counts the kernel launches either way.
struct PhaseScope {
  eph_ctx *c;
  int phase;
  cudaEvent_t b = nullptr;
  PhaseScope(eph_ctx *ctx, int ph) : c(ctx), phase(ph) {
    if (c->profiling) {
      b = take_event(c);
      cudaEventRecord(b, c->stream);
    }
  }
  void launched(int k = 1) {
    c->launches += k;
    c->phase_launches[phase] += k;
  }
  ~PhaseScope() {
    if (c->profiling && b) {
      cudaEvent_t e = take_event(c);
      cudaEventRecord(e, c->stream);
      c->marks.push_back({phase, b, e});
    }
  }
};

}  // namespace ctxi
}  // namespace ephgb

#define CUDA_TRY(ctx, call)                                                                           \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) return ephgb::ctxi::fail((ctx), EPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
