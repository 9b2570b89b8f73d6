// Reverse-mode gradient of a trajectory loss through the fix-eph step
// (eph_adjoint_* in include/eph_gb.h).  The reference computes no
// derivatives; what is differentiated is the plain step of this library
// (fix_eph.cpp:305-348 integrator, :431-466 density, :687-837 force_prl,
// :364-404 deposition, eph_fdm.h:267-400 grid solve), so a trajectory run here
// is the eph_step trajectory bit for bit.
//
// One step maps (x, v, f, T) to (x', v', f', T').  With a_i = alpha(rho_i)/rho_i,
// H_ij = rho_{type j}(r^2)/r^2, E_ij = e e^T (e = x_j - x_i):
//   w_i   = a_i sum_j H_ij E_ij (v_i - v_j)                     (stage 1: w = W[v])
//   F[y]_i = sum_j E_ij (a_i H_ij y_i - a_j H_ji y_j)            (stages 2, 3)
//   f_EPH = -F[w],  f_RNG_i = eta sqrt(T_e(x_i)) F[xi]_i
// F is the transpose of W, so the adjoint of w is W applied to the cotangent
// of f_EPH and the adjoint of v through w is F applied to that: the reverse
// sweeps reuse the forward's pair structure.  The reverse of one step is
//   grid solve (substeps in reverse) -> per-atom energy/force cotangents ->
//   pair sweep 1 (adjoint of w, of a_i and rho_i) -> pair sweep 2 (adjoints of
//   positions and velocities, spline-coefficient gradients) -> integrator,
// each a gather over the atom's own full pair list (no scatter between
// atoms).  Gradients of the rho(r^2) and alpha tables come out per spline
// coefficient and are chained to the beta file's knot columns on the host
// (Beta::knot_gradient); C_e and kappa_e per cell, summed on the host.
//
// Memory: checkpoints of (x, v, f, xhold, T, Philox counter) every K steps,
// and for the segment being reversed, K recorded steps (positions and
// velocities at post_force, per-atom records, forces, the pair list, the grid
// at every substep).  A segment is recomputed once from its checkpoint.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "eph_ctx_impl.hpp"
#include "eph_df_pair.cuh"

using namespace ephgb;

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int ABLOCK = 128;
// rho(r^2) coefficient gradients go to per-thread accumulators in shared
// memory (deterministic) when the tables hold at most this many knots
// (x 4 coefficients x 128 threads x 8 B = 96 KB); else global atomics
constexpr int PRIV_MAX_KNOTS = 24;
// alpha coefficient gradients: per-warp accumulators in shared memory
// (deterministic) up to this many knots (x 4 x 4 warps x 8 B = 48 KB)
constexpr int WARP_MAX_KNOTS = 384;

inline int nb_of(long n, int b = ABLOCK) { return (int)((n + b - 1) / b); }

// device pointers of one recorded step
struct Slot {
  const D4 *x1, *v1, *v2, *A, *Bw, *fE, *fR;
  const int *cell, *ns;
  const double *Te;
  const unsigned *pj;
};

struct GridArgs {
  long n[3];
  long nc;
  double h[3];
  double ih2[3];  // 1/h^2 per axis
  double inner_dt;
  const double *kappa, *rhoC, *irhoC, *rho_e, *S;  // irhoC = 1/(rho_e C_e)
  const signed char *flag;
};

// value, derivative and knot of a spline at x (index as eph_spline.h:134-142).
// The reverse sweeps are FP64-issue bound: products and sums are fused
// explicitly (this file is compiled without contraction).
__device__ __forceinline__ void spline_vd(const D4 *__restrict__ tab, double inv_dx, int n, double x, double &val,
                                          double &der, int &idx) {
  unsigned long long k = trunc_index(x * inv_dx);
  if (k >= (unsigned long long)n) k = (unsigned long long)(n - 1);
  const D4 c = tab[k];
  val = fma(x, fma(x, fma(x, c.w, c.z), c.y), c.x);
  der = fma(x, fma(3.0 * x, c.w, 2.0 * c.z), c.y);
  idx = (int)k;
}

__device__ __forceinline__ double dotf(double ax, double ay, double az, double bx, double by, double bz) {
  return fma(az, bz, fma(ay, by, ax * bx));
}

// e = x_j (periodic image of the pair code) - x_i, as the density sweep forms it
__device__ __forceinline__ void pair_vector(const StepParams &P, const D4 &xi, const D4 &xj, unsigned code,
                                            double &ex, double &ey, double &ez) {
  double cx = xj.x, cy = xj.y, cz = xj.z;
  if (code != CODE_NOSHIFT) {
    const int mx = (int)(code % 3u) - 1, my = (int)((code / 3u) % 3u) - 1, mz = (int)(code / 9u) - 1;
    if (mx) cx = xj.x + (mx > 0 ? P.prd[0] : -P.prd[0]);
    if (my) cy = xj.y + (my > 0 ? P.prd[1] : -P.prd[1]);
    if (mz) cz = xj.z + (mz > 0 ? P.prd[2] : -P.prd[2]);
  }
  ex = cx - xi.x;
  ey = cy - xi.y;
  ez = cz - xi.z;
}

// Sum (c0..c3) of the lanes that share a key into base[4 key ..]; lanes with
// key < 0 take no part.  Called by all 32 lanes; one lane writes per key, so
// warps that own separate accumulators need no atomics and the sums do not
// depend on timing.
__device__ __forceinline__ void warp_add4(double *base, int key, double c0, double c1, double c2, double c3,
                                          int lane) {
  unsigned todo = __ballot_sync(FULL, key >= 0);
  while (todo) {
    const int src = __ffs(todo) - 1;
    const int k = __shfl_sync(FULL, key, src);
    const bool mine = key == k;
    double a0 = mine ? c0 : 0.0, a1 = mine ? c1 : 0.0, a2 = mine ? c2 : 0.0, a3 = mine ? c3 : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(FULL, a0, o);
      a1 += __shfl_xor_sync(FULL, a1, o);
      a2 += __shfl_xor_sync(FULL, a2, o);
      a3 += __shfl_xor_sync(FULL, a3, o);
    }
    if (lane == src) {
      base[4 * k + 0] += a0;
      base[4 * k + 1] += a1;
      base[4 * k + 2] += a2;
      base[4 * k + 3] += a3;
    }
    todo &= ~__ballot_sync(FULL, mine);
  }
}

// ------------------------------------------------------------ grid solve

// neighbours p, q of cell s along axis a, with the ZERO_DERIVATIVE rule of
// eph_fdm.h:325-367 (a wall neighbour is replaced by the cell itself)
__device__ __forceinline__ void axis_pq(const GridArgs &G, long s, int a, long &p, long &q) {
  const long st = a == 0 ? 1 : (a == 1 ? G.n[0] : G.n[0] * G.n[1]);
  const long na = G.n[a];
  const long c = (s / st) % na;
  p = c > 0 ? s - st : s + (na - 1) * st;
  q = c < na - 1 ? s + st : s - (na - 1) * st;
  if (G.flag[q] == 2) q = s;
  else if (G.flag[p] == 2) p = s;
}

// the stencil sum ddT of cell r at temperatures T and its derivative with
// respect to a change of every cell's kappa by the same amount (lap)
__device__ __forceinline__ void cell_ddT(const GridArgs &G, const double *__restrict__ T, long r, double &ddT,
                                         double &lap) {
  ddT = 0.0;
  lap = 0.0;
  if (G.flag[r] == 2) return;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    long p, q;
    axis_pq(G, r, a, p, q);
    const double ih2 = G.ih2[a];
    const double l = (T[q] + T[p] - 2.0 * T[r]) * ih2;
    ddT += (G.kappa[q] - G.kappa[p]) * (T[q] - T[p]) * 0.25 * ih2 + G.kappa[r] * l;
    lap += l;
  }
}

// Substep T_k -> T_k+1 at cell r, reversed: lam = dL/dT_k+1[r]; returns
// u = lam unless the forward clamped the cell at T = 0, and adds the substep's
// share to the source, C_e and kappa_e gradients of the cell.
__device__ __forceinline__ double substep_reverse(const GridArgs &G, const double *__restrict__ Tk,
                                                  const double *__restrict__ src, long r, double lam,
                                                  double *__restrict__ srcbar, double *__restrict__ gC,
                                                  double *__restrict__ gK, bool first) {
  double ddT, lap;
  cell_ddT(G, Tk, r, ddT, lap);
  const bool dyn = G.flag[r] == 1;
  const double rate = ddT + src[r] + G.S[r];
  const double pre = dyn ? Tk[r] + rate * G.irhoC[r] * G.inner_dt : Tk[r];
  const double u = pre >= 0.0 ? lam : 0.0;
  double w = 0.0;
  if (dyn) {
    w = u * G.inner_dt * G.irhoC[r];
    gC[r] -= w * rate * G.rho_e[r] * G.irhoC[r];
    gK[r] += w * lap;
  }
  srcbar[r] = first ? w : srcbar[r] + w;
  return u;
}

// last substep of a step: u = dL/dT after the step (+ the mean-T cotangent)
__global__ void k_adj_fdm_first(GridArgs G, const double *__restrict__ Tk, const double *__restrict__ src,
                                const double *__restrict__ Tb, const double *__restrict__ tau, double *__restrict__ u,
                                double *__restrict__ srcbar, double *__restrict__ gC, double *__restrict__ gK) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= G.nc) return;
  u[r] = substep_reverse(G, Tk, src, r, Tb[r] + *tau, srcbar, gC, gK, true);
}

// The transpose of one substep's Jacobian, as 7 weights per cell (self,
// -x, +x, -y, +y, -z, +z neighbour): lam[r] = u[r] + sum_m W[m][r] u[s_m] with
// W = dddT_s/dT_r * dt'/(rho_e C_e)_s on DYNAMIC cells s.  The same for every
// substep while kappa, C_e and the flags stay, so it is built once per pass.
// On axes of 1 or 2 cells the neighbours coincide; each distinct cell is
// counted once (in the self or the -axis slot).
__global__ void k_adj_fdm_weights(GridArgs G, double *__restrict__ W) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= G.nc) return;
  double w[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int a = 0; a < 3; ++a) {
    const long st = a == 0 ? 1 : (a == 1 ? G.n[0] : G.n[0] * G.n[1]);
    const long na = G.n[a];
    const long c = (r / st) % na;
    long cand[3];
    int slot[3];
    int ncand = 0;
    cand[ncand] = r;
    slot[ncand++] = 0;
    if (na >= 2) {
      cand[ncand] = c > 0 ? r - st : r + (na - 1) * st;
      slot[ncand++] = 1 + 2 * a;
    }
    if (na >= 3) {
      cand[ncand] = c < na - 1 ? r + st : r - (na - 1) * st;
      slot[ncand++] = 2 + 2 * a;
    }
    const double ih2 = G.ih2[a];
    for (int m = 0; m < ncand; ++m) {
      const long s = cand[m];
      if (G.flag[s] != 1) continue;  // only DYNAMIC cells move (eph_fdm.h:375-387)
      long p, q;
      axis_pq(G, s, a, p, q);
      const double dk = G.kappa[q] - G.kappa[p];
      double coef = 0.0;
      if (q == r) coef += 0.25 * ih2 * dk + G.kappa[s] * ih2;
      if (p == r) coef += -0.25 * ih2 * dk + G.kappa[s] * ih2;
      if (s == r) coef -= 2.0 * G.kappa[s] * ih2;
      w[slot[m]] += coef * G.inner_dt * G.irhoC[s];
    }
  }
  for (int m = 0; m < 7; ++m) W[(size_t)m * G.nc + r] = w[m];
}

// lam_k = the transposed substep applied to u_k; then u_k-1 of the substep
// before (Tprev = T_k-1), or, after the first substep, the cotangent of the
// grid at the start of the step (Tb).
__global__ void k_adj_fdm_back(GridArgs G, const double *__restrict__ W, const double *__restrict__ u,
                               const double *__restrict__ Tprev, const double *__restrict__ src,
                               double *__restrict__ u_out, double *__restrict__ Tb, double *__restrict__ srcbar,
                               double *__restrict__ gC, double *__restrict__ gK) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= G.nc) return;
  const long nx = G.n[0], nxy = G.n[0] * G.n[1];
  const long i = r % nx, j = (r / nx) % G.n[1], k = r / nxy;
  const long nb[6] = {i > 0 ? r - 1 : r + (nx - 1), i < nx - 1 ? r + 1 : r - (nx - 1),
                      j > 0 ? r - nx : r + (G.n[1] - 1) * nx, j < G.n[1] - 1 ? r + nx : r - (G.n[1] - 1) * nx,
                      k > 0 ? r - nxy : r + (G.n[2] - 1) * nxy, k < G.n[2] - 1 ? r + nxy : r - (G.n[2] - 1) * nxy};
  const double ur = u[r];
  double lam = fma(W[r], ur, ur);
#pragma unroll
  for (int m = 0; m < 6; ++m) lam = fma(W[(size_t)(m + 1) * G.nc + r], u[nb[m]], lam);
  if (Tprev)
    u_out[r] = substep_reverse(G, Tprev, src, r, lam, srcbar, gC, gK, false);
  else
    Tb[r] = lam;
}

__global__ void k_adj_add(double *__restrict__ a, long n, const double *__restrict__ v) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) a[r] += *v;
}

// mean of the grid (one block, fixed summation order)
__global__ void k_adj_mean(const double *__restrict__ T, long nc, double *__restrict__ out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (long r = threadIdx.x; r < nc; r += blockDim.x) acc += T[r];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0] / (double)nc;
}

// ------------------------------------------------------------ per atom

// Reverse of end_of_step's deposition and of final_integrate, and the
// cotangents the pair sweeps need.  eb = dL/dE of this step, srcbar =
// dL/d(grid source) (src = sum dE / (dV dt)).  In: vb = dL/dv', fb = dL/df'.
// Out: cE = -dL/dF_EPH... as the cotangent of F[w] (zero on atoms whose
// forces the forward skipped), cR = eta sqrt(T_e) dL/df_RNG (cotangent of
// F[xi]), vb = the part of dL/dv at post_force that does not go through the
// pair sums, Tb += dL/dT_e through sqrt(T_e).
template <bool FRIC, bool RAND>
__global__ void k_adj_energy(StepParams P, Slot S, const int *__restrict__ mask, const int *__restrict__ type,
                             const double *__restrict__ ebp, double src_scale, const double *__restrict__ srcbar,
                             D4 *__restrict__ vb,
                             const D4 *__restrict__ fb, D4 *__restrict__ cE, D4 *__restrict__ cR,
                             double *__restrict__ tbc, int *__restrict__ tb_exp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  D4 ce{0.0, 0.0, 0.0, 0.0}, cr{0.0, 0.0, 0.0, 0.0};
  double tc = 0.0;
  if (mask[i] & P.groupbit) {
    const bool integ = !(P.flags & 0x08);
    const double dtfm = integ ? P.dtfm[type[i]] : 0.0;
    const int cell = S.cell[i];
    const double G = *ebp + (srcbar ? srcbar[cell] * src_scale : 0.0);
    const D4 V = vb[i], F = fb[i], v2 = S.v2[i];
    const double gdt = P.dt * G;
    const D4 fe = FRIC ? S.fE[i] : D4{0.0, 0.0, 0.0, 0.0};
    const D4 fr = RAND ? S.fR[i] : D4{0.0, 0.0, 0.0, 0.0};
    // dL/dv' in total: from the next step and from dE = -dt f.v'
    D4 vn = V;
    vn.x -= gdt * (fe.x + fr.x);
    vn.y -= gdt * (fe.y + fr.y);
    vn.z -= gdt * (fe.z + fr.z);
    // dL/df of the force the engine integrates (v' = v + dtf/m f)
    const double tx = F.x + dtfm * vn.x, ty = F.y + dtfm * vn.y, tz = F.z + dtfm * vn.z;
    const bool live = S.A[i].x > 0.0;
    if (FRIC) {
      const bool applied = !(P.flags & 0x10);
      const double ax = (applied ? tx : 0.0) - gdt * v2.x, ay = (applied ? ty : 0.0) - gdt * v2.y,
                   az = (applied ? tz : 0.0) - gdt * v2.z;
      if (live) ce = D4{-ax, -ay, -az, 0.0};
    }
    if (RAND) {
      const bool applied = !(P.flags & 0x20);
      const double bx = (applied ? tx : 0.0) - gdt * v2.x, by = (applied ? ty : 0.0) - gdt * v2.y,
                   bz = (applied ? tz : 0.0) - gdt * v2.z;
      const double Te = S.Te[i];
      if (live && Te > 0.0) {
        const double s = P.eta * sqrt(Te);
        cr = D4{s * bx, s * by, s * bz, 0.0};
        // f_RNG = eta sqrt(T) F[xi]: d f_RNG / dT = f_RNG / (2 T)
        tc = (bx * fr.x + by * fr.y + bz * fr.z) / (2.0 * Te);
      }
    }
    vb[i] = vn;
  }
  cE[i] = ce;
  cR[i] = cr;
  tbc[i] = tc;
  // largest binary exponent of the step's contributions (integer max: order-free)
  const int ex = (int)((__double_as_longlong(tc) >> 52) & 0x7ff);
  if (ex) atomicMax(tb_exp, ex);
}

// The contributions to the grid's cotangent, summed per cell exactly: each
// becomes a 128-bit fixed-point integer on a scale that puts the step's
// largest at about 2^40 (2^-104 of it resolved) and integer adds do not depend
// on the order, so the backward pass is reproducible bit for bit.
__global__ void k_adj_tb_fixed(int n, const double *__restrict__ tbc, const int *__restrict__ cell,
                               const int *__restrict__ tb_exp, U128 *__restrict__ acc, unsigned *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = *tb_exp;
  if (i >= n || e == 0) return;
  const double c = tbc[i];
  if (c == 0.0) return;
  const U128 q = to_fixed(scalbn(c, 40 - (e - 1023)), err);
  atomic_add128(acc + cell[i], q);
}

__global__ void k_adj_tb_apply(long nc, const int *__restrict__ tb_exp, U128 *__restrict__ acc,
                               double *__restrict__ Tb) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int e = *tb_exp;
  if (r >= nc || e == 0) return;
  const U128 q = acc[r];
  if (q.lo | q.hi) Tb[r] += scalbn(from_fixed(q), (e - 1023) - 40);
  acc[r] = U128{0ull, 0ull};
}

// Pair sweep 1: U_i = sum_j H_ij (e.(cE_i - cE_j)) e and V_i (same with cR)
// over neighbours whose forces the forward computed (rho_j > 0).  Then
//   dL/dw_i     = a_i U_i
//   dL/da_i     = 2 w_i.U_i + xi_i.V_i
//   dL/drho_i   = dL/da_i (alpha'(rho_i) - a_i) / rho_i
// and the alpha-table coefficient gradient dL/da_i / rho_i (1, rho, rho^2, rho^3)
// (AMODE 0: added to this block's own partial row, summed once per pass).
// adjW = {dL/dw_i, dL/drho_i}.
template <bool FAST, int AMODE>
__global__ void __launch_bounds__(ABLOCK)
    k_adj_sweep1(StepParams P, Slot S, const int *__restrict__ mask, const D4 *__restrict__ cE,
                 const D4 *__restrict__ cR, D4 *__restrict__ adjW, double *__restrict__ gpart,
                 double *__restrict__ gglob, int nt4) {
  extern __shared__ double s_w[];  // AMODE 0: [warps][nt4]
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (AMODE == 0) {
    for (int q = t; q < (int)(blockDim.x >> 5) * nt4; q += blockDim.x) s_w[q] = 0.0;
    __syncthreads();
  }
  const int i = blockIdx.x * blockDim.x + t;
  const bool valid = i < P.n;
  D4 Ai{0.0, 0.0, 0.0, 0.0};
  bool act = false;
  if (valid) {
    Ai = S.A[i];
    act = (mask[i] & P.groupbit) && Ai.x > 0.0;
  }
  double Ux = 0.0, Uy = 0.0, Uz = 0.0, Vx = 0.0, Vy = 0.0, Vz = 0.0;
  D4 xi{0.0, 0.0, 0.0, 0.0};
  if (act) {
    xi = S.x1[i];
    const D4 ce = cE[i], cr = cR[i];
    const int ns = S.ns[i];
    for (int k = 0; k < ns; ++k) {
      const unsigned u = S.pj[(size_t)k * P.n + i];
      const unsigned j = u & IDX_MASK;
      const D4 Aj = S.A[j];
      if (!(Aj.x > 0.0)) continue;
      const D4 xj = S.x1[j];
      double ex, ey, ez;
      pair_vector(P, xi, xj, u >> IDX_BITS, ex, ey, ez);
      const double r2 = dotf(ex, ey, ez, ex, ey, ez);
      double g, gd;
      int idx;
      spline_vd(P.tab_rho_r_sq + (size_t)(int)xj.w * P.n_rho, P.inv_dr_sq, P.n_rho, r2, g, gd, idx);
      const double H = g * recip_nr(r2);
      const D4 cej = cE[j], crj = cR[j];
      const double dE = H * dotf(ex, ey, ez, ce.x - cej.x, ce.y - cej.y, ce.z - cej.z);
      const double dR = H * dotf(ex, ey, ez, cr.x - crj.x, cr.y - crj.y, cr.z - crj.z);
      Ux = fma(dE, ex, Ux);
      Uy = fma(dE, ey, Uy);
      Uz = fma(dE, ez, Uz);
      Vx = fma(dR, ex, Vx);
      Vy = fma(dR, ey, Vy);
      Vz = fma(dR, ez, Vz);
    }
  }
  D4 out{0.0, 0.0, 0.0, 0.0};
  int key = -1;
  double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
  if (act) {
    const D4 Bi = S.Bw[i];
    const double rho = Ai.x;
    const double a = FAST ? Ai.y : Ai.y / rho;
    const double ab = fma(2.0, dotf(Bi.y, Bi.z, Bi.w, Ux, Uy, Uz), dotf(Ai.z, Ai.w, Bi.x, Vx, Vy, Vz));
    out.x = a * Ux;
    out.y = a * Uy;
    out.z = a * Uz;
    if (rho <= P.rho_cutoff) {  // above it alpha is the constant 0 (eph_beta.h:174-197)
      const int ei = (int)xi.w;
      double al, ald;
      int idx;
      spline_vd(P.tab_alpha + (size_t)ei * P.n_beta, P.inv_drho, P.n_beta, rho, al, ald, idx);
      const double q = ab / rho;
      out.w = q * (ald - a);
      key = ei * P.n_beta + idx;
      c0 = q;
      c1 = q * rho;
      c2 = c1 * rho;
      c3 = c2 * rho;
    }
  }
  if (valid) adjW[i] = out;
  if (AMODE == 0) {
    warp_add4(s_w + warp * nt4, key, c0, c1, c2, c3, lane);
    __syncthreads();
    for (int q = t; q < nt4; q += blockDim.x) {
      double sum = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += s_w[w * nt4 + q];
      gpart[(size_t)blockIdx.x * nt4 + q] += sum;
    }
  } else if (key >= 0) {
    atomicAdd(gglob + 4 * key + 0, c0);
    atomicAdd(gglob + 4 * key + 1, c1);
    atomicAdd(gglob + 4 * key + 2, c2);
    atomicAdd(gglob + 4 * key + 3, c3);
  }
}

// Pair sweep 2: for the unordered pair {i, j} the linearised pair terms are
//   Q = P_i B_i + P_j B_j,  P_i = a_i H_ij,  P_j = a_j H_ji,
//   B_i =  L [(e.w_i)(e.dcE) + (e.xi_i)(e.dcR)] + (e.dv)(e.om_i)
//   B_j = -L [(e.w_j)(e.dcE) + (e.xi_j)(e.dcR)] - (e.dv)(e.om_j)
// (dv = v_i - v_j, dcE = cE_i - cE_j, dcR = cR_i - cR_j, om = dL/dw, L = both
// atoms' forces computed).  Atom i gathers dQ/dx_i (through e, and through
// r^2 in H and in rho_i, rho_j), dQ/dv_i = F[om]_i, and for its ordered pairs
// the rho(r^2)-table coefficient gradient (a_i B_i / r^2 + dL/drho_i) (1, r^2,
// r^4, r^6); then the integrator in reverse: x = x0 + dt v, v = v0 + dtf/m f0.
// dQ/de at fixed H is P_i V_i - P_j V_j + dv (e.Od) + L [dcE (e.Wd) + dcR (e.Xd)]
// with V_a = (e.dv) om_a + L [(e.dcE) w_a + (e.dcR) xi_a] and Od, Wd, Xd the
// P-weighted differences of om, w, xi.
template <bool FAST, bool MULTI, int RMODE>
__global__ void __launch_bounds__(ABLOCK)
    k_adj_sweep2(StepParams P, Slot S, const int *__restrict__ mask, const int *__restrict__ type,
                 const D4 *__restrict__ cE, const D4 *__restrict__ cR, const D4 *__restrict__ adjW,
                 D4 *__restrict__ xb, D4 *__restrict__ vb, D4 *__restrict__ fb, double *__restrict__ gpart,
                 double *__restrict__ gglob, int nt4) {
  extern __shared__ double s_p[];  // RMODE 0: [nt4][blockDim]
  const int t = threadIdx.x, nt = blockDim.x;
  if (RMODE == 0)
    for (int q = 0; q < nt4; ++q) s_p[q * nt + t] = 0.0;
  const int i = blockIdx.x * blockDim.x + t;
  const bool grp = i < P.n && (mask[i] & P.groupbit);
  if (grp) {
    const D4 xi = S.x1[i], vi = S.v1[i], Ai = S.A[i], Bi = S.Bw[i], cei = cE[i], cri = cR[i], Wi = adjW[i];
    const bool live_i = Ai.x > 0.0;
    const double ai = live_i ? (FAST ? Ai.y : Ai.y / Ai.x) : 0.0;
    const int ei = (int)xi.w;
    double gxx = 0.0, gxy = 0.0, gxz = 0.0, gvx = 0.0, gvy = 0.0, gvz = 0.0;
    const int ns = S.ns[i];
    for (int k = 0; k < ns; ++k) {
      const unsigned u = S.pj[(size_t)k * P.n + i];
      const unsigned j = u & IDX_MASK;
      const D4 xj = S.x1[j];
      double ex, ey, ez;
      pair_vector(P, xi, xj, u >> IDX_BITS, ex, ey, ez);
      const double r2 = dotf(ex, ey, ez, ex, ey, ez);
      const double rinv = recip_nr(r2);
      const int ej = (int)xj.w;
      double gj, gjd;
      int idx;
      spline_vd(P.tab_rho_r_sq + (size_t)ej * P.n_rho, P.inv_dr_sq, P.n_rho, r2, gj, gjd, idx);
      const double Hij = gj * rinv, Hpij = (gjd - Hij) * rinv;
      double gid = gjd, Hji = Hij, Hpji = Hpij;
      if (MULTI && ej != ei) {
        double gi;
        int idx2;
        spline_vd(P.tab_rho_r_sq + (size_t)ei * P.n_rho, P.inv_dr_sq, P.n_rho, r2, gi, gid, idx2);
        Hji = gi * rinv;
        Hpji = (gid - Hji) * rinv;
      }
      const D4 Aj = S.A[j], Wj = adjW[j], vj = S.v1[j];
      const bool live_j = Aj.x > 0.0;
      const double aj = live_j ? (FAST ? Aj.y : Aj.y / Aj.x) : 0.0;
      const double dvx = vi.x - vj.x, dvy = vi.y - vj.y, dvz = vi.z - vj.z;
      const double e_dv = dotf(ex, ey, ez, dvx, dvy, dvz);
      const double Pi = ai * Hij, Pj = aj * Hji;
      const double eoi = dotf(ex, ey, ez, Wi.x, Wi.y, Wi.z), eoj = dotf(ex, ey, ez, Wj.x, Wj.y, Wj.z);
      const double eOd = fma(Pi, eoi, -Pj * eoj);
      double Bi_ = e_dv * eoi, Bj_ = -e_dv * eoj;
      double Vix = e_dv * Wi.x, Viy = e_dv * Wi.y, Viz = e_dv * Wi.z;
      double Vjx = e_dv * Wj.x, Vjy = e_dv * Wj.y, Vjz = e_dv * Wj.z;
      double gx = dvx * eOd, gy = dvy * eOd, gz = dvz * eOd;
      if (live_i && live_j) {
        const D4 Bj = S.Bw[j], cej = cE[j], crj = cR[j];
        const double dEx = cei.x - cej.x, dEy = cei.y - cej.y, dEz = cei.z - cej.z;
        const double dRx = cri.x - crj.x, dRy = cri.y - crj.y, dRz = cri.z - crj.z;
        const double e_dE = dotf(ex, ey, ez, dEx, dEy, dEz), e_dR = dotf(ex, ey, ez, dRx, dRy, dRz);
        const double ewi = dotf(ex, ey, ez, Bi.y, Bi.z, Bi.w), ewj = dotf(ex, ey, ez, Bj.y, Bj.z, Bj.w);
        const double exi = dotf(ex, ey, ez, Ai.z, Ai.w, Bi.x), exj = dotf(ex, ey, ez, Aj.z, Aj.w, Bj.x);
        Bi_ = fma(ewi, e_dE, fma(exi, e_dR, Bi_));
        Bj_ = Bj_ - fma(ewj, e_dE, exj * e_dR);
        Vix = fma(e_dE, Bi.y, fma(e_dR, Ai.z, Vix));
        Viy = fma(e_dE, Bi.z, fma(e_dR, Ai.w, Viy));
        Viz = fma(e_dE, Bi.w, fma(e_dR, Bi.x, Viz));
        Vjx = fma(e_dE, Bj.y, fma(e_dR, Aj.z, Vjx));
        Vjy = fma(e_dE, Bj.z, fma(e_dR, Aj.w, Vjy));
        Vjz = fma(e_dE, Bj.w, fma(e_dR, Bj.x, Vjz));
        const double eWd = fma(Pi, ewi, -Pj * ewj), eXd = fma(Pi, exi, -Pj * exj);
        gx = fma(dEx, eWd, fma(dRx, eXd, gx));
        gy = fma(dEy, eWd, fma(dRy, eXd, gy));
        gz = fma(dEz, eWd, fma(dRz, eXd, gz));
      }
      gx = fma(Pi, Vix, fma(-Pj, Vjx, gx));
      gy = fma(Pi, Viy, fma(-Pj, Vjy, gy));
      gz = fma(Pi, Viz, fma(-Pj, Vjz, gz));
      const double aBi = ai * Bi_;
      const double s2 = 2.0 * fma(aBi, Hpij, fma(aj * Bj_, Hpji, fma(Wi.w, gjd, Wj.w * gid)));
      gxx -= fma(s2, ex, gx);  // e = x_j - x_i
      gxy -= fma(s2, ey, gy);
      gxz -= fma(s2, ez, gz);
      gvx = fma(ex, eOd, gvx);
      gvy = fma(ey, eOd, gvy);
      gvz = fma(ez, eOd, gvz);
      const double cS = fma(aBi, rinv, Wi.w);
      const int slot = 4 * (ej * P.n_rho + idx);
      const double c2 = cS * r2, c4 = c2 * r2;
      if (RMODE == 0) {
        s_p[(slot + 0) * nt + t] += cS;
        s_p[(slot + 1) * nt + t] += c2;
        s_p[(slot + 2) * nt + t] += c4;
        s_p[(slot + 3) * nt + t] = fma(c4, r2, s_p[(slot + 3) * nt + t]);
      } else {
        atomicAdd(gglob + slot + 0, cS);
        atomicAdd(gglob + slot + 1, c2);
        atomicAdd(gglob + slot + 2, c4);
        atomicAdd(gglob + slot + 3, c4 * r2);
      }
    }
    const bool integ = !(P.flags & 0x08);
    const D4 X = xb[i], V = vb[i];
    const double xbx = X.x + gxx, xby = X.y + gxy, xbz = X.z + gxz;
    double vbx = V.x + gvx, vby = V.y + gvy, vbz = V.z + gvz;
    if (integ) {
      vbx = fma(P.dtv, xbx, vbx);
      vby = fma(P.dtv, xby, vby);
      vbz = fma(P.dtv, xbz, vbz);
    }
    const double dtfm = integ ? P.dtfm[type[i]] : 0.0;
    xb[i] = D4{xbx, xby, xbz, 0.0};
    vb[i] = D4{vbx, vby, vbz, 0.0};
    fb[i] = D4{dtfm * vbx, dtfm * vby, dtfm * vbz, 0.0};
  }
  if (RMODE == 0) {
    __syncthreads();
    for (int q = t; q < nt4; q += nt) {
      double sum = 0.0;
      for (int tt = 0; tt < nt; ++tt) sum += s_p[q * nt + tt];
      gpart[(size_t)blockIdx.x * nt4 + q] += sum;
    }
  }
}

// ------------------------------------------------ reverse sweeps in df64
// The same two sweeps with every per-pair operation in df64 on the FP32 pipe
// (the FP64 versions above are bound by FP64 issue): per step, k_adj_split
// turns each atom's FP64 records into double-float records that the pair
// loops gather (12 float4 per atom, rows R_*), the pair terms and their sums
// are formed in df64, and the per-atom work stays FP64.  Positions are split
// as they are (the boxes of the adjoint's workloads are < 100 A, so the lo
// parts carry them to ~1e-13 A); the spline is the forward's local-form df64
// table (value and derivative from the same interval, whose knot receives the
// coefficient gradient).  Results agree with the FP64 sweeps to ~1e-12.
constexpr int R_X = 0, R_V = 2, R_WX = 4, R_C = 7, R_W = 10, R_N = 12;

// rows R_X (x, a_i = alpha_i / rho_i or 0), R_V (v, element, live flag),
// R_WX (w, xi), R_C (cotangents cE, cR) of atom i
template <bool FAST>
__global__ void k_adj_split(int n, Slot S, const D4 *__restrict__ cE, const D4 *__restrict__ cR,
                            float4 *__restrict__ rec) {
  using namespace df64;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const D4 x = S.x1[i], v = S.v1[i], A = S.A[i], B = S.Bw[i], ce = cE[i], cr = cR[i];
  const bool live = A.x > 0.0;
  const df a = from_double(live ? (FAST ? A.y : A.y / A.x) : 0.0);
  float4 *r = rec + (size_t)R_N * i;
  const df x0 = from_double(x.x), x1 = from_double(x.y), x2 = from_double(x.z);
  r[R_X] = make_float4(x0.hi, x1.hi, x2.hi, a.hi);
  r[R_X + 1] = make_float4(x0.lo, x1.lo, x2.lo, a.lo);
  const df v0 = from_double(v.x), v1 = from_double(v.y), v2 = from_double(v.z);
  r[R_V] = make_float4(v0.hi, v1.hi, v2.hi, __int_as_float((int)x.w));
  r[R_V + 1] = make_float4(v0.lo, v1.lo, v2.lo, live ? 1.0f : 0.0f);
  const df w0 = from_double(B.y), w1 = from_double(B.z), w2 = from_double(B.w);
  const df q0 = from_double(A.z), q1 = from_double(A.w), q2 = from_double(B.x);
  r[R_WX] = make_float4(w0.hi, w1.hi, w2.hi, q0.hi);
  r[R_WX + 1] = make_float4(w0.lo, w1.lo, w2.lo, q0.lo);
  r[R_WX + 2] = make_float4(q1.hi, q2.hi, q1.lo, q2.lo);
  const df e0 = from_double(ce.x), e1 = from_double(ce.y), e2 = from_double(ce.z);
  const df c0 = from_double(cr.x), c1 = from_double(cr.y), c2 = from_double(cr.z);
  r[R_C] = make_float4(e0.hi, e1.hi, e2.hi, c0.hi);
  r[R_C + 1] = make_float4(e0.lo, e1.lo, e2.lo, c0.lo);
  r[R_C + 2] = make_float4(c1.hi, c2.hi, c1.lo, c2.lo);
}

struct df3 {
  df64::df x, y, z;
};
__device__ __forceinline__ df3 df3_of(float4 hi, float4 lo) {
  return df3{df64::df{hi.x, lo.x}, df64::df{hi.y, lo.y}, df64::df{hi.z, lo.z}};
}
// the third-row layout {a.hi, b.hi, a.lo, b.lo} with the first component in .w
__device__ __forceinline__ df3 df3_split(float4 hi, float4 lo, float4 rest) {
  return df3{df64::df{hi.w, lo.w}, df64::df{rest.x, rest.z}, df64::df{rest.y, rest.w}};
}
__device__ __forceinline__ df64::df ddot(const df3 &a, const df3 &b) {
  return df64::dot3(a.x, a.y, a.z, b.x, b.y, b.z);
}
__device__ __forceinline__ df3 dsub(const df3 &a, const df3 &b) {
  return df3{df64::sub(a.x, b.x), df64::sub(a.y, b.y), df64::sub(a.z, b.z)};
}
__device__ __forceinline__ df3 dscale(df64::df s, const df3 &a) {
  return df3{df64::mul(s, a.x), df64::mul(s, a.y), df64::mul(s, a.z)};
}
__device__ __forceinline__ df3 daxpy(df64::df s, const df3 &a, const df3 &y) {  // s a + y
  return df3{df64::fma(s, a.x, y.x), df64::fma(s, a.y, y.y), df64::fma(s, a.z, y.z)};
}
// (x_j + image of code) - x_i from df64 positions
__device__ __forceinline__ df3 adj_disp(const StepParams &P, float4 jh, float4 jl, float4 ih, float4 il,
                                        unsigned code) {
  const int mx = (int)(code % 3u) - 1, my = (int)((code / 3u) % 3u) - 1, mz = (int)(code / 9u) - 1;
  return df3{pair_disp(mx, jh.x, jl.x, ih.x, il.x, P.prd_hi[0], P.prd_lo[0]),
             pair_disp(my, jh.y, jl.y, ih.y, il.y, P.prd_hi[1], P.prd_lo[1]),
             pair_disp(mz, jh.z, jl.z, ih.z, il.z, P.prd_hi[2], P.prd_lo[2])};
}

// k_adj_sweep1 with the pair loop in df64 (rows R_X, R_V, R_C of k_adj_split);
// also writes the df64 row R_W of its result for k_adj_sweep2_df
template <bool FAST, int AMODE>
__global__ void __launch_bounds__(ABLOCK)
    k_adj_sweep1_df(StepParams P, Slot S, const int *__restrict__ mask, float4 *__restrict__ rec,
                    D4 *__restrict__ adjW, double *__restrict__ gpart, double *__restrict__ gglob, int nt4,
                    unsigned *__restrict__ err) {
  using namespace df64;
  extern __shared__ double s_w[];  // AMODE 0: [warps][nt4]
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (AMODE == 0) {
    for (int q = t; q < (int)(blockDim.x >> 5) * nt4; q += blockDim.x) s_w[q] = 0.0;
    __syncthreads();
  }
  const int i = blockIdx.x * blockDim.x + t;
  const bool valid = i < P.n;
  D4 Ai{0.0, 0.0, 0.0, 0.0};
  bool act = false;
  if (valid) {
    Ai = S.A[i];
    act = (mask[i] & P.groupbit) && Ai.x > 0.0;
  }
  acc U[3] = {acc_zero(), acc_zero(), acc_zero()}, V[3] = {acc_zero(), acc_zero(), acc_zero()};
  D4 xi{0.0, 0.0, 0.0, 0.0};
  if (act) {
    xi = S.x1[i];
    const float4 *ri = rec + (size_t)R_N * i;
    const float4 ih = ri[R_X], il = ri[R_X + 1];
    const df3 cei = df3_of(ri[R_C], ri[R_C + 1]), cri = df3_split(ri[R_C], ri[R_C + 1], ri[R_C + 2]);
    const int ns = S.ns[i];
    for (int k = 0; k < ns; ++k) {
      const unsigned u = S.pj[(size_t)k * P.n + i];
      const unsigned j = u & IDX_MASK;
      const float4 *rj = rec + (size_t)R_N * j;
      const float4 vl = rj[R_V + 1];
      if (!(vl.w > 0.0f)) continue;  // rho_j <= 0
      const df3 e = adj_disp(P, rj[R_X], rj[R_X + 1], ih, il, u >> IDX_BITS);
      const df r2 = ddot(e, e);
      const df H = mul(spline_rho_df(P, __float_as_int(rj[R_V].w), r2, err), recip(r2, rcp_estimate(r2.hi)));
      const float4 ch = rj[R_C], cl = rj[R_C + 1];
      const df3 cej = df3_of(ch, cl), crj = df3_split(ch, cl, rj[R_C + 2]);
      const df dE = mul(H, ddot(e, dsub(cei, cej)));
      const df dR = mul(H, ddot(e, dsub(cri, crj)));
      acc_fma(U[0], dE, e.x);
      acc_fma(U[1], dE, e.y);
      acc_fma(U[2], dE, e.z);
      acc_fma(V[0], dR, e.x);
      acc_fma(V[1], dR, e.y);
      acc_fma(V[2], dR, e.z);
    }
  }
  const double Ux = to_double(acc_value(U[0])), Uy = to_double(acc_value(U[1])), Uz = to_double(acc_value(U[2]));
  const double Vx = to_double(acc_value(V[0])), Vy = to_double(acc_value(V[1])), Vz = to_double(acc_value(V[2]));
  D4 out{0.0, 0.0, 0.0, 0.0};
  int key = -1;
  double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
  if (act) {
    const D4 Bi = S.Bw[i];
    const double rho = Ai.x;
    const double a = FAST ? Ai.y : Ai.y / rho;
    const double ab = fma(2.0, dotf(Bi.y, Bi.z, Bi.w, Ux, Uy, Uz), dotf(Ai.z, Ai.w, Bi.x, Vx, Vy, Vz));
    out.x = a * Ux;
    out.y = a * Uy;
    out.z = a * Uz;
    if (rho <= P.rho_cutoff) {  // above it alpha is the constant 0 (eph_beta.h:174-197)
      const int ei = (int)xi.w;
      double al, ald;
      int idx;
      spline_vd(P.tab_alpha + (size_t)ei * P.n_beta, P.inv_drho, P.n_beta, rho, al, ald, idx);
      const double q = ab / rho;
      out.w = q * (ald - a);
      key = ei * P.n_beta + idx;
      c0 = q;
      c1 = q * rho;
      c2 = c1 * rho;
      c3 = c2 * rho;
    }
  }
  if (valid) {
    adjW[i] = out;
    const df o0 = from_double(out.x), o1 = from_double(out.y), o2 = from_double(out.z), o3 = from_double(out.w);
    rec[(size_t)R_N * i + R_W] = make_float4(o0.hi, o1.hi, o2.hi, o3.hi);
    rec[(size_t)R_N * i + R_W + 1] = make_float4(o0.lo, o1.lo, o2.lo, o3.lo);
  }
  if (AMODE == 0) {
    warp_add4(s_w + warp * nt4, key, c0, c1, c2, c3, lane);
    __syncthreads();
    for (int q = t; q < nt4; q += blockDim.x) {
      double sum = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += s_w[w * nt4 + q];
      gpart[(size_t)blockIdx.x * nt4 + q] += sum;
    }
  } else if (key >= 0) {
    atomicAdd(gglob + 4 * key + 0, c0);
    atomicAdd(gglob + 4 * key + 1, c1);
    atomicAdd(gglob + 4 * key + 2, c2);
    atomicAdd(gglob + 4 * key + 3, c3);
  }
}

// k_adj_sweep2 with the pair loop in df64 (the same terms, in the same
// grouping; rows of k_adj_split and R_W of k_adj_sweep1_df).  RMODE 0 keeps
// its per-thread coefficient accumulators as df64 pairs in shared memory.
template <bool FAST, bool MULTI, int RMODE>
__global__ void __launch_bounds__(ABLOCK)
    k_adj_sweep2_df(StepParams P, Slot S, const int *__restrict__ mask, const int *__restrict__ type,
                    const float4 *__restrict__ rec, D4 *__restrict__ xb, D4 *__restrict__ vb, D4 *__restrict__ fb,
                    double *__restrict__ gpart, double *__restrict__ gglob, int nt4) {
  using namespace df64;
  extern __shared__ double s_p[];  // RMODE 0: [nt4][blockDim] (hi, lo) pairs
  float2 *s_pf = reinterpret_cast<float2 *>(s_p);
  const int t = threadIdx.x, nt = blockDim.x;
  if (RMODE == 0)
    for (int q = 0; q < nt4; ++q) s_pf[q * nt + t] = make_float2(0.f, 0.f);
  const int i = blockIdx.x * blockDim.x + t;
  const bool grp = i < P.n && (mask[i] & P.groupbit);
  if (grp) {
    const float4 *ri = rec + (size_t)R_N * i;
    const float4 ih = ri[R_X], il = ri[R_X + 1], vh = ri[R_V], vl = ri[R_V + 1];
    const bool live_i = vl.w > 0.0f;
    const df ai{ih.w, il.w};
    const int ei = __float_as_int(vh.w);
    const df3 vi = df3_of(vh, vl);
    const float4 wxh = ri[R_WX], wxl = ri[R_WX + 1];
    const df3 wi = df3_of(wxh, wxl), xii = df3_split(wxh, wxl, ri[R_WX + 2]);
    const float4 ch = ri[R_C], cl = ri[R_C + 1];
    const df3 cei = df3_of(ch, cl), cri = df3_split(ch, cl, ri[R_C + 2]);
    const float4 Oh = ri[R_W], Ol = ri[R_W + 1];
    const df3 Wi = df3_of(Oh, Ol);
    const df Wwi{Oh.w, Ol.w};
    acc gx[3] = {acc_zero(), acc_zero(), acc_zero()}, gv[3] = {acc_zero(), acc_zero(), acc_zero()};
    const int ns = S.ns[i];
    for (int k = 0; k < ns; ++k) {
      const unsigned u = S.pj[(size_t)k * P.n + i];
      const unsigned j = u & IDX_MASK;
      const float4 *rj = rec + (size_t)R_N * j;
      const float4 jxh = rj[R_X], jxl = rj[R_X + 1], jvh = rj[R_V], jvl = rj[R_V + 1];
      const df3 e = adj_disp(P, jxh, jxl, ih, il, u >> IDX_BITS);
      const df r2 = ddot(e, e);
      const df rinv = recip(r2, rcp_estimate(r2.hi));
      const int ej = __float_as_int(jvh.w);
      df gj, gjd;
      int idx;
      spline_rho_df_vd(P, ej, r2, gj, gjd, idx);
      const df Hij = mul(gj, rinv), Hpij = mul(sub(gjd, Hij), rinv);
      df gid = gjd, Hji = Hij, Hpji = Hpij;
      if (MULTI && ej != ei) {
        df gi;
        int idx2;
        spline_rho_df_vd(P, ei, r2, gi, gid, idx2);
        Hji = mul(gi, rinv);
        Hpji = mul(sub(gid, Hji), rinv);
      }
      const bool live_j = jvl.w > 0.0f;
      const df aj{jxh.w, jxl.w};
      const float4 jOh = rj[R_W], jOl = rj[R_W + 1];
      const df3 Wj = df3_of(jOh, jOl);
      const df Wwj{jOh.w, jOl.w};
      const df3 dv = dsub(vi, df3_of(jvh, jvl));
      const df e_dv = ddot(e, dv);
      const df Pi = mul(ai, Hij), Pj = mul(aj, Hji);
      const df eoi = ddot(e, Wi), eoj = ddot(e, Wj);
      const df eOd = sub(mul(Pi, eoi), mul(Pj, eoj));
      df Bi_ = mul(e_dv, eoi), Bj_ = neg(mul(e_dv, eoj));
      df3 Vi = dscale(e_dv, Wi), Vj = dscale(e_dv, Wj);
      df3 g = dscale(eOd, dv);
      if (live_i && live_j) {
        const float4 jwh = rj[R_WX], jwl = rj[R_WX + 1], jch = rj[R_C], jcl = rj[R_C + 1];
        const df3 wj = df3_of(jwh, jwl), xij = df3_split(jwh, jwl, rj[R_WX + 2]);
        const df3 dE = dsub(cei, df3_of(jch, jcl)), dR = dsub(cri, df3_split(jch, jcl, rj[R_C + 2]));
        const df e_dE = ddot(e, dE), e_dR = ddot(e, dR);
        const df ewi = ddot(e, wi), ewj = ddot(e, wj), exi = ddot(e, xii), exj = ddot(e, xij);
        Bi_ = add(Bi_, add(mul(ewi, e_dE), mul(exi, e_dR)));
        Bj_ = sub(Bj_, add(mul(ewj, e_dE), mul(exj, e_dR)));
        Vi = daxpy(e_dE, wi, daxpy(e_dR, xii, Vi));
        Vj = daxpy(e_dE, wj, daxpy(e_dR, xij, Vj));
        const df eWd = sub(mul(Pi, ewi), mul(Pj, ewj)), eXd = sub(mul(Pi, exi), mul(Pj, exj));
        g = daxpy(eWd, dE, daxpy(eXd, dR, g));
      }
      g = daxpy(Pi, Vi, daxpy(neg(Pj), Vj, g));
      const df aBi = mul(ai, Bi_);
      const df s2h = add(add(mul(aBi, Hpij), mul(mul(aj, Bj_), Hpji)), add(mul(Wwi, gjd), mul(Wwj, gid)));
      const df s2 = add(s2h, s2h);
      // x cotangent: -(s2 e + g) summed (e = x_j - x_i); v cotangent: e (e.Od)
      const df3 gs = daxpy(s2, e, g);
      acc_add(gx[0], gs.x);
      acc_add(gx[1], gs.y);
      acc_add(gx[2], gs.z);
      acc_fma(gv[0], e.x, eOd);
      acc_fma(gv[1], e.y, eOd);
      acc_fma(gv[2], e.z, eOd);
      const df cS = fma(aBi, rinv, Wwi);
      const int slot = 4 * (ej * P.n_rho + idx);
      const df c2 = mul(cS, r2), c4 = mul(c2, r2), c6 = mul(c4, r2);
      if (RMODE == 0) {
        const df cs[4] = {cS, c2, c4, c6};
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          float2 &cell = s_pf[(slot + m) * nt + t];
          const df sum = add(df{cell.x, cell.y}, cs[m]);
          cell = make_float2(sum.hi, sum.lo);
        }
      } else {
        atomicAdd(gglob + slot + 0, to_double(cS));
        atomicAdd(gglob + slot + 1, to_double(c2));
        atomicAdd(gglob + slot + 2, to_double(c4));
        atomicAdd(gglob + slot + 3, to_double(c6));
      }
    }
    const double gxx = -to_double(acc_value(gx[0])), gxy = -to_double(acc_value(gx[1])),
                 gxz = -to_double(acc_value(gx[2]));
    const double gvx = to_double(acc_value(gv[0])), gvy = to_double(acc_value(gv[1])),
                 gvz = to_double(acc_value(gv[2]));
    const bool integ = !(P.flags & 0x08);
    const D4 X = xb[i], V = vb[i];
    const double xbx = X.x + gxx, xby = X.y + gxy, xbz = X.z + gxz;
    double vbx = V.x + gvx, vby = V.y + gvy, vbz = V.z + gvz;
    if (integ) {
      vbx = fma(P.dtv, xbx, vbx);
      vby = fma(P.dtv, xby, vby);
      vbz = fma(P.dtv, xbz, vbz);
    }
    const double dtfm = integ ? P.dtfm[type[i]] : 0.0;
    xb[i] = D4{xbx, xby, xbz, 0.0};
    vb[i] = D4{vbx, vby, vbz, 0.0};
    fb[i] = D4{dtfm * vbx, dtfm * vby, dtfm * vbz, 0.0};
  }
  if (RMODE == 0) {
    __syncthreads();
    for (int q = t; q < nt4; q += nt) {
      double sum = 0.0;
      for (int tt = 0; tt < nt; ++tt) {
        const float2 cell = s_pf[q * nt + tt];
        sum += to_double(df64::df{cell.x, cell.y});
      }
      gpart[(size_t)blockIdx.x * nt4 + q] += sum;
    }
  }
}

// sum of the blocks' partial rows, in block order
__global__ void k_adj_reduce(const double *__restrict__ gpart, int nparts, int nt4, double *__restrict__ acc) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nt4) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += gpart[(size_t)b * nt4 + q];
  acc[q] += s;
}

}  // namespace

// =================================================================== driver

struct eph_adjoint {
  std::string err;
  eph_ctx *c = nullptr;
  int K = 20;
  int n = 0, kcap = 0;
  long nc = 0;
  unsigned nsub = 0;
  bool fric = false, rand = false, fdm = false;
  // start of every trajectory
  DevBuf<D4> s_x, s_v, s_f, s_xh;
  DevBuf<double> s_T;
  DevBuf<unsigned long long> s_step;
  // checkpoints, one per segment of K steps
  long nck = 0;
  DevBuf<D4> k_x, k_v, k_f, k_xh;
  DevBuf<double> k_T;
  DevBuf<unsigned long long> k_step;
  // K recorded steps
  DevBuf<D4> r_x1, r_v1, r_v2, r_A, r_Bw, r_fE, r_fR;
  DevBuf<int> r_cell, r_ns;
  DevBuf<double> r_Te, r_T0, r_src, r_Tsub;
  DevBuf<unsigned> r_pj;
  unsigned r_nsub = 0;
  // trajectory
  long nsteps = 0;
  DevBuf<double> d_E, d_Tm;
  // adjoint state and work arrays
  DevBuf<D4> xb, vb, fb, cE, cR, W;
  DevBuf<float4> dfr;  // df64 rows of the reverse sweeps (R_N per atom), the pair arithmetic is df64
  DevBuf<double> Tb, u0, u1, srcbar, gC, gK, rho_e;
  DevBuf<double> fdmW;  // [7][ncells]: transposed substep stencil, see k_adj_fdm_weights
  DevBuf<double> g_rho, g_alpha, part_rho, part_alpha;
  DevBuf<double> tbc;     // per atom: contribution to the grid's cotangent
  DevBuf<U128> tb_acc;    // per cell: its exact sum
  DevBuf<int> tb_exp;     // per step: the largest exponent among the contributions
  DevBuf<unsigned> d_err;
  int nt4_rho = 0, nt4_alpha = 0, amode = 0, rmode = 0;
  // gradients
  bool have_grad = false;
  std::vector<std::vector<double>> grad_rho, grad_beta;
  double grad_C = 0.0, grad_K = 0.0;
  // timing
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double fwd_ms = 0.0, bwd_ms = 0.0;
  long fwd_launches = 0, bwd_launches = 0, launches = 0;
  // cotangents of the backward pass on the device (the reverse kernels read
  // them, so one captured pass serves every loss) and their pinned staging
  DevBuf<double> d_eb, d_tau;
  double *h_cot = nullptr;
  long h_cot_n = 0;
  unsigned long long own_gen = 0;  // bumped when the adjoint reallocates
  // each pass is captured once as a CUDA graph and replayed while its shape,
  // the step constants and every buffer address stay the same
  struct Shape {
    long nsteps = -1;
    unsigned nsub = 0;
    unsigned long long ctx_gen = 0, own_gen = 0;
    StepParams P{};
    double inner_dt = 0.0;
    bool fext = false;
  };
  bool use_graph = true;
  // passes: 0 forward (records the last segment as it goes), 1 backward that
  // recomputes every segment, 2 backward that finds the last segment recorded
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
  Shape shape[3];
  long graph_launches[3] = {0, 0, 0};
  bool last_recorded = false;  // the record slots hold the last segment of the trajectory
};

namespace {

int afail(eph_adjoint *a, int code, const std::string &msg) {
  if (a) a->err = msg;
  return code;
}

#define ADJ_TRY(a, call)                                                                                     \
  do {                                                                                                       \
    cudaError_t e_ = (call);                                                                                 \
    if (e_ != cudaSuccess) return afail((a), EPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// a context call failed: carry its message over
int from_ctx(eph_adjoint *a, int r) {
  if (r) a->err = a->c->err;
  return r;
}

template <typename T>
cudaError_t d2d(T *dst, const T *src, size_t count, cudaStream_t s) {
  return cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyDeviceToDevice, s);
}

int save_state(eph_adjoint *a, D4 *x, D4 *v, D4 *f, D4 *xh, double *T, unsigned long long *step) {
  eph_ctx *c = a->c;
  const size_t N = (size_t)a->n;
  ADJ_TRY(a, d2d(x, c->x.p, N, c->stream));
  ADJ_TRY(a, d2d(v, c->v.p, N, c->stream));
  ADJ_TRY(a, d2d(f, c->f.p, N, c->stream));
  ADJ_TRY(a, d2d(xh, c->xhold.p, N, c->stream));
  ADJ_TRY(a, d2d(T, c->T0.p, (size_t)a->nc, c->stream));
  ADJ_TRY(a, d2d(step, c->step_ctr.p, 1, c->stream));
  return EPH_OK;
}

int load_state(eph_adjoint *a, const D4 *x, const D4 *v, const D4 *f, const D4 *xh, const double *T,
               const unsigned long long *step) {
  eph_ctx *c = a->c;
  const size_t N = (size_t)a->n;
  ADJ_TRY(a, d2d(c->x.p, x, N, c->stream));
  ADJ_TRY(a, d2d(c->v.p, v, N, c->stream));
  ADJ_TRY(a, d2d(c->f.p, f, N, c->stream));
  ADJ_TRY(a, d2d(c->xhold.p, xh, N, c->stream));
  ADJ_TRY(a, d2d(c->T0.p, T, (size_t)a->nc, c->stream));
  ADJ_TRY(a, d2d(c->step_ctr.p, step, 1, c->stream));
  ADJ_TRY(a, cudaMemsetAsync(c->wrapflag.p, 0, sizeof(int), c->stream));
  ADJ_TRY(a, cudaMemsetAsync(c->acc.p, 0, sizeof(U128) * (size_t)a->nc, c->stream));
  return EPH_OK;
}

// the plain engine step (the sequence of eph_step), optionally recording slot s
int run_step(eph_adjoint *a, int s) {
  eph_ctx *c = a->c;
  const size_t N = (size_t)a->n;
  const long before = c->launches;
  int r;
  if ((r = ctxi::launch_initial(c, 1))) return from_ctx(a, r);
  if (c->have_fext)
    ADJ_TRY(a, d2d(c->f.p, c->fext.p, N, c->stream));
  else
    ADJ_TRY(a, cudaMemsetAsync(c->f.p, 0, sizeof(D4) * N, c->stream));
  if ((r = ctxi::launch_post_force(c, 0))) return from_ctx(a, r);
  if (s >= 0) {
    const size_t o = (size_t)s * N;
    ADJ_TRY(a, d2d(a->r_x1.p + o, c->x.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_v1.p + o, c->v.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_A.p + o, c->A.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_Bw.p + o, c->Bw.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_Te.p + o, c->Te_i.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_cell.p + o, c->cell.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_ns.p + o, c->nshort.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_pj.p + (size_t)s * a->kcap * N, c->pj.p, (size_t)a->kcap * N, c->stream));
    ADJ_TRY(a, d2d(a->r_T0.p + (size_t)s * a->nc, c->T0.p, (size_t)a->nc, c->stream));
  }
  if ((r = ctxi::launch_final(c))) return from_ctx(a, r);
  if (s >= 0) {
    const size_t o = (size_t)s * N;
    ADJ_TRY(a, d2d(a->r_v2.p + o, c->v.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_fE.p + o, c->f_eph.p, N, c->stream));
    ADJ_TRY(a, d2d(a->r_fR.p + o, c->f_rng.p, N, c->stream));
    if (a->fdm) c->fdm_rec = a->r_Tsub.p + (size_t)s * a->nsub * (size_t)a->nc;
  }
  r = ctxi::launch_end_of_step(c);
  c->fdm_rec = nullptr;
  if (r) return from_ctx(a, r);
  if (s >= 0 && a->fdm) ADJ_TRY(a, d2d(a->r_src.p + (size_t)s * a->nc, c->dT.p, (size_t)a->nc, c->stream));
  a->launches += c->launches - before;
  c->launches = before;
  return EPH_OK;
}

Slot slot_view(eph_adjoint *a, int s) {
  const size_t o = (size_t)s * (size_t)a->n;
  Slot S;
  S.x1 = a->r_x1.p + o;
  S.v1 = a->r_v1.p + o;
  S.v2 = a->r_v2.p + o;
  S.A = a->r_A.p + o;
  S.Bw = a->r_Bw.p + o;
  S.fE = a->r_fE.p + o;
  S.fR = a->r_fR.p + o;
  S.cell = a->r_cell.p + o;
  S.ns = a->r_ns.p + o;
  S.Te = a->r_Te.p + o;
  S.pj = a->r_pj.p + (size_t)s * a->kcap * (size_t)a->n;
  return S;
}

GridArgs grid_args(eph_adjoint *a) {
  const eph_ctx *c = a->c;
  const Grid &g = c->grid;
  GridArgs G;
  G.n[0] = g.nx;
  G.n[1] = g.ny;
  G.n[2] = g.nz;
  G.nc = a->nc;
  G.h[0] = g.dx;
  G.h[1] = g.dy;
  G.h[2] = g.dz;
  for (int k = 0; k < 3; ++k) G.ih2[k] = 1.0 / (G.h[k] * G.h[k]);
  G.inner_dt = c->inner_dt;
  G.kappa = c->kappa.p;
  G.rhoC = c->rhoC.p;
  G.irhoC = c->irhoC.p;
  G.rho_e = a->rho_e.p;
  G.S = c->S.p;
  G.flag = c->gflag.p;
  return G;
}

template <bool FAST>
void launch_sweeps_df(eph_adjoint *a, const Slot &S) {
  eph_ctx *c = a->c;
  const int nb = nb_of(a->n);
  k_adj_split<FAST><<<nb, ABLOCK, 0, c->stream>>>(a->n, S, a->cE.p, a->cR.p, a->dfr.p);
  const size_t sh1 = a->amode == 0 ? sizeof(double) * 4 * (size_t)a->nt4_alpha : 0;
  if (a->amode == 0)
    k_adj_sweep1_df<FAST, 0><<<nb, ABLOCK, sh1, c->stream>>>(c->P, S, c->mask.p, a->dfr.p, a->W.p, a->part_alpha.p,
                                                              a->g_alpha.p, a->nt4_alpha, a->d_err.p);
  else
    k_adj_sweep1_df<FAST, 1><<<nb, ABLOCK, 0, c->stream>>>(c->P, S, c->mask.p, a->dfr.p, a->W.p, a->part_alpha.p,
                                                            a->g_alpha.p, a->nt4_alpha, a->d_err.p);
  const size_t sh2 = a->rmode == 0 ? sizeof(double) * (size_t)a->nt4_rho * ABLOCK : 0;
#define ADJ_SWEEP2(M, R)                                                                                        \
  k_adj_sweep2_df<FAST, M, R><<<nb, ABLOCK, sh2, c->stream>>>(c->P, S, c->mask.p, c->type.p, a->dfr.p, a->xb.p, \
                                                              a->vb.p, a->fb.p, a->part_rho.p, a->g_rho.p,      \
                                                              a->nt4_rho)
  if (c->multi) {
    if (a->rmode == 0) ADJ_SWEEP2(true, 0);
    else ADJ_SWEEP2(true, 1);
  } else {
    if (a->rmode == 0) ADJ_SWEEP2(false, 0);
    else ADJ_SWEEP2(false, 1);
  }
#undef ADJ_SWEEP2
  a->launches += 3;
}

template <bool FAST>
void launch_sweeps(eph_adjoint *a, const Slot &S) {
  eph_ctx *c = a->c;
  if (c->pair_arith == EPH_PAIRS_DF64) {
    launch_sweeps_df<FAST>(a, S);
    return;
  }
  const int nb = nb_of(a->n);
  const size_t sh1 = a->amode == 0 ? sizeof(double) * 4 * (size_t)a->nt4_alpha : 0;
  if (a->amode == 0)
    k_adj_sweep1<FAST, 0><<<nb, ABLOCK, sh1, c->stream>>>(c->P, S, c->mask.p, a->cE.p, a->cR.p, a->W.p,
                                                           a->part_alpha.p, a->g_alpha.p, a->nt4_alpha);
  else
    k_adj_sweep1<FAST, 1><<<nb, ABLOCK, 0, c->stream>>>(c->P, S, c->mask.p, a->cE.p, a->cR.p, a->W.p,
                                                         a->part_alpha.p, a->g_alpha.p, a->nt4_alpha);
  a->launches += 1;
  const size_t sh2 = a->rmode == 0 ? sizeof(double) * (size_t)a->nt4_rho * ABLOCK : 0;
#define ADJ_SWEEP2(M, R)                                                                                    \
  k_adj_sweep2<FAST, M, R><<<nb, ABLOCK, sh2, c->stream>>>(c->P, S, c->mask.p, c->type.p, a->cE.p, a->cR.p, \
                                                           a->W.p, a->xb.p, a->vb.p, a->fb.p, a->part_rho.p, \
                                                           a->g_rho.p, a->nt4_rho)
  if (c->multi) {
    if (a->rmode == 0) ADJ_SWEEP2(true, 0);
    else ADJ_SWEEP2(true, 1);
  } else {
    if (a->rmode == 0) ADJ_SWEEP2(false, 0);
    else ADJ_SWEEP2(false, 1);
  }
#undef ADJ_SWEEP2
  a->launches += 1;
}

// reverse of the recorded step in slot s; eb, tau: device addresses of
// dL/dE and dL/dT_mean / ncells of the step
int reverse_step(eph_adjoint *a, int s, const double *eb, const double *tau) {
  eph_ctx *c = a->c;
  const long nc = a->nc;
  const int gb = nb_of(nc, 64);
  const double *src = a->r_src.p + (size_t)s * nc;
  if (a->fdm) {
    const GridArgs G = grid_args(a);
    const unsigned ns = a->nsub;
    // grid at the start of substep m of this step
    auto Tat = [&](unsigned m) -> const double * {
      return m == 0 ? a->r_T0.p + (size_t)s * nc : a->r_Tsub.p + ((size_t)s * ns + (m - 1)) * (size_t)nc;
    };
    double *ub[2] = {a->u0.p, a->u1.p};
    const int gb32 = nb_of(nc, 32);  // small grids: spread the cells over more SMs
    k_adj_fdm_first<<<gb32, 32, 0, c->stream>>>(G, Tat(ns - 1), src, a->Tb.p, tau, ub[0], a->srcbar.p, a->gC.p,
                                                a->gK.p);
    a->launches += 1;
    int cur = 0;
    for (int k = (int)ns - 1; k >= 0; --k) {
      const double *Tprev = k >= 1 ? Tat((unsigned)k - 1) : nullptr;
      k_adj_fdm_back<<<gb32, 32, 0, c->stream>>>(G, a->fdmW.p, ub[cur], Tprev, src, ub[cur ^ 1], a->Tb.p,
                                                 a->srcbar.p, a->gC.p, a->gK.p);
      a->launches += 1;
      cur ^= 1;
    }
  } else {
    k_adj_add<<<gb, 64, 0, c->stream>>>(a->Tb.p, nc, tau);
    a->launches += 1;
  }
  const Slot S = slot_view(a, s);
  const int nb = nb_of(a->n);
  const double scale = a->fdm ? 1.0 / c->P.prescale : 0.0;
  const double *sb = a->fdm ? a->srcbar.p : nullptr;
  int *texp = a->tb_exp.p + (eb - a->d_eb.p);  // this step's slot
#define ADJ_ENERGY(F, R)                                                                                          \
  k_adj_energy<F, R><<<nb, ABLOCK, 0, c->stream>>>(c->P, S, c->mask.p, c->type.p, eb, scale, sb, a->vb.p, a->fb.p, \
                                                   a->cE.p, a->cR.p, a->tbc.p, texp)
  if (a->fric && a->rand) ADJ_ENERGY(true, true);
  else if (a->fric) ADJ_ENERGY(true, false);
  else if (a->rand) ADJ_ENERGY(false, true);
  else ADJ_ENERGY(false, false);
#undef ADJ_ENERGY
  a->launches += 1;
  if (a->rand) {
    k_adj_tb_fixed<<<nb, ABLOCK, 0, c->stream>>>(a->n, a->tbc.p, S.cell, texp, a->tb_acc.p, a->d_err.p);
    k_adj_tb_apply<<<gb, 64, 0, c->stream>>>(nc, texp, a->tb_acc.p, a->Tb.p);
    a->launches += 2;
  }
  if (c->mode == EPH_MODE_FAST) launch_sweeps<true>(a, S);
  else launch_sweeps<false>(a, S);
  ADJ_TRY(a, cudaGetLastError());
  return EPH_OK;
}

template <typename T>
int ensure(eph_adjoint *a, DevBuf<T> &b, size_t count) {
  if (b.n >= count && b.p) return EPH_OK;
  a->own_gen += 1;
  ADJ_TRY(a, b.alloc(count));
  return EPH_OK;
}

eph_adjoint::Shape shape_now(const eph_adjoint *a, long nsteps) {
  const eph_ctx *c = a->c;
  eph_adjoint::Shape s;
  s.nsteps = nsteps;
  s.nsub = c->nsub;
  s.ctx_gen = c->buf_gen;
  s.own_gen = a->own_gen;
  s.P = c->P;
  s.inner_dt = c->inner_dt;
  s.fext = c->have_fext;
  return s;
}

bool same_shape(const eph_adjoint::Shape &x, const eph_adjoint::Shape &y) {
  return x.nsteps == y.nsteps && x.nsub == y.nsub && x.ctx_gen == y.ctx_gen && x.own_gen == y.own_gen &&
         x.inner_dt == y.inner_dt && x.fext == y.fext && std::memcmp(&x.P, &y.P, sizeof(StepParams)) == 0;
}

// the forward pass: from the start state, nsteps plain steps with a
// checkpoint every K steps and E, T_mean of each step; the steps of the last
// segment are recorded as they run (the backward pass starts there)
int issue_forward(eph_adjoint *a, long nsteps) {
  eph_ctx *c = a->c;
  const size_t N = (size_t)a->n, nc = (size_t)a->nc;
  const long last0 = ((nsteps - 1) / a->K) * a->K;
  int r;
  if ((r = load_state(a, a->s_x.p, a->s_v.p, a->s_f.p, a->s_xh.p, a->s_T.p, a->s_step.p))) return r;
  for (long t = 0; t < nsteps; ++t) {
    if (t % a->K == 0) {
      const long k = t / a->K;
      if ((r = save_state(a, a->k_x.p + k * N, a->k_v.p + k * N, a->k_f.p + k * N, a->k_xh.p + k * N,
                          a->k_T.p + k * nc, a->k_step.p + k)))
        return r;
    }
    if ((r = run_step(a, t >= last0 ? (int)(t - last0) : -1))) return r;
    if (a->fric || a->rand) ADJ_TRY(a, d2d(a->d_E.p + t, c->scal.p + 1, 1, c->stream));
    else ADJ_TRY(a, cudaMemsetAsync(a->d_E.p + t, 0, sizeof(double), c->stream));
    k_adj_mean<<<1, 256, 0, c->stream>>>(c->T0.p, a->nc, a->d_Tm.p + t);
    a->launches += 1;
  }
  ADJ_TRY(a, cudaGetLastError());
  return EPH_OK;
}

// the backward pass over the last trajectory, cotangents in d_eb / d_tau;
// skip_last: the last segment is still recorded from the forward pass
int issue_backward(eph_adjoint *a, bool skip_last) {
  eph_ctx *c = a->c;
  const size_t N = (size_t)a->n, nc = (size_t)a->nc;
  int r;
  for (DevBuf<D4> *b : {&a->xb, &a->vb, &a->fb}) ADJ_TRY(a, cudaMemsetAsync(b->p, 0, sizeof(D4) * N, c->stream));
  for (DevBuf<double> *b : {&a->Tb, &a->gC, &a->gK})
    ADJ_TRY(a, cudaMemsetAsync(b->p, 0, sizeof(double) * nc, c->stream));
  ADJ_TRY(a, cudaMemsetAsync(a->g_rho.p, 0, sizeof(double) * (size_t)a->nt4_rho, c->stream));
  ADJ_TRY(a, cudaMemsetAsync(a->g_alpha.p, 0, sizeof(double) * (size_t)a->nt4_alpha, c->stream));
  ADJ_TRY(a, cudaMemsetAsync(a->tb_exp.p, 0, sizeof(int) * (size_t)a->nsteps, c->stream));
  const int nb = nb_of(a->n);
  if (a->rmode == 0)
    ADJ_TRY(a, cudaMemsetAsync(a->part_rho.p, 0, sizeof(double) * (size_t)nb * a->nt4_rho, c->stream));
  if (a->amode == 0)
    ADJ_TRY(a, cudaMemsetAsync(a->part_alpha.p, 0, sizeof(double) * (size_t)nb * a->nt4_alpha, c->stream));
  if (a->fdm) {
    k_adj_fdm_weights<<<nb_of(a->nc, 64), 64, 0, c->stream>>>(grid_args(a), a->fdmW.p);
    a->launches += 1;
  }
  const long nseg = (a->nsteps + a->K - 1) / a->K;
  for (long seg = nseg - 1; seg >= 0; --seg) {
    const long t0 = seg * a->K, t1 = std::min(t0 + a->K, a->nsteps);
    if (!(skip_last && seg == nseg - 1)) {
      if ((r = load_state(a, a->k_x.p + seg * N, a->k_v.p + seg * N, a->k_f.p + seg * N, a->k_xh.p + seg * N,
                          a->k_T.p + seg * nc, a->k_step.p + seg)))
        return r;
      for (long t = t0; t < t1; ++t)
        if ((r = run_step(a, (int)(t - t0)))) return r;
    }
    for (long t = t1 - 1; t >= t0; --t)
      if ((r = reverse_step(a, (int)(t - t0), a->d_eb.p + t, a->d_tau.p + t))) return r;
  }
  // the blocks' partial rows of the table-coefficient gradients, once per pass
  if (a->amode == 0) {
    k_adj_reduce<<<nb_of(a->nt4_alpha), ABLOCK, 0, c->stream>>>(a->part_alpha.p, nb, a->nt4_alpha, a->g_alpha.p);
    a->launches += 1;
  }
  if (a->rmode == 0) {
    k_adj_reduce<<<nb_of(a->nt4_rho), ABLOCK, 0, c->stream>>>(a->part_rho.p, nb, a->nt4_rho, a->g_rho.p);
    a->launches += 1;
  }
  ADJ_TRY(a, cudaGetLastError());
  return EPH_OK;
}

// Run a pass: replay its graph, capturing it first when none fits; or issue
// it directly.  The context's profiling is off meanwhile (its event marks
// cannot live inside a graph).
int run_pass(eph_adjoint *a, int pass, long nsteps, cudaEvent_t e0, cudaEvent_t e1) {
  eph_ctx *c = a->c;
  const bool prof = c->profiling;
  c->profiling = false;
  int r = EPH_OK;
  cudaGraphExec_t &ex = a->exec[pass];
  eph_adjoint::Shape &sh = a->shape[pass];
  long &gl = a->graph_launches[pass];
  auto issue = [&]() { return pass == 0 ? issue_forward(a, nsteps) : issue_backward(a, pass == 2); };
  if (a->use_graph) {
    const eph_adjoint::Shape now = shape_now(a, nsteps);
    if (!ex || !same_shape(sh, now)) {
      if (ex) cudaGraphExecDestroy(ex);
      ex = nullptr;
      a->launches = 0;
      cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) r = afail(a, EPH_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(e));
      if (!r) {
        r = issue();
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(c->stream, &g);
        if (!r && e != cudaSuccess) r = afail(a, EPH_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
        if (!r) {
          e = cudaGraphInstantiate(&ex, g, 0);
          if (e != cudaSuccess) r = afail(a, EPH_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
        }
        if (g) cudaGraphDestroy(g);
      }
      if (!r) {
        sh = now;
        gl = a->launches;
      } else {
        cudaGetLastError();  // a failed capture leaves its error behind for the next caller
      }
    }
    if (!r) {
      cudaEventRecord(e0, c->stream);
      cudaError_t e = cudaGraphLaunch(ex, c->stream);
      cudaEventRecord(e1, c->stream);
      if (e != cudaSuccess) r = afail(a, EPH_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
      a->launches = gl;
    }
  } else {
    a->launches = 0;
    cudaEventRecord(e0, c->stream);
    r = issue();
    cudaEventRecord(e1, c->stream);
  }
  c->profiling = prof;
  return r;
}

int ensure_records(eph_adjoint *a) {
  eph_ctx *c = a->c;
  const size_t N = (size_t)a->n, K = (size_t)a->K;
  int r;
  a->nsub = c->nsub;
  for (DevBuf<D4> *b : {&a->r_x1, &a->r_v1, &a->r_v2, &a->r_A, &a->r_Bw, &a->r_fE, &a->r_fR})
    if ((r = ensure(a, *b, K * N))) return r;
  if ((r = ensure(a, a->r_cell, K * N)) || (r = ensure(a, a->r_ns, K * N)) || (r = ensure(a, a->r_Te, K * N)))
    return r;
  if ((r = ensure(a, a->r_pj, K * (size_t)a->kcap * N))) return r;
  if ((r = ensure(a, a->r_T0, K * (size_t)a->nc)) || (r = ensure(a, a->r_src, K * (size_t)a->nc))) return r;
  if ((r = ensure(a, a->r_Tsub, K * (size_t)a->nsub * (size_t)a->nc))) return r;
  return EPH_OK;
}

// ---------------------------------------------------------- pass pieces

// checks and allocations of a forward pass
int fwd_prepare(eph_adjoint *a, long nsteps) {
  eph_ctx *c = a->c;
  if (c->n != a->n || c->kcap != a->kcap)
    return afail(a, EPH_ERR_STATE, "the context's atoms changed since the adjoint was created");
  ADJ_TRY(a, cudaSetDevice(c->device));
  const long nseg = (nsteps + a->K - 1) / a->K;
  const size_t N = (size_t)a->n, nc = (size_t)a->nc;
  int r;
  if (nseg > a->nck) {
    a->own_gen += 1;
    for (DevBuf<D4> *b : {&a->k_x, &a->k_v, &a->k_f, &a->k_xh}) ADJ_TRY(a, b->alloc((size_t)nseg * N));
    ADJ_TRY(a, a->k_T.alloc((size_t)nseg * nc));
    ADJ_TRY(a, a->k_step.alloc((size_t)nseg));
    a->nck = nseg;
  }
  if ((r = ensure(a, a->d_E, (size_t)nsteps)) || (r = ensure(a, a->d_Tm, (size_t)nsteps))) return r;
  if (c->nsub != a->nsub || !a->r_x1.p)
    if ((r = ensure_records(a))) return r;
  a->last_recorded = false;
  return EPH_OK;
}

// after a forward pass on `st`: E and T_mean to the host, device checks
int fwd_finish(eph_adjoint *a, long nsteps, double *E, double *T_mean, cudaStream_t st) {
  eph_ctx *c = a->c;
  int r;
  if (E) ADJ_TRY(a, cudaMemcpyAsync(E, a->d_E.p, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, st));
  if (T_mean) ADJ_TRY(a, cudaMemcpyAsync(T_mean, a->d_Tm.p, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, st));
  ADJ_TRY(a, cudaStreamSynchronize(st));
  if ((r = ctxi::check_device(c))) return from_ctx(a, r);
  a->nsteps = nsteps;
  a->have_grad = false;
  a->last_recorded = true;
  return EPH_OK;
}

// allocations of a backward pass and the cotangents to the device (on `st`)
int bwd_prepare(eph_adjoint *a, const double *dL_dE, const double *dL_dT_mean, cudaStream_t st, bool *skip_last) {
  if (a->nsteps < 1) return afail(a, EPH_ERR_STATE, "no trajectory: call eph_adjoint_forward first");
  eph_ctx *c = a->c;
  ADJ_TRY(a, cudaSetDevice(c->device));
  int r;
  if (c->nsub != a->nsub || !a->r_x1.p)
    if ((r = ensure_records(a))) return r;
  const long ns = a->nsteps;
  if ((r = ensure(a, a->d_eb, (size_t)ns)) || (r = ensure(a, a->d_tau, (size_t)ns)) ||
      (r = ensure(a, a->tb_exp, (size_t)ns)))
    return r;
  if (a->h_cot_n < 2 * ns) {
    if (a->h_cot) cudaFreeHost(a->h_cot);
    a->h_cot = nullptr;
    a->h_cot_n = 0;
    ADJ_TRY(a, cudaMallocHost(&a->h_cot, sizeof(double) * 2 * (size_t)ns));
    a->h_cot_n = 2 * ns;
  }
  const double inv_nc = 1.0 / (double)a->nc;
  for (long t = 0; t < ns; ++t) {
    a->h_cot[t] = dL_dE ? dL_dE[t] : 0.0;
    a->h_cot[ns + t] = dL_dT_mean ? dL_dT_mean[t] * inv_nc : 0.0;
  }
  ADJ_TRY(a, cudaMemcpyAsync(a->d_eb.p, a->h_cot, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  ADJ_TRY(a, cudaMemcpyAsync(a->d_tau.p, a->h_cot + ns, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  *skip_last = a->last_recorded && c->nsub == a->nsub;
  return EPH_OK;
}

// after a backward pass on `st`: gradients to the host, chained to the knots
int bwd_finish(eph_adjoint *a, bool skip_last, cudaStream_t st) {
  eph_ctx *c = a->c;
  const size_t nc = (size_t)a->nc;
  int r;
  // the records now hold the first segment (or still the last, if only one)
  a->last_recorded = (a->nsteps + a->K - 1) / a->K == 1 && skip_last;
  unsigned herr = 0;
  const Beta &B = c->beta;
  std::vector<double> hr((size_t)a->nt4_rho), ha((size_t)a->nt4_alpha), hC(nc), hK(nc);
  ADJ_TRY(a, cudaMemcpyAsync(&herr, a->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  ADJ_TRY(a, cudaMemcpyAsync(hr.data(), a->g_rho.p, hr.size() * 8, cudaMemcpyDeviceToHost, st));
  ADJ_TRY(a, cudaMemcpyAsync(ha.data(), a->g_alpha.p, ha.size() * 8, cudaMemcpyDeviceToHost, st));
  ADJ_TRY(a, cudaMemcpyAsync(hC.data(), a->gC.p, nc * 8, cudaMemcpyDeviceToHost, st));
  ADJ_TRY(a, cudaMemcpyAsync(hK.data(), a->gK.p, nc * 8, cudaMemcpyDeviceToHost, st));
  ADJ_TRY(a, cudaStreamSynchronize(st));
  if ((r = ctxi::check_device(c))) return from_ctx(a, r);
  if (herr) {
    cudaMemset(a->d_err.p, 0, sizeof(unsigned));
    return afail(a, EPH_ERR_RANGE, "device: a grid cotangent sum left the fixed-point range");
  }
  a->grad_rho.assign(B.n_elements, std::vector<double>(B.n_rho, 0.0));
  a->grad_beta.assign(B.n_elements, std::vector<double>(B.n_beta, 0.0));
  for (int e = 0; e < B.n_elements; ++e)
    B.knot_gradient(e, hr.data() + (size_t)e * B.n_rho * 4, ha.data() + (size_t)e * B.n_beta * 4,
                    a->grad_rho[e].data(), a->grad_beta[e].data());
  a->grad_C = 0.0;
  a->grad_K = 0.0;
  for (size_t i = 0; i < nc; ++i) {
    a->grad_C += hC[i];
    a->grad_K += hK[i];
  }
  a->have_grad = true;
  return EPH_OK;
}

}  // namespace

extern "C" {

int eph_adjoint_create(eph_ctx *c, int checkpoint_every, eph_adjoint **out) {
  if (!c || !out || checkpoint_every < 1) return EPH_ERR_ARG;
  *out = nullptr;
  if (c->n <= 0) return ctxi::fail(c, EPH_ERR_STATE, "no atoms: call eph_set_atoms first");
  if (c->args.model != 4) return ctxi::fail(c, EPH_ERR_UNSUPPORTED_MODEL, "the adjoint follows force_prl (model 4)");
  if (c->args.coloured) return ctxi::fail(c, EPH_ERR_UNSUPPORTED_MODEL, "the adjoint follows fix eph, not eph/coloured/exp");
  if (c->td.tdyn) return ctxi::fail(c, EPH_ERR_STATE, "the adjoint needs a grid without temperature-dependent cells");
  if (c->eam) return ctxi::fail(c, EPH_ERR_UNSUPPORTED_MODEL, "the adjoint does not differentiate the EAM pair force");
  if (c->beta.n_elements * c->beta.n_beta > 65536)
    return ctxi::fail(c, EPH_ERR_CAPACITY, "alpha tables too large for the adjoint's accumulators");
  // recomputed segments must repeat the recorded steps bit for bit: every
  // step searches the bins (a kept candidate list would carry state across
  // checkpoints)
  c->list_block = true;
  if (int rl = ctxi::configure_list(c)) return rl;
  eph_adjoint *a = new (std::nothrow) eph_adjoint();
  if (!a) return EPH_ERR_ARG;
  *out = a;
  a->c = c;
  a->K = checkpoint_every;
  a->n = c->n;
  a->kcap = c->kcap;
  a->nc = c->grid.ntotal;
  a->fric = c->P.flags & FLAG_FRICTION;
  a->rand = c->P.flags & FLAG_RANDOM;
  a->fdm = c->P.flags & FLAG_FDM;
  ADJ_TRY(a, cudaSetDevice(c->device));
  const size_t N = (size_t)a->n, nc = (size_t)a->nc;
  for (DevBuf<D4> *b : {&a->s_x, &a->s_v, &a->s_f, &a->s_xh, &a->xb, &a->vb, &a->fb, &a->cE, &a->cR, &a->W})
    ADJ_TRY(a, b->alloc(N));
  for (DevBuf<double> *b : {&a->s_T, &a->Tb, &a->u0, &a->u1, &a->srcbar, &a->gC, &a->gK, &a->rho_e})
    ADJ_TRY(a, b->alloc(nc));
  ADJ_TRY(a, a->fdmW.alloc(7 * nc));
  ADJ_TRY(a, a->dfr.alloc((size_t)R_N * N));
  ADJ_TRY(a, a->s_step.alloc(1));
  ADJ_TRY(a, a->tbc.alloc(N));
  ADJ_TRY(a, a->tb_acc.alloc(nc));
  ADJ_TRY(a, a->d_err.alloc(1));
  ADJ_TRY(a, cudaMemset(a->tb_acc.p, 0, sizeof(U128) * nc));
  ADJ_TRY(a, cudaMemset(a->d_err.p, 0, sizeof(unsigned)));
  ADJ_TRY(a, cudaMemcpy(a->rho_e.p, c->grid.rho.data(), nc * sizeof(double), cudaMemcpyHostToDevice));
  const Beta &B = c->beta;
  a->nt4_rho = 4 * B.n_elements * (int)B.n_rho;
  a->nt4_alpha = 4 * B.n_elements * (int)B.n_beta;
  a->rmode = B.n_elements * B.n_rho <= PRIV_MAX_KNOTS ? 0 : 1;
  a->amode = B.n_elements * B.n_beta <= WARP_MAX_KNOTS ? 0 : 1;
  const int nb = nb_of(a->n);
  ADJ_TRY(a, a->g_rho.alloc((size_t)a->nt4_rho));
  ADJ_TRY(a, a->g_alpha.alloc((size_t)a->nt4_alpha));
  if (a->rmode == 0) ADJ_TRY(a, a->part_rho.alloc((size_t)nb * a->nt4_rho));
  if (a->amode == 0) ADJ_TRY(a, a->part_alpha.alloc((size_t)nb * a->nt4_alpha));
  if (a->rmode == 0) {
    const int sh = (int)(sizeof(double) * (size_t)a->nt4_rho * ABLOCK);
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2<true, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2<true, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2<false, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2<false, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2_df<true, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2_df<true, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2_df<false, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    sh));
    ADJ_TRY(a, cudaFuncSetAttribute(k_adj_sweep2_df<false, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    sh));
  }
  for (cudaEvent_t &e : a->ev) ADJ_TRY(a, cudaEventCreate(&e));
  // the start of every trajectory: the context as it is now
  int r = save_state(a, a->s_x.p, a->s_v.p, a->s_f.p, a->s_xh.p, a->s_T.p, a->s_step.p);
  if (r) return r;
  ADJ_TRY(a, cudaStreamSynchronize(c->stream));
  return EPH_OK;
}

void eph_adjoint_destroy(eph_adjoint *a) {
  if (!a) return;
  // the context may already be gone: touch nothing of it (cudaFree below
  // waits for the device's outstanding work)
  for (cudaEvent_t e : a->ev)
    if (e) cudaEventDestroy(e);
  for (cudaGraphExec_t e : a->exec)
    if (e) cudaGraphExecDestroy(e);
  if (a->h_cot) cudaFreeHost(a->h_cot);
  delete a;
}

const char *eph_adjoint_last_error(const eph_adjoint *a) { return a ? a->err.c_str() : "null adjoint"; }

int eph_adjoint_forward(eph_adjoint *a, long nsteps, double *E, double *T_mean) {
  if (!a || nsteps < 1) return EPH_ERR_ARG;
  int r;
  if ((r = fwd_prepare(a, nsteps))) return r;
  if ((r = run_pass(a, 0, nsteps, a->ev[0], a->ev[1]))) return r;
  if ((r = fwd_finish(a, nsteps, E, T_mean, a->c->stream))) return r;
  float ms = 0.f;
  ADJ_TRY(a, cudaEventElapsedTime(&ms, a->ev[0], a->ev[1]));
  a->fwd_ms = ms;
  a->fwd_launches = a->launches;
  return EPH_OK;
}

int eph_adjoint_backward(eph_adjoint *a, const double *dL_dE, const double *dL_dT_mean) {
  if (!a) return EPH_ERR_ARG;
  int r;
  bool skip_last = false;
  if ((r = bwd_prepare(a, dL_dE, dL_dT_mean, a->c->stream, &skip_last))) return r;
  if ((r = run_pass(a, skip_last ? 2 : 1, a->nsteps, a->ev[2], a->ev[3]))) return r;
  if ((r = bwd_finish(a, skip_last, a->c->stream))) return r;
  float ms = 0.f;
  ADJ_TRY(a, cudaEventElapsedTime(&ms, a->ev[2], a->ev[3]));
  a->bwd_ms = ms;
  a->bwd_launches = a->launches;
  return EPH_OK;
}

int eph_adjoint_set_graph(eph_adjoint *a, int on) {
  if (!a) return EPH_ERR_ARG;
  a->use_graph = on != 0;
  return EPH_OK;
}

int eph_adjoint_gradient(eph_adjoint *a, int which, int elem, double *out, long n) {
  if (!a || !out) return EPH_ERR_ARG;
  if (!a->have_grad) return afail(a, EPH_ERR_STATE, "no gradient: call eph_adjoint_backward first");
  const Beta &B = a->c->beta;
  switch (which) {
    case EPH_GRAD_RHO_KNOTS:
      if (elem < 0 || elem >= B.n_elements || n != B.n_rho) return afail(a, EPH_ERR_ARG, "rho(r) column: element or size");
      std::memcpy(out, a->grad_rho[elem].data(), sizeof(double) * (size_t)n);
      return EPH_OK;
    case EPH_GRAD_BETA_KNOTS:
      if (elem < 0 || elem >= B.n_elements || n != B.n_beta) return afail(a, EPH_ERR_ARG, "beta(rho) column: element or size");
      std::memcpy(out, a->grad_beta[elem].data(), sizeof(double) * (size_t)n);
      return EPH_OK;
    case EPH_GRAD_C_E:
      if (n != 1) return afail(a, EPH_ERR_ARG, "one value");
      *out = a->grad_C;
      return EPH_OK;
    case EPH_GRAD_KAPPA:
      if (n != 1) return afail(a, EPH_ERR_ARG, "one value");
      *out = a->grad_K;
      return EPH_OK;
    default: return afail(a, EPH_ERR_ARG, "unknown gradient");
  }
}

int eph_adjoint_timing(eph_adjoint *a, double *forward_ms, double *backward_ms, long *forward_launches,
                       long *backward_launches) {
  if (!a) return EPH_ERR_ARG;
  if (forward_ms) *forward_ms = a->fwd_ms;
  if (backward_ms) *backward_ms = a->bwd_ms;
  if (forward_launches) *forward_launches = a->fwd_launches;
  if (backward_launches) *backward_launches = a->bwd_launches;
  return EPH_OK;
}

// ----------------------------------------------------------- batched passes

struct eph_adjoint_batch {
  std::vector<eph_adjoint *> a;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
  std::vector<eph_adjoint::Shape> shape[3];
  long graph_launches[3] = {0, 0, 0};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double fwd_ms = 0.0, bwd_ms = 0.0;
  long fwd_launches = 0, bwd_launches = 0;
  std::string err;
};

static int bfail(eph_adjoint_batch *b, int code, const std::string &msg) {
  b->err = msg;
  return code;
}

// One pass of every adjoint as parallel branches of one graph launched on
// b->main (fork event -> each context's stream -> join events).
static int batch_pass(eph_adjoint_batch *b, int pass, long nsteps, cudaEvent_t e0, cudaEvent_t e1) {
  std::vector<eph_adjoint::Shape> now;
  for (eph_adjoint *a : b->a) now.push_back(shape_now(a, nsteps));
  bool fits = b->exec[pass] && b->shape[pass].size() == now.size();
  for (size_t r = 0; fits && r < now.size(); ++r) fits = same_shape(b->shape[pass][r], now[r]);
  // work already queued on the contexts' streams comes first
  for (eph_adjoint *a : b->a)
    if (cudaStreamSynchronize(a->c->stream) != cudaSuccess) return bfail(b, EPH_ERR_CUDA, "stream synchronise");
  std::vector<bool> prof;
  for (eph_adjoint *a : b->a) {
    prof.push_back(a->c->profiling);
    a->c->profiling = false;
  }
  int rc = EPH_OK;
  if (!fits) {
    if (b->exec[pass]) cudaGraphExecDestroy(b->exec[pass]);
    b->exec[pass] = nullptr;
    long total = 0;
    if (cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal) != cudaSuccess ||
        cudaEventRecord(b->fork, b->main) != cudaSuccess)
      rc = bfail(b, EPH_ERR_CUDA, "begin capture");
    for (size_t r = 0; r < b->a.size() && !rc; ++r) {
      eph_adjoint *a = b->a[r];
      if (cudaStreamWaitEvent(a->c->stream, b->fork, 0) != cudaSuccess) {
        rc = bfail(b, EPH_ERR_CUDA, "fork");
        break;
      }
      a->launches = 0;
      rc = pass == 0 ? issue_forward(a, nsteps) : issue_backward(a, pass == 2);
      total += a->launches;
      if (rc) {
        b->err = "adjoint " + std::to_string(r) + ": " + a->err;
        break;
      }
      if (cudaEventRecord(b->joins[r], a->c->stream) != cudaSuccess ||
          cudaStreamWaitEvent(b->main, b->joins[r], 0) != cudaSuccess)
        rc = bfail(b, EPH_ERR_CUDA, "join");
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->main, &g);
    if (!rc && e != cudaSuccess) rc = bfail(b, EPH_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
    if (!rc && cudaGraphInstantiate(&b->exec[pass], g, 0) != cudaSuccess)
      rc = bfail(b, EPH_ERR_CUDA, "cannot instantiate the batched graph");
    if (g) cudaGraphDestroy(g);
    if (!rc) {
      b->shape[pass] = now;
      b->graph_launches[pass] = total;
    } else {
      cudaGetLastError();
    }
  }
  if (!rc) {
    cudaEventRecord(e0, b->main);
    if (cudaGraphLaunch(b->exec[pass], b->main) != cudaSuccess) rc = bfail(b, EPH_ERR_CUDA, "graph launch");
    cudaEventRecord(e1, b->main);
  }
  for (size_t r = 0; r < b->a.size(); ++r) b->a[r]->c->profiling = prof[r];
  return rc;
}

int eph_adjoint_batch_create(int nadj, eph_adjoint *const *adj, eph_adjoint_batch **out) {
  if (!out || nadj < 1 || !adj) return EPH_ERR_ARG;
  *out = nullptr;
  eph_adjoint_batch *b = new (std::nothrow) eph_adjoint_batch();
  if (!b) return EPH_ERR_ARG;
  *out = b;
  for (int r = 0; r < nadj; ++r) {
    if (!adj[r]) return bfail(b, EPH_ERR_ARG, "null adjoint");
    if (adj[r]->c->device != adj[0]->c->device) return bfail(b, EPH_ERR_ARG, "all adjoints of a batch on one device");
    for (int q = 0; q < r; ++q)
      if (adj[q] == adj[r] || adj[q]->c == adj[r]->c) return bfail(b, EPH_ERR_ARG, "one adjoint per context");
    b->a.push_back(adj[r]);
  }
  if (cudaSetDevice(adj[0]->c->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    return bfail(b, EPH_ERR_CUDA, "cannot create the batch stream");
  b->joins.assign(nadj, nullptr);
  for (auto &e : b->joins)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bfail(b, EPH_ERR_CUDA, "events");
  for (auto &e : b->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return bfail(b, EPH_ERR_CUDA, "events");
  return EPH_OK;
}

void eph_adjoint_batch_destroy(eph_adjoint_batch *b) {
  if (!b) return;
  if (b->main) cudaStreamSynchronize(b->main);
  for (cudaGraphExec_t e : b->exec)
    if (e) cudaGraphExecDestroy(e);
  for (auto e : b->joins)
    if (e) cudaEventDestroy(e);
  for (auto e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->main) cudaStreamDestroy(b->main);
  delete b;
}

const char *eph_adjoint_batch_last_error(const eph_adjoint_batch *b) { return b ? b->err.c_str() : "null batch"; }

int eph_adjoint_batch_forward(eph_adjoint_batch *b, long nsteps, double *E, double *T_mean) {
  if (!b || nsteps < 1) return EPH_ERR_ARG;
  int rc;
  for (size_t r = 0; r < b->a.size(); ++r)
    if ((rc = fwd_prepare(b->a[r], nsteps))) return bfail(b, rc, "adjoint " + std::to_string(r) + ": " + b->a[r]->err);
  if ((rc = batch_pass(b, 0, nsteps, b->ev[0], b->ev[1]))) return rc;
  for (size_t r = 0; r < b->a.size(); ++r)
    if ((rc = fwd_finish(b->a[r], nsteps, E ? E + r * nsteps : nullptr, T_mean ? T_mean + r * nsteps : nullptr,
                         b->main)))
      return bfail(b, rc, "adjoint " + std::to_string(r) + ": " + b->a[r]->err);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
  b->fwd_ms = ms;
  b->fwd_launches = b->graph_launches[0];
  return EPH_OK;
}

int eph_adjoint_batch_backward(eph_adjoint_batch *b, const double *dL_dE, const double *dL_dT_mean) {
  if (!b) return EPH_ERR_ARG;
  const long ns = b->a[0]->nsteps;
  for (eph_adjoint *a : b->a)
    if (a->nsteps != ns || ns < 1) return bfail(b, EPH_ERR_STATE, "run eph_adjoint_batch_forward first");
  int rc;
  bool all_skip = true;
  for (size_t r = 0; r < b->a.size(); ++r) {
    bool sk = false;
    if ((rc = bwd_prepare(b->a[r], dL_dE ? dL_dE + r * ns : nullptr, dL_dT_mean ? dL_dT_mean + r * ns : nullptr,
                          b->main, &sk)))
      return bfail(b, rc, "adjoint " + std::to_string(r) + ": " + b->a[r]->err);
    all_skip = all_skip && sk;
  }
  if ((rc = batch_pass(b, all_skip ? 2 : 1, ns, b->ev[2], b->ev[3]))) return rc;
  for (size_t r = 0; r < b->a.size(); ++r)
    if ((rc = bwd_finish(b->a[r], all_skip, b->main)))
      return bfail(b, rc, "adjoint " + std::to_string(r) + ": " + b->a[r]->err);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev[2], b->ev[3]);
  b->bwd_ms = ms;
  b->bwd_launches = b->graph_launches[all_skip ? 2 : 1];
  return EPH_OK;
}

int eph_adjoint_batch_timing(eph_adjoint_batch *b, double *forward_ms, double *backward_ms, long *forward_launches,
                             long *backward_launches) {
  if (!b) return EPH_ERR_ARG;
  if (forward_ms) *forward_ms = b->fwd_ms;
  if (backward_ms) *backward_ms = b->bwd_ms;
  if (forward_launches) *forward_launches = b->fwd_launches;
  if (backward_launches) *backward_launches = b->bwd_launches;
  return EPH_OK;
}

}  // extern "C"
