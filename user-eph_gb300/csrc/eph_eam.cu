// The engine's pair force for standalone runs: eam/alloy (a LAMMPS setfl
// file; E = sum_i F_a(rho_i) + 1/2 sum_{i != j} phi_ab(r_ij), rho_i = sum_j
// f_b(r_ij)), evaluated on the GPU from the fix's own spatial bins each step
// before post_force, as LAMMPS's Verlet computes the pair force between
// initial_integrate and post_force.  No reference counterpart: the reference
// fix receives the pair force from LAMMPS (Tests/MD_Run/run.lmp uses
// pair_style eam/alloy with Ni.eam); this gives the standalone driver the
// same physics.  Tables: cubic Hermite per interval (host hermite_table).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "eph_ctx_impl.hpp"
#include "eph_df64.cuh"
#include "eph_df_pair.cuh"

using namespace ephgb;

struct EamDevice {
  Eam host;
  DevBuf<D4> F, f, z2r;  // [element][nrho], [element][nr], [pair][nr]
  // f and z2r as double-floats for the df64 pair sums (FAST mode with
  // EPH_PAIRS_DF64): two float4 per interval, hi and lo parts
  DevBuf<float4> fd, zd;
  DevBuf<float2> fpd;  // F'(rho_i) / dr as a double-float, gathered per pair
  DevBuf<double> fp, energy, esum;
  DevBuf<unsigned> pj;    // pair list, [kcap][n]
  DevBuf<int> ns;         // pairs per atom
  int kcap = 0;
  int map[65] = {0};      // LAMMPS type -> setfl element
  double rc2_band = 0.0;  // FP32 candidate threshold
};

namespace {

constexpr unsigned FULL = 0xffffffffu;

struct EamParams {
  const D4 *F, *f, *z2r;
  const float4 *fd, *zd;
  int nel, nrho, nr;
  double inv_drho, inv_dr, rho_max, rc2;
  float rc2_band;
  float inv_dr_hi, inv_dr_lo, rc2_hi, rc2_lo;  // 1/dr and rc^2 as double-floats
  int map[65];
};

// value and d/d(index) of a Hermite table at x (in units of the knot spacing)
__device__ __forceinline__ void herm(const D4 *__restrict__ t, int n, double x, double &v, double &dv) {
  int m = x > 0.0 ? (int)x : 0;  // below the table: its first interval
  if (m > n - 2) m = n - 2;
  double p = x - (double)m;
  if (p > 1.0) p = 1.0;
  const D4 c = t[m];
  v = fma(p, fma(p, fma(p, c.w, c.z), c.y), c.x);
  dv = fma(p, fma(3.0 * p, c.w, 2.0 * c.z), c.y);
}

// e = x_j (periodic image of the pair code) - x_i
__device__ __forceinline__ void image_vector(const StepParams &P, const D4 &xi, const D4 &xj, unsigned code,
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

// Pass 1 of the EAM density sweeps: atom i's candidates in the 27 bins
// around it (FP32/integer work, warp-uniform loop bounds), stored by cset as
// neighbour index | periodic-image code << 27; returns their count
template <class Set>
__device__ __forceinline__ int eam_candidates(const StepParams &P, const EamParams &E, int i, bool valid, int4 Bi,
                                              float4 oi, const int *__restrict__ bin_count,
                                              const BinEntry *__restrict__ bins, int kcap, unsigned *__restrict__ err,
                                              Set cset) {
  int nc = 0;
  for (int dz = -1; dz <= 1; ++dz) {
    const int Tz = Bi.z + dz, tz = Tz < 0 ? Tz + P.nb[2] : (Tz >= P.nb[2] ? Tz - P.nb[2] : Tz);
    const int kz = Tz < 0 ? -1 : (Tz >= P.nb[2] ? 1 : 0);
    const float bz = (float)dz * P.wf[2] - oi.z;
    for (int dy = -1; dy <= 1; ++dy) {
      const int Ty = Bi.y + dy, ty = Ty < 0 ? Ty + P.nb[1] : (Ty >= P.nb[1] ? Ty - P.nb[1] : Ty);
      const int ky = Ty < 0 ? -1 : (Ty >= P.nb[1] ? 1 : 0);
      const float by = (float)dy * P.wf[1] - oi.y;
      for (int dx = -1; dx <= 1; ++dx) {
        const int Tx = Bi.x + dx, tx = Tx < 0 ? Tx + P.nb[0] : (Tx >= P.nb[0] ? Tx - P.nb[0] : Tx);
        const int kx = Tx < 0 ? -1 : (Tx >= P.nb[0] ? 1 : 0);
        const float bx = (float)dx * P.wf[0] - oi.x;
        const int flat = tx + P.nb[0] * (ty + P.nb[1] * tz);
        int cnt = 0;
        if (valid) {
          cnt = bin_count[flat];
          cnt = cnt < P.bcap ? cnt : P.bcap;
        }
        const int cmax = __reduce_max_sync(FULL, cnt);
        const BinEntry *be = bins + (size_t)flat * P.bcap;
        for (int s = 0; s < cmax; ++s) {
          if (s >= cnt) continue;
          const BinEntry b = be[s];
          const unsigned j = b.idx & IDX_MASK;
          const float fx = bx + b.ox, fy = by + b.oy, fz = bz + b.oz;
          if (j == (unsigned)i || fx * fx + fy * fy + fz * fz >= E.rc2_band) continue;
          const unsigned wc = b.idx >> IDX_BITS;
          const int mx = kx - ((int)(wc % 3u) - 1), my = ky - ((int)((wc / 3u) % 3u) - 1),
                    mz = kz - ((int)(wc / 9u) - 1);
          if (mx < -1 || mx > 1 || my < -1 || my > 1 || mz < -1 || mz > 1) {
            atomicOr(err, ERR_DRIFT);
          } else if (nc >= kcap) {
            atomicOr(err, ERR_PAIR_OVERFLOW);
          } else {
            cset(nc++, j | ((unsigned)((mx + 1) + 3 * (my + 1) + 9 * (mz + 1)) << IDX_BITS));
          }
        }
      }
    }
  }
  return nc;
}

// rho_i = sum_j f_b(r_ij) over the 27 bins around atom i (bin edge >= the
// cutoff), the pairs within the cutoff written to the EAM pair list
// (u32: neighbour index | periodic-image code << 27, row k of atom i at
// k * n + i), then F_a(rho_i) and F'_a(rho_i) (beyond the table F continues
// linearly with the slope at its end).  Two passes as in the fix's density
// sweep: FP32/integer candidates (warp-uniform loop bounds) kept in shared
// memory with the overflow in the list rows, then the FP64 pass over the
// candidates in lockstep.
__global__ void __launch_bounds__(128)
    k_eam_density(StepParams P, EamParams E, const D4 *__restrict__ x, const int *__restrict__ type,
                  const int *__restrict__ bin_count, const BinEntry *__restrict__ bins,
                  const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
                  unsigned *__restrict__ epj, int *__restrict__ ens, int kcap, double *__restrict__ fp,
                  double *__restrict__ energy, unsigned *__restrict__ err) {
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  const bool valid = i < P.n;
  auto cget = [&](int k) -> unsigned { return k < CAND_SMEM ? s_cand[k * nt + t] : epj[(size_t)k * P.n + i]; };
  auto cset = [&](int k, unsigned u) {
    if (k < CAND_SMEM)
      s_cand[k * nt + t] = u;
    else
      epj[(size_t)k * P.n + i] = u;
  };
  const D4 xi = valid ? x[i] : D4{0.0, 0.0, 0.0, 0.0};
  int4 Bi = make_int4(0, 0, 0, 0);
  float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
  if (valid) {
    Bi = atom_bin[i];
    oi = atom_off[i];
  }
  const int nc = eam_candidates(P, E, i, valid, Bi, oi, bin_count, bins, kcap, err, cset);
  __syncwarp();
  double rho = 0.0;
  int ns = 0;
  const int nmax = __reduce_max_sync(FULL, nc);
  for (int k = 0; k < nmax; ++k) {
    if (k >= nc) continue;
    const unsigned u = cget(k);
    const unsigned j = u & IDX_MASK;
    double ex, ey, ez;
    image_vector(P, xi, x[j], u >> IDX_BITS, ex, ey, ez);
    const double r2 = fma(ez, ez, fma(ey, ey, ex * ex));
    if (r2 < E.rc2) {
      epj[(size_t)ns * P.n + i] = u;  // ns <= k: the candidate there is consumed
      ++ns;
      double v, dv;
      herm(E.f + (size_t)E.map[type[j]] * E.nr, E.nr, sqrt(r2) * E.inv_dr, v, dv);
      rho += v;
    }
  }
  if (!valid) return;
  ens[i] = ns;
  const int a = E.map[type[i]];
  double F, dF;
  herm(E.F + (size_t)a * E.nrho, E.nrho, rho * E.inv_drho, F, dF);
  dF *= E.inv_drho;
  if (rho > E.rho_max) F += dF * (rho - E.rho_max);
  fp[i] = dF;
  energy[i] = F;
}

// f_i = sum_j [F'_a(rho_i) f_b'(r) + F'_b(rho_j) f_a'(r) + phi_ab'(r)] e / r over
// the EAM pair list, added to the external force (if any); energy[i] +=
// 1/2 sum_j phi_ab(r)
__global__ void __launch_bounds__(128)
    k_eam_force(StepParams P, EamParams E, const D4 *__restrict__ x, const int *__restrict__ type,
                const unsigned *__restrict__ epj, const int *__restrict__ ens, const double *__restrict__ fp,
                const D4 *__restrict__ fext, D4 *__restrict__ f, double *__restrict__ energy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const D4 xi = x[i];
  const int a = E.map[type[i]];
  const double fpi = fp[i];
  double fx = 0.0, fy = 0.0, fz = 0.0, ep = 0.0;
  const int ns = ens[i];
  for (int k = 0; k < ns; ++k) {
    const unsigned u = epj[(size_t)k * P.n + i];
    const unsigned j = u & IDX_MASK;
    double ex, ey, ez;
    image_vector(P, xi, x[j], u >> IDX_BITS, ex, ey, ez);
    const double r2 = fma(ez, ez, fma(ey, ey, ex * ex));
    const double rinv = rsqrt(r2), r = r2 * rinv, q = r * E.inv_dr;
    const int b = E.map[type[j]];
    double fb, dfb, fa, dfa, z, dz;
    herm(E.f + (size_t)b * E.nr, E.nr, q, fb, dfb);
    dfa = dfb;
    if (a != b) herm(E.f + (size_t)a * E.nr, E.nr, q, fa, dfa);
    const int hi = a > b ? a : b, lo = a > b ? b : a;
    herm(E.z2r + (size_t)(hi * (hi + 1) / 2 + lo) * E.nr, E.nr, q, z, dz);
    const double phi = z * rinv;
    const double dphi = fma(dz, E.inv_dr, -phi) * rinv;
    const double dEdr = fma(fpi * E.inv_dr, dfb, fma(fp[j] * E.inv_dr, dfa, dphi));
    const double s = dEdr * rinv;
    fx = fma(s, ex, fx);
    fy = fma(s, ey, fy);
    fz = fma(s, ez, fz);
    ep = fma(0.5, phi, ep);
  }
  D4 out{fx, fy, fz, 0.0};
  if (fext) {
    const D4 g = fext[i];
    out.x += g.x;
    out.y += g.y;
    out.z += g.z;
  }
  f[i] = out;
  energy[i] += ep;
}

// ---------------------------------------------- df64 pair sums (FAST mode)

// herm() on a double-float table at q >= 0 (knot units): the interval from
// the FP32 part of q settled by the sign of the double-float remainder, the
// same clamps (at most the last interval, p at most 1), the value and the
// derivative per knot unit
__device__ __forceinline__ void herm_df(const float4 *__restrict__ t, int n, df64::df q, df64::df &v,
                                        df64::df &dv) {
  using namespace df64;
  const df one{1.0f, 0.0f};
  const float kr = floor_estimate(q.hi);
  int m = floor_estimate_int(kr);
  float th, te;
  two_sum(q.hi, -kr, th, te);
  df p = make(th, te + q.lo);
  if (lt(p, df{0.0f, 0.0f})) {
    m -= 1;
    p = add(p, one);
  } else if (!lt(p, one)) {
    m += 1;
    p = sub(p, one);
  }
  if (m > n - 2) {
    p = add(p, df{(float)(m - (n - 2)), 0.0f});
    m = n - 2;
    if (!lt(p, one)) p = one;
  }
  if (m < 0) m = 0;
  const float4 hi = t[2 * (size_t)m], lo = t[2 * (size_t)m + 1];
  const df c0{hi.x, lo.x}, c1{hi.y, lo.y}, c2{hi.z, lo.z}, c3{hi.w, lo.w};
  v = horner(c0, c1, c2, c3, p);
  dv = fma(p, fma(p, mul(df{3.0f, 0.0f}, c3), mul(df{2.0f, 0.0f}, c2)), c1);
}

// A pair's displacement as double-floats: from the atoms' df64 records of
// this step's bins when there are any (the bin difference with the periodic
// image plus the offsets in the bins, no FP64 work), else from the FP64
// positions as k_eam_density forms it
__device__ __forceinline__ void pair_e_df(const StepParams &P, const float4 *__restrict__ rec, int4 Bi, float4 oi,
                                          float4 ol, const D4 &xi, const D4 *__restrict__ x, unsigned j,
                                          unsigned code, df64::df &ex, df64::df &ey, df64::df &ez) {
  if (rec) {
    const float4 R0 = rec[2 * (size_t)j], R1 = rec[2 * (size_t)j + 1];
    const unsigned pk = __float_as_uint(R0.w);
    const int dx = (int)(pk & 1023u) - 1 + ((int)(code % 3u) - 1) * P.nb[0] - Bi.x;
    const int dy = (int)((pk >> 10) & 1023u) - 1 + ((int)((code / 3u) % 3u) - 1) * P.nb[1] - Bi.y;
    const int dz = (int)((pk >> 20) & 1023u) - 1 + ((int)(code / 9u) - 1) * P.nb[2] - Bi.z;
    ex = pair_disp(dx, R0.x, R1.x, oi.x, ol.x, P.w_hi[0], P.w_lo[0]);
    ey = pair_disp(dy, R0.y, R1.y, oi.y, ol.y, P.w_hi[1], P.w_lo[1]);
    ez = pair_disp(dz, R0.z, R1.z, oi.z, ol.z, P.w_hi[2], P.w_lo[2]);
  } else {
    double a, b, c;
    image_vector(P, xi, x[j], code, a, b, c);
    ex = df64::from_double(a);
    ey = df64::from_double(b);
    ez = df64::from_double(c);
  }
}

// k_eam_density with the pair arithmetic in double-float: e from the FP64
// positions (the periodic image added as k_eam_density adds it), then r^2,
// the cut-off test, r and f_b(r) in df64, rho_i in blocked sums; F and F'
// per atom in FP64; F' / dr also as a double-float for k_eam_force_df
__global__ void __launch_bounds__(128)
    k_eam_density_df(StepParams P, EamParams E, const D4 *__restrict__ x, const int *__restrict__ type,
                     const int *__restrict__ bin_count, const BinEntry *__restrict__ bins,
                     const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
                     unsigned *__restrict__ epj, int *__restrict__ ens, int kcap, double *__restrict__ fp,
                     float2 *__restrict__ fpd, double *__restrict__ energy, unsigned *__restrict__ err,
                     const float4 *__restrict__ rec) {
  using namespace df64;
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  const bool valid = i < P.n;
  auto cget = [&](int k) -> unsigned { return k < CAND_SMEM ? s_cand[k * nt + t] : epj[(size_t)k * P.n + i]; };
  auto cset = [&](int k, unsigned u) {
    if (k < CAND_SMEM)
      s_cand[k * nt + t] = u;
    else
      epj[(size_t)k * P.n + i] = u;
  };
  const D4 xi = valid ? x[i] : D4{0.0, 0.0, 0.0, 0.0};
  int4 Bi = make_int4(0, 0, 0, 0);
  float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
  if (valid) {
    Bi = atom_bin[i];
    oi = atom_off[i];
  }
  const int nc = eam_candidates(P, E, i, valid, Bi, oi, bin_count, bins, kcap, err, cset);
  __syncwarp();
  float4 rh = make_float4(0.f, 0.f, 0.f, 0.f), rl = rh;
  if (rec && valid) {
    rh = rec[2 * (size_t)i];
    rl = rec[2 * (size_t)i + 1];
  }
  const df rc2{E.rc2_hi, E.rc2_lo}, inv_dr{E.inv_dr_hi, E.inv_dr_lo};
  bsum rs = bsum_zero();
  int ns = 0;
  const int nmax = __reduce_max_sync(FULL, nc);
  for (int k = 0; k < nmax; ++k) {
    if (k >= nc) continue;
    const unsigned u = cget(k);
    const unsigned j = u & IDX_MASK;
    df dx, dy, dz;
    pair_e_df(P, rec, Bi, rh, rl, xi, x, j, u >> IDX_BITS, dx, dy, dz);
    const df r2 = dot3(dx, dy, dz, dx, dy, dz);
    if (lt(r2, rc2)) {
      epj[(size_t)ns * P.n + i] = u;  // ns <= k: the candidate there is consumed
      ++ns;
      df v, dv;
      const df q = mul(df64::sqrt(r2, rsqrt_estimate(r2.hi)), inv_dr);
      herm_df(E.fd + 2 * (size_t)E.map[type[j]] * E.nr, E.nr, q, v, dv);
      acc_add(rs.blk, v);
      if ((ns & 7) == 0) bsum_fold(rs);
    }
  }
  if (!valid) return;
  const double rho = to_double(bsum_value(rs));
  ens[i] = ns;
  const int a = E.map[type[i]];
  double F, dF;
  herm(E.F + (size_t)a * E.nrho, E.nrho, rho * E.inv_drho, F, dF);
  dF *= E.inv_drho;
  if (rho > E.rho_max) F += dF * (rho - E.rho_max);
  fp[i] = dF;
  const df g = from_double(dF * E.inv_dr);
  fpd[i] = make_float2(g.hi, g.lo);
  energy[i] = F;
}

// k_eam_force with the pair arithmetic in double-float: per pair r, 1/r,
// the Hermite tables f_b, f_a and z2r = r phi, dE/dr and (dE/dr / r) e in
// df64, the force and 1/2 sum phi in blocked sums
__global__ void __launch_bounds__(128)
    k_eam_force_df(StepParams P, EamParams E, const D4 *__restrict__ x, const int *__restrict__ type,
                   const unsigned *__restrict__ epj, const int *__restrict__ ens, const float2 *__restrict__ fpd,
                   const D4 *__restrict__ fext, D4 *__restrict__ f, double *__restrict__ energy,
                   const float4 *__restrict__ rec, const int4 *__restrict__ atom_bin) {
  using namespace df64;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const D4 xi = x[i];
  int4 Bi = make_int4(0, 0, 0, 0);
  float4 rh = make_float4(0.f, 0.f, 0.f, 0.f), rl = rh;
  if (rec) {
    Bi = atom_bin[i];
    rh = rec[2 * (size_t)i];
    rl = rec[2 * (size_t)i + 1];
  }
  const int a = E.map[type[i]];
  const float2 gi = fpd[i];
  const df fpi{gi.x, gi.y}, inv_dr{E.inv_dr_hi, E.inv_dr_lo};
  bsum sx = bsum_zero(), sy = bsum_zero(), sz = bsum_zero(), se = bsum_zero();
  const int ns = ens[i];
  for (int k = 0; k < ns; ++k) {
    const unsigned u = epj[(size_t)k * P.n + i];
    const unsigned j = u & IDX_MASK;
    df dx, dy, dz;
    pair_e_df(P, rec, Bi, rh, rl, xi, x, j, u >> IDX_BITS, dx, dy, dz);
    const df r2 = dot3(dx, dy, dz, dx, dy, dz);
    const df r = df64::sqrt(r2, rsqrt_estimate(r2.hi));
    const df rinv = recip(r, rcp_estimate(r.hi));
    const df q = mul(r, inv_dr);
    const int b = E.map[type[j]];
    df fb, dfb, fa, dfa, z, dzz;
    herm_df(E.fd + 2 * (size_t)b * E.nr, E.nr, q, fb, dfb);
    dfa = dfb;
    if (a != b) herm_df(E.fd + 2 * (size_t)a * E.nr, E.nr, q, fa, dfa);
    const int hi = a > b ? a : b, lo = a > b ? b : a;
    herm_df(E.zd + 2 * (size_t)(hi * (hi + 1) / 2 + lo) * E.nr, E.nr, q, z, dzz);
    const df phi = mul(z, rinv);
    const df dphi = mul(sub(mul(dzz, inv_dr), phi), rinv);
    const float2 gj = fpd[j];
    const df dEdr = add(add(mul(fpi, dfb), mul(df{gj.x, gj.y}, dfa)), dphi);
    const df s = mul(dEdr, rinv);
    acc_fma(sx.blk, s, dx);
    acc_fma(sy.blk, s, dy);
    acc_fma(sz.blk, s, dz);
    acc_add(se.blk, df{0.5f * phi.hi, 0.5f * phi.lo});
    if ((k & 7) == 7) {
      bsum_fold(sx);
      bsum_fold(sy);
      bsum_fold(sz);
      bsum_fold(se);
    }
  }
  D4 out{to_double(bsum_value(sx)), to_double(bsum_value(sy)), to_double(bsum_value(sz)), 0.0};
  if (fext) {
    const D4 g = fext[i];
    out.x += g.x;
    out.y += g.y;
    out.z += g.z;
  }
  f[i] = out;
  energy[i] += to_double(bsum_value(se));
}

// sum of the per-atom energies, one block, fixed order
__global__ void k_eam_energy_sum(const double *__restrict__ e, int n, double *__restrict__ out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += e[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

EamParams eam_params(const eph_ctx *c) {
  const EamDevice *d = c->eam;
  EamParams E;
  E.F = d->F.p;
  E.f = d->f.p;
  E.z2r = d->z2r.p;
  E.nel = d->host.nel;
  E.nrho = (int)d->host.nrho;
  E.nr = (int)d->host.nr;
  E.inv_drho = 1.0 / d->host.drho;
  E.inv_dr = 1.0 / d->host.dr;
  E.rho_max = d->host.drho * (double)(d->host.nrho - 1);
  E.rc2 = d->host.rc * d->host.rc;
  E.rc2_band = (float)d->rc2_band;
  E.fd = d->fd.p;
  E.zd = d->zd.p;
  const df64::df idr = df64::from_double(E.inv_dr), rc2 = df64::from_double(E.rc2);
  E.inv_dr_hi = idr.hi;
  E.inv_dr_lo = idr.lo;
  E.rc2_hi = rc2.hi;
  E.rc2_lo = rc2.lo;
  std::memcpy(E.map, d->map, sizeof(E.map));
  return E;
}

// The Hermite tables in FP64 (D4 {c0, c1, c2, c3} per interval) and, with
// df not NULL, as double-floats (float4 hi parts, float4 lo parts per
// interval; each coefficient the nearest float plus the nearest float to
// the rest)
int upload_table(eph_ctx *c, DevBuf<D4> &dst, const std::vector<std::vector<double>> &tabs,
                 DevBuf<float4> *dfo = nullptr) {
  std::vector<double> all;
  for (const auto &t : tabs) {
    std::vector<double> coef;
    hermite_table(t, coef);
    all.insert(all.end(), coef.begin(), coef.end());
  }
  CUDA_TRY(c, dst.alloc(all.size() / 4));
  CUDA_TRY(c, cudaMemcpy(dst.p, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
  if (dfo) {
    std::vector<float> split(2 * all.size());
    for (size_t m = 0; m < all.size() / 4; ++m)
      for (int k = 0; k < 4; ++k) {
        const df64::df v = df64::from_double(all[4 * m + k]);
        split[8 * m + k] = v.hi;
        split[8 * m + 4 + k] = v.lo;
      }
    CUDA_TRY(c, dfo->alloc(all.size() / 2));
    CUDA_TRY(c, cudaMemcpy(dfo->p, split.data(), split.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  return EPH_OK;
}

}  // namespace

namespace ephgb {
namespace ctxi {

void eam_free(eph_ctx *c) {
  delete c->eam;
  c->eam = nullptr;
}

int eam_resize(eph_ctx *c) {
  EamDevice *d = c->eam;
  if (!d || d->fp.n == (size_t)c->n) return EPH_OK;
  const size_t N = (size_t)c->n;
  CUDA_TRY(c, d->fp.alloc(N));
  CUDA_TRY(c, d->energy.alloc(N));
  CUDA_TRY(c, d->ns.alloc(N));
  CUDA_TRY(c, d->fpd.alloc(N));
  CUDA_TRY(c, cudaMemset(d->energy.p, 0, sizeof(double) * N));
  // pair rows from the number density: twice the cut-off sphere, plus slack
  const double dens = (double)c->n / (c->prd[0] * c->prd[1] * c->prd[2]);
  const double rc = d->host.rc;
  d->kcap = ((int)std::ceil(2.0 * dens * 4.18879020478639 * rc * rc * rc + 32.0) + 7) / 8 * 8;
  CUDA_TRY(c, d->pj.alloc((size_t)d->kcap * N));
  return EPH_OK;
}

bool eam_pair_list(const eph_ctx *c, const unsigned **pj, const int **ns) {
  const EamDevice *d = c->eam;
  if (!d || !d->pj.p || !d->ns.p || d->ns.n < (size_t)c->n) return false;
  // every pair within the fix's FP32 candidate threshold must be in the list
  // (within the EAM cut-off, by the FP64 test), with room for FP32 rounding
  if (!((double)c->P.rc2_band * (1.0 + 1e-5) < d->host.rc * d->host.rc)) return false;
  *pj = d->pj.p;
  *ns = d->ns.p;
  return true;
}

int launch_eam(eph_ctx *c) {
  EamDevice *d = c->eam;
  const EamParams E = eam_params(c);
  const int nb = nblocks(c->n);
  if (d->fp.n < (size_t)c->n) return fail(c, EPH_ERR_STATE, "pair force buffers not sized for the atoms");
  PhaseScope ps(c, EPH_PHASE_PAIR);
  ps.launched(2);
  const D4 *fext = c->have_fext ? c->fext.p : nullptr;
  if (c->mode == EPH_MODE_FAST && c->pair_arith == EPH_PAIRS_DF64) {
    // the atoms' df64 records of this step's bins, where k_bin wrote them
    const float4 *rec = ctxi::df_active(c) ? c->dfrec.p : nullptr;
    k_eam_density_df<<<nb, BLOCK, 0, c->stream>>>(c->P, E, c->x.p, c->type.p, c->bin_count.p, c->bins.p,
                                                   c->atom_bin.p, c->atom_off.p, d->pj.p, d->ns.p, d->kcap, d->fp.p,
                                                   d->fpd.p, d->energy.p, c->d_err.p, rec);
    k_eam_force_df<<<nb, BLOCK, 0, c->stream>>>(c->P, E, c->x.p, c->type.p, d->pj.p, d->ns.p, d->fpd.p, fext,
                                                 c->f.p, d->energy.p, rec, c->atom_bin.p);
  } else {
    k_eam_density<<<nb, BLOCK, 0, c->stream>>>(c->P, E, c->x.p, c->type.p, c->bin_count.p, c->bins.p,
                                                c->atom_bin.p, c->atom_off.p, d->pj.p, d->ns.p, d->kcap, d->fp.p,
                                                d->energy.p, c->d_err.p);
    k_eam_force<<<nb, BLOCK, 0, c->stream>>>(c->P, E, c->x.p, c->type.p, d->pj.p, d->ns.p, d->fp.p, fext, c->f.p,
                                              d->energy.p);
  }
  CUDA_TRY(c, cudaGetLastError());
  c->eam_list_fresh = true;  // this step's pairs: the fix's density sweep may read them
  return EPH_OK;
}

}  // namespace ctxi
}  // namespace ephgb

extern "C" {

int eph_set_pair_eam(eph_ctx *c, const char *path, int ntypes, const char *const *elements) {
  if (!c || !path || !elements) return EPH_ERR_ARG;
  if (c->n > 0) return ctxi::fail(c, EPH_ERR_STATE, "set the pair force before the atoms (eph_set_atoms)");
  if (ntypes != c->ntypes) return ctxi::fail(c, EPH_ERR_ARG, "one setfl element name per atom type");
  EamDevice *d = new (std::nothrow) EamDevice();
  if (!d) return EPH_ERR_ARG;
  std::string e = d->host.load(path);
  if (!e.empty()) {
    delete d;
    return ctxi::fail(c, EPH_ERR_FILE, e);
  }
  for (int t = 1; t <= ntypes; ++t) {
    int m = -1;
    for (int k = 0; k < d->host.nel; ++k)
      if (d->host.names[k] == elements[t - 1]) m = k;
    if (m < 0) {
      delete d;
      return ctxi::fail(c, EPH_ERR_ARG, std::string("element ") + elements[t - 1] + " not in the setfl file");
    }
    d->map[t] = m;
  }
  ctxi::eam_free(c);
  ctxi::drop_list(c);  // the pair force needs this step's bins every step
  c->eam = d;
  int r;
  CUDA_TRY(c, cudaSetDevice(c->device));
  if ((r = upload_table(c, d->F, d->host.F)) || (r = upload_table(c, d->f, d->host.f, &d->fd)) ||
      (r = upload_table(c, d->z2r, d->host.z2r, &d->zd)))
    return r;
  CUDA_TRY(c, d->esum.alloc(1));
  d->rc2_band = d->host.rc * d->host.rc * (1.0 + 1e-4);
  // the bins must hold every pair within the larger of the two cutoffs (all
  // of their geometry: the FP64, FP32 and double-float bin edges)
  if ((r = ctxi::set_bin_geometry(c, std::max(c->beta.r_cutoff, d->host.rc))))
    return ctxi::fail(c, EPH_ERR_ARG, "box edge shorter than three EAM cutoffs");
  c->bin_count.free();
  c->bcap = 0;
  ctxi::drop_graph(c);
  c->buf_gen += 1;
  return EPH_OK;
}

int eph_pair_energy(eph_ctx *c, double *E) {
  if (!c || !E) return EPH_ERR_ARG;
  *E = 0.0;
  if (!c->eam || !c->eam->energy.p) return EPH_OK;
  k_eam_energy_sum<<<1, 256, 0, c->stream>>>(c->eam->energy.p, c->n, c->eam->esum.p);
  CUDA_TRY(c, cudaMemcpyAsync(E, c->eam->esum.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return ctxi::check_device(c);
}

}  // extern "C"
