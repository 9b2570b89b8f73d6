// Types, step constants and device helpers shared by the sm_103a kernels of
// the fix-eph path (eph_kernels.cuh) and of its adjoint (eph_adjoint.cu).
// Everything here is a type or an inline device function, so several
// translation units may include it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ephgb {

struct __align__(32) D4 {
  double x, y, z, w;
};

struct __align__(16) BinEntry {
  unsigned idx;  // atom index | wrap code << 27
  float ox, oy, oz;  // offset of the atom inside its unwrapped bin
};

struct __align__(16) U128 {
  unsigned long long lo, hi;  // two's-complement 128-bit fixed point, 2^-64 units
};

constexpr int KMAX = 128;   // largest pair capacity (rows of one atom in the pair arrays)
constexpr int CAND_SMEM = 48;  // candidate rows of one atom kept in shared memory
constexpr unsigned IDX_BITS = 27;
constexpr unsigned IDX_MASK = (1u << IDX_BITS) - 1u;
constexpr unsigned CODE_NOSHIFT = 13;  // (0,0,0) image of the 3x3x3 code
constexpr int LIST_FMAX = 32;          // moved atoms handled between two list builds (one warp)

enum : unsigned {
  ERR_BIN_OVERFLOW = 1u,
  ERR_PAIR_OVERFLOW = 2u,
  ERR_DRIFT = 4u,
  ERR_Q_RANGE = 8u,
  ERR_SPLINE_RANGE = 16u,
  ERR_TIMEOUT = 32u
};

enum : int { CNT_RHO_CUTOFF = 0, CNT_T_CLAMP = 1, CNT_BUILD = 2, CNT_WRAP = 3, NCOUNTERS = 4 };

// Everything a step's kernels read besides the big arrays.
struct StepParams {
  int n;
  int flags;
  int groupbit;
  int nelem;
  double lo[3], hi[3], prd[3];
  double rc2;         // r_cutoff^2 (eph_beta.h:85)
  float rc2_band;     // FP32 candidate threshold, rc^2 (1 + 1e-4)
  int nb[3];          // bins per axis (>= 3), bin edge >= r_cutoff (1 + 5e-5)
  double inv_w[3], w[3];
  float wf[3];
  int bcap, kcap;
  // candidate-list reuse (FAST mode, one lane per atom): the candidates within
  // r_list = r_cutoff + s stay complete for every pair of atoms that moved
  // less than s/2 since the list was built (bins then have edge >= r_list)
  float rl2_band;     // r_list^2 (1 + 1e-4): candidates kept in the list
  float rmark2_band;  // (r_cutoff + s/2)^2 (1 + 1e-4): atoms this close to a moved atom search afresh
  double lslow2;      // (s/2)^2: squared displacement from which an atom counts as moved
  double half_prd[3];
  float half_prdf[3];
  int lcap;           // rows of the candidate list
  // FAST pair sums in df64 (k_density_df, k_forces_df): the bin widths, the
  // cut-off and the rho(r^2) knot spacing as double-floats (hi, lo), and the
  // rho(r^2) tables in local form about each knot (two float4 per knot:
  // hi and lo parts of a', b', c', d' with y = a' + t (b' + t (c' + t d')),
  // t = x - k dx)
  float w_hi[3], w_lo[3];
  float prd_hi[3], prd_lo[3];  // box edges (the adjoint's df64 sweeps: periodic images)
  float rc2_hi, rc2_lo;
  float dxr_hi, dxr_lo, inv_dxr_f;
  const float4 *tab_rho_df;
  // splines: tables of element e start at e * n_knots
  const D4 *tab_rho_r_sq;
  const D4 *tab_beta;
  const D4 *tab_alpha;
  double inv_dr_sq, inv_drho;
  int n_rho, n_beta;
  double rho_cutoff;
  // integrator and forces
  double dtv, dt, eta, triggersq;
  double dtfm[65];  // dtf / mass[type], type 1..64 (fix_eph.cpp:314)
  int type_map[65];  // LAMMPS type -> element
  // grid
  long gnx, gny, gnz, ncells;
  double gx0, gy0, gz0, gdx, gdy, gdz;
  double prescale;  // dV * dt (eph_fdm.h:176)
  // coloured noise (fix_eph_coloured_exp.cpp:190): exponential memory on
  // f_EPH and f_RNG, zeta = 1 - exp(-dt / tau0)
  int coloured;
  double zeta;
  // random numbers: Philox key = seed, counter = (atom, *step) with *step the
  // number of post_force calls so far, kept on the device so a captured
  // step replays with fresh numbers
  unsigned seed;
  unsigned long long *step;
};

// ------------------------------------------------------------------ helpers

// v > 0 and w < c for non-negative c, on the bit patterns: integer compares
// keep these tests off the FP64 pipe (IEEE order of non-negative doubles is
// the order of their bits).
__device__ __forceinline__ bool pos_double(double v) { return __double_as_longlong(v) > 0; }

// Wait until the grids this one depends on programmatically have completed
// and their memory is visible (griddepcontrol.wait; returns at once for a
// kernel launched without a programmatic dependency).
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ bool below(double v, double c) { return __double_as_longlong(v) < __double_as_longlong(c); }

// (size_t)y for a non-negative double y, by integer work on its bits (the
// conversion instruction runs on the FP64 pipe); y >= 2^53, negative or NaN
// gives ~0ull.
__device__ __forceinline__ unsigned long long trunc_index(double y) {
  const long long b = __double_as_longlong(y);
  const int e = (int)((b >> 52) & 0x7ff);
  if (b < 0 || e > 1075) return ~0ull;
  if (e < 1023) return 0ull;
  return (((unsigned long long)b & ((1ull << 52) - 1ull)) | (1ull << 52)) >> (1075 - e);
}

// v truncated to float by integer work on its bits (the conversion
// instruction would run on the FP64 pipe): exponent rebased, top 23 mantissa
// bits; |v| < 2^-126 gives 0.  Good to 2^-23 relative (truncated): for image
// tests, not for arithmetic.
__device__ __forceinline__ float float_bits(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hi = (unsigned)(b >> 32);
  int e = (int)((hi >> 20) & 0x7ffu);
  if (e < 897) return 0.f;
  e = e > 1150 ? 1150 : e;
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)(e - 896) << 23) | ((hi & 0xfffffu) << 3) |
                         ((unsigned)b >> 29));
}

template <bool FAST>
__device__ __forceinline__ double spline_eval(const D4 *__restrict__ tab, double inv_dx, int n, double x,
                                              unsigned *err) {
  // eph_spline.h:134-142: index floor(x/dx), value a + x(b + x(c + x d))
  unsigned long long idx = trunc_index(x * inv_dx);
  if (idx >= (unsigned long long)n) {
    atomicOr(err, ERR_SPLINE_RANGE);
    idx = (unsigned long long)(n - 1);
  }
  const D4 c = tab[idx];
  if (FAST) return fma(x, fma(x, fma(x, c.w, c.z), c.y), c.x);
  return c.x + x * (c.y + x * (c.z + x * c.w));
}

// 1/x for FAST mode, x > 0 inside the normal float range (x = r^2 here):
// x truncated to float by its bits (exponent rebased, top 23 mantissa bits),
// the FP32 hardware reciprocal estimate (rcp.approx.ftz.f32, ~2^-23), widened
// back to double by its bits, then one Newton-Raphson step
// r <- r + r (1 - x r), which squares the relative error: ~2^-44 against
// the correctly rounded 1/x.  Two FP64 instructions; the rest runs on the
// integer and FP32 pipes, which GB300 has ~60 times more of.
__device__ __forceinline__ double recip_nr(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned fb = (hi & 0x80000000u) | ((((hi >> 20) & 0x7ffu) - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(fb)));
  const unsigned rb = __float_as_uint(rf);
  const unsigned rhi = (rb & 0x80000000u) | ((((rb >> 23) & 0xffu) + 896u) << 20) | ((rb & 0x7fffffu) >> 3);
  const double r = __longlong_as_double((long long)(((unsigned long long)rhi << 32) | (unsigned long long)(rb << 29)));
  return fma(r, fma(-x, r, 1.0), r);
}

__device__ __forceinline__ double dot3(double ax, double ay, double az, double bx, double by, double bz) {
  return ax * bx + ay * by + az * bz;  // ((ax bx + ay by) + az bz), fix_eph.h:160-163
}

__device__ __forceinline__ double dot3_fma(double ax, double ay, double az, double bx, double by, double bz) {
  return fma(az, bz, fma(ay, by, ax * bx));
}

// eph_fdm.h:494-509: cell of a position, floor-wrapped into the grid
__device__ __forceinline__ long grid_index(const StepParams &P, double x, double y, double z) {
  int lx = (int)floor((x - P.gx0) / P.gdx);
  int px = (int)floor(((double)lx) / (double)P.gnx);
  lx -= px * (int)P.gnx;
  int ly = (int)floor((y - P.gy0) / P.gdy);
  int py = (int)floor(((double)ly) / (double)P.gny);
  ly -= py * (int)P.gny;
  int lz = (int)floor((z - P.gz0) / P.gdz);
  int pz = (int)floor(((double)lz) / (double)P.gnz);
  lz -= pz * (int)P.gnz;
  return (long)lx + (long)ly * P.gnx + (long)lz * P.gnx * P.gny;
}

// ---------------------------------------------------- fixed-point deposits

// Round t * 2^64 to the nearest integer as a 128-bit two's-complement value.
// Integer work only.  |t| must stay below 2^62.
__device__ __forceinline__ U128 to_fixed(double t, unsigned *err) {
  U128 r{0ull, 0ull};
  const unsigned long long bits = (unsigned long long)__double_as_longlong(t);
  const int e = (int)((bits >> 52) & 0x7ffu);
  if (e == 0) return r;  // zero or subnormal: far below one unit
  const unsigned long long m = (bits & ((1ull << 52) - 1ull)) | (1ull << 52);
  const int sh = e - 1011;  // value * 2^64 = m * 2^(e - 1075 + 64)
  unsigned long long lo, hi;
  if (sh >= 74) {
    atomicOr(err, ERR_Q_RANGE);
    return r;
  } else if (sh >= 64) {
    lo = 0ull;
    hi = m << (sh - 64);
  } else if (sh > 11) {
    lo = m << sh;
    hi = m >> (64 - sh);
  } else if (sh >= 0) {
    lo = m << sh;
    hi = 0ull;
  } else if (sh > -54) {
    const int s = -sh;
    lo = (m + (1ull << (s - 1))) >> s;  // round half up on the magnitude
    hi = 0ull;
  } else {
    return r;
  }
  if ((long long)bits < 0) {  // negate: ~v + 1
    lo = ~lo;
    hi = ~hi;
    lo += 1ull;
    if (lo == 0ull) hi += 1ull;
  }
  r.lo = lo;
  r.hi = hi;
  return r;
}

__device__ __forceinline__ U128 add128(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
  return r;
}

__device__ __forceinline__ void atomic_add128(U128 *dst, U128 v) {
  const unsigned long long old = atomicAdd(&dst->lo, v.lo);
  const unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
  atomicAdd(&dst->hi, v.hi + carry);
}

__device__ __forceinline__ double from_fixed(U128 v) {
  // v * 2^-64 = (signed hi) + lo * 2^-64
  return (double)(long long)v.hi + (double)v.lo * 5.421010862427522170037264e-20;
}

__device__ __forceinline__ U128 shfl_down128(U128 v, int d) {
  U128 r;
  r.lo = __shfl_down_sync(0xffffffffu, v.lo, d);
  r.hi = __shfl_down_sync(0xffffffffu, v.hi, d);
  return r;
}

// ------------------------------------------------------------ random numbers

// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11): ten rounds of two
// 32x32->64 multiplies with a Weyl-sequence key schedule.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k.x += W0;
      k.y += W1;
    }
    const unsigned hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const unsigned hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

// A uniform in (0, 1) with 53 random bits from two 32-bit words:
// (27 bits of a, 26 of b, + 1/2) * 2^-53.
__device__ __forceinline__ double uniform53(unsigned a, unsigned b) {
  const unsigned long long m = ((unsigned long long)(a >> 5) << 26) | (unsigned long long)(b >> 6);
  return ((double)m + 0.5) * 1.1102230246251565404236316680908203125e-16;
}

// Three standard normal deviates for atom i at step s: Box-Muller in FP64 on
// 53-bit uniforms (two Philox4x32-10 blocks, counters differing in their last
// word), as the reference draws FP64 deviates from RanMars
// (fix_eph.cpp:854-860).  CUDA's FP64 log, sqrt and sincospi.
__device__ __forceinline__ void gaussian3(unsigned seed, unsigned long long step, unsigned i, double *g) {
  const uint2 key = make_uint2(seed, 0x9e3779b9u);
  const uint4 r = philox4x32_10(make_uint4(i, (unsigned)step, (unsigned)(step >> 32), 0x45504847u), key);
  const uint4 q = philox4x32_10(make_uint4(i, (unsigned)step, (unsigned)(step >> 32), 0x45504848u), key);
  const double u0 = uniform53(r.x, r.y), u1 = uniform53(r.z, r.w);
  const double u2 = uniform53(q.x, q.y), u3 = uniform53(q.z, q.w);
  const double ra = sqrt(-2.0 * log(u0)), rb = sqrt(-2.0 * log(u2));
  double sa, ca;
  sincospi(2.0 * u1, &sa, &ca);
  g[0] = ra * ca;
  g[1] = ra * sa;
  g[2] = rb * cospi(2.0 * u3);
}

// ------------------------------------------------- grid parameter tables


// Temperature-dependent cells (T_dynamic): tables of the grid parameter file.
struct TdynTables {
  const unsigned char *tdyn;  // per cell, nonzero: C_e(T), kappa_e(T), E_e(T) apply
  const D4 *C_T, *K_T;        // splines of C_e and kappa_e over T (eph_fdm.h:94-95)
  const double *E_y, *E_dy;   // E_e(T) = integral of C_e dT, piecewise linear (eph_fdm.h:97-103)
  const double *rho;          // rho_e per cell
  double dT, inv_dT;
  int n;
};

// eph_linear.h:41-48
__device__ __forceinline__ double linear_eval(const TdynTables &t, double x) {
  const unsigned long long idx = trunc_index(x / t.dT);
  if (idx < (unsigned long long)t.n) {
    const double delta = x - (double)idx * t.dT;
    return t.E_y[idx] + t.E_dy[idx] * delta;
  }
  return 0.;
}

// eph_linear.h:51-60: first knot above v (upper bound), linear inverse
__device__ __forceinline__ double linear_reverse(const TdynTables &t, double v) {
  int lo = 0, hi = t.n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (!(v < t.E_y[mid]))
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo != t.n && lo > 0) {
    const int idx = lo - 1;
    return (double)idx * t.dT + 1. / t.E_dy[idx] * (v - t.E_y[idx]);
  }
  return 0.;
}


}  // namespace ephgb
