// Pair helpers of the df64 sweeps, shared by the forward sweeps
// (eph_kernels.cuh) and the reverse sweeps of the adjoint (eph_adjoint.cu):
// the rho(r^2) spline of the local-form df64 tables and a pair's
// displacement from double-float coordinates.
#pragma once

#include "eph_device.cuh"
#include "eph_df64.cuh"

namespace ephgb {

// rho_e(x) of element e at x = r^2 from the local-form df64 table: knot
// k = floor(x / dx) from the FP32 quotient, moved by one where the df64
// offset t = x - k dx falls outside [0, dx) (so the interval is that of the
// df64 x, not of its FP32 part), then y = a' + t (b' + t (c' + t d')).  The
// local form was expanded from the reference's absolute-form cubic on the
// host (the same polynomial), so the value is the reference's spline to
// ~1e-14 without the cancellation of evaluating the absolute form at large x.
__device__ __forceinline__ df64::df spline_rho_df(const StepParams &P, int e, df64::df x, unsigned *err) {
  using namespace df64;
  // floor(x / dx) from the FP32 quotient without a conversion instruction
  // (floor_estimate; off by one at most, settled by the sign of t below)
  const float q = x.hi * P.inv_dxr_f;
  const float kr = floor_estimate(q);
  int k = floor_estimate_int(kr);
  float p, pe;
  two_prod(kr, P.dxr_hi, p, pe);
  pe = fmaf(kr, P.dxr_lo, pe);
  float th, te;
  two_sum(x.hi, -p, th, te);
  df t = make(th, (te + x.lo) - pe);
  const df dx = df{P.dxr_hi, P.dxr_lo};
  if (t.hi < 0.0f) {
    k -= 1;
    t = add(t, dx);
  } else if (!(t.hi < P.dxr_hi)) {
    k += 1;
    t = sub(t, dx);
  }
  if (k < 0 || k >= P.n_rho) {
    atomicOr(err, ERR_SPLINE_RANGE);
    k = k < 0 ? 0 : P.n_rho - 1;
  }
  const float4 *c = P.tab_rho_df + 2 * ((size_t)e * P.n_rho + k);
  const float4 hi = c[0], lo = c[1];
  return horner(df{hi.x, lo.x}, df{hi.y, lo.y}, df{hi.z, lo.z}, df{hi.w, lo.w}, t);
}

// The same spline's value and derivative d rho / d x at x, and its knot k
// (the interval whose coefficients the value comes from)
__device__ __forceinline__ void spline_rho_df_vd(const StepParams &P, int e, df64::df x, df64::df &val,
                                                 df64::df &der, int &k) {
  using namespace df64;
  const float q = x.hi * P.inv_dxr_f;
  const float kr = floor_estimate(q);
  k = floor_estimate_int(kr);
  float p, pe;
  two_prod(kr, P.dxr_hi, p, pe);
  pe = fmaf(kr, P.dxr_lo, pe);
  float th, te;
  two_sum(x.hi, -p, th, te);
  df t = make(th, (te + x.lo) - pe);
  const df dx = df{P.dxr_hi, P.dxr_lo};
  if (t.hi < 0.0f) {
    k -= 1;
    t = add(t, dx);
  } else if (!(t.hi < P.dxr_hi)) {
    k += 1;
    t = sub(t, dx);
  }
  k = k < 0 ? 0 : (k >= P.n_rho ? P.n_rho - 1 : k);
  const float4 *c = P.tab_rho_df + 2 * ((size_t)e * P.n_rho + k);
  const float4 hi = c[0], lo = c[1];
  const df a0{hi.x, lo.x}, a1{hi.y, lo.y}, a2{hi.z, lo.z}, a3{hi.w, lo.w};
  val = horner(a0, a1, a2, a3, t);
  // d/dt of a' + b' t + c' t^2 + d' t^3
  der = fma(t, fma(t, mul(df{3.0f, 0.0f}, a3), mul(df{2.0f, 0.0f}, a2)), a1);
}

// displacement component d w + (o_j - o_i) of a pair from the bin offsets
__device__ __forceinline__ df64::df pair_disp(int d, float ojh, float ojl, float oih, float oil, float wh,
                                              float wl) {
  using namespace df64;
  float s, se;
  two_sum(ojh, -oih, s, se);
  const float dw = (float)d * wh;  // exact: d is -1, 0 or 1
  float s2, se2;
  two_sum(s, dw, s2, se2);
  return make(s2, ((ojl - oil) + se) + (se2 + (float)d * wl));
}


}  // namespace ephgb
