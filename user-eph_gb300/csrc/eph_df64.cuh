// Double-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of
// two IEEE binary32 numbers, |lo| <= ulp(hi)/2 when normalised, which carries
// 48 significand bits (unit roundoff u ~ 2^-48 = 3.6e-15).  Built only from
// correctly rounded FP32 additions, multiplications and fused multiply-adds,
// following the error-free transformations of T. J. Dekker, "A floating-point
// technique for extending the available precision", Numer. Math. 18 (1971)
// 224-242, and D. E. Knuth, TAOCP vol. 2, 4.2.2 (TwoSum), with the FMA form of
// the exact product (J.-M. Muller et al., Handbook of Floating-Point
// Arithmetic, 2nd ed., ch. 4-5).
//
// Why: GB300 issues FP32 at 128 lanes per SM per clock and FP64 at 2, so the
// FAST-mode pair sweeps, which were bound by FP64 issue, do their per-pair
// arithmetic here instead; per-atom work (splines of rho_i, alpha, the
// epilogues) stays FP64.
//
// The translation units are compiled without FP contraction (-fmad=false),
// which these transformations need: every a * b + c below rounds twice unless
// written as fmaf.  Host and device versions are the same code (the host
// build is the CPU check of the precision, tests/native/df64_check.cpp).
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define DF_FN __host__ __device__ __forceinline__
#else
#define DF_FN inline
#endif

namespace df64 {

struct df {
  float hi, lo;
};

// s + e = a + b exactly (Knuth's TwoSum, no precondition)
DF_FN void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker's FastTwoSum)
DF_FN void fast_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  e = b - (s - a);
}

// p + e = a * b exactly (the FMA gives the product's rounding error)
DF_FN void two_prod(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

DF_FN df make(float hi, float lo) {
  df r;
  fast_two_sum(hi, lo, r.hi, r.lo);
  return r;
}

#if defined(__CUDA_ARCH__)
// double -> nearest float by integer work on the bits (the conversion
// instruction would take an FP64-pipe slot): the 29 dropped significand bits
// rounded half away from zero, the exponent rebased; |v| below 2^-126 gives
// 0 and no value here reaches 2^128.
__device__ __forceinline__ float round_to_float_bits(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v) + 0x10000000ull;
  const unsigned hi = (unsigned)(b >> 32);
  const int e = (int)((hi >> 20) & 0x7ffu);
  if (e < 897) return __uint_as_float(hi & 0x80000000u);
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)(e - 896) << 23) | ((hi & 0xfffffu) << 3) |
                         ((unsigned)b >> 29));
}

// float -> double exactly by integer work on the bits (zero and normal
// floats; the df64 parts here are never subnormal)
__device__ __forceinline__ double widen_bits(float f) {
  const unsigned u = __float_as_uint(f);
  if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((unsigned long long)u << 32));
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long e = (unsigned long long)(((u >> 23) & 0xffu) + 896u) << 52;
  const unsigned long long m = (unsigned long long)(u & 0x7fffffu) << 29;
  return __longlong_as_double((long long)(s | e | m));
}
#endif

// the nearest df64 to x (hi the nearest float, lo the nearest float to the
// rest, which hi subtracts exactly); one FP64 addition on the device
DF_FN df from_double(double x) {
  df r;
#if defined(__CUDA_ARCH__)
  r.hi = round_to_float_bits(x);
  r.lo = round_to_float_bits(x - widen_bits(r.hi));
#else
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
#endif
  return r;
}

DF_FN double to_double(df a) {
#if defined(__CUDA_ARCH__)
  return widen_bits(a.hi) + widen_bits(a.lo);
#else
  return (double)a.hi + (double)a.lo;
#endif
}

DF_FN df neg(df a) { return df{-a.hi, -a.lo}; }

// a + b within ~2 u of |a| + |b| (Dekker's add; the error relative to the sum
// grows only where a + b cancels)
DF_FN df add(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  df r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

DF_FN df sub(df a, df b) { return add(a, neg(b)); }

// a * b, relative error ~3 u
DF_FN df mul(df a, df b) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  df r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}

// a * b + c
DF_FN df fma(df a, df b, df c) { return add(mul(a, b), c); }

// a < b for normalised values
DF_FN bool lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// 1/a for a > 0 in the FP32 normal range: the FP32 reciprocal y0 and one
// Newton-Raphson step y0 + y0 (1 - a y0) with the residual formed exactly
// (a.hi y0 by TwoProd; 1 - p is exact since p = 1 within a few ulps): the
// relative error is that of y0 squared (y0 correctly rounded on the host,
// within 2^-23 on the device: ~2^-46 = 1.4e-14) plus ~2 u.
DF_FN df recip(df a, float y0) {
  float p, pe;
  two_prod(a.hi, y0, p, pe);
  const float t = ((1.0f - p) - pe) - a.lo * y0;
  df r;
  fast_two_sum(y0, y0 * t, r.hi, r.lo);
  return r;
}

// FP32 reciprocal estimate: the hardware's rcp.approx.ftz.f32 (within 2^-23)
// on the device, the correctly rounded quotient on the host
DF_FN float rcp_estimate(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}

// FP32 reciprocal square root estimate: rsqrt.approx.ftz.f32 on the device,
// 1 / sqrtf on the host
DF_FN float rsqrt_estimate(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / sqrtf(x);
#endif
}

// sqrt(a) for a > 0 in the FP32 normal range from y ~ 1/sqrt(a.hi): the
// estimate s0 = a.hi y, then twice s + y (a - s^2) / 2 (Karp and Markstein's
// form of Newton's iteration, "High-precision division and square root",
// ACM TOMS 23 (1997)) with the first residual formed exactly by TwoProd; the
// second step takes the error from ~(2^-23)^2 to a few u
DF_FN df sqrt(df a, float y) {
  const float s0 = a.hi * y;
  float p, pe;
  two_prod(s0, s0, p, pe);
  const float res = ((a.hi - p) - pe) + a.lo;
  df s;
  fast_two_sum(s0, 0.5f * y * res, s.hi, s.lo);
  const df r2 = sub(a, mul(s, s));
  return add(s, df{0.5f * y * r2.hi, 0.0f});
}

// round(q - 0.5) as an integer-valued float for 0 <= q < 2^22 without a
// conversion instruction: adding 1.5 * 2^23 puts the sum where FP32 spacing
// is exactly 1, so the addition rounds to an integer (ties to even), and
// subtracting the constant again is exact.  The result is floor(q) or, at
// an exact integer q, one less; it is never negative.  The integer itself is
// the low bits of (result + 1.5 * 2^23).
DF_FN float floor_estimate(float q) { return ((q - 0.5f) + 12582912.0f) - 12582912.0f; }
DF_FN int floor_estimate_int(float kr) {
  union {
    float f;
    int i;
  } u;
  u.f = kr + 12582912.0f;
  return u.i - 0x4B400000;
}

// A running sum of products kept as an unnormalised pair: hi carries the
// rounded sum, lo collects every rounding error (each product's by TwoProd,
// each addition's by TwoSum) -- the cascaded "Dot2" of Ogita, Rump and Oishi
// ("Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005)
// 1955-1988), extended to df64 factors.  Its lo part rounds at ~u |sum| per
// addition, so its error grows with the number of terms: use it for a few.
struct acc {
  float hi, lo;
};

DF_FN acc acc_zero() { return acc{0.0f, 0.0f}; }

// s += a * b
DF_FN void acc_fma(acc &s, df a, df b) {
  float p, pe;
  two_prod(a.hi, b.hi, p, pe);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  float t, te;
  two_sum(s.hi, p, t, te);
  s.hi = t;
  s.lo += te + pe;
}

// s += a
DF_FN void acc_add(acc &s, df a) {
  float t, te;
  two_sum(s.hi, a.hi, t, te);
  s.hi = t;
  s.lo += te + a.lo;
}

DF_FN df acc_value(acc s) {
  df r;
  fast_two_sum(s.hi, s.lo, r.hi, r.lo);
  return r;
}

// Blocked summation: a cascaded acc takes a handful of products, then folds
// into a normalised df64 total by one Dekker addition.  With blocks of 8, 42
// products of random sign sum to ~1.5 u of sum |terms| (one cascaded acc over
// all 42: ~11 u; FP64 recursive summation: ~0.13 u), measured by
// tests/native/df64_check.cpp.
struct bsum {
  acc blk;
  df tot;
};

DF_FN bsum bsum_zero() { return bsum{acc{0.0f, 0.0f}, df{0.0f, 0.0f}}; }

DF_FN void bsum_fold(bsum &s) {
  s.tot = add(s.tot, acc_value(s.blk));
  s.blk = acc{0.0f, 0.0f};
}

DF_FN df bsum_value(bsum s) { return add(s.tot, acc_value(s.blk)); }

// a . b of two df64 3-vectors, normalised
DF_FN df dot3(df ax, df ay, df az, df bx, df by, df bz) {
  acc s = acc_zero();
  acc_fma(s, ax, bx);
  acc_fma(s, ay, by);
  acc_fma(s, az, bz);
  return acc_value(s);
}

// Cubic c0 + t (c1 + t (c2 + t c3)), Horner in df64 (the spline tables in
// local form, t measured from the interval's knot, so the terms decrease and
// nothing cancels).
DF_FN df horner(df c0, df c1, df c2, df c3, df t) { return fma(t, fma(t, fma(t, c3, c2), c1), c0); }

}  // namespace df64
