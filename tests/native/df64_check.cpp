// CPU check of the df64 arithmetic the FAST pair sweeps use
// (user-eph_gb300/csrc/eph_df64.cuh, host build of the same code): each
// operation against long double on seeded random operands, and the pair sums
// of one atom (the density sweep's M_i and S_i, the force sweep's sum) with
// realistic magnitudes, summed in blocks of 8 as the sweeps do.  Prints
// "name max_relative_error" lines.
#include <cmath>
#include <cstdio>
#include <random>

#include "eph_df64.cuh"

using namespace df64;
typedef long double ld;

static ld L(df a) { return (ld)a.hi + (ld)a.lo; }
static df D(ld x) {
  df r;
  r.hi = (float)x;
  r.lo = (float)(x - (ld)r.hi);
  return r;
}
static ld rel(ld got, ld want, ld scale) { return fabsl(got - want) / scale; }

int main() {
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.0, 1.0);
  ld e_add = 0, e_mul = 0, e_rcp = 0, e_dot = 0, e_hor = 0, e_disp = 0, e_M = 0, e_S = 0, e_w = 0, e_f = 0;
  const int N = 200000;
  for (int t = 0; t < N; ++t) {
    const ld a = (ld)U(g) * powl(2.0L, (int)(U(g) * 20)), b = (ld)U(g) * powl(2.0L, (int)(U(g) * 20));
    const df A = D(a), B = D(b);
    const ld aa = L(A), bb = L(B);
    e_add = fmaxl(e_add, rel(L(add(A, B)), aa + bb, fabsl(aa) + fabsl(bb)));
    e_mul = fmaxl(e_mul, rel(L(mul(A, B)), aa * bb, fabsl(aa * bb)));
    const ld x = 0.01L + 30.0L * (ld)P(g);
    const df X = D(x);
    e_rcp = fmaxl(e_rcp, rel(L(recip(X, rcp_estimate(X.hi))), 1.0L / L(X), 1.0L / L(X)));
    // displacement d w + (o_j - o_i) from bin offsets, as the density sweep forms it
    const double w = 4.70123456789, oi = 4.7 * P(g), oj = 4.7 * P(g);
    const int d = (int)(3 * P(g)) - 1;
    const df Oi = from_double(oi), Oj = from_double(oj), Wd = from_double(w);
    float s, se;
    two_sum(Oj.hi, -Oi.hi, s, se);
    float s2, se2;
    two_sum(s, (float)d * Wd.hi, s2, se2);
    const df E = make(s2, ((Oj.lo - Oi.lo) + se) + (se2 + (float)d * Wd.lo));
    const ld ex = (ld)d * (ld)w + ((ld)oj - (ld)oi);
    if (fabsl(ex) > 0.5L) e_disp = fmaxl(e_disp, rel(L(E), ex, fabsl(ex)));
    const df V[3] = {D(U(g)), D(U(g)), D(U(g))}, Q[3] = {D(U(g)), D(U(g)), D(U(g))};
    const ld dd = L(V[0]) * L(Q[0]) + L(V[1]) * L(Q[1]) + L(V[2]) * L(Q[2]);
    const ld sc = fabsl(L(V[0]) * L(Q[0])) + fabsl(L(V[1]) * L(Q[1])) + fabsl(L(V[2]) * L(Q[2]));
    e_dot = fmaxl(e_dot, rel(L(dot3(V[0], V[1], V[2], Q[0], Q[1], Q[2])), dd, sc));
  }
  // a spline interval in local form about its knot x0 (values ~exp(-r/0.6) at
  // r^2 = x, t = x - x0 in [0, dx)), as the density sweep evaluates it
  for (int t = 0; t < N; ++t) {
    const ld x0 = 0.5L + 20.0L * (ld)P(g), h = 0.0106L;
    const ld r0 = sqrtl(x0), y = expl(-r0 / 0.6L);
    const ld y1 = -y / (1.2L * r0), y2 = y / (2.88L * x0), y3 = -y / (10.0L * x0 * r0);
    const df c[4] = {D(y), D(y1), D(y2), D(y3)};
    const df T = D(h * (ld)P(g));
    const ld tt = L(T);
    const ld want = L(c[0]) + tt * (L(c[1]) + tt * (L(c[2]) + tt * L(c[3])));
    e_hor = fmaxl(e_hor, rel(L(horner(c[0], c[1], c[2], c[3], T)), want, fabsl(want)));
  }
  // one atom: 42 neighbours on the fcc shells, H ~ rho/r^2, thermal velocities;
  // the density sweep's M_i = sum H e e^T, S_i = sum H (e.v_j) e,
  // w_i = M_i v_i - S_i, and the force sweep's sum_j (e.W_j) H e
  const ld shells[3] = {2.489L, 3.52L, 4.311L};
  const int counts[3] = {12, 6, 24};
  const int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  for (int t = 0; t < 20000; ++t) {
    bsum M[6], S[3], F[3];
    for (int k = 0; k < 6; ++k) M[k] = bsum_zero();
    for (int k = 0; k < 3; ++k) S[k] = F[k] = bsum_zero();
    ld Ml[6] = {0}, Sl[3] = {0}, Fl[3] = {0};
    const ld vi[3] = {5 * U(g), 5 * U(g), 5 * U(g)};
    int npair = 0;
    for (int sh = 0; sh < 3; ++sh)
      for (int c = 0; c < counts[sh]; ++c) {
        ld ev[3] = {U(g), U(g), U(g)};
        const ld nn = sqrtl(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]);
        const ld r = shells[sh] + 0.05L * U(g);
        df e[3];
        ld el[3];
        for (int k = 0; k < 3; ++k) {
          e[k] = D(ev[k] / nn * r);
          el[k] = L(e[k]);
        }
        const df H = D(expl(-r / 0.6L) / (r * r));
        df h[3];
        for (int k = 0; k < 3; ++k) h[k] = mul(H, e[k]);
        const ld hl[3] = {L(H) * el[0], L(H) * el[1], L(H) * el[2]};
        for (int k = 0; k < 6; ++k) {
          acc_fma(M[k].blk, h[ij[k][0]], e[ij[k][1]]);
          Ml[k] += hl[ij[k][0]] * el[ij[k][1]];
        }
        df vj[3], Wj[3];
        for (int k = 0; k < 3; ++k) {
          vj[k] = D(5 * U(g));
          Wj[k] = D(U(g));
        }
        const df dv = dot3(e[0], e[1], e[2], vj[0], vj[1], vj[2]);
        const ld dvl = el[0] * L(vj[0]) + el[1] * L(vj[1]) + el[2] * L(vj[2]);
        const df dw = dot3(e[0], e[1], e[2], Wj[0], Wj[1], Wj[2]);
        const ld dwl = el[0] * L(Wj[0]) + el[1] * L(Wj[1]) + el[2] * L(Wj[2]);
        for (int k = 0; k < 3; ++k) {
          acc_fma(S[k].blk, dv, h[k]);
          Sl[k] += dvl * hl[k];
          acc_fma(F[k].blk, dw, h[k]);
          Fl[k] += dwl * hl[k];
        }
        if ((++npair & 7) == 0) {
          for (int k = 0; k < 6; ++k) bsum_fold(M[k]);
          for (int k = 0; k < 3; ++k) {
            bsum_fold(S[k]);
            bsum_fold(F[k]);
          }
        }
      }
    ld msc = 0;
    for (int k = 0; k < 6; ++k) msc = fmaxl(msc, fabsl(Ml[k]));
    for (int k = 0; k < 6; ++k) e_M = fmaxl(e_M, rel(to_double(bsum_value(M[k])), Ml[k], msc));
    const ld ssc = fmaxl(fabsl(Sl[0]), fmaxl(fabsl(Sl[1]), fabsl(Sl[2])));
    for (int k = 0; k < 3; ++k) e_S = fmaxl(e_S, rel(to_double(bsum_value(S[k])), Sl[k], ssc));
    // w = M v_i - S (the M-form's cancellation), in double from the df64 sums as the epilogue forms it
    const int row[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    ld wsc = 0, werr = 0;
    for (int a = 0; a < 3; ++a) {
      ld wl = -Sl[a];
      double wd = -to_double(bsum_value(S[a]));
      for (int b = 0; b < 3; ++b) {
        wl += Ml[row[a][b]] * vi[b];
        wd += to_double(bsum_value(M[row[a][b]])) * (double)vi[b];
      }
      wsc = fmaxl(wsc, fabsl(wl));
      werr = fmaxl(werr, fabsl((ld)wd - wl));
    }
    e_w = fmaxl(e_w, werr / wsc);
    const ld fsc = fmaxl(fabsl(Fl[0]), fmaxl(fabsl(Fl[1]), fabsl(Fl[2])));
    for (int k = 0; k < 3; ++k) e_f = fmaxl(e_f, rel(to_double(bsum_value(F[k])), Fl[k], fsc));
  }
  // the square root of the EAM sweeps (r from r^2), with the host's seed and
  // with seeds off by +-2^-22 relative (the device estimate's error class)
  ld e_sqrt = 0, e_sqrt_seed = 0;
  for (int t = 0; t < N; ++t) {
    const ld x = 0.01L + 60.0L * (ld)P(g);
    const df X = D(x);
    const ld want = sqrtl(L(X));
    e_sqrt = fmaxl(e_sqrt, rel(L(sqrt(X, rsqrt_estimate(X.hi))), want, want));
    const float y = rsqrt_estimate(X.hi) * (t & 1 ? 1.0f + 2.384185791015625e-7f : 1.0f - 2.384185791015625e-7f);
    e_sqrt_seed = fmaxl(e_sqrt_seed, rel(L(sqrt(X, y)), want, want));
  }
  // the spline index estimate: floor(q) or one less, never negative, for
  // 0 <= q < 2^22 (the knot counts of the beta files are far below that)
  int bad_floor = 0;
  for (int t = 0; t < N; ++t) {
    const float q = t < 1000 ? (float)t * 0.25f : (float)(4.0e6 * P(g) * P(g) * P(g));
    const float kr = floor_estimate(q);
    const int k = floor_estimate_int(kr);
    const int f = (int)floorf(q);
    if (!(kr == (float)k && k >= 0 && (k == f || k == f - 1))) ++bad_floor;
  }
  printf("floor_estimate_bad %d\n", bad_floor);
  printf("add %.3Le\nmul %.3Le\nrecip %.3Le\ndisplacement %.3Le\ndot3 %.3Le\nhorner %.3Le\n", e_add, e_mul, e_rcp,
         e_disp, e_dot, e_hor);
  printf("atom_M %.3Le\natom_S %.3Le\natom_w %.3Le\natom_force_sum %.3Le\n", e_M, e_S, e_w, e_f);
  printf("sqrt %.3Le\nsqrt_seed_2e-7 %.3Le\n", e_sqrt, e_sqrt_seed);
  return 0;
}
