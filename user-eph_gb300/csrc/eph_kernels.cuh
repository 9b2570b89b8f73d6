// sm_103a kernels of the fix-eph hot path.
//
// One thread per atom for every per-atom sweep.  The FP64 pipe of GB300
// issues about two instructions per clock per SM, so these kernels are bound
// by FP64 instruction issue, not by HBM: the design removes FP64 work
// (in-cutoff pairs compacted per step so the warps sweep them in lockstep,
// pair geometry and rho(r^2) cached once per step, alpha/beta per atom once)
// and keeps integer/FP32 work (binning, candidate tests, sorting) off the
// FP64 pipe.
//
// This translation unit is compiled with -fmad=false: in EXACT mode every
// product and sum rounds separately, in the reference's order, so forces and
// densities equal the reference's bit for bit; FAST mode writes its FMAs
// explicitly.
#pragma once

#include "eph_device.cuh"
#include "eph_df64.cuh"
#include "eph_df_pair.cuh"

namespace ephgb {

// ------------------------------------------------------------- integrator

// The half kick and drift of FixEPH::initial_integrate (fix_eph.cpp:305-328)
// for one atom of the group
template <bool FAST>
__device__ __forceinline__ void kick_drift(const StepParams &P, double dtfm, const D4 &fi, D4 &xi, D4 &vi) {
  if (FAST) {
    vi.x = fma(dtfm, fi.x, vi.x);
    vi.y = fma(dtfm, fi.y, vi.y);
    vi.z = fma(dtfm, fi.z, vi.z);
    xi.x = fma(P.dtv, vi.x, xi.x);
    xi.y = fma(P.dtv, vi.y, xi.y);
    xi.z = fma(P.dtv, vi.z, xi.z);
  } else {
    vi.x += dtfm * fi.x;
    vi.y += dtfm * fi.y;
    vi.z += dtfm * fi.z;
    xi.x += P.dtv * vi.x;
    xi.y += P.dtv * vi.y;
    xi.z += P.dtv * vi.z;
  }
}

// The half kick of FixEPH::final_integrate (fix_eph.cpp:330-348)
template <bool FAST>
__device__ __forceinline__ void kick(double dtfm, const D4 &fi, D4 &vi) {
  if (FAST) {
    vi.x = fma(dtfm, fi.x, vi.x);
    vi.y = fma(dtfm, fi.y, vi.y);
    vi.z = fma(dtfm, fi.z, vi.z);
  } else {
    vi.x += dtfm * fi.x;
    vi.y += dtfm * fi.y;
    vi.z += dtfm * fi.z;
  }
}

// FixEPH::initial_integrate (fix_eph.cpp:305-328) and the engine's rebuild
// test (an atom moved more than skin/2 since the last wrap).
template <bool FAST>
__global__ void k_initial_integrate(StepParams P, D4 *__restrict__ x, D4 *__restrict__ v,
                                    const D4 *__restrict__ f, const int *__restrict__ type,
                                    const int *__restrict__ mask, const D4 *__restrict__ xhold, int check_wrap,
                                    int *__restrict__ wrapflag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool moved = false;
  if (i < P.n) {
    D4 xi = x[i];
    if (!(P.flags & 0x08) && (mask[i] & P.groupbit)) {
      D4 vi = v[i];
      kick_drift<FAST>(P, P.dtfm[type[i]], f[i], xi, vi);
      v[i] = vi;
      x[i] = xi;
    }
    if (check_wrap) {
      const D4 h = xhold[i];
      const double dx = xi.x - h.x, dy = xi.y - h.y, dz = xi.z - h.z;
      moved = dx * dx + dy * dy + dz * dz > P.triggersq;
    }
  }
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(wrapflag, 1);
}

// FixEPH::final_integrate (fix_eph.cpp:330-348)
template <bool FAST>
__global__ void k_final_integrate(StepParams P, D4 *__restrict__ v, const D4 *__restrict__ f,
                                  const int *__restrict__ type, const int *__restrict__ mask) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n || (P.flags & 0x08) || !(mask[i] & P.groupbit)) return;
  D4 vi = v[i];
  kick<FAST>(P.dtfm[type[i]], f[i], vi);
  v[i] = vi;
}

// The hooks with the engine's host arrays (eph_initial_integrate_host,
// eph_final_integrate_host), one chunk of `count` atoms per launch (the
// pointers start at the chunk): the staged host rows (n x 3 doubles) go into
// the D4 records (x.w, the element, kept), the hook's arithmetic runs, and
// the rows the engine reads back are written to staging for the
// device->host copies -- the work of k_pack3, the hook's kernel and
// k_unpack3 in one pass.
template <bool FAST>
__global__ void k_initial_host(StepParams P, int count, const double *__restrict__ sx, const double *__restrict__ sv,
                               D4 *__restrict__ x, D4 *__restrict__ v, const D4 *__restrict__ f,
                               const int *__restrict__ type, const int *__restrict__ mask, double *__restrict__ ox,
                               double *__restrict__ ov) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const size_t r = 3 * (size_t)i;
  D4 xi = x[i];
  xi.x = sx[r];
  xi.y = sx[r + 1];
  xi.z = sx[r + 2];
  D4 vi = v[i];
  vi.x = sv[r];
  vi.y = sv[r + 1];
  vi.z = sv[r + 2];
  if (!(P.flags & 0x08) && (mask[i] & P.groupbit)) kick_drift<FAST>(P, P.dtfm[type[i]], f[i], xi, vi);
  x[i] = xi;
  v[i] = vi;
  ox[r] = xi.x;
  ox[r + 1] = xi.y;
  ox[r + 2] = xi.z;
  ov[r] = vi.x;
  ov[r + 1] = vi.y;
  ov[r + 2] = vi.z;
}

template <bool FAST>
__global__ void k_final_host(StepParams P, int count, const double *__restrict__ sf, D4 *__restrict__ f,
                             D4 *__restrict__ v, const int *__restrict__ type, const int *__restrict__ mask,
                             double *__restrict__ ov) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const size_t r = 3 * (size_t)i;
  D4 fi = f[i];
  fi.x = sf[r];
  fi.y = sf[r + 1];
  fi.z = sf[r + 2];
  f[i] = fi;
  D4 vi = v[i];
  if (!(P.flags & 0x08) && (mask[i] & P.groupbit)) {
    kick<FAST>(P.dtfm[type[i]], fi, vi);
    v[i] = vi;
  }
  ov[r] = vi.x;
  ov[r + 1] = vi.y;
  ov[r + 2] = vi.z;
}

// ------------------------------------------------------------------ binning

// LAMMPS Domain::pbc for an orthogonal box: a position into [lo, hi)
__device__ __forceinline__ void wrap_into_box(const StepParams &P, D4 &xi) {
  double *c[3] = {&xi.x, &xi.y, &xi.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double q = *c[k];
    if (q < P.lo[k]) q += P.prd[k];
    if (q >= P.hi[k]) {
      q -= P.prd[k];
      q = q > P.lo[k] ? q : P.lo[k];
    }
    *c[k] = q;
  }
}

// Wrap positions into [lo, hi) when the engine rebuilds, then drop every
// atom into its spatial bin.  A bin edge is at least the cutoff (with list
// reuse: the list radius), so all pairs inside it are found in the 27 bins
// around an atom.  Bins keep unwrapped coordinates: an atom that drifted up
// to one bin outside the box carries a wrap code and the offset from its own
// (unwrapped) bin corner.
// With a gate (candidate-list reuse): nothing unless *gate (a build step),
// no wrap (k_list_check did it), and the positions are kept in xref.
// The records of atom i for the df64 pair sums (k_density_df,
// k_density_list_df) in bins B of the current geometry: rec[2i] = {offset
// x - lo - B w, hi parts; B + 1 packed 10 bits per axis}, rec[2i+1] =
// {offset, lo parts; element}, vrec[2i], vrec[2i+1] = velocity, hi and lo.
// The offset is formed with one rounding; a pair's displacement is then
// d w + (o_j - o_i), d its bin difference.
__device__ __forceinline__ void df_records(const StepParams &P, int i, const D4 &xi, const int *B,
                                           const D4 *__restrict__ v, float4 *__restrict__ rec,
                                           float4 *__restrict__ vrec) {
  const double p[3] = {xi.x, xi.y, xi.z};
  df64::df o[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) o[k] = df64::from_double(fma(-(double)B[k], P.w[k], p[k] - P.lo[k]));
  const unsigned packed = (unsigned)(B[0] + 1) | ((unsigned)(B[1] + 1) << 10) | ((unsigned)(B[2] + 1) << 20);
  rec[2 * (size_t)i] = make_float4(o[0].hi, o[1].hi, o[2].hi, __uint_as_float(packed));
  rec[2 * (size_t)i + 1] = make_float4(o[0].lo, o[1].lo, o[2].lo, __int_as_float((int)xi.w));
  const D4 vi = v[i];
  const df64::df vx = df64::from_double(vi.x), vy = df64::from_double(vi.y), vz = df64::from_double(vi.z);
  vrec[2 * (size_t)i] = make_float4(vx.hi, vy.hi, vz.hi, 0.f);
  vrec[2 * (size_t)i + 1] = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
}

// With rec (the df64 pair sums), also the atom's records for them: rec[2i] =
// {offset in its bin, hi parts; bin + 1 packed 10 bits per axis},
// rec[2i+1] = {offset, lo parts; element}, vrec[2i], vrec[2i+1] = velocity,
// hi and lo parts.  The offset is x - lo - b w with one rounding; a pair's
// displacement is then d w + (o_j - o_i), d the bin difference.
__global__ void k_bin(StepParams P, D4 *__restrict__ x, D4 *__restrict__ xhold, const int *__restrict__ wrapflag,
                      int *__restrict__ bin_count, BinEntry *__restrict__ bins, int4 *__restrict__ atom_bin,
                      float4 *__restrict__ atom_off, unsigned *__restrict__ err,
                      unsigned long long *__restrict__ counters, int bump_step, const int *__restrict__ gate = nullptr,
                      D4 *__restrict__ xref = nullptr, float4 *__restrict__ rec = nullptr,
                      float4 *__restrict__ vrec = nullptr, const D4 *__restrict__ v = nullptr) {
  if (gate && !*gate) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && bump_step) *P.step += 1ull;  // read by the density sweep that follows
  if (i >= P.n) return;
  D4 xi = x[i];
  if (!gate && *wrapflag) {
    wrap_into_box(P, xi);
    x[i] = xi;
    xhold[i] = xi;
    if (i == 0) atomicAdd(&counters[CNT_WRAP], 1ull);
  }
  if (xref) xref[i] = xi;
  const double p[3] = {xi.x, xi.y, xi.z};
  int B[3], t[3], wc[3];
  float o[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double s = p[k] - P.lo[k];
    int b = (int)floor(s * P.inv_w[k]);
    if (b < -1 || b > P.nb[k]) {
      atomicOr(err, ERR_DRIFT);
      b = b < -1 ? -1 : P.nb[k];
    }
    B[k] = b;
    t[k] = b < 0 ? b + P.nb[k] : (b >= P.nb[k] ? b - P.nb[k] : b);
    wc[k] = (b - t[k]) / P.nb[k];
    o[k] = (float)(s - (double)b * P.w[k]);
  }
  const int flat = t[0] + P.nb[0] * (t[1] + P.nb[1] * t[2]);
  const unsigned code = (unsigned)((wc[0] + 1) + 3 * (wc[1] + 1) + 9 * (wc[2] + 1));
  const int slot = atomicAdd(&bin_count[flat], 1);
  if (slot < P.bcap) {
    BinEntry be;
    be.idx = (unsigned)i | (code << IDX_BITS);
    be.ox = o[0];
    be.oy = o[1];
    be.oz = o[2];
    bins[(size_t)flat * P.bcap + slot] = be;
  } else {
    atomicOr(err, ERR_BIN_OVERFLOW);
  }
  atom_bin[i] = make_int4(B[0], B[1], B[2], flat);
  atom_off[i] = make_float4(o[0], o[1], o[2], 0.f);
  if (rec) df_records(P, i, xi, B, v, rec, vrec);
}

// -------------------------------------------------------- density sweep

// Candidates of atom i in the bin at stencil offset (dx, dy, dz) from its
// own: the entries whose FP32 distance passes the widened cut-off, appended
// through cset (FAST: in bin order; EXACT: kept in ascending neighbour index
// by insertion) while nc < cap.  Contains a warp-wide max: every lane of the
// warp calls it the same number of times (look = false for a lane with
// nothing to search).  r2band is the FP32 threshold (the cutoff's, or the
// candidate list's); with SKIP, entries of atoms flagged as moved (skip[j] &
// 2) are left out.
template <bool FAST, bool SKIP = false, class Get, class Set>
__device__ __forceinline__ void bin_candidates(const StepParams &P, int i, bool look, int4 Bi, float4 oi, int dx,
                                               int dy, int dz, const int *__restrict__ bin_count,
                                               const BinEntry *__restrict__ bins, unsigned *__restrict__ err,
                                               int &nc, int cap, Get cget, Set cset, float r2band,
                                               const int *__restrict__ skip = nullptr, float r2lo = -1.f) {
  const int Tz = Bi.z + dz, tz = Tz < 0 ? Tz + P.nb[2] : (Tz >= P.nb[2] ? Tz - P.nb[2] : Tz);
  const int kz = Tz < 0 ? -1 : (Tz >= P.nb[2] ? 1 : 0);
  const float bz = (float)dz * P.wf[2] - oi.z;
  const int Ty = Bi.y + dy, ty = Ty < 0 ? Ty + P.nb[1] : (Ty >= P.nb[1] ? Ty - P.nb[1] : Ty);
  const int ky = Ty < 0 ? -1 : (Ty >= P.nb[1] ? 1 : 0);
  const float by = (float)dy * P.wf[1] - oi.y;
  const int Tx = Bi.x + dx, tx = Tx < 0 ? Tx + P.nb[0] : (Tx >= P.nb[0] ? Tx - P.nb[0] : Tx);
  const int kx = Tx < 0 ? -1 : (Tx >= P.nb[0] ? 1 : 0);
  const float bx = (float)dx * P.wf[0] - oi.x;
  const int flat = tx + P.nb[0] * (ty + P.nb[1] * tz);
  int cnt = 0;
  if (look) {
    cnt = bin_count[flat];
    cnt = cnt < P.bcap ? cnt : P.bcap;
  }
  const int cmax = __reduce_max_sync(0xffffffffu, cnt);
  const BinEntry *be = bins + (size_t)flat * P.bcap;
  for (int s = 0; s < cmax; ++s) {
    if (s < cnt) {
      const BinEntry b = be[s];
      const unsigned j = b.idx & IDX_MASK;
      const float ex = bx + b.ox, ey = by + b.oy, ez = bz + b.oz;
      const float r2 = ex * ex + ey * ey + ez * ez;
      if (j != (unsigned)i && r2 < r2band && r2 >= r2lo && !(SKIP && (skip[j] & 2))) {
        const unsigned wc = b.idx >> IDX_BITS;
        const int mx = kx - ((int)(wc % 3u) - 1), my = ky - ((int)((wc / 3u) % 3u) - 1),
                  mz = kz - ((int)(wc / 9u) - 1);
        if (mx < -1 || mx > 1 || my < -1 || my > 1 || mz < -1 || mz > 1) {
          atomicOr(err, ERR_DRIFT);
        } else if (nc >= cap) {
          atomicOr(err, ERR_PAIR_OVERFLOW);
        } else {
          const unsigned u = j | ((unsigned)((mx + 1) + 3 * (my + 1) + 9 * (mz + 1)) << IDX_BITS);
          int pos = nc++;
          if (!FAST) {  // ascending neighbour index
            while (pos > 0) {
              const unsigned prev = cget(pos - 1);
              if ((prev & IDX_MASK) <= j) break;
              cset(pos, prev);
              --pos;
            }
          }
          cset(pos, u);
        }
      }
    }
  }
}

// Pass 1 of the density sweep for atom i: the candidates of the 27 bins
// around its own within the FP32 thresholds r2lo <= r^2 < r2band, appended
// after the first nc0 (at most cap in all).  Returns their number.
template <bool FAST, bool SKIP = false, class Get, class Set>
__device__ __forceinline__ int collect_candidates(const StepParams &P, int i, bool active, int4 Bi, float4 oi,
                                                  const int *__restrict__ bin_count,
                                                  const BinEntry *__restrict__ bins, unsigned *__restrict__ err,
                                                  Get cget, Set cset, float r2band, int cap,
                                                  const int *__restrict__ skip = nullptr, float r2lo = -1.f,
                                                  int nc0 = 0) {
  int nc = nc0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx)
        bin_candidates<FAST, SKIP>(P, i, active, Bi, oi, dx, dy, dz, bin_count, bins, err, nc, cap, cget, cset,
                                   r2band, skip, r2lo);
  return nc;
}

// Pass 1 from the standalone engine's EAM pair list of this step
// (k_eam_density's rows: the same bins, the same stencil order, every pair
// within the EAM cut-off, which exceeds r2band): its entries within the
// FP32 threshold r2band, tested with bin_candidates' arithmetic on the
// neighbours' bins and offsets -- the candidates of the bin search, in its
// order, without scanning the bins.  Returns their number.
template <class Set>
__device__ __forceinline__ int list_candidates(const StepParams &P, int i, bool active, int4 Bi, float4 oi,
                                               const unsigned *__restrict__ elist, const int *__restrict__ ens,
                                               const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
                                               unsigned *__restrict__ err, Set cset, float r2band, int cap) {
  int nc = 0;
  const int ne = active ? ens[i] : 0;
  const int nmax = __reduce_max_sync(0xffffffffu, ne);
  for (int k = 0; k < nmax; ++k) {
    if (k >= ne) continue;
    const unsigned u = elist[(size_t)k * P.n + i];
    const unsigned j = u & IDX_MASK, code = u >> IDX_BITS;
    const int4 Bj = atom_bin[j];
    const float4 oj = atom_off[j];
    // the stencil cell of the pair: j's (unwrapped) bin moved by its image
    const int dx = Bj.x + ((int)(code % 3u) - 1) * P.nb[0] - Bi.x;
    const int dy = Bj.y + ((int)((code / 3u) % 3u) - 1) * P.nb[1] - Bi.y;
    const int dz = Bj.z + ((int)(code / 9u) - 1) * P.nb[2] - Bi.z;
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) {
      atomicOr(err, ERR_DRIFT);
      continue;
    }
    const float bx = (float)dx * P.wf[0] - oi.x, by = (float)dy * P.wf[1] - oi.y, bz = (float)dz * P.wf[2] - oi.z;
    const float ex = bx + oj.x, ey = by + oj.y, ez = bz + oj.z;
    if (ex * ex + ey * ey + ez * ez < r2band) {
      if (nc >= cap)
        atomicOr(err, ERR_PAIR_OVERFLOW);
      else
        cset(nc++, u);
    }
  }
  return nc;
}

// The same sort with one warp per bin, for bins of at most 64 entries: lane l
// holds entries l and l + 32, each entry's place is the number of entries
// with a smaller atom index (indices are distinct), found by broadcasting
// every entry's key across the warp; all loads happen before any store.
__global__ void k_bin_sort_warp(int nbins, int bcap, const int *__restrict__ bin_count, BinEntry *__restrict__ bins,
                                const int *__restrict__ gate = nullptr) {
  if (gate && !*gate) return;
  const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nbins) return;  // whole warps leave together
  int cnt = bin_count[w];
  cnt = cnt < bcap ? cnt : bcap;
  BinEntry *e = bins + (size_t)w * bcap;
  const bool h0 = lane < cnt, h1 = lane + 32 < cnt;
  BinEntry a{}, b{};
  if (h0) a = e[lane];
  if (h1) b = e[lane + 32];
  const unsigned ka = h0 ? (a.idx & IDX_MASK) : 0xffffffffu, kb = h1 ? (b.idx & IDX_MASK) : 0xffffffffu;
  int ra = 0, rb = 0;
  for (int s = 0; s < 32; ++s) {
    const unsigned k0 = __shfl_sync(0xffffffffu, ka, s), k1 = __shfl_sync(0xffffffffu, kb, s);
    ra += (k0 < ka) + (k1 < ka);
    rb += (k0 < kb) + (k1 < kb);
  }
  __syncwarp();
  if (h0) e[ra] = a;
  if (h1) e[rb] = b;
}

// Sort every bin's entries by atom index (one thread per bin, a handful of
// entries each), so the candidate order below is fixed run to run.
__global__ void k_bin_sort(int nbins, int bcap, const int *__restrict__ bin_count, BinEntry *__restrict__ bins,
                           const int *__restrict__ gate = nullptr) {
  if (gate && !*gate) return;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  int cnt = bin_count[b];
  cnt = cnt < bcap ? cnt : bcap;
  BinEntry *e = bins + (size_t)b * bcap;
  for (int k = 1; k < cnt; ++k) {
    const BinEntry v = e[k];
    const unsigned key = v.idx & IDX_MASK;
    int p = k;
    while (p > 0 && (e[p - 1].idx & IDX_MASK) > key) {
      e[p] = e[p - 1];
      --p;
    }
    e[p] = v;
  }
}

// One in-cutoff pair (i, j) of the density sweep: rho_j(r^2) into rho_i, the
// pair cache row at `slot`, and with FUSE_W the sums of M_i and S_i.
template <bool FAST, bool MULTI, bool FUSE_W>
__device__ __forceinline__ void density_pair(const StepParams &P, int ei, unsigned u, int ej, double ex, double ey,
                                             double ez, double r2, size_t slot, unsigned *__restrict__ pj,
                                             D4 *__restrict__ pe, double2 *__restrict__ pg,
                                             const D4 *__restrict__ v, unsigned *__restrict__ err, double &rho,
                                             double &mxx, double &mxy, double &mxz, double &myy, double &myz,
                                             double &mzz, double &Sx, double &Sy, double &Sz) {
  const double rji = spline_eval<FAST>(P.tab_rho_r_sq + (size_t)ej * P.n_rho, P.inv_dr_sq, P.n_rho, r2, err);
  double rij = rji;
  if (MULTI && ej != ei)
    rij = spline_eval<FAST>(P.tab_rho_r_sq + (size_t)ei * P.n_rho, P.inv_dr_sq, P.n_rho, r2, err);
  // with M_i summed (FAST, FUSE_W) rho_i is its trace, sum_j H_ij r^2
  // (density_epilogue): one FP64 add per pair less
  if (!(FAST && FUSE_W)) rho += rji;
  pj[slot] = u;
  if (FAST) {
    const double inv_r2 = recip_nr(r2);
    const double H = rji * inv_r2;
    const double hx = H * ex, hy = H * ey, hz = H * ez;
    if (FUSE_W && !MULTI) {
      // one element: H_ij = H_ji, and the force sweep takes the pair's
      // H e from here instead of multiplying by H per pair
      pe[slot] = D4{ex, ey, ez, hx};
      pg[slot] = make_double2(hy, hz);
    } else {
      pe[slot] = D4{ex, ey, ez, H};
      if (MULTI) pg[slot] = make_double2(rij * inv_r2, 0.0);
    }
    if (FUSE_W) {
      const D4 vj = v[u & IDX_MASK];
      mxx = fma(hx, ex, mxx);
      mxy = fma(hx, ey, mxy);
      mxz = fma(hx, ez, mxz);
      myy = fma(hy, ey, myy);
      myz = fma(hy, ez, myz);
      mzz = fma(hz, ez, mzz);
      const double d = dot3_fma(ex, ey, ez, vj.x, vj.y, vj.z);
      Sx = fma(d, hx, Sx);
      Sy = fma(d, hy, Sy);
      Sz = fma(d, hz, Sz);
    }
  } else {
    pe[slot] = D4{ex, ey, ez, r2};
    pg[slot] = make_double2(rji, rij);
  }
}

// e = x_j (periodic image of the pair code) - x_i, as the engine's ghost
// atoms give it: (x_j + image shift) - x_i
__device__ __forceinline__ void density_vector(const StepParams &P, const D4 &xi, const D4 &xj, unsigned code,
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

// The end of the density sweep for atom i (its pairs summed): alpha, beta,
// the deviates, its grid cell and T_e, and the per-atom records.
// With DFG (the df64 force sweep follows) the gathered records go to G as
// double-floats, three float4 per atom: {W hi, X_x hi}, {W lo, X_x lo},
// {X_y hi, X_z hi, X_y lo, X_z lo} (W = a_i w_i, X = a_i xi_i); an atom the
// reference skips as a neighbour (rho <= 0 or outside the group) is marked
// by a NaN in its first word.
template <bool FAST, bool FUSE_W, bool DFG = false>
__device__ __forceinline__ void density_epilogue(
    const StepParams &P, int i, bool active, const D4 &xi, int ei, double rho, int ns, double mxx, double mxy,
    double mxz, double myy, double myz, double mzz, double Sx, double Sy, double Sz,
    const D4 *__restrict__ xi_given, int xi_mode, const double *__restrict__ T_e, int *__restrict__ nshort,
    D4 *__restrict__ A, D4 *__restrict__ Bw, double *__restrict__ rho_out, double *__restrict__ beta_out,
    int *__restrict__ cell, double *__restrict__ Te_i, unsigned *__restrict__ err,
    unsigned long long *__restrict__ counters, const D4 *__restrict__ v, D4 *__restrict__ Mm,
    D4 *__restrict__ G) {
  nshort[i] = ns;
  // FAST with M_i: rho_i = trace M_i = sum_j rho_j(r^2) / r^2 * r^2, within
  // the reciprocal's error (~6e-14) of the sum of rho_j(r^2)
  if (FAST && FUSE_W) rho = mxx + myy + mzz;
  // per-atom quantities
  double alpha = 0.0, beta = 0.0, xi3[3] = {0.0, 0.0, 0.0};
  if (active) {
    if (rho > P.rho_cutoff) {  // eph_beta.h:174-197
      atomicAdd(&counters[CNT_RHO_CUTOFF], 1ull);
    } else {
      beta = spline_eval<FAST>(P.tab_beta + (size_t)ei * P.n_beta, P.inv_drho, P.n_beta, rho, err);
      if (rho > 0) alpha = spline_eval<FAST>(P.tab_alpha + (size_t)ei * P.n_beta, P.inv_drho, P.n_beta, rho, err);
    }
    if (FAST && rho > 0) alpha = alpha / rho;
    if (P.flags & 0x02) {
      if (xi_mode == 0) {
        gaussian3(P.seed, *P.step, (unsigned)i, xi3);
      } else {
        const D4 g = xi_given[i];
        xi3[0] = g.x;
        xi3[1] = g.y;
        xi3[2] = g.z;
      }
    }
    const long c = grid_index(P, xi.x, xi.y, xi.z);
    cell[i] = (int)c;
    Te_i[i] = T_e[c];
  }
  A[i] = D4{rho, alpha, xi3[0], xi3[1]};
  if (FUSE_W) {
    // w_i = a_i (M_i v_i - S_i), a_i = alpha_i/rho_i; k_friction_w's rule: w
    // stays 0 unless rho_i > 0.  For k_forces_m: M_i, and the records
    // G_i = {a_i w_i, a_i xi_i, rho_i} that the neighbours gather.
    double wx = 0.0, wy = 0.0, wz = 0.0;
    if (active && pos_double(rho)) {
      const D4 vi = v[i];
      wx = alpha * (fma(mxx, vi.x, fma(mxy, vi.y, mxz * vi.z)) - Sx);
      wy = alpha * (fma(mxy, vi.x, fma(myy, vi.y, myz * vi.z)) - Sy);
      wz = alpha * (fma(mxz, vi.x, fma(myz, vi.y, mzz * vi.z)) - Sz);
    }
    Bw[i] = D4{xi3[2], wx, wy, wz};
    Mm[i] = D4{mxx, mxy, mxz, myy};
    Mm[(size_t)P.n + i] = D4{myz, mzz, 0.0, 0.0};
    if (DFG) {
      const df64::df W[3] = {df64::from_double(alpha * wx), df64::from_double(alpha * wy),
                             df64::from_double(alpha * wz)};
      const df64::df X[3] = {df64::from_double(alpha * xi3[0]), df64::from_double(alpha * xi3[1]),
                             df64::from_double(alpha * xi3[2])};
      const bool live = active && pos_double(rho);
      float4 *g = reinterpret_cast<float4 *>(G) + 3 * (size_t)i;
      g[0] = make_float4(live ? W[0].hi : __int_as_float(0x7fc00000), W[1].hi, W[2].hi, X[0].hi);
      g[1] = make_float4(W[0].lo, W[1].lo, W[2].lo, X[0].lo);
      g[2] = make_float4(X[1].hi, X[2].hi, X[1].lo, X[2].lo);
    } else {
      G[2 * (size_t)i] = D4{alpha * wx, alpha * wy, alpha * wz, alpha * xi3[0]};
      G[2 * (size_t)i + 1] = D4{alpha * xi3[1], alpha * xi3[2], active ? rho : 0.0, 0.0};
    }
  } else {
    Bw[i] = D4{xi3[2], 0.0, 0.0, 0.0};
  }
  rho_out[i] = rho;
  beta_out[i] = beta;
}

// calculate_environment (fix_eph.cpp:431-466) plus everything per atom the
// later sweeps need.  One thread per atom, warps kept converged: a warp FP64
// instruction costs the same whether 1 or 32 lanes are active, so the FP64
// work must run in lockstep.
//   pass 1 (FP32/integer): candidates from the 27 bins around the atom with an
//     FP32 distance test padded by 1e-4 of rc^2, kept in shared memory; EXACT
//     mode keeps them in ascending neighbour index (the order of the
//     reference's list, so sums round identically), FAST mode in the fixed
//     bin-stencil order of index-sorted bins
//   pass 2 (FP64): the exact test r^2 < rc^2 with e = (x_j + image) - x_i, the
//     density sum, and the pair cache of the in-cutoff pairs
// Pair cache row k of atom i sits at k*n + i (coalesced across the warp):
//   pj: neighbour index | image code << 27
//   pe: e_ij and (EXACT) r^2 or (FAST) rho_j(r^2)/r^2
//   pg: (EXACT) rho_j(r^2), rho_i(r^2); (FAST, several elements) rho_i(r^2)/r^2
// A[i] = {rho_i, alpha_i (EXACT) | alpha_i/rho_i (FAST), xi_x, xi_y}
// Bw[i] = {xi_z, w_i} (w written by the friction sweep, or here with FUSE_W)
// Candidates: the first CAND_SMEM rows of an atom live in shared memory
// ([CAND_SMEM][blockDim]), further ones in the atom's own rows of pj (read
// back before pass 2 overwrites them: pair slot <= candidate slot).
// FUSE_W (FAST mode, one lane per atom): the friction pre-vector of stage 1
// in the same pass — it needs only this atom's density, so its sums ride
// along with rho and the separate sweep over the pair cache is saved:
// M_i = sum_j H_ij e e^T and S_i = sum_j H_ij (e.v_j) e (H_ij = rho_j(r^2)/r^2),
// then w_i = (alpha_i / rho_i) (M_i v_i - S_i).  It also leaves M_i and the
// records G_i = {a_i w_i, a_i xi_i, rho_i} for k_forces_m.
template <bool FAST, bool MULTI, bool FUSE_W = false>
__global__ void __launch_bounds__(128) k_density(
    StepParams P, const D4 *__restrict__ x, const int *__restrict__ mask, const int *__restrict__ bin_count,
    const BinEntry *__restrict__ bins, const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
    const D4 *__restrict__ xi_given, int xi_mode, const double *__restrict__ T_e, unsigned *__restrict__ pj,
    D4 *__restrict__ pe, double2 *__restrict__ pg, int *__restrict__ nshort, D4 *__restrict__ A,
    D4 *__restrict__ Bw, double *__restrict__ rho_out, double *__restrict__ beta_out, int *__restrict__ cell,
    double *__restrict__ Te_i, int *__restrict__ wrapflag, unsigned *__restrict__ err,
    unsigned long long *__restrict__ counters, const D4 *__restrict__ v = nullptr, D4 *__restrict__ Mm = nullptr,
    D4 *__restrict__ G = nullptr) {
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  if (i == 0) *wrapflag = 0;  // the binning kernel has read it
  const bool valid = i < P.n;
  const bool active = valid && (mask[i] & P.groupbit) != 0;
  auto cget = [&](int k) -> unsigned { return k < CAND_SMEM ? s_cand[k * nt + t] : pj[(size_t)k * P.n + i]; };
  auto cset = [&](int k, unsigned u) {
    if (k < CAND_SMEM)
      s_cand[k * nt + t] = u;
    else
      pj[(size_t)k * P.n + i] = u;
  };
  D4 xi = D4{0.0, 0.0, 0.0, 0.0};
  if (valid) xi = x[i];
  const int ei = (int)xi.w;
  double rho = 0.0;
  int ns = 0, nc = 0;
  // pass 1: candidates, FP32/integer work only, warp-uniform loop bounds
  {
    int4 Bi = make_int4(0, 0, 0, 0);
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
      Bi = atom_bin[i];
      oi = atom_off[i];
    }
    nc = collect_candidates<FAST>(P, i, active, Bi, oi, bin_count, bins, err, cget, cset, P.rc2_band, P.kcap);
  }
  __syncwarp();
  // pass 2: exact FP64 test, density and pair cache, in lockstep
  // FUSE_W: M_i = sum_j H_ij e e^T over all pairs and S_i = sum_j H_ij (e.v_j) e
  double Sx = 0.0, Sy = 0.0, Sz = 0.0;
  double mxx = 0.0, mxy = 0.0, mxz = 0.0, myy = 0.0, myz = 0.0, mzz = 0.0;
  const int nmax = __reduce_max_sync(0xffffffffu, nc);
  for (int k = 0; k < nmax; ++k) {
    if (k < nc) {
      const unsigned u = cget(k);
      const D4 xj = x[u & IDX_MASK];
      double ex, ey, ez;
      density_vector(P, xi, xj, u >> IDX_BITS, ex, ey, ez);
      const double r2 = FAST ? dot3_fma(ex, ey, ez, ex, ey, ez) : dot3(ex, ey, ez, ex, ey, ez);
      if (below(r2, P.rc2)) {  // r2 >= 0
        density_pair<FAST, MULTI, FUSE_W>(P, ei, u, (int)xj.w, ex, ey, ez, r2, (size_t)ns * P.n + i, pj, pe, pg,
                                          v, err, rho, mxx, mxy, mxz, myy, myz, mzz, Sx, Sy, Sz);
        ++ns;
      }
    }
  }
  if (!valid) return;
  density_epilogue<FAST, FUSE_W>(P, i, active, xi, ei, rho, ns, mxx, mxy, mxz, myy, myz, mzz, Sx, Sy, Sz, xi_given,
                                 xi_mode, T_e, nshort, A, Bw, rho_out, beta_out, cell, Te_i, err, counters, v, Mm, G);
}

// ------------------------------------------- FAST pair sweeps in df64

// resident blocks of 128 threads per SM the df64 sweeps are compiled for
// (their register budget: 65,536 / (128 x blocks)); measured on GB300 at
// 2,048,000 atoms: density 6 and 7 alike, 8 spills and is 17 % slower;
// forces 6 / 7 / 8: 1.51 / 1.36 / 1.50 ms
#ifndef EPH_DF_DENSITY_BLOCKS
#define EPH_DF_DENSITY_BLOCKS 6
#endif
#ifndef EPH_DF_FORCES_BLOCKS
#define EPH_DF_FORCES_BLOCKS 7
#endif
// candidates per iteration of the df64 density sweep's pass 2 (measured on
// GB300 at 2,048,000 atoms: 1 -> 3.89 ms, 2 -> 3.91 ms; the sweep waits on
// the neighbours' records and its pair-cache writes more than on its chains)
#ifndef DF_UNROLL
#define DF_UNROLL 1
#endif

// The FAST density sweep of k_density<true, MULTI, true> (one lane per atom,
// stage 1 and M_i folded) with every per-pair operation in df64 on the FP32
// pipe: pass 1 is k_density's; pass 2 forms e = d w + (o_j - o_i) from the
// atoms' bin offsets (k_bin's records, 48 significant bits), r^2, the exact
// cut-off test, rho_j(r^2) (spline_rho_df), H = rho_j(r^2) / r^2 (a df64
// Newton reciprocal), H e, and the sums of M_i and S_i (blocked df64 sums,
// folded every 8 candidates); the epilogue is k_density's in FP64 and writes
// the records G for k_forces_df.  Pair cache (row k of atom i at k*n + i):
// pa = {e hi, (H e)_x hi | H_ji hi}, pb = the lo parts, pc = {(H e)_y, (H e)_z}
// hi, hi, lo, lo with one element, {H_ij hi, H_ij lo} with several.
template <bool MULTI>
__global__ void __launch_bounds__(128, EPH_DF_DENSITY_BLOCKS) k_density_df(
    StepParams P, const int *__restrict__ mask, const int *__restrict__ bin_count, const BinEntry *__restrict__ bins,
    const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off, const float4 *__restrict__ rec,
    const float4 *__restrict__ vrec, const D4 *__restrict__ x, const D4 *__restrict__ xi_given, int xi_mode,
    const double *__restrict__ T_e, unsigned *__restrict__ pj, float4 *__restrict__ pa, float4 *__restrict__ pb,
    float4 *__restrict__ pc, int *__restrict__ nshort, D4 *__restrict__ A, D4 *__restrict__ Bw,
    double *__restrict__ rho_out, double *__restrict__ beta_out, int *__restrict__ cell, double *__restrict__ Te_i,
    int *__restrict__ wrapflag, unsigned *__restrict__ err, unsigned long long *__restrict__ counters,
    const D4 *__restrict__ v, D4 *__restrict__ Mm, D4 *__restrict__ G, const unsigned *__restrict__ elist = nullptr,
    const int *__restrict__ ens = nullptr) {
  using namespace df64;
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  if (i == 0) *wrapflag = 0;  // the binning kernel has read it
  const bool valid = i < P.n;
  const bool active = valid && (mask[i] & P.groupbit) != 0;
  auto cget = [&](int k) -> unsigned { return k < CAND_SMEM ? s_cand[k * nt + t] : pj[(size_t)k * P.n + i]; };
  auto cset = [&](int k, unsigned u) {
    if (k < CAND_SMEM)
      s_cand[k * nt + t] = u;
    else
      pj[(size_t)k * P.n + i] = u;
  };
  int4 Bi = make_int4(0, 0, 0, 0);
  float4 oi = make_float4(0.f, 0.f, 0.f, 0.f), Ri1 = make_float4(0.f, 0.f, 0.f, 0.f);
  int ns = 0, nc = 0;
  if (valid) {
    Bi = atom_bin[i];
    oi = rec[2 * (size_t)i];
    Ri1 = rec[2 * (size_t)i + 1];
  }
  const int ei = __float_as_int(Ri1.w);
  // pass 1: candidates, FP32/integer work only, warp-uniform loop bounds;
  // from the EAM pair list when the standalone engine made one this step
  {
    float4 of = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) of = atom_off[i];
    if (elist)
      nc = list_candidates(P, i, active, Bi, of, elist, ens, atom_bin, atom_off, err, cset, P.rc2_band, P.kcap);
    else
      nc = collect_candidates<true>(P, i, active, Bi, of, bin_count, bins, err, cget, cset, P.rc2_band, P.kcap);
  }
  __syncwarp();
  // pass 2 in df64: M_i (xx, xy, xz, yy, yz, zz) and S_i (x, y, z), DF_UNROLL
  // candidates per iteration with no branch around their arithmetic: a
  // candidate outside the cut-off (or past the lane's list) is evaluated at
  // r^2 = 1 with H forced to 0, so its terms add exact zeros and it writes no
  // pair.
  bsum sm[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) sm[q] = bsum_zero();
  const df rc2{P.rc2_hi, P.rc2_lo};
  const int nmax = __reduce_max_sync(0xffffffffu, nc);
  for (int k = 0; k < nmax; k += DF_UNROLL) {
    unsigned uu[DF_UNROLL];
    df ex[DF_UNROLL], ey[DF_UNROLL], ez[DF_UNROLL], r2[DF_UNROLL];
    int ej[DF_UNROLL];
    bool in[DF_UNROLL];
#pragma unroll
    for (int c = 0; c < DF_UNROLL; ++c) {
      const bool have = k + c < nc;
      const unsigned u = have ? cget(k + c) : 0u;
      const unsigned j = u & IDX_MASK, code = have ? u >> IDX_BITS : CODE_NOSHIFT;
      const float4 R0 = rec[2 * (size_t)j], R1 = rec[2 * (size_t)j + 1];
      const unsigned pk = __float_as_uint(R0.w);
      // bin difference of the pair: j's bin + its periodic image - i's bin
      const int dx = (int)(pk & 1023u) - 1 + ((int)(code % 3u) - 1) * P.nb[0] - Bi.x;
      const int dy = (int)((pk >> 10) & 1023u) - 1 + ((int)((code / 3u) % 3u) - 1) * P.nb[1] - Bi.y;
      const int dz = (int)((pk >> 20) & 1023u) - 1 + ((int)(code / 9u) - 1) * P.nb[2] - Bi.z;
      ex[c] = pair_disp(dx, R0.x, R1.x, oi.x, Ri1.x, P.w_hi[0], P.w_lo[0]);
      ey[c] = pair_disp(dy, R0.y, R1.y, oi.y, Ri1.y, P.w_hi[1], P.w_lo[1]);
      ez[c] = pair_disp(dz, R0.z, R1.z, oi.z, Ri1.z, P.w_hi[2], P.w_lo[2]);
      r2[c] = dot3(ex[c], ey[c], ez[c], ex[c], ey[c], ez[c]);
      in[c] = have && lt(r2[c], rc2);
      if (!in[c]) r2[c] = df{1.0f, 0.0f};
      ej[c] = __float_as_int(R1.w);
      uu[c] = u;
    }
#pragma unroll
    for (int c = 0; c < DF_UNROLL; ++c) {
      const df rji = spline_rho_df(P, ej[c], r2[c], err);
      const df inv = recip(r2[c], rcp_estimate(r2[c].hi));
      df H = mul(rji, inv);
      if (!in[c]) H = df{0.0f, 0.0f};
      const df hx = mul(H, ex[c]), hy = mul(H, ey[c]), hz = mul(H, ez[c]);
      if (in[c]) {
        const size_t slot = (size_t)ns * P.n + i;
        pj[slot] = uu[c];
        if (MULTI) {
          const df rij = ej[c] != ei ? spline_rho_df(P, ei, r2[c], err) : rji;
          const df Hji = mul(rij, inv);
          pa[slot] = make_float4(ex[c].hi, ey[c].hi, ez[c].hi, Hji.hi);
          pb[slot] = make_float4(ex[c].lo, ey[c].lo, ez[c].lo, Hji.lo);
          pc[slot] = make_float4(H.hi, H.lo, 0.f, 0.f);
        } else {
          pa[slot] = make_float4(ex[c].hi, ey[c].hi, ez[c].hi, hx.hi);
          pb[slot] = make_float4(ex[c].lo, ey[c].lo, ez[c].lo, hx.lo);
          pc[slot] = make_float4(hy.hi, hz.hi, hy.lo, hz.lo);
        }
        ++ns;
      }
      acc_fma(sm[0].blk, hx, ex[c]);
      acc_fma(sm[1].blk, hx, ey[c]);
      acc_fma(sm[2].blk, hx, ez[c]);
      acc_fma(sm[3].blk, hy, ey[c]);
      acc_fma(sm[4].blk, hy, ez[c]);
      acc_fma(sm[5].blk, hz, ez[c]);
      const unsigned j = uu[c] & IDX_MASK;
      const float4 V0 = vrec[2 * (size_t)j], V1 = vrec[2 * (size_t)j + 1];
      const df d = dot3(ex[c], ey[c], ez[c], df{V0.x, V1.x}, df{V0.y, V1.y}, df{V0.z, V1.z});
      acc_fma(sm[6].blk, d, hx);
      acc_fma(sm[7].blk, d, hy);
      acc_fma(sm[8].blk, d, hz);
    }
    if ((k & 7) == 8 - DF_UNROLL) {
#pragma unroll
      for (int q = 0; q < 9; ++q) bsum_fold(sm[q]);
    }
  }
  if (!valid) return;
  double mq[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) mq[q] = to_double(bsum_value(sm[q]));
  const D4 xi = x[i];
  density_epilogue<true, true, true>(P, i, active, xi, ei, 0.0, ns, mq[0], mq[1], mq[2], mq[3], mq[4], mq[5], mq[6],
                                     mq[7], mq[8], xi_given, xi_mode, T_e, nshort, A, Bw, rho_out, beta_out, cell,
                                     Te_i, err, counters, v, Mm, G);
}

// The FAST density sweep with TPA lanes per atom (TPA = 2, 4, 8) for small
// systems, where one lane per atom leaves the SMs a few warps each and the
// sweep waits on its loads.  Lane g of an atom searches bins g, g + TPA, ...
// of the 27 (its candidates in its own shared-memory column, at most
// CAND_SMEM), tests them exactly, and after a prefix sum over the atom's
// lanes writes its in-cutoff pairs to rows [offset_g, offset_g + count_g)
// of the pair cache; rho (and with FUSE_W, M_i and S_i) are summed over the
// lanes by a butterfly and lane 0 finishes the atom.  Sums in a fixed order
// (the same every run), within rounding of the one-lane sweep.
template <bool MULTI, bool FUSE_W, int TPA>
__global__ void __launch_bounds__(128) k_density_tpa(
    StepParams P, const D4 *__restrict__ x, const int *__restrict__ mask, const int *__restrict__ bin_count,
    const BinEntry *__restrict__ bins, const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
    const D4 *__restrict__ xi_given, int xi_mode, const double *__restrict__ T_e, unsigned *__restrict__ pj,
    D4 *__restrict__ pe, double2 *__restrict__ pg, int *__restrict__ nshort, D4 *__restrict__ A,
    D4 *__restrict__ Bw, double *__restrict__ rho_out, double *__restrict__ beta_out, int *__restrict__ cell,
    double *__restrict__ Te_i, int *__restrict__ wrapflag, unsigned *__restrict__ err,
    unsigned long long *__restrict__ counters, const D4 *__restrict__ v, D4 *__restrict__ Mm,
    D4 *__restrict__ G) {
  static_assert(CAND_SMEM <= 64, "candidate masks are 64 bits");
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const long gt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(gt / TPA), g = (int)(gt % TPA);
  const int t = threadIdx.x, nt = blockDim.x;
  if (gt == 0) *wrapflag = 0;  // the binning kernel has read it
  const bool valid = i < P.n;
  const bool active = valid && (mask[i] & P.groupbit) != 0;
  auto cget = [&](int k) -> unsigned { return s_cand[k * nt + t]; };
  auto cset = [&](int k, unsigned u) { s_cand[k * nt + t] = u; };
  D4 xi = D4{0.0, 0.0, 0.0, 0.0};
  if (valid) xi = x[i];
  const int ei = (int)xi.w;
  // pass 1: this lane's bins (the same number of rounds on every lane)
  int nc = 0;
  {
    int4 Bi = make_int4(0, 0, 0, 0);
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
      Bi = atom_bin[i];
      oi = atom_off[i];
    }
    for (int m = 0; m < (27 + TPA - 1) / TPA; ++m) {
      const int b = g + m * TPA;  // (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)
      const bool look = active && b < 27;
      const int bb = b < 27 ? b : 13;
      bin_candidates<true>(P, i, look, Bi, oi, bb % 3 - 1, (bb / 3) % 3 - 1, bb / 9 - 1, bin_count, bins, err, nc,
                           CAND_SMEM, cget, cset, P.rc2_band);
    }
  }
  __syncwarp();
  // pass 2a: the exact test of this lane's candidates
  unsigned long long keep = 0ull;
  const int nmax = __reduce_max_sync(0xffffffffu, nc);
  for (int k = 0; k < nmax; ++k) {
    if (k < nc) {
      const unsigned u = cget(k);
      double ex, ey, ez;
      density_vector(P, xi, x[u & IDX_MASK], u >> IDX_BITS, ex, ey, ez);
      if (below(dot3_fma(ex, ey, ez, ex, ey, ez), P.rc2)) keep |= 1ull << k;
    }
  }
  // rows of this lane's pairs: an exclusive prefix sum over the atom's lanes
  const int count = __popcll(keep);
  int incl = count;
#pragma unroll
  for (int d = 1; d < TPA; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, d);
    if (g >= d) incl += y;
  }
  const int ns = __shfl_sync(0xffffffffu, incl, (int)(threadIdx.x & 31) | (TPA - 1));
  const int off = incl - count;
  if (ns > P.kcap && g == 0 && valid) atomicOr(err, ERR_PAIR_OVERFLOW);
  // pass 2b: the kept pairs
  double rho = 0.0, Sx = 0.0, Sy = 0.0, Sz = 0.0;
  double mxx = 0.0, mxy = 0.0, mxz = 0.0, myy = 0.0, myz = 0.0, mzz = 0.0;
  unsigned long long rest = keep;
  const int n2 = __reduce_max_sync(0xffffffffu, count);
  for (int m = 0; m < n2; ++m) {
    if (m < count) {
      const int k = __ffsll((long long)rest) - 1;
      rest &= rest - 1ull;
      const unsigned u = cget(k);
      const D4 xj = x[u & IDX_MASK];
      double ex, ey, ez;
      density_vector(P, xi, xj, u >> IDX_BITS, ex, ey, ez);
      const double r2 = dot3_fma(ex, ey, ez, ex, ey, ez);
      if (off + m < P.kcap)
        density_pair<true, MULTI, FUSE_W>(P, ei, u, (int)xj.w, ex, ey, ez, r2, (size_t)(off + m) * P.n + i, pj, pe,
                                          pg, v, err, rho, mxx, mxy, mxz, myy, myz, mzz, Sx, Sy, Sz);
    }
  }
#pragma unroll
  for (int o = TPA / 2; o > 0; o >>= 1) {
    if (!FUSE_W) rho += __shfl_xor_sync(0xffffffffu, rho, o);  // with M_i: its trace
    if (FUSE_W) {
      mxx += __shfl_xor_sync(0xffffffffu, mxx, o);
      mxy += __shfl_xor_sync(0xffffffffu, mxy, o);
      mxz += __shfl_xor_sync(0xffffffffu, mxz, o);
      myy += __shfl_xor_sync(0xffffffffu, myy, o);
      myz += __shfl_xor_sync(0xffffffffu, myz, o);
      mzz += __shfl_xor_sync(0xffffffffu, mzz, o);
      Sx += __shfl_xor_sync(0xffffffffu, Sx, o);
      Sy += __shfl_xor_sync(0xffffffffu, Sy, o);
      Sz += __shfl_xor_sync(0xffffffffu, Sz, o);
    }
  }
  if (!valid || g != 0) return;
  density_epilogue<true, FUSE_W>(P, i, active, xi, ei, rho, ns < P.kcap ? ns : P.kcap, mxx, mxy, mxz, myy, myz, mzz,
                                 Sx, Sy, Sz, xi_given, xi_mode, T_e, nshort, A, Bw, rho_out, beta_out, cell, Te_i,
                                 err, counters, v, Mm, G);
}

// ------------------------------------------------ candidate-list reuse

// FAST mode, one lane per atom.  The candidates of atom i within r_list =
// r_cutoff + s (s the list skin) are kept from a build step on: while atoms
// i and j both moved less than s/2 since the build, |x_i - x_j| < r_cutoff
// implies that j is in i's list.  Atoms that moved farther ("moved", at most
// LIST_FMAX of them) are handled every step instead: they and every atom
// within r_cutoff + s/2 of one of them (from the bins of the build) search
// the bins afresh, leave moved atoms' bin entries out and take the moved
// atoms as extra candidates.  More moved atoms, or a request from the host,
// make the step a build step.  Decisions live on the device (rb[0] build
// requested, rb[1] moved atoms this step, rb[2] this step builds), so a
// captured step replays them.  Lists hold atom indices; the periodic image of
// a pair is the minimum image of the current positions, decided in FP32 (the
// box is at least three list radii wide, so it is the image within the
// cutoff), and e = (x_j +- L) - x_i rounds as the engine's ghost atoms give
// it.

__device__ __forceinline__ double min_image(double d, double L, double h) {
  return d > h ? d - L : (d < -h ? d + L : d);
}

// The 3x3x3 image code of x_j seen from x_i: the image of x_j within half a
// box of x_i on every axis, decided in FP32 (the box is at least three list
// radii wide, so a pair within the list radius is far from the threshold).
// The pair vector then comes from density_vector, the rounding of the bin
// search path.
__device__ __forceinline__ unsigned image_code(const StepParams &P, float xi, float yi, float zi, const D4 &xj) {
  const float dx = float_bits(xj.x) - xi, dy = float_bits(xj.y) - yi, dz = float_bits(xj.z) - zi;
  const int mx = dx > P.half_prdf[0] ? -1 : (dx < -P.half_prdf[0] ? 1 : 0);
  const int my = dy > P.half_prdf[1] ? -1 : (dy < -P.half_prdf[1] ? 1 : 0);
  const int mz = dz > P.half_prdf[2] ? -1 : (dz < -P.half_prdf[2] ? 1 : 0);
  return (unsigned)((mx + 1) + 3 * (my + 1) + 9 * (mz + 1));
}

// The bin and FP32 offset of a position wrapped into the box (an atom whose
// bins entry is stale: it moved since the build)
__device__ __forceinline__ void current_bin(const StepParams &P, const D4 &xi, int4 &B, float4 &o) {
  const double p[3] = {xi.x, xi.y, xi.z};
  int b[3];
  float of[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double q = p[k] - P.lo[k];
    q -= floor(q / P.prd[k]) * P.prd[k];
    if (q >= P.prd[k]) q -= P.prd[k];
    if (q < 0.0) q = 0.0;
    int bb = (int)floor(q * P.inv_w[k]);
    bb = bb < 0 ? 0 : (bb >= P.nb[k] ? P.nb[k] - 1 : bb);
    b[k] = bb;
    of[k] = (float)(q - (double)bb * P.w[k]);
  }
  B = make_int4(b[0], b[1], b[2], b[0] + P.nb[0] * (b[1] + P.nb[1] * b[2]));
  o = make_float4(of[0], of[1], of[2], 0.f);
}

// First kernel of a step with list reuse: the engine's wrap (as k_bin does
// it), then each atom's displacement since the list build; moved atoms get
// state 2 and join the list of moved atoms (state 0 otherwise).  With rec
// (the df64 density sweep), also every atom's records for it from its
// current position, in the bins of the current geometry (df_records).
__global__ void k_list_check(StepParams P, D4 *__restrict__ x, D4 *__restrict__ xhold,
                             const int *__restrict__ wrapflag, const D4 *__restrict__ xref, int *__restrict__ state,
                             int *__restrict__ rb, int *__restrict__ flist, unsigned long long *__restrict__ counters,
                             float4 *__restrict__ rec = nullptr, float4 *__restrict__ vrec = nullptr,
                             const D4 *__restrict__ v = nullptr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *P.step += 1ull;  // read by the density sweep that follows
  bool moved = false;
  if (i < P.n) {
    D4 xi = x[i];
    if (*wrapflag) {
      wrap_into_box(P, xi);
      x[i] = xi;
      xhold[i] = xi;
      if (i == 0) atomicAdd(&counters[CNT_WRAP], 1ull);
    }
    if (rec) {
      const double p[3] = {xi.x, xi.y, xi.z};
      int B[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int b = (int)floor((p[k] - P.lo[k]) * P.inv_w[k]);
        B[k] = b < -1 ? -1 : (b > P.nb[k] ? P.nb[k] : b);
      }
      df_records(P, i, xi, B, v, rec, vrec);
    }
    const D4 r = xref[i];
    const double dx = min_image(xi.x - r.x, P.prd[0], P.half_prd[0]);
    const double dy = min_image(xi.y - r.y, P.prd[1], P.half_prd[1]);
    const double dz = min_image(xi.z - r.z, P.prd[2], P.half_prd[2]);
    moved = dx * dx + dy * dy + dz * dz >= P.lslow2;
    state[i] = moved ? 2 : 0;
  }
  // one atomic per warp (after a long run without a build most atoms move)
  const unsigned mv = __ballot_sync(0xffffffffu, moved);
  if (mv) {
    const int lane = threadIdx.x & 31, lead = __ffs(mv) - 1;
    int base = 0;
    if (lane == lead) base = atomicAdd(&rb[1], __popc(mv));
    base = __shfl_sync(0xffffffffu, base, lead);
    const int k = base + __popc(mv & ((1u << lane) - 1u));
    if (moved && k < LIST_FMAX) flist[k] = i;
  }
}

// One warp: build or not, and the moved atoms in index order (they were
// appended in any order; the order of the extra candidates must not change
// from run to run).
__global__ void k_list_decide(int *__restrict__ rb, int *__restrict__ flist,
                              unsigned long long *__restrict__ counters) {
  const int lane = threadIdx.x;
  const int cnt = rb[1];
  const bool build = rb[0] != 0 || cnt > LIST_FMAX;
  if (!build && cnt > 1) {
    const int v = lane < cnt ? flist[lane] : 0x7fffffff;
    int rank = 0;
    for (int s = 0; s < 32; ++s) rank += __shfl_sync(0xffffffffu, v, s) < v;
    __syncwarp();
    if (lane < cnt) flist[rank] = v;
  }
  if (lane == 0) {
    rb[2] = build ? 1 : 0;
    rb[0] = 0;
    if (build) atomicAdd(&counters[CNT_BUILD], 1ull);
  }
}

__global__ void k_zero_if(int *__restrict__ p, int n, const int *__restrict__ gate) {
  if (!*gate) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0;
}

// Block b: moved atom flist[b] flags (state |= 1) every atom whose position
// at the build lies within r_cutoff + s/2 of its current position — the
// only unmoved atoms it can now be within r_cutoff of.
__global__ void k_list_mark(StepParams P, const D4 *__restrict__ x, const int *__restrict__ rb,
                            const int *__restrict__ flist, const int *__restrict__ bin_count,
                            const BinEntry *__restrict__ bins, int *__restrict__ state) {
  if (rb[2] || (int)blockIdx.x >= rb[1]) return;
  const int f = flist[blockIdx.x];
  int4 B;
  float4 o;
  current_bin(P, x[f], B, o);
  const int per = 27 * P.bcap;
  for (int q = threadIdx.x; q < per; q += blockDim.x) {
    const int slot = q % P.bcap, b = q / P.bcap;
    const int dx = b % 3 - 1, dy = (b / 3) % 3 - 1, dz = b / 9 - 1;
    const int Tx = B.x + dx, Ty = B.y + dy, Tz = B.z + dz;
    const int tx = Tx < 0 ? Tx + P.nb[0] : (Tx >= P.nb[0] ? Tx - P.nb[0] : Tx);
    const int ty = Ty < 0 ? Ty + P.nb[1] : (Ty >= P.nb[1] ? Ty - P.nb[1] : Ty);
    const int tz = Tz < 0 ? Tz + P.nb[2] : (Tz >= P.nb[2] ? Tz - P.nb[2] : Tz);
    const int flat = tx + P.nb[0] * (ty + P.nb[1] * tz);
    const int cnt = min(bin_count[flat], P.bcap);
    if (slot >= cnt) continue;
    const BinEntry e = bins[(size_t)flat * P.bcap + slot];
    const float ex = ((float)dx * P.wf[0] - o.x) + e.ox;
    const float ey = ((float)dy * P.wf[1] - o.y) + e.oy;
    const float ez = ((float)dz * P.wf[2] - o.z) + e.oz;
    if (ex * ex + ey * ey + ez * ez < P.rmark2_band) atomicOr(&state[e.idx & IDX_MASK], 1);
  }
}

// k_density (FAST, stage 1 and M_i folded in) over the kept candidate lists:
// on a build step pass 1 searches the bins within r_list for every atom and
// writes the lists (rows k * n + i of cl, counts in cl_n); otherwise an atom
// reads its list, except the atoms flagged by k_list_check / k_list_mark,
// which search the bins of the build afresh (their candidates in shared
// memory, spilling into their pj rows as in k_density) and add the moved
// atoms.  Pass 2 and the epilogue are k_density's.
// (128 threads a block; 64 registers as k_density has: with
// __launch_bounds__(128) ptxas settled on 56 and spilled)
template <bool MULTI>
__global__ void __maxnreg__(64) k_density_list(
    StepParams P, const D4 *__restrict__ x, const int *__restrict__ mask, const int *__restrict__ bin_count,
    const BinEntry *__restrict__ bins, const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
    const D4 *__restrict__ xi_given, int xi_mode, const double *__restrict__ T_e, unsigned *__restrict__ pj,
    D4 *__restrict__ pe, double2 *__restrict__ pg, int *__restrict__ nshort, D4 *__restrict__ A,
    D4 *__restrict__ Bw, double *__restrict__ rho_out, double *__restrict__ beta_out, int *__restrict__ cell,
    double *__restrict__ Te_i, int *__restrict__ wrapflag, unsigned *__restrict__ err,
    unsigned long long *__restrict__ counters, const D4 *__restrict__ v, D4 *__restrict__ Mm, D4 *__restrict__ G,
    unsigned *__restrict__ cl, int *__restrict__ cl_n, const int *__restrict__ state, const int *__restrict__ rb,
    const int *__restrict__ flist) {
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  if (i == 0) *wrapflag = 0;  // k_list_check has read it
  const bool valid = i < P.n;
  const bool active = valid && (mask[i] & P.groupbit) != 0;
  const size_t n = (size_t)P.n;
  auto sget = [&](int k) -> unsigned { return k < CAND_SMEM ? s_cand[k * nt + t] : pj[(size_t)k * n + i]; };
  auto sset = [&](int k, unsigned u) {
    if (k < CAND_SMEM)
      s_cand[k * nt + t] = u;
    else
      pj[(size_t)k * n + i] = u;
  };
  // build steps: the list rows, their first CAND_SMEM also in shared memory
  auto lset = [&](int k, unsigned u) {
    if (k < CAND_SMEM) s_cand[k * nt + t] = u;
    cl[(size_t)k * n + i] = u;
  };
  auto lget = [&](int k) -> unsigned { return cl[(size_t)k * n + i]; };
  D4 xi = D4{0.0, 0.0, 0.0, 0.0};
  if (valid) xi = x[i];
  const int ei = (int)xi.w;
  const bool build = rb[2] != 0;
  int nc = 0;
  bool fresh = false;
  if (build) {
    int4 Bi = make_int4(0, 0, 0, 0);
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
      Bi = atom_bin[i];
      oi = atom_off[i];
    }
    // the candidates inside the cut-off first, the shell out to r_list after
    // them: the shell's pairs mostly fail the exact test, and at the end of
    // the lists whole warps skip them
    nc = collect_candidates<true>(P, i, active, Bi, oi, bin_count, bins, err, lget, lset, P.rc2_band, P.lcap);
    nc = collect_candidates<true>(P, i, active, Bi, oi, bin_count, bins, err, lget, lset, P.rl2_band, P.lcap,
                                  nullptr, P.rc2_band, nc);
    if (valid) cl_n[i] = nc;
  } else {
    const int st = active ? state[i] : 0;
    fresh = st != 0;
    if (__any_sync(0xffffffffu, fresh)) {
      int4 Bi = make_int4(0, 0, 0, 0);
      float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
      if (fresh) {
        if (st & 2) {
          current_bin(P, xi, Bi, oi);
        } else {
          Bi = atom_bin[i];
          oi = atom_off[i];
        }
      }
      nc = collect_candidates<true, true>(P, i, fresh, Bi, oi, bin_count, bins, err, sget, sset, P.rl2_band, P.kcap,
                                          state);
      // the moved atoms near enough (a widened test; pass 2 decides)
      const int nf = rb[1];  // <= LIST_FMAX on a step without a build
      for (int q = 0; q < nf; ++q) {
        const int f = flist[q];
        if (fresh && f != i) {
          const D4 xf = x[f];
          const double dx = min_image(xf.x - xi.x, P.prd[0], P.half_prd[0]);
          const double dy = min_image(xf.y - xi.y, P.prd[1], P.half_prd[1]);
          const double dz = min_image(xf.z - xi.z, P.prd[2], P.half_prd[2]);
          if (dx * dx + dy * dy + dz * dz < P.rc2 * (1.0 + 1e-4)) {
            if (nc < P.kcap)
              sset(nc++, (unsigned)f | (CODE_NOSHIFT << IDX_BITS));
            else
              atomicOr(err, ERR_PAIR_OVERFLOW);
          }
        }
      }
    }
    if (active && !fresh) {
      // the list's head into shared memory: independent loads up front
      // instead of one DRAM round trip in front of every pair
      nc = cl_n[i];
      const int nh = nc < CAND_SMEM ? nc : CAND_SMEM;
#pragma unroll 8
      for (int k = 0; k < nh; ++k) s_cand[k * nt + t] = __ldcs(cl + (size_t)k * n + i);  // read once a step
    }
  }
  __syncwarp();
  // candidate k: shared memory, then the list rows (or, for an atom that
  // searched afresh, its pj rows)
  const unsigned *__restrict__ tail = fresh ? pj : cl;
  double rho = 0.0, Sx = 0.0, Sy = 0.0, Sz = 0.0;
  double mxx = 0.0, mxy = 0.0, mxz = 0.0, myy = 0.0, myz = 0.0, mzz = 0.0;
  int ns = 0;
  // pass 2: the image of each candidate from FP32 copies of the positions
  // (integer and FP32 work), then k_density's FP64 work per pair
  const float xif = float_bits(xi.x), yif = float_bits(xi.y), zif = float_bits(xi.z);
  const int nmax = __reduce_max_sync(0xffffffffu, nc);
  for (int k = 0; k < nmax; ++k) {
    if (k < nc) {
      const unsigned j = (k < CAND_SMEM ? s_cand[k * nt + t] : __ldcs(tail + (size_t)k * n + i)) & IDX_MASK;
      const D4 xj = x[j];
      const unsigned code = image_code(P, xif, yif, zif, xj);
      double ex, ey, ez;
      density_vector(P, xi, xj, code, ex, ey, ez);
      const double r2 = dot3_fma(ex, ey, ez, ex, ey, ez);
      if (below(r2, P.rc2)) {
        if (ns < P.kcap)
          density_pair<true, MULTI, true>(P, ei, j | (code << IDX_BITS), (int)xj.w, ex, ey, ez, r2,
                                          (size_t)ns * n + i, pj, pe, pg, v, err, rho, mxx, mxy, mxz, myy, myz, mzz,
                                          Sx, Sy, Sz);
        else
          atomicOr(err, ERR_PAIR_OVERFLOW);
        ++ns;
      }
    }
  }
  if (!valid) return;
  density_epilogue<true, true>(P, i, active, xi, ei, rho, ns < P.kcap ? ns : P.kcap, mxx, mxy, mxz, myy, myz, mzz, Sx, Sy, Sz, xi_given,
                               xi_mode, T_e, nshort, A, Bw, rho_out, beta_out, cell, Te_i, err, counters, v, Mm, G);
}

// k_density_list with k_density_df's pass 2: the candidates come from the
// kept lists as there (build steps search the bins, atoms flagged near moved
// ones search afresh), then every pair term and sum in df64 from the records
// k_list_check wrote this step (bins of the current positions); the periodic
// image of a candidate comes from FP32 positions rebuilt from those records
// (B w + o, good to ~1e-6 of the box: the image test has a margin of
// tens of angstroms).
template <bool MULTI>
__global__ void __launch_bounds__(128, EPH_DF_DENSITY_BLOCKS) k_density_list_df(
    StepParams P, const D4 *__restrict__ x, const int *__restrict__ mask, const int *__restrict__ bin_count,
    const BinEntry *__restrict__ bins, const int4 *__restrict__ atom_bin, const float4 *__restrict__ atom_off,
    const float4 *__restrict__ rec, const float4 *__restrict__ vrec, const D4 *__restrict__ xi_given, int xi_mode,
    const double *__restrict__ T_e, unsigned *__restrict__ pj, float4 *__restrict__ pa, float4 *__restrict__ pb,
    float4 *__restrict__ pc, int *__restrict__ nshort, D4 *__restrict__ A, D4 *__restrict__ Bw,
    double *__restrict__ rho_out, double *__restrict__ beta_out, int *__restrict__ cell, double *__restrict__ Te_i,
    int *__restrict__ wrapflag, unsigned *__restrict__ err, unsigned long long *__restrict__ counters,
    const D4 *__restrict__ v, D4 *__restrict__ Mm, D4 *__restrict__ G, unsigned *__restrict__ cl,
    int *__restrict__ cl_n, const int *__restrict__ state, const int *__restrict__ rb,
    const int *__restrict__ flist) {
  using namespace df64;
  __shared__ unsigned s_cand[CAND_SMEM * 128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = threadIdx.x, nt = blockDim.x;
  if (i == 0) *wrapflag = 0;  // k_list_check has read it
  const bool valid = i < P.n;
  const bool active = valid && (mask[i] & P.groupbit) != 0;
  const size_t n = (size_t)P.n;
  auto sget = [&](int k) -> unsigned { return k < CAND_SMEM ? s_cand[k * nt + t] : pj[(size_t)k * n + i]; };
  auto sset = [&](int k, unsigned u) {
    if (k < CAND_SMEM)
      s_cand[k * nt + t] = u;
    else
      pj[(size_t)k * n + i] = u;
  };
  auto lset = [&](int k, unsigned u) {
    if (k < CAND_SMEM) s_cand[k * nt + t] = u;
    cl[(size_t)k * n + i] = u;
  };
  auto lget = [&](int k) -> unsigned { return cl[(size_t)k * n + i]; };
  D4 xi = D4{0.0, 0.0, 0.0, 0.0};
  if (valid) xi = x[i];
  const bool build = rb[2] != 0;
  int nc = 0;
  bool fresh = false;
  if (build) {
    int4 Bi = make_int4(0, 0, 0, 0);
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
      Bi = atom_bin[i];
      oi = atom_off[i];
    }
    nc = collect_candidates<true>(P, i, active, Bi, oi, bin_count, bins, err, lget, lset, P.rc2_band, P.lcap);
    nc = collect_candidates<true>(P, i, active, Bi, oi, bin_count, bins, err, lget, lset, P.rl2_band, P.lcap,
                                  nullptr, P.rc2_band, nc);
    if (valid) cl_n[i] = nc;
  } else {
    const int st = active ? state[i] : 0;
    fresh = st != 0;
    if (__any_sync(0xffffffffu, fresh)) {
      int4 Bi = make_int4(0, 0, 0, 0);
      float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
      if (fresh) {
        if (st & 2) {
          current_bin(P, xi, Bi, oi);
        } else {
          Bi = atom_bin[i];
          oi = atom_off[i];
        }
      }
      nc = collect_candidates<true, true>(P, i, fresh, Bi, oi, bin_count, bins, err, sget, sset, P.rl2_band, P.kcap,
                                          state);
      const int nf = rb[1];  // <= LIST_FMAX on a step without a build
      for (int q = 0; q < nf; ++q) {
        const int f = flist[q];
        if (fresh && f != i) {
          const D4 xf = x[f];
          const double dx = min_image(xf.x - xi.x, P.prd[0], P.half_prd[0]);
          const double dy = min_image(xf.y - xi.y, P.prd[1], P.half_prd[1]);
          const double dz = min_image(xf.z - xi.z, P.prd[2], P.half_prd[2]);
          if (dx * dx + dy * dy + dz * dz < P.rc2 * (1.0 + 1e-4)) {
            if (nc < P.kcap)
              sset(nc++, (unsigned)f | (CODE_NOSHIFT << IDX_BITS));
            else
              atomicOr(err, ERR_PAIR_OVERFLOW);
          }
        }
      }
    }
    if (active && !fresh) {
      nc = cl_n[i];
      const int nh = nc < CAND_SMEM ? nc : CAND_SMEM;
#pragma unroll 8
      for (int k = 0; k < nh; ++k) s_cand[k * nt + t] = __ldcs(cl + (size_t)k * n + i);  // read once a step
    }
  }
  __syncwarp();
  const unsigned *__restrict__ tail = fresh ? pj : cl;
  // atom i's records; its FP32 position B w + o for the image test
  float4 oi = make_float4(0.f, 0.f, 0.f, 0.f), Ri1 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (valid) {
    oi = rec[2 * (size_t)i];
    Ri1 = rec[2 * (size_t)i + 1];
  }
  const unsigned pki = __float_as_uint(oi.w);
  const int bix = (int)(pki & 1023u) - 1, biy = (int)((pki >> 10) & 1023u) - 1, biz = (int)((pki >> 20) & 1023u) - 1;
  const float pix = (float)bix * P.wf[0] + oi.x, piy = (float)biy * P.wf[1] + oi.y, piz = (float)biz * P.wf[2] + oi.z;
  const int ei = __float_as_int(Ri1.w);
  bsum sm[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) sm[q] = bsum_zero();
  const df rc2{P.rc2_hi, P.rc2_lo};
  int ns = 0;
  const int nmax = __reduce_max_sync(0xffffffffu, nc);
  for (int k = 0; k < nmax; ++k) {
    const bool have = k < nc;
    const unsigned j = have ? (k < CAND_SMEM ? s_cand[k * nt + t] : __ldcs(tail + (size_t)k * n + i)) & IDX_MASK : 0u;
    const float4 R0 = rec[2 * (size_t)j], R1 = rec[2 * (size_t)j + 1];
    const unsigned pk = __float_as_uint(R0.w);
    const int bjx = (int)(pk & 1023u) - 1, bjy = (int)((pk >> 10) & 1023u) - 1, bjz = (int)((pk >> 20) & 1023u) - 1;
    const float qx = (float)bjx * P.wf[0] + R0.x - pix, qy = (float)bjy * P.wf[1] + R0.y - piy,
                qz = (float)bjz * P.wf[2] + R0.z - piz;
    const int mx = qx > P.half_prdf[0] ? -1 : (qx < -P.half_prdf[0] ? 1 : 0);
    const int my = qy > P.half_prdf[1] ? -1 : (qy < -P.half_prdf[1] ? 1 : 0);
    const int mz = qz > P.half_prdf[2] ? -1 : (qz < -P.half_prdf[2] ? 1 : 0);
    const unsigned code = (unsigned)((mx + 1) + 3 * (my + 1) + 9 * (mz + 1));
    const df ex = pair_disp(bjx + mx * P.nb[0] - bix, R0.x, R1.x, oi.x, Ri1.x, P.w_hi[0], P.w_lo[0]);
    const df ey = pair_disp(bjy + my * P.nb[1] - biy, R0.y, R1.y, oi.y, Ri1.y, P.w_hi[1], P.w_lo[1]);
    const df ez = pair_disp(bjz + mz * P.nb[2] - biz, R0.z, R1.z, oi.z, Ri1.z, P.w_hi[2], P.w_lo[2]);
    df r2 = dot3(ex, ey, ez, ex, ey, ez);
    const bool in = have && lt(r2, rc2);
    // the shell beyond the cut-off sits at the end of the lists: where no
    // lane of the warp has a pair inside, the iteration would add only zeros
    if (!__any_sync(0xffffffffu, in)) {
      if ((k & 7) == 7) {
#pragma unroll
        for (int q = 0; q < 9; ++q) bsum_fold(sm[q]);
      }
      continue;
    }
    if (!in) r2 = df{1.0f, 0.0f};
    const int ej = __float_as_int(R1.w);
    const df rji = spline_rho_df(P, ej, r2, err);
    const df inv = recip(r2, rcp_estimate(r2.hi));
    df H = mul(rji, inv);
    if (!in) H = df{0.0f, 0.0f};
    const df hx = mul(H, ex), hy = mul(H, ey), hz = mul(H, ez);
    if (in) {
      if (ns < P.kcap) {
        const size_t slot = (size_t)ns * n + i;
        pj[slot] = j | (code << IDX_BITS);
        if (MULTI) {
          const df rij = ej != ei ? spline_rho_df(P, ei, r2, err) : rji;
          const df Hji = mul(rij, inv);
          pa[slot] = make_float4(ex.hi, ey.hi, ez.hi, Hji.hi);
          pb[slot] = make_float4(ex.lo, ey.lo, ez.lo, Hji.lo);
          pc[slot] = make_float4(H.hi, H.lo, 0.f, 0.f);
        } else {
          pa[slot] = make_float4(ex.hi, ey.hi, ez.hi, hx.hi);
          pb[slot] = make_float4(ex.lo, ey.lo, ez.lo, hx.lo);
          pc[slot] = make_float4(hy.hi, hz.hi, hy.lo, hz.lo);
        }
      } else {
        atomicOr(err, ERR_PAIR_OVERFLOW);
      }
      ++ns;
    }
    acc_fma(sm[0].blk, hx, ex);
    acc_fma(sm[1].blk, hx, ey);
    acc_fma(sm[2].blk, hx, ez);
    acc_fma(sm[3].blk, hy, ey);
    acc_fma(sm[4].blk, hy, ez);
    acc_fma(sm[5].blk, hz, ez);
    const float4 V0 = vrec[2 * (size_t)j], V1 = vrec[2 * (size_t)j + 1];
    const df d = dot3(ex, ey, ez, df{V0.x, V1.x}, df{V0.y, V1.y}, df{V0.z, V1.z});
    acc_fma(sm[6].blk, d, hx);
    acc_fma(sm[7].blk, d, hy);
    acc_fma(sm[8].blk, d, hz);
    if ((k & 7) == 7) {
#pragma unroll
      for (int q = 0; q < 9; ++q) bsum_fold(sm[q]);
    }
  }
  if (!valid) return;
  double mq[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) mq[q] = to_double(bsum_value(sm[q]));
  density_epilogue<true, true, true>(P, i, active, xi, ei, 0.0, ns < P.kcap ? ns : P.kcap, mq[0], mq[1], mq[2],
                                     mq[3], mq[4], mq[5], mq[6], mq[7], mq[8], xi_given, xi_mode, T_e, nshort, A,
                                     Bw, rho_out, beta_out, cell, Te_i, err, counters, v, Mm, G);
}

// -------------------------------------------------------- friction sweep 1

// force_prl stage 1 (fix_eph.cpp:699-741) in the reference's expression order
// (EXACT mode; FAST mode folds it into the density sweep):
// w_i = sum_j p_ij [(e.v_i) - (e.v_j)] e,  p_ij = alpha_i rho_j(r^2) / (rho_i r^2)
__global__ void __launch_bounds__(128) k_friction_w(StepParams P, const int *__restrict__ mask,
                                                     const D4 *__restrict__ v, const unsigned *__restrict__ pj,
                                                     const D4 *__restrict__ pe, const double2 *__restrict__ pg,
                                                     const int *__restrict__ nshort, const D4 *__restrict__ A,
                                                     D4 *__restrict__ Bw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const D4 Ai = A[i];
  if (!(mask[i] & P.groupbit) || !pos_double(Ai.x)) return;  // Bw[i].yzw stays 0
  const D4 vi = v[i];
  const int ns = nshort[i];
  double wx = 0.0, wy = 0.0, wz = 0.0;
  for (int k = 0; k < ns; ++k) {
    const size_t slot = (size_t)k * P.n + i;
    const unsigned j = pj[slot] & IDX_MASK;
    const D4 e = pe[slot];
    const D4 vj = v[j];
    const double rji = pg[slot].x;
    const double prescaler = Ai.y * rji / (Ai.x * e.w);
    const double var1 = prescaler * dot3(e.x, e.y, e.z, vi.x, vi.y, vi.z);
    const double var2 = prescaler * dot3(e.x, e.y, e.z, vj.x, vj.y, vj.z);
    const double dvar = var1 - var2;
    wx += dvar * e.x;
    wy += dvar * e.y;
    wz += dvar * e.z;
  }
  const double xiz = Bw[i].x;
  Bw[i] = D4{xiz, wx, wy, wz};
}

// ------------------------------------------------ friction + random sweep

// The end of post_force for atom i: the coloured-noise memory of
// eph/coloured/exp (fix_eph_coloured_exp.cpp:562-568, :619-625), f_EPH and
// f_RNG, and their addition to the engine's force unless NOFRICTION /
// NORANDOM keep them out (fix_eph.cpp:892-906).
template <bool FRIC, bool RAND>
__device__ __forceinline__ void store_forces(const StepParams &P, int i, bool live, double fex, double fey,
                                             double fez, double frx, double fry, double frz, D4 *__restrict__ f,
                                             D4 *__restrict__ f_eph, D4 *__restrict__ f_rng, D4 *__restrict__ f_dis,
                                             D4 *__restrict__ f_sto) {
  if (P.coloured && live) {
    if (FRIC) {
      D4 d = f_dis[i];
      d.x = d.x * (1. - P.zeta) + P.zeta * fex;
      d.y = d.y * (1. - P.zeta) + P.zeta * fey;
      d.z = d.z * (1. - P.zeta) + P.zeta * fez;
      f_dis[i] = d;
      fex = d.x;
      fey = d.y;
      fez = d.z;
    }
    if (RAND) {
      D4 d = f_sto[i];
      d.x = d.x * (1. - P.zeta) + P.zeta * frx;
      d.y = d.y * (1. - P.zeta) + P.zeta * fry;
      d.z = d.z * (1. - P.zeta) + P.zeta * frz;
      f_sto[i] = d;
      frx = d.x;
      fry = d.y;
      frz = d.z;
    }
  }
  f_eph[i] = D4{fex, fey, fez, 0.0};
  f_rng[i] = D4{frx, fry, frz, 0.0};
  D4 fi = f[i];
  if (FRIC && !(P.flags & 0x10)) {
    fi.x += fex;
    fi.y += fey;
    fi.z += fez;
  }
  if (RAND && !(P.flags & 0x20)) {
    fi.x += frx;
    fi.y += fry;
    fi.z += frz;
  }
  f[i] = fi;
}

// force_prl stages 2 and 3 (fix_eph.cpp:748-836) in one pass over the pairs,
// then the force update of post_force (fix_eph.cpp:892-906):
//   f_EPH_i -= sum_j [a_i rho_j(r^2) (e.w_i)/(rho_i r^2) - a_j rho_i(r^2) (e.w_j)/(rho_j r^2)] e
//   f_RNG_i  = eta sqrt(T_e(x_i)) sum_j [same with xi] e
template <bool FAST, bool MULTI, bool FRIC, bool RAND>
__global__ void __launch_bounds__(128) k_forces(StepParams P, const int *__restrict__ mask,
                                                const unsigned *__restrict__ pj, const D4 *__restrict__ pe,
                                                const double2 *__restrict__ pg, const int *__restrict__ nshort,
                                                const D4 *__restrict__ A, const D4 *__restrict__ Bw,
                                                const double *__restrict__ Te_i, D4 *__restrict__ f,
                                                D4 *__restrict__ f_eph, D4 *__restrict__ f_rng,
                                                D4 *__restrict__ f_dis, D4 *__restrict__ f_sto) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double fex = 0.0, fey = 0.0, fez = 0.0, frx = 0.0, fry = 0.0, frz = 0.0;
  const D4 Ai = A[i];
  const bool live = (mask[i] & P.groupbit) && pos_double(Ai.x);
  if (live) {
    const D4 Bi = Bw[i];
    const double xix = Ai.z, xiy = Ai.w, xiz = Bi.x;
    const int ns = nshort[i];
    for (int k = 0; k < ns; ++k) {
      const size_t slot = (size_t)k * P.n + i;
      const unsigned j = pj[slot] & IDX_MASK;
      const D4 Aj = A[j];
      if (!pos_double(Aj.x)) continue;
      const D4 e = pe[slot];
      // FAST mode with one element has no pg rows (the buffer is not allocated)
      const double2 g = (FAST && !MULTI) ? make_double2(0.0, 0.0) : pg[slot];
      const D4 Bj = Bw[j];
      if (FAST) {
        const double a = Ai.y * e.w;                  // alpha_i/rho_i * rho_j(r^2)/r^2
        const double b = Aj.y * (MULTI ? g.x : e.w);  // alpha_j/rho_j * rho_i(r^2)/r^2
        if (FRIC) {
          const double di = dot3_fma(e.x, e.y, e.z, Bi.y, Bi.z, Bi.w);
          const double dj = dot3_fma(e.x, e.y, e.z, Bj.y, Bj.z, Bj.w);
          const double dvar = fma(a, di, -(b * dj));
          fex = fma(-dvar, e.x, fex);
          fey = fma(-dvar, e.y, fey);
          fez = fma(-dvar, e.z, fez);
        }
        if (RAND) {
          const double di = dot3_fma(e.x, e.y, e.z, xix, xiy, xiz);
          const double dj = dot3_fma(e.x, e.y, e.z, Aj.z, Aj.w, Bj.x);
          const double dvar = fma(a, di, -(b * dj));
          frx = fma(dvar, e.x, frx);
          fry = fma(dvar, e.y, fry);
          frz = fma(dvar, e.z, frz);
        }
      } else {
        const double r2 = e.w;
        const double ai = Ai.y * g.x;                 // alpha_i * rho_j(r^2)
        const double aj = Aj.y * (MULTI ? g.y : g.x);  // alpha_j * rho_i(r^2)
        const double den_i = Ai.x * r2, den_j = Aj.x * r2;
        if (FRIC) {
          const double var1 = ai * dot3(e.x, e.y, e.z, Bi.y, Bi.z, Bi.w) / den_i;
          const double var2 = aj * dot3(e.x, e.y, e.z, Bj.y, Bj.z, Bj.w) / den_j;
          const double dvar = var1 - var2;
          fex -= dvar * e.x;
          fey -= dvar * e.y;
          fez -= dvar * e.z;
        }
        if (RAND) {
          const double var1 = ai * dot3(e.x, e.y, e.z, xix, xiy, xiz) / den_i;
          const double var2 = aj * dot3(e.x, e.y, e.z, Aj.z, Aj.w, Bj.x) / den_j;
          const double dvar = var1 - var2;
          frx += dvar * e.x;
          fry += dvar * e.y;
          frz += dvar * e.z;
        }
      }
    }
    if (RAND) {
      const double var = P.eta * sqrt(Te_i[i]);
      frx *= var;
      fry *= var;
      frz *= var;
    }
  }
  store_forces<FRIC, RAND>(P, i, live, fex, fey, fez, frx, fry, frz, f, f_eph, f_rng, f_dis, f_sto);
}

// Stages 2 and 3 in FAST mode after k_density<.., true> (same sums as
// k_forces, split into the atom's own part and the neighbours' part); TPA
// lanes per atom take rows g, g + TPA, ... of the neighbours' part and
// combine by a butterfly, as k_forces_tpa does.  With W_i = a_i w_i, X_i = a_i xi_i (a_i = alpha_i/rho_i)
// and M_i = sum_j H_ij e e^T over all of the atom's pairs:
//   f_EPH_i = -M_i W_i + sum_{j live} H_ji (e.W_j) e + sum_{j not live} H_ij (e.W_i) e
//   f_RNG_i = eta sqrt(T_e) [M_i X_i - sum_{j live} H_ji (e.X_j) e - sum_{j not live} H_ij (e.X_i) e]
// ("live": rho_j > 0, the reference's test; the last sums take back the
// pairs it skips).  Per pair 14 FP64 instructions instead of 24.
template <bool MULTI, bool RAND, int TPA = 1>
__global__ void __launch_bounds__(128) k_forces_m(StepParams P, const unsigned *__restrict__ pj,
                                                  const D4 *__restrict__ pe, const double2 *__restrict__ pg,
                                                  const int *__restrict__ nshort, const D4 *__restrict__ Mm,
                                                  const D4 *__restrict__ G, const double *__restrict__ Te_i,
                                                  D4 *__restrict__ f, D4 *__restrict__ f_eph, D4 *__restrict__ f_rng,
                                                  D4 *__restrict__ f_dis, D4 *__restrict__ f_sto) {
  const long gt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(gt / TPA), g = (int)(gt % TPA);
  if (TPA == 1 && i >= P.n) return;  // with TPA > 1 every lane joins the butterfly
  double fex = 0.0, fey = 0.0, fez = 0.0, frx = 0.0, fry = 0.0, frz = 0.0;
  bool live = false;
  int ns = 0, skipped = 0;
  if (i < P.n) {
    live = pos_double(G[2 * (size_t)i + 1].z);  // rho_i > 0 (0 outside the group)
    if (live) ns = nshort[i];
  }
  for (int k = g; k < ns; k += TPA) {
    const size_t slot = (size_t)k * P.n + i;
    const unsigned j = pj[slot] & IDX_MASK;
    const D4 e = pe[slot];
    const D4 Gj1 = G[2 * (size_t)j], Gj2 = G[2 * (size_t)j + 1];
    if (!pos_double(Gj2.z)) {  // a pair the reference skips (handled below)
      skipped = 1;
      continue;
    }
    if (MULTI) {
      const double Hji = pg[slot].x;  // rho_i(r^2)/r^2
      const double sw = Hji * dot3_fma(e.x, e.y, e.z, Gj1.x, Gj1.y, Gj1.z);
      fex = fma(sw, e.x, fex);
      fey = fma(sw, e.y, fey);
      fez = fma(sw, e.z, fez);
      if (RAND) {
        const double sx = Hji * dot3_fma(e.x, e.y, e.z, Gj1.w, Gj2.x, Gj2.y);
        frx = fma(sx, e.x, frx);
        fry = fma(sx, e.y, fry);
        frz = fma(sx, e.z, frz);
      }
    } else {  // the pair's H e: {e.w, pg.x, pg.y}
      const double2 h = pg[slot];
      const double sw = dot3_fma(e.x, e.y, e.z, Gj1.x, Gj1.y, Gj1.z);
      fex = fma(sw, e.w, fex);
      fey = fma(sw, h.x, fey);
      fez = fma(sw, h.y, fez);
      if (RAND) {
        const double sx = dot3_fma(e.x, e.y, e.z, Gj1.w, Gj2.x, Gj2.y);
        frx = fma(sx, e.w, frx);
        fry = fma(sx, h.x, fry);
        frz = fma(sx, h.y, frz);
      }
    }
  }
  if (TPA > 1) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) {
      fex += __shfl_xor_sync(0xffffffffu, fex, o);
      fey += __shfl_xor_sync(0xffffffffu, fey, o);
      fez += __shfl_xor_sync(0xffffffffu, fez, o);
      if (RAND) {
        frx += __shfl_xor_sync(0xffffffffu, frx, o);
        fry += __shfl_xor_sync(0xffffffffu, fry, o);
        frz += __shfl_xor_sync(0xffffffffu, frz, o);
      }
      skipped |= __shfl_xor_sync(0xffffffffu, skipped, o);
    }
    if (i >= P.n || g != 0) return;
  }
  if (live) {
    double cex = 0.0, cey = 0.0, cez = 0.0, crx = 0.0, cry = 0.0, crz = 0.0;
    const D4 Gi1 = G[2 * (size_t)i], Gi2 = G[2 * (size_t)i + 1];
    if (skipped) {  // rare: the skipped pairs' shares of M_i come back out (a second
                    // pass keeps this work out of the main loop's instruction stream)
      for (int k = 0; k < ns; ++k) {
        const size_t slot = (size_t)k * P.n + i;
        const unsigned j = pj[slot] & IDX_MASK;
        if (pos_double(G[2 * (size_t)j + 1].z)) continue;
        const D4 e = pe[slot];
        // H_ij e: {H e.x, e.y, e.z} with several elements, {e.w, pg} with one
        double hx = e.x, hy = e.y, hz = e.z, H = e.w;
        if (!MULTI) {
          const double2 h = pg[slot];
          hx = e.w;
          hy = h.x;
          hz = h.y;
          H = 1.0;
        }
        const double sw = H * dot3_fma(e.x, e.y, e.z, Gi1.x, Gi1.y, Gi1.z);
        cex = fma(sw, hx, cex);
        cey = fma(sw, hy, cey);
        cez = fma(sw, hz, cez);
        if (RAND) {
          const double sx = H * dot3_fma(e.x, e.y, e.z, Gi1.w, Gi2.x, Gi2.y);
          crx = fma(sx, hx, crx);
          cry = fma(sx, hy, cry);
          crz = fma(sx, hz, crz);
        }
      }
    }
    const D4 M1 = Mm[i], M2 = Mm[(size_t)P.n + i];  // {xx, xy, xz, yy}, {yz, zz}
    fex += cex - fma(M1.x, Gi1.x, fma(M1.y, Gi1.y, M1.z * Gi1.z));
    fey += cey - fma(M1.y, Gi1.x, fma(M1.w, Gi1.y, M2.x * Gi1.z));
    fez += cez - fma(M1.z, Gi1.x, fma(M2.x, Gi1.y, M2.y * Gi1.z));
    if (RAND) {
      const double var = P.eta * sqrt(Te_i[i]);
      frx = var * (fma(M1.x, Gi1.w, fma(M1.y, Gi2.x, M1.z * Gi2.y)) - crx - frx);
      fry = var * (fma(M1.y, Gi1.w, fma(M1.w, Gi2.x, M2.x * Gi2.y)) - cry - fry);
      frz = var * (fma(M1.z, Gi1.w, fma(M2.x, Gi2.x, M2.y * Gi2.y)) - crz - frz);
    }
  }
  store_forces<true, RAND>(P, i, live, fex, fey, fez, frx, fry, frz, f, f_eph, f_rng, f_dis, f_sto);
}

// k_forces_m over the df64 pair cache and records of k_density_df: per pair
// (e.W_j) H e and (e.X_j) H e (several elements: H_ji (e.W_j) e) in df64
// with blocked sums; the per-atom part (-M_i W_i, the pairs the reference
// skips, eta sqrt(T_e), the force update) in FP64 as k_forces_m does it, with
// W_i = a_i w_i and X_i = a_i xi_i formed from A and Bw exactly as the FP64
// records are.  A neighbour the reference skips (rho_j <= 0 or outside the
// group) carries a NaN in its record's first word.
template <bool MULTI, bool RAND, int TPA = 1>
__global__ void __launch_bounds__(128, EPH_DF_FORCES_BLOCKS)
    k_forces_df(StepParams P, const unsigned *__restrict__ pj, const float4 *__restrict__ pa,
                const float4 *__restrict__ pb, const float4 *__restrict__ pc, const int *__restrict__ nshort,
                const D4 *__restrict__ Mm, const float4 *__restrict__ Gf, const D4 *__restrict__ A,
                const D4 *__restrict__ Bw, const double *__restrict__ Te_i, D4 *__restrict__ f,
                D4 *__restrict__ f_eph, D4 *__restrict__ f_rng, D4 *__restrict__ f_dis, D4 *__restrict__ f_sto) {
  using namespace df64;
  const long gt = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(gt / TPA), g = (int)(gt % TPA);
  if (TPA == 1 && i >= P.n) return;  // with TPA > 1 every lane joins the butterfly
  bsum se[3], sr[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) se[q] = sr[q] = bsum_zero();
  bool live = false;
  int ns = 0, skipped = 0;
  if (i < P.n) {
    const float g0 = Gf[3 * (size_t)i].x;
    live = g0 == g0;  // not NaN: rho_i > 0 and in the group
    if (live) ns = nshort[i];
  }
  int m = 0;
  for (int k = g; k < ns; k += TPA, ++m) {
    const size_t slot = (size_t)k * P.n + i;
    const unsigned j = pj[slot] & IDX_MASK;
    const float4 G0 = Gf[3 * (size_t)j];
    if (G0.x != G0.x) {  // a pair the reference skips (handled below)
      skipped = 1;
    } else {
      const float4 a = pa[slot], b = pb[slot];
      const float4 G1 = Gf[3 * (size_t)j + 1];
      const df ex{a.x, b.x}, ey{a.y, b.y}, ez{a.z, b.z};
      df hx, hy, hz;
      if (MULTI) {
        const df Hji{a.w, b.w};
        hx = mul(Hji, ex);
        hy = mul(Hji, ey);
        hz = mul(Hji, ez);
      } else {
        const float4 c = pc[slot];
        hx = df{a.w, b.w};
        hy = df{c.x, c.z};
        hz = df{c.y, c.w};
      }
      const df sw = dot3(ex, ey, ez, df{G0.x, G1.x}, df{G0.y, G1.y}, df{G0.z, G1.z});
      acc_fma(se[0].blk, sw, hx);
      acc_fma(se[1].blk, sw, hy);
      acc_fma(se[2].blk, sw, hz);
      if (RAND) {
        const float4 G2 = Gf[3 * (size_t)j + 2];
        const df sx = dot3(ex, ey, ez, df{G0.w, G1.w}, df{G2.x, G2.z}, df{G2.y, G2.w});
        acc_fma(sr[0].blk, sx, hx);
        acc_fma(sr[1].blk, sx, hy);
        acc_fma(sr[2].blk, sx, hz);
      }
    }
    if ((m & 7) == 7) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        bsum_fold(se[q]);
        if (RAND) bsum_fold(sr[q]);
      }
    }
  }
  double fex = to_double(bsum_value(se[0])), fey = to_double(bsum_value(se[1])), fez = to_double(bsum_value(se[2]));
  double frx = 0.0, fry = 0.0, frz = 0.0;
  if (RAND) {
    frx = to_double(bsum_value(sr[0]));
    fry = to_double(bsum_value(sr[1]));
    frz = to_double(bsum_value(sr[2]));
  }
  if (TPA > 1) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) {
      fex += __shfl_xor_sync(0xffffffffu, fex, o);
      fey += __shfl_xor_sync(0xffffffffu, fey, o);
      fez += __shfl_xor_sync(0xffffffffu, fez, o);
      if (RAND) {
        frx += __shfl_xor_sync(0xffffffffu, frx, o);
        fry += __shfl_xor_sync(0xffffffffu, fry, o);
        frz += __shfl_xor_sync(0xffffffffu, frz, o);
      }
      skipped |= __shfl_xor_sync(0xffffffffu, skipped, o);
    }
    if (i >= P.n || g != 0) return;
  }
  if (live) {
    double cex = 0.0, cey = 0.0, cez = 0.0, crx = 0.0, cry = 0.0, crz = 0.0;
    const D4 Ai = A[i], Bi = Bw[i];
    const double a = Ai.y;  // alpha_i / rho_i
    const double Wx = a * Bi.y, Wy = a * Bi.z, Wz = a * Bi.w;
    const double Xx = a * Ai.z, Xy = a * Ai.w, Xz = a * Bi.x;
    if (skipped) {  // rare: the skipped pairs' shares of M_i come back out
      for (int k = 0; k < ns; ++k) {
        const size_t slot = (size_t)k * P.n + i;
        const unsigned j = pj[slot] & IDX_MASK;
        const float g0 = Gf[3 * (size_t)j].x;
        if (g0 == g0) continue;
        const float4 pa4 = pa[slot], pb4 = pb[slot], pc4 = pc[slot];
        const double ex = to_double(df{pa4.x, pb4.x}), ey = to_double(df{pa4.y, pb4.y}),
                     ez = to_double(df{pa4.z, pb4.z});
        double hx, hy, hz, H;
        if (MULTI) {  // H_ij e
          H = to_double(df{pc4.x, pc4.y});
          hx = ex;
          hy = ey;
          hz = ez;
        } else {
          hx = to_double(df{pa4.w, pb4.w});
          hy = to_double(df{pc4.x, pc4.z});
          hz = to_double(df{pc4.y, pc4.w});
          H = 1.0;
        }
        const double sw = H * dot3_fma(ex, ey, ez, Wx, Wy, Wz);
        cex = fma(sw, hx, cex);
        cey = fma(sw, hy, cey);
        cez = fma(sw, hz, cez);
        if (RAND) {
          const double sx = H * dot3_fma(ex, ey, ez, Xx, Xy, Xz);
          crx = fma(sx, hx, crx);
          cry = fma(sx, hy, cry);
          crz = fma(sx, hz, crz);
        }
      }
    }
    const D4 M1 = Mm[i], M2 = Mm[(size_t)P.n + i];  // {xx, xy, xz, yy}, {yz, zz}
    fex += cex - fma(M1.x, Wx, fma(M1.y, Wy, M1.z * Wz));
    fey += cey - fma(M1.y, Wx, fma(M1.w, Wy, M2.x * Wz));
    fez += cez - fma(M1.z, Wx, fma(M2.x, Wy, M2.y * Wz));
    if (RAND) {
      const double var = P.eta * sqrt(Te_i[i]);
      frx = var * (fma(M1.x, Xx, fma(M1.y, Xy, M1.z * Xz)) - crx - frx);
      fry = var * (fma(M1.y, Xx, fma(M1.w, Xy, M2.x * Xz)) - cry - fry);
      frz = var * (fma(M1.z, Xx, fma(M2.x, Xy, M2.y * Xz)) - crz - frz);
    }
  }
  store_forces<true, RAND>(P, i, live, fex, fey, fez, frx, fry, frz, f, f_eph, f_rng, f_dis, f_sto);
}

// ------------------------------------- pair sweeps, several lanes per atom

// FAST mode with TPA lanes per atom (TPA = 2, 4, 8): lane g of an atom takes
// rows g, g + TPA, ...; the lanes' sums are combined by a butterfly over the
// TPA neighbouring lanes.  Small systems (tens of thousands of atoms) leave
// the SMs with a few warps each and the one-lane sweeps wait on their loads;
// TPA times more warps hide that.  The order of the sums depends on TPA
// (results within rounding of the one-lane sweeps, the same every run).
template <bool MULTI, bool FRIC, bool RAND, int TPA>
__global__ void __launch_bounds__(128) k_forces_tpa(StepParams P, const int *__restrict__ mask,
                                                     const unsigned *__restrict__ pj, const D4 *__restrict__ pe,
                                                     const double2 *__restrict__ pg, const int *__restrict__ nshort,
                                                     const D4 *__restrict__ A, const D4 *__restrict__ Bw,
                                                     const double *__restrict__ Te_i, D4 *__restrict__ f,
                                                     D4 *__restrict__ f_eph, D4 *__restrict__ f_rng,
                                                     D4 *__restrict__ f_dis, D4 *__restrict__ f_sto) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gt / TPA, g = gt % TPA;
  double fex = 0.0, fey = 0.0, fez = 0.0, frx = 0.0, fry = 0.0, frz = 0.0;
  D4 Ai{0.0, 0.0, 0.0, 0.0};
  bool live = false;
  if (i < P.n) {
    Ai = A[i];
    live = (mask[i] & P.groupbit) && pos_double(Ai.x);
  }
  if (live) {
    const D4 Bi = Bw[i];
    const double xix = Ai.z, xiy = Ai.w, xiz = Bi.x;
    const int ns = nshort[i];
    for (int k = g; k < ns; k += TPA) {
      const size_t slot = (size_t)k * P.n + i;
      const unsigned j = pj[slot] & IDX_MASK;
      const D4 Aj = A[j];
      if (!pos_double(Aj.x)) continue;
      const D4 e = pe[slot];
      const D4 Bj = Bw[j];
      const double a = Ai.y * e.w;
      const double b = Aj.y * (MULTI ? pg[slot].x : e.w);
      if (FRIC) {
        const double di = dot3_fma(e.x, e.y, e.z, Bi.y, Bi.z, Bi.w);
        const double dj = dot3_fma(e.x, e.y, e.z, Bj.y, Bj.z, Bj.w);
        const double dvar = fma(a, di, -(b * dj));
        fex = fma(-dvar, e.x, fex);
        fey = fma(-dvar, e.y, fey);
        fez = fma(-dvar, e.z, fez);
      }
      if (RAND) {
        const double di = dot3_fma(e.x, e.y, e.z, xix, xiy, xiz);
        const double dj = dot3_fma(e.x, e.y, e.z, Aj.z, Aj.w, Bj.x);
        const double dvar = fma(a, di, -(b * dj));
        frx = fma(dvar, e.x, frx);
        fry = fma(dvar, e.y, fry);
        frz = fma(dvar, e.z, frz);
      }
    }
  }
#pragma unroll
  for (int o = TPA / 2; o > 0; o >>= 1) {
    if (FRIC) {
      fex += __shfl_xor_sync(0xffffffffu, fex, o);
      fey += __shfl_xor_sync(0xffffffffu, fey, o);
      fez += __shfl_xor_sync(0xffffffffu, fez, o);
    }
    if (RAND) {
      frx += __shfl_xor_sync(0xffffffffu, frx, o);
      fry += __shfl_xor_sync(0xffffffffu, fry, o);
      frz += __shfl_xor_sync(0xffffffffu, frz, o);
    }
  }
  if (i >= P.n || g != 0) return;
  if (live && RAND) {
    const double var = P.eta * sqrt(Te_i[i]);
    frx *= var;
    fry *= var;
    frz *= var;
  }
  store_forces<FRIC, RAND>(P, i, live, fex, fey, fez, frx, fry, frz, f, f_eph, f_rng, f_dis, f_sto);
}

// --------------------------------------------------------- model 1 (TTM)

// force_ttm (fix_eph.cpp:468-503): a local Langevin thermostat with the
// site's beta(rho_i): f_EPH = -beta v_i, f_RNG = eta alpha(rho_i) sqrt(T_e) xi_i;
// then the force update of post_force (:892-906).
template <bool FAST, bool FRIC, bool RAND>
__global__ void k_forces_ttm(StepParams P, const int *__restrict__ mask, const D4 *__restrict__ x,
                             const D4 *__restrict__ v,
                             const D4 *__restrict__ A, const D4 *__restrict__ Bw, const double *__restrict__ rho,
                             const double *__restrict__ beta, const double *__restrict__ Te_i, D4 *__restrict__ f,
                             D4 *__restrict__ f_eph, D4 *__restrict__ f_rng, unsigned *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  D4 fe = D4{0.0, 0.0, 0.0, 0.0}, fr = D4{0.0, 0.0, 0.0, 0.0};
  if (mask[i] & P.groupbit) {
    if (FRIC) {
      const double var = -beta[i];
      const D4 vi = v[i];
      fe = D4{var * vi.x, var * vi.y, var * vi.z, 0.0};
    }
    if (RAND) {
      const double r = rho[i];
      double alpha = 0.0;
      if (!(r > P.rho_cutoff)) {  // eph_beta.h:188-197
        const int e = (int)x[i].w;
        alpha = spline_eval<FAST>(P.tab_alpha + (size_t)e * P.n_beta, P.inv_drho, P.n_beta, r, err);
      }
      const double var = P.eta * alpha * sqrt(Te_i[i]);
      fr = D4{var * A[i].z, var * A[i].w, var * Bw[i].x, 0.0};
    }
  }
  f_eph[i] = fe;
  f_rng[i] = fr;
  D4 fi = f[i];
  if (FRIC && !(P.flags & 0x10)) {
    fi.x += fe.x;
    fi.y += fe.y;
    fi.z += fe.z;
  }
  if (RAND && !(P.flags & 0x20)) {
    fi.x += fr.x;
    fi.y += fr.y;
    fi.z += fr.z;
  }
  f[i] = fi;
}

// ------------------------------------------------------- energy deposition

// end_of_step deposition (fix_eph.cpp:364-390, eph_fdm.h:172-179): per atom
// dE = -f.v dt for the friction and the random force, dT_e[cell] += dE/(dV dt).
// The grid sums are exact: every term becomes a 128-bit fixed-point integer
// (2^-64 units) and integer addition is order-free, so the grid and the
// energy total are the same whatever order the atoms arrive in; the block
// totals of the energy go to `part` and are summed by k_energy_total.
template <bool FRIC, bool RAND, bool GRID>
__global__ void __launch_bounds__(256) k_deposit(StepParams P, const int *__restrict__ mask,
                                                 const D4 *__restrict__ v, const D4 *__restrict__ f_eph,
                                                 const D4 *__restrict__ f_rng, const int *__restrict__ cell,
                                                 U128 *__restrict__ acc, U128 *__restrict__ part,
                                                 unsigned *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  U128 e{0ull, 0ull};
  if (i < P.n && (mask[i] & P.groupbit)) {
    const D4 vi = v[i];
    U128 g{0ull, 0ull};
    if (FRIC) {
      const D4 fe = f_eph[i];
      double dE = 0.0;
      dE -= fe.x * vi.x * P.dt;
      dE -= fe.y * vi.y * P.dt;
      dE -= fe.z * vi.z * P.dt;
      e = add128(e, to_fixed(dE, err));
      if (GRID) g = add128(g, to_fixed(dE / P.prescale, err));
    }
    if (RAND) {
      const D4 fr = f_rng[i];
      double dE = 0.0;
      dE -= fr.x * vi.x * P.dt;
      dE -= fr.y * vi.y * P.dt;
      dE -= fr.z * vi.z * P.dt;
      e = add128(e, to_fixed(dE, err));
      if (GRID) g = add128(g, to_fixed(dE / P.prescale, err));
    }
    if (GRID && (g.lo | g.hi)) atomic_add128(acc + cell[i], g);
  }
  // block total of the energy, integer adds
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) e = add128(e, shfl_down128(e, d));
  __shared__ U128 warp_tot[8];
  if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    U128 t{0ull, 0ull};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = add128(t, warp_tot[w]);
    part[blockIdx.x] = t;
  }
}

// Sum the block totals, add the step's exchange to Ee (fix_eph.cpp:402-404).
__global__ void k_energy_total(const U128 *__restrict__ part, int nparts, double *__restrict__ E_local,
                               double *__restrict__ Ee) {
  U128 t{0ull, 0ull};
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) t = add128(t, part[b]);
  for (int d = 16; d > 0; d >>= 1) t = add128(t, shfl_down128(t, d));
  __shared__ U128 warp_tot[32];
  if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    U128 s{0ull, 0ull};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = add128(s, warp_tot[w]);
    const double e = from_fixed(s);
    *E_local = e;
    *Ee += e;
  }
}

// ------------------------------------------------------------- FDM solve
// eph_fdm.h:280-287: C_e and kappa_e of the T-dependent cells from T, before
// the stability test; the prescaler rho_e C_e follows.
__global__ void k_fdm_tdyn_params(long ncells, TdynTables t, const double *__restrict__ T, double *__restrict__ C,
                                  double *__restrict__ kappa, double *__restrict__ rhoC, unsigned *__restrict__ err) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ncells || !t.tdyn[r]) return;
  const double c = spline_eval<false>(t.C_T, t.inv_dT, t.n, T[r], err);
  C[r] = c;
  kappa[r] = spline_eval<false>(t.K_T, t.inv_dT, t.n, T[r], err);
  rhoC[r] = t.rho[r] * c;
}

// c_min, rho_min, kappa_max of the stability rule (eph_fdm.h:290-300): cell 0
// whatever its flag, then every cell that is not CONSTANT_VALUE.  One block.
__global__ void k_fdm_bounds(long ncells, const double *__restrict__ C, const double *__restrict__ rho,
                             const double *__restrict__ kappa, const signed char *__restrict__ flag,
                             double *__restrict__ out) {
  double c_min = C[0], r_min = rho[0], k_max = kappa[0];
  for (long i = 1 + threadIdx.x; i < ncells; i += blockDim.x)
    if (flag[i] != 0) {
      c_min = fmin(c_min, C[i]);
      r_min = fmin(r_min, rho[i]);
      k_max = fmax(k_max, kappa[i]);
    }
  __shared__ double s[3][256];
  s[0][threadIdx.x] = c_min;
  s[1][threadIdx.x] = r_min;
  s[2][threadIdx.x] = k_max;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + h]);
      s[1][threadIdx.x] = fmin(s[1][threadIdx.x], s[1][threadIdx.x + h]);
      s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s[0][0];
    out[1] = s[1][0];
    out[2] = s[2][0];
  }
}

// T of cell r after one substep of EPH_FDM::solve (eph_fdm.h:315-396) with
// the reference's expression order: the variable-kappa 7-point stencil with
// periodic wrap and ZERO_DERIVATIVE walls, then T += (ddT + dT + S)/(rho_e C_e)
// dt' on DYNAMIC cells and the clamp at T = 0.  FAST: ih2 = 1/h^2 per axis and
// irhoC = 1/(rho_e C_e) per cell come precomputed (the same correctly rounded
// quotients as 1.0 / x here).  CG: read the temperatures through L2 only
// (other blocks wrote them in the substep before).
template <bool FAST, bool CG>
__device__ __forceinline__ double fdm_cell(long r, long nx, long ny, long nz, double dx, double dy, double dz,
                                           double inner_dt, const double *__restrict__ T,
                                           const double *__restrict__ kappa, const double *__restrict__ rhoC,
                                           const double *__restrict__ S, const signed char *__restrict__ flag,
                                           double dTr, unsigned long long *__restrict__ counters,
                                           const TdynTables &td, double3 ih2, const double *__restrict__ irhoC) {
  auto ldT = [&](long k) -> double { return CG ? __ldcg(T + k) : T[k]; };
  const long i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
  const double Tr = ldT(r);
  double ddT = 0.0;
  if (flag[r] != 2) {
    long p, q;
    const long pr[3] = {(i > 0) ? r - 1 : r + (nx - 1), (j > 0) ? r - nx : r + (ny - 1) * nx,
                        (k > 0) ? r - nx * ny : r + (nz - 1) * nx * ny};
    const long qr[3] = {(i < nx - 1) ? r + 1 : r - (nx - 1), (j < ny - 1) ? r + nx : r - (ny - 1) * nx,
                        (k < nz - 1) ? r + nx * ny : r - (nz - 1) * nx * ny};
    const double h[3] = {dx, dy, dz};
    const double ih2s[3] = {ih2.x, ih2.y, ih2.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      p = pr[a];
      q = qr[a];
      if (flag[q] == 2) q = r;
      else if (flag[p] == 2) p = r;
      const double Tq = ldT(q), Tp = ldT(p);
      if (FAST) {  // reciprocals instead of the reference's divisions (within 1e-15 of them)
        const double ih2v = ih2s[a];
        ddT = fma((kappa[q] - kappa[p]) * (Tq - Tp), 0.25 * ih2v, ddT);
        ddT = fma(kappa[r] * ih2v, Tq + Tp - 2.0 * Tr, ddT);
      } else {
        ddT += (kappa[q] - kappa[p]) * (Tq - Tp) / h[a] / h[a] / 4.0;
        ddT += kappa[r] * ((Tq + Tp - 2.0 * Tr) / h[a] / h[a]);
      }
    }
  }
  double t = Tr;
  if (FAST && flag[r] == 1 && !(td.tdyn && td.tdyn[r] == 1)) {
    t = fma((ddT + dTr + S[r]) * inner_dt, irhoC[r], t);
  } else if (flag[r] == 1) {
    if (td.tdyn && td.tdyn[r] == 1) {  // eph_fdm.h:378-382: through E_e(T)
      double E = linear_eval(td, t);
      E += (ddT + dTr + S[r]) / td.rho[r] * inner_dt;
      t = linear_reverse(td, E);
    } else {
      t += (ddT + dTr + S[r]) / rhoC[r] * inner_dt;
    }
  }
  if (t < 0.0) {
    t = 0.0;
    atomicAdd(&counters[CNT_T_CLAMP], 1ull);
  }
  return t;
}

// One substep over the grid, one thread per cell: reads T, writes Tout.  The
// first substep turns the fixed-point deposits into dT and clears them.
// Launched as a programmatic dependent of the kernel before it (its launch
// overlaps that kernel's tail): waits for that kernel's results before
// touching memory.
template <bool FAST>
__global__ void k_fdm_substep(long nx, long ny, long nz, double dx, double dy, double dz, double inner_dt,
                              const double *__restrict__ T, double *__restrict__ Tout,
                              const double *__restrict__ kappa, const double *__restrict__ rhoC,
                              const double *__restrict__ S, const signed char *__restrict__ flag,
                              double *__restrict__ dT, U128 *__restrict__ acc, int first,
                              unsigned long long *__restrict__ counters, TdynTables td, double3 ih2,
                              const double *__restrict__ irhoC) {
  griddep_wait();
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long ntotal = nx * ny * nz;
  if (r >= ntotal) return;
  double dTr;
  if (first) {
    U128 a = acc[r];
    dTr = from_fixed(a);
    dT[r] = dTr;
    acc[r] = U128{0ull, 0ull};
  } else {
    dTr = dT[r];
  }
  Tout[r] = fdm_cell<FAST, false>(r, nx, ny, nz, dx, dy, dz, inner_dt, T, kappa, rhoC, S, flag, dTr, counters, td,
                                  ih2, irhoC);
}

// All substeps of a small grid in one launch of one thread-block cluster of
// FDM_CLUSTER blocks (one per SM), block b holding the cells
// [b * blockDim, (b + 1) * blockDim) (one cell per thread).  Substeps are
// separated by a device-scope fence and the cluster's hardware barrier,
// which every thread of every block reaches the same number of times (the
// loop bound is a launch argument).  Substep s reads src, writes dst as the
// per-substep launches do (rec: substep s writes rec + s * ncells);
// temperatures are read through L2.  Results are those of nsub launches of
// k_fdm_substep.
constexpr int FDM_CLUSTER = 8;
template <bool FAST>
__global__ void __launch_bounds__(1024, 1)
    k_fdm_cluster(long nx, long ny, long nz, double dx, double dy, double dz, double inner_dt, unsigned nsub,
                  double *__restrict__ T0, double *__restrict__ T1, double *__restrict__ rec,
                  const double *__restrict__ kappa, const double *__restrict__ rhoC, const double *__restrict__ S,
                  const signed char *__restrict__ flag, double *__restrict__ dT, U128 *__restrict__ acc,
                  unsigned long long *__restrict__ counters, TdynTables td, double3 ih2,
                  const double *__restrict__ irhoC) {
  const long ntotal = nx * ny * nz;
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool mine = r < ntotal;
  double dTr = 0.0;
  if (mine) {
    U128 a = acc[r];
    dTr = from_fixed(a);
    dT[r] = dTr;
    acc[r] = U128{0ull, 0ull};
  }
  const double *src = T0;
  double *dst = T1;
  for (unsigned s = 0; s < nsub; ++s) {
    if (rec) dst = rec + (size_t)s * (size_t)ntotal;
    if (mine)
      dst[r] = fdm_cell<FAST, true>(r, nx, ny, nz, dx, dy, dz, inner_dt, src, kappa, rhoC, S, flag, dTr, counters,
                                    td, ih2, irhoC);
    __threadfence();
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    double *next = rec ? nullptr : const_cast<double *>(src);
    src = dst;
    if (!rec) dst = next;
  }
}

// Exact sum of the grid temperatures (EPH_FDM::get_T_total, eph_fdm.h:189-196).
__global__ void k_grid_sum(const double *__restrict__ T, long ncells, U128 *__restrict__ out,
                           unsigned *__restrict__ err) {
  U128 t{0ull, 0ull};
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < ncells; r += (long)gridDim.x * blockDim.x)
    t = add128(t, to_fixed(T[r], err));
  for (int d = 16; d > 0; d >>= 1) t = add128(t, shfl_down128(t, d));
  if ((threadIdx.x & 31) == 0 && (t.lo | t.hi)) atomic_add128(out, t);
}

__global__ void k_from_fixed(const U128 *__restrict__ in, double *__restrict__ out) { *out = from_fixed(*in); }

// ------------------------------------------------------------ layout moves

// engine layout (n x 3) <-> padded device layout; w is kept
__global__ void k_pack3(int n, const double *__restrict__ src, D4 *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  D4 d = dst[i];
  d.x = src[3 * (size_t)i + 0];
  d.y = src[3 * (size_t)i + 1];
  d.z = src[3 * (size_t)i + 2];
  dst[i] = d;
}

__global__ void k_unpack3(int n, const D4 *__restrict__ src, double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const D4 s = src[i];
  dst[3 * (size_t)i + 0] = s.x;
  dst[3 * (size_t)i + 1] = s.y;
  dst[3 * (size_t)i + 2] = s.z;
}

// per-atom array of the fix (fix_eph.cpp:406-428): rho, beta(rho), f_EPH, f_RNG
__global__ void k_peratom(int n, int groupbit, const int *__restrict__ mask, const double *__restrict__ rho,
                          const double *__restrict__ beta, const D4 *__restrict__ f_eph,
                          const D4 *__restrict__ f_rng, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *o = out + 8 * (size_t)i;
  if (mask[i] & groupbit) {
    const D4 a = f_eph[i], b = f_rng[i];
    o[0] = rho[i];
    o[1] = beta[i];
    o[2] = a.x;
    o[3] = a.y;
    o[4] = a.z;
    o[5] = b.x;
    o[6] = b.y;
    o[7] = b.z;
  } else {
    for (int k = 0; k < 8; ++k) o[k] = 0.0;
  }
}

// rho and w in the engine layout
__global__ void k_get_w(int n, const D4 *__restrict__ Bw, double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const D4 b = Bw[i];
  dst[3 * (size_t)i + 0] = b.y;
  dst[3 * (size_t)i + 1] = b.z;
  dst[3 * (size_t)i + 2] = b.w;
}

// the deviates the last post_force used (A.z, A.w, Bw.x)
__global__ void k_get_xi(int n, const D4 *__restrict__ A, const D4 *__restrict__ Bw, double *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[3 * (size_t)i + 0] = A[i].z;
  dst[3 * (size_t)i + 1] = A[i].w;
  dst[3 * (size_t)i + 2] = Bw[i].x;
}

__global__ void k_set_elem(int n, const int *__restrict__ type, const int *__restrict__ type_map,
                           D4 *__restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i].w = (double)type_map[type[i]];
}

}  // namespace ephgb
