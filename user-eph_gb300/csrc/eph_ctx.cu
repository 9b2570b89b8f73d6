// Context, launches and the C ABI (include/eph_gb.h) of the GB300 fix-eph
// path.  One context = one fix instance on one GPU; all its work is ordered
// on one CUDA stream.  Device layout (n atoms, K = pair capacity):
//   x, v, f, xhold, f_eph, f_rng, xi   D4[n]       (x.w holds the element index)
//   A, Bw                              D4[n]       per-atom records read by neighbours
//   Mm, G                              D4[2n]      FAST one-lane sweeps: M_i, gathered records
//   pj, pe, pg                         [K][n]      in-cutoff pairs of the step
//   bins                               [nbins][bcap] BinEntry
//   grid T (two buffers), kappa, rho_e*C_e, S, flag, dT, fixed-point deposits
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "eph_ctx_impl.hpp"
#include "eph_kernels.cuh"

using namespace ephgb;


namespace ephgb {
namespace ctxi {

bool fused_friction(const eph_ctx *c);
bool df_active(const eph_ctx *c);

// pg rows per pair: {rho_j(r^2), rho_i(r^2)} in EXACT mode, {rho_i(r^2)/r^2, 0}
// in FAST mode with several elements, the y and z of H e with one element
// when stage 1 is folded into the density sweep (the force sweep then needs
// no H per pair); none otherwise
cudaError_t alloc_pg(eph_ctx *c) {
  if (c->mode == EPH_MODE_EXACT || c->multi || fused_friction(c))
    return c->pg.alloc((size_t)c->kcap * (size_t)c->n);
  c->pg.free();
  return cudaSuccess;
}

int fail(eph_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}


int upload_tables(eph_ctx *c) {
  const Beta &b = c->beta;
  auto up = [&](DevBuf<D4> &dst, int which, long nk) -> cudaError_t {
    std::vector<double> h((size_t)b.n_elements * nk * 4);
    for (int e = 0; e < b.n_elements; ++e) {
      const Spline &s = b.table(which, e);
      std::memcpy(&h[(size_t)e * nk * 4], s.c.data(), sizeof(double) * 4 * nk);
    }
    if (dst.n != (size_t)b.n_elements * nk) {  // same size: keep the buffer (captured graphs hold its address)
      c->buf_gen += 1;
      cudaError_t r = dst.alloc((size_t)b.n_elements * nk);
      if (r != cudaSuccess) return r;
    }
    return cudaMemcpy(dst.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  };
  CUDA_TRY(c, up(c->tab_rho_r_sq, EPH_SPLINE_RHO_R_SQ, b.n_rho));
  CUDA_TRY(c, up(c->tab_beta, EPH_SPLINE_BETA, b.n_beta));
  CUDA_TRY(c, up(c->tab_alpha, EPH_SPLINE_ALPHA, b.n_beta));
  // the rho(r^2) tables for the df64 density sweep: each interval's cubic
  // a + b x + c x^2 + d x^3 (the reference's absolute form) re-expanded about
  // the knot X_k the device forms (k dx as a double-float product) in long
  // double: a' = a + X (b + X (c + X d)), b' = b + X (2c + 3 d X),
  // c' = c + 3 d X, d' = d; each split into FP32 hi and lo parts
  {
    const long nk = b.n_rho;
    const double dx = 1.0 / b.rho_r_sq[0].inv_dx;
    const float dx_hi = (float)dx, dx_lo = (float)(dx - (double)dx_hi);
    c->P.dxr_hi = dx_hi;
    c->P.dxr_lo = dx_lo;
    c->P.inv_dxr_f = (float)b.rho_r_sq[0].inv_dx;
    std::vector<float4> h((size_t)b.n_elements * nk * 2);
    for (int e = 0; e < b.n_elements; ++e) {
      const Spline &sp = b.table(EPH_SPLINE_RHO_R_SQ, e);
      for (long k = 0; k < nk; ++k) {
        const float kr = (float)k;
        const float p = kr * dx_hi;
        float pe = std::fma(kr, dx_hi, -p);
        pe = std::fma(kr, dx_lo, pe);
        const long double X = (long double)p + (long double)pe;
        const long double a = sp.c[4 * k], bb = sp.c[4 * k + 1], cc = sp.c[4 * k + 2], d = sp.c[4 * k + 3];
        const long double q[4] = {a + X * (bb + X * (cc + X * d)), bb + X * (2 * cc + 3 * d * X), cc + 3 * d * X, d};
        float hi[4], lo[4];
        for (int m = 0; m < 4; ++m) {
          hi[m] = (float)q[m];
          lo[m] = (float)(q[m] - (long double)hi[m]);
        }
        h[2 * ((size_t)e * nk + k)] = make_float4(hi[0], hi[1], hi[2], hi[3]);
        h[2 * ((size_t)e * nk + k) + 1] = make_float4(lo[0], lo[1], lo[2], lo[3]);
      }
    }
    if (c->tab_rho_df.n != h.size()) {
      c->buf_gen += 1;
      CUDA_TRY(c, c->tab_rho_df.alloc(h.size()));
    }
    CUDA_TRY(c, cudaMemcpy(c->tab_rho_df.p, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice));
    c->P.tab_rho_df = c->tab_rho_df.p;
  }
  return EPH_OK;
}

// 1/(rho_e C_e) per cell for the FAST substeps (IEEE quotients, as on the device)
cudaError_t upload_inverse(eph_ctx *c, const std::vector<double> &rc) {
  std::vector<double> inv(rc.size());
  for (size_t i = 0; i < rc.size(); ++i) inv[i] = 1.0 / rc[i];
  return cudaMemcpy(c->irhoC.p, inv.data(), inv.size() * 8, cudaMemcpyHostToDevice);
}

int upload_grid(eph_ctx *c) {
  Grid &g = c->grid;
  const size_t nc = (size_t)g.ntotal;
  CUDA_TRY(c, c->T0.alloc(nc));
  CUDA_TRY(c, c->T1.alloc(nc));
  CUDA_TRY(c, c->kappa.alloc(nc));
  CUDA_TRY(c, c->rhoC.alloc(nc));
  CUDA_TRY(c, c->irhoC.alloc(nc));
  CUDA_TRY(c, c->S.alloc(nc));
  CUDA_TRY(c, c->dT.alloc(nc));
  CUDA_TRY(c, c->gflag.alloc(nc));
  CUDA_TRY(c, c->acc.alloc(nc));
  std::vector<double> rc(nc);
  std::vector<signed char> fl(nc);
  for (size_t i = 0; i < nc; ++i) {
    rc[i] = g.rho[i] * g.C[i];  // eph_fdm.h:372 prescaler
    fl[i] = (signed char)g.flag[i];
  }
  CUDA_TRY(c, cudaMemcpy(c->T0.p, g.T.data(), nc * 8, cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->kappa.p, g.kappa.data(), nc * 8, cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->rhoC.p, rc.data(), nc * 8, cudaMemcpyHostToDevice));
  CUDA_TRY(c, upload_inverse(c, rc));
  CUDA_TRY(c, cudaMemcpy(c->S.p, g.S.data(), nc * 8, cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->gflag.p, fl.data(), nc, cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemset(c->dT.p, 0, nc * 8));
  CUDA_TRY(c, cudaMemset(c->acc.p, 0, nc * sizeof(U128)));
  c->td = TdynTables{};
  bool any = false;
  for (size_t i = 0; i < nc; ++i) any = any || g.T_dynamic[i];
  if (g.has_tdyn && any) {
    const size_t nt = (size_t)g.E_T.y.size();
    std::vector<unsigned char> td(nc);
    for (size_t i = 0; i < nc; ++i) td[i] = (unsigned char)std::min<unsigned>(g.T_dynamic[i], 255u);
    CUDA_TRY(c, c->tdyn.alloc(nc));
    CUDA_TRY(c, c->gC.alloc(nc));
    CUDA_TRY(c, c->grho.alloc(nc));
    CUDA_TRY(c, c->E_y.alloc(nt));
    CUDA_TRY(c, c->E_dy.alloc(nt));
    CUDA_TRY(c, c->C_T.alloc(nt));
    CUDA_TRY(c, c->K_T.alloc(nt));
    CUDA_TRY(c, c->bounds.alloc(4));
    CUDA_TRY(c, cudaMemcpy(c->tdyn.p, td.data(), nc, cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->gC.p, g.C.data(), nc * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->grho.p, g.rho.data(), nc * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->E_y.p, g.E_T.y.data(), nt * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->E_dy.p, g.E_T.dy.data(), nt * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->C_T.p, g.C_T.c.data(), nt * sizeof(D4), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->K_T.p, g.kappa_T.c.data(), nt * sizeof(D4), cudaMemcpyHostToDevice));
    if (!c->h_bounds) CUDA_TRY(c, cudaMallocHost(&c->h_bounds, 4 * sizeof(double)));
    c->td = TdynTables{c->tdyn.p, c->C_T.p, c->K_T.p, c->E_y.p, c->E_dy.p, c->grho.p, g.E_T.dx, g.C_T.inv_dx, (int)nt};
  }
  return EPH_OK;
}

void set_time_params(eph_ctx *c) {
  // fix_eph.cpp:200-205 and reset_dt (:909-916)
  c->P.eta = std::sqrt(2.0 * c->boltz / c->dt);
  c->P.dtv = c->dt;
  c->P.dt = c->dt;
  const double dtf = 0.5 * c->dt * c->ftm2v;
  for (int t = 1; t <= c->ntypes; ++t) c->P.dtfm[t] = dtf / c->mass[t];
  c->grid.dt = c->dt;  // EPH_FDM::set_dt
  c->nsub = c->grid.substeps(&c->inner_dt);
  c->P.prescale = c->grid.dV * c->dt;
  if (c->args.coloured) c->P.zeta = 1.0 - std::exp(-c->dt / c->args.tau0);  // fix_eph_coloured_exp.cpp:190, :685
}

// read back the device error word; returns EPH_OK or the matching status
int check_device(eph_ctx *c) {
  CUDA_TRY(c, cudaMemcpyAsync(c->h_err, c->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const unsigned e = *c->h_err;
  if (!e) return EPH_OK;
  cudaMemsetAsync(c->d_err.p, 0, sizeof(unsigned), c->stream);
  if (e & (ERR_BIN_OVERFLOW | ERR_PAIR_OVERFLOW))
    return fail(c, EPH_ERR_CAPACITY,
                std::string("device: ") + ((e & ERR_BIN_OVERFLOW) ? "bin capacity exceeded " : "") +
                    ((e & ERR_PAIR_OVERFLOW) ? "pair capacity exceeded" : ""));
  if (e & ERR_TIMEOUT) return fail(c, EPH_ERR_TIMEOUT, "device: a bounded wait gave up");
  if (e & ERR_DRIFT) return fail(c, EPH_ERR_RANGE, "device: an atom drifted more than one bin outside the box");
  if (e & ERR_SPLINE_RANGE) return fail(c, EPH_ERR_RANGE, "device: spline argument outside its table");
  return fail(c, EPH_ERR_RANGE, "device: energy deposit outside the fixed-point range");
}

void collect_marks(eph_ctx *c) {
  for (auto &m : c->marks) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) c->phase_ms[m.phase] += ms;
    c->event_pool.push_back(m.a);
    c->event_pool.push_back(m.b);
  }
  c->marks.clear();
}

int require_atoms(eph_ctx *c) {
  if (c->n <= 0) return fail(c, EPH_ERR_STATE, "no atoms: call eph_set_atoms first");
  return EPH_OK;
}

// --------------------------------------------------------------- launches

int launch_initial(eph_ctx *c, int check_wrap) {
  PhaseScope ps(c, EPH_PHASE_INTEGRATE);
  ps.launched();
  const int nb = nblocks(c->n);
  if (c->mode == EPH_MODE_FAST)
    k_initial_integrate<true><<<nb, BLOCK, 0, c->stream>>>(c->P, c->x.p, c->v.p, c->f.p, c->type.p, c->mask.p,
                                                           c->xhold.p, check_wrap, c->wrapflag.p);
  else
    k_initial_integrate<false><<<nb, BLOCK, 0, c->stream>>>(c->P, c->x.p, c->v.p, c->f.p, c->type.p, c->mask.p,
                                                            c->xhold.p, check_wrap, c->wrapflag.p);
  CUDA_TRY(c, cudaGetLastError());
  return EPH_OK;
}

int launch_final(eph_ctx *c) {
  PhaseScope ps(c, EPH_PHASE_INTEGRATE);
  ps.launched();
  const int nb = nblocks(c->n);
  if (c->mode == EPH_MODE_FAST)
    k_final_integrate<true><<<nb, BLOCK, 0, c->stream>>>(c->P, c->v.p, c->f.p, c->type.p, c->mask.p);
  else
    k_final_integrate<false><<<nb, BLOCK, 0, c->stream>>>(c->P, c->v.p, c->f.p, c->type.p, c->mask.p);
  CUDA_TRY(c, cudaGetLastError());
  return EPH_OK;
}

// FAST mode folds stage 1 (the friction pre-vector) and M_i into the density
// sweep (one lane per atom, or below 16,384 atoms the lanes of
// k_density_tpa), and stages 2 and 3 run as k_forces_m with the same lanes.
bool fused_friction(const eph_ctx *c) {
  return c->mode == EPH_MODE_FAST && c->args.model == 4 && (c->P.flags & FLAG_FRICTION) && c->fuse_w;
}

// FAST pair sums in df64: the one-lane density sweep with stage 1 folded,
// over the bin search (k_density_df) or the kept lists (k_density_list_df),
// then k_forces_df at any lanes per atom; bins of at most 1022 per axis
// (the records pack them in 10 bits each)
bool df_active(const eph_ctx *c) {
  return c->pair_arith == EPH_PAIRS_DF64 && c->mode == EPH_MODE_FAST && fused_friction(c) &&
         !(c->tpa > 1 && c->n < 16384) && c->P.nb[0] <= 1022 && c->P.nb[1] <= 1022 && c->P.nb[2] <= 1022;
}

template <bool FAST, bool MULTI, bool FUSE>
void launch_density_f(eph_ctx *c, int xi_mode) {
  // several lanes per atom in the density sweep too below 16,384 atoms, where
  // one lane per atom leaves it latency bound (measured on GB300: 4,000 atoms
  // 0.289 -> 0.210 ms per step; from 16,384 atoms on the extra exact-test pass
  // and lane sums cost more than they hide: 32,000 atoms 71 -> 81 ms per 200
  // steps, so the one-lane sweep stays there)
  if constexpr (FAST) {
    // not over the EAM engine's bins: they are sized for its cut-off, and a
    // lane's share of 27 such bins can hold more candidates than its
    // shared-memory column (the one-lane sweeps spill to the pair rows)
    if (c->tpa > 1 && c->n < 16384 && !c->eam) {
#define EPH_DENSITY_TPA(T)                                                                                         \
  k_density_tpa<MULTI, FUSE, T><<<nblocks((long)c->n * T), BLOCK, 0, c->stream>>>(                                  \
      c->P, c->x.p, c->mask.p, c->bin_count.p, c->bins.p, c->atom_bin.p, c->atom_off.p, c->xi.p, xi_mode, c->T0.p, \
      c->pj.p, c->pe.p, c->pg.p, c->nshort.p, c->A.p, c->Bw.p, c->rho.p, c->beta_i.p, c->cell.p, c->Te_i.p,        \
      c->wrapflag.p, c->d_err.p, c->counters.p, c->v.p, c->Mm.p, c->G.p)
      if (c->tpa == 2) EPH_DENSITY_TPA(2);
      else if (c->tpa == 4) EPH_DENSITY_TPA(4);
      else EPH_DENSITY_TPA(8);
#undef EPH_DENSITY_TPA
      return;
    }
  }
  if constexpr (FAST && FUSE) {
    if (c->reuse && df_active(c)) {
      float4 *pa = reinterpret_cast<float4 *>(c->pe.p), *pb = pa + (size_t)c->kcap * c->n;
      k_density_list_df<MULTI><<<nblocks(c->n), BLOCK, 0, c->stream>>>(
          c->P, c->x.p, c->mask.p, c->bin_count.p, c->bins.p, c->atom_bin.p, c->atom_off.p, c->dfrec.p, c->dfvrec.p,
          c->xi.p, xi_mode, c->T0.p, c->pj.p, pa, pb, reinterpret_cast<float4 *>(c->pg.p), c->nshort.p, c->A.p,
          c->Bw.p, c->rho.p, c->beta_i.p, c->cell.p, c->Te_i.p, c->wrapflag.p, c->d_err.p, c->counters.p, c->v.p,
          c->Mm.p, c->G.p, c->cl.p, c->cl_n.p, c->state.p, c->rb.p, c->flist.p);
      return;
    }
    if (c->reuse) {
      k_density_list<MULTI><<<nblocks(c->n), BLOCK, 0, c->stream>>>(
          c->P, c->x.p, c->mask.p, c->bin_count.p, c->bins.p, c->atom_bin.p, c->atom_off.p, c->xi.p, xi_mode,
          c->T0.p, c->pj.p, c->pe.p, c->pg.p, c->nshort.p, c->A.p, c->Bw.p, c->rho.p, c->beta_i.p, c->cell.p,
          c->Te_i.p, c->wrapflag.p, c->d_err.p, c->counters.p, c->v.p, c->Mm.p, c->G.p, c->cl.p, c->cl_n.p,
          c->state.p, c->rb.p, c->flist.p);
      return;
    }
  }
  if constexpr (FAST && FUSE) {
    if (df_active(c)) {
      float4 *pa = reinterpret_cast<float4 *>(c->pe.p), *pb = pa + (size_t)c->kcap * c->n;
      // with the standalone engine's EAM force the candidates come from its
      // pair list of this step (the same bins and order; no bin scan)
      const unsigned *elist = nullptr;
      const int *ens = nullptr;
      if (!(c->eam_list_fresh && eam_pair_list(c, &elist, &ens))) elist = nullptr, ens = nullptr;
      k_density_df<MULTI><<<nblocks(c->n), BLOCK, 0, c->stream>>>(
          c->P, c->mask.p, c->bin_count.p, c->bins.p, c->atom_bin.p, c->atom_off.p, c->dfrec.p, c->dfvrec.p, c->x.p,
          c->xi.p, xi_mode, c->T0.p, c->pj.p, pa, pb, reinterpret_cast<float4 *>(c->pg.p), c->nshort.p, c->A.p,
          c->Bw.p, c->rho.p, c->beta_i.p, c->cell.p, c->Te_i.p, c->wrapflag.p, c->d_err.p, c->counters.p, c->v.p,
          c->Mm.p, c->G.p, elist, ens);
      c->eam_list_fresh = false;
      return;
    }
  }
  k_density<FAST, MULTI, FUSE><<<nblocks(c->n), BLOCK, 0, c->stream>>>(
      c->P, c->x.p, c->mask.p, c->bin_count.p, c->bins.p, c->atom_bin.p, c->atom_off.p, c->xi.p, xi_mode, c->T0.p,
      c->pj.p, c->pe.p, c->pg.p, c->nshort.p, c->A.p, c->Bw.p, c->rho.p, c->beta_i.p, c->cell.p, c->Te_i.p,
      c->wrapflag.p, c->d_err.p, c->counters.p, c->v.p, c->Mm.p, c->G.p);
}

template <bool FAST, bool MULTI>
void launch_density_t(eph_ctx *c, int xi_mode) {
  if (FAST && fused_friction(c)) launch_density_f<FAST, MULTI, true>(c, xi_mode);
  else launch_density_f<FAST, MULTI, false>(c, xi_mode);
}

template <bool FAST, bool MULTI, bool FRIC, bool RAND>
void launch_forces_t(eph_ctx *c) {
  const int tpa = FAST ? c->tpa : 1;
  if (FAST && FRIC && df_active(c)) {
    const float4 *pa = reinterpret_cast<const float4 *>(c->pe.p), *pb = pa + (size_t)c->kcap * c->n;
#define EPH_FORCES_DF(T)                                                                                          \
  k_forces_df<MULTI, RAND, T><<<nblocks((long)c->n * T), BLOCK, 0, c->stream>>>(                                   \
      c->P, c->pj.p, pa, pb, reinterpret_cast<const float4 *>(c->pg.p), c->nshort.p, c->Mm.p,                    \
      reinterpret_cast<const float4 *>(c->G.p), c->A.p, c->Bw.p, c->Te_i.p, c->f.p, c->f_eph.p, c->f_rng.p,       \
      c->f_dis.p, c->f_sto.p)
    if (tpa == 1) EPH_FORCES_DF(1);
    else if (tpa == 2) EPH_FORCES_DF(2);
    else if (tpa == 4) EPH_FORCES_DF(4);
    else EPH_FORCES_DF(8);
#undef EPH_FORCES_DF
    return;
  }
  if (FAST && FRIC && fused_friction(c)) {
#define EPH_FORCES_M(T)                                                                                      \
  k_forces_m<MULTI, RAND, T><<<nblocks((long)c->n * T), BLOCK, 0, c->stream>>>(                               \
      c->P, c->pj.p, c->pe.p, c->pg.p, c->nshort.p, c->Mm.p, c->G.p, c->Te_i.p, c->f.p, c->f_eph.p, c->f_rng.p, \
      c->f_dis.p, c->f_sto.p)
    if (tpa == 1) EPH_FORCES_M(1);
    else if (tpa == 2) EPH_FORCES_M(2);
    else if (tpa == 4) EPH_FORCES_M(4);
    else EPH_FORCES_M(8);
#undef EPH_FORCES_M
    return;
  }
  if (tpa == 1) {
    k_forces<FAST, MULTI, FRIC, RAND><<<nblocks(c->n), BLOCK, 0, c->stream>>>(
        c->P, c->mask.p, c->pj.p, c->pe.p, c->pg.p, c->nshort.p, c->A.p, c->Bw.p, c->Te_i.p, c->f.p, c->f_eph.p,
        c->f_rng.p, c->f_dis.p, c->f_sto.p);
    return;
  }
#define EPH_FORCES_TPA(T)                                                                                     \
  k_forces_tpa<MULTI, FRIC, RAND, T><<<nblocks((long)c->n * T), BLOCK, 0, c->stream>>>(                       \
      c->P, c->mask.p, c->pj.p, c->pe.p, c->pg.p, c->nshort.p, c->A.p, c->Bw.p, c->Te_i.p, c->f.p, c->f_eph.p, \
      c->f_rng.p, c->f_dis.p, c->f_sto.p)
  if (tpa == 2) EPH_FORCES_TPA(2);
  else if (tpa == 4) EPH_FORCES_TPA(4);
  else EPH_FORCES_TPA(8);
#undef EPH_FORCES_TPA
}

// lanes per atom of the FAST pair sweeps for n atoms: more lanes where the
// one-lane sweeps leave the SMs with too few warps to hide their loads
// (measured on GB300, µs per step with 2 / 4 / 8 lanes: 2,048 atoms
// 207 / 171 / 148; 4,000 atoms 220 / 185 / 177; 8,788 atoms 226 / 213 / 235;
// 16,384 atoms 282 / 280 / 284; above ~65,000 atoms one lane)
int auto_tpa(long n) { return n <= 6144 ? 8 : (n <= 65536 ? 4 : 1); }

// Bins of edge >= r (1 + 5e-5), at least three per axis; 0 or an error
int set_bin_geometry(eph_ctx *c, double r) {
  const double edge = r * (1.0 + 5e-5);
  int nb[3];
  for (int k = 0; k < 3; ++k) {
    nb[k] = (int)(c->prd[k] / edge);
    if (nb[k] < 3) return fail(c, EPH_ERR_ARG, "box edge shorter than three bin edges: too small for minimum-image bins");
  }
  for (int k = 0; k < 3; ++k) {
    c->P.nb[k] = nb[k];
    c->P.w[k] = c->prd[k] / nb[k];
    c->P.inv_w[k] = 1.0 / c->P.w[k];
    c->P.wf[k] = (float)c->P.w[k];
    c->P.w_hi[k] = (float)c->P.w[k];
    c->P.w_lo[k] = (float)(c->P.w[k] - (double)c->P.w_hi[k]);
  }
  c->nbins = nb[0] * nb[1] * nb[2];
  return EPH_OK;
}

// a bin's capacity from the number density: ~density * w^3 atoms
int auto_bcap(const eph_ctx *c) {
  const double dens = c->n / (c->prd[0] * c->prd[1] * c->prd[2]);
  const double per_bin = dens * c->P.w[0] * c->P.w[1] * c->P.w[2];
  return ((int)std::ceil(2.0 * per_bin + 16.0) + 7) / 8 * 8;
}

// Kept candidate lists: FAST mode, model 4 with friction, the one-lane
// density sweep (one lane per atom, or 16,384 atoms and more), no pair force
// of the engine (it needs bins every step) and no adjoint.  By default from
// 2^15 to 2^20 atoms: the lists save the bin search, which the density
// sweep's FP64 pass hides less well in small systems, and cost four small
// launches a step plus the atoms near moved ones (measured on GB300 with a
// 0.3 A skin, step time: 16,384 atoms +18 %, 62,500 atoms -8 %, 131,072 atoms
// -9 %, 256,000 atoms -5 %, 500,000 atoms -2 %, 1,000,188 atoms -1 %,
// 2,048,000 atoms +0.2 %, where both sweeps already run at the FP64 issue
// limit); a skin set through eph_set_list_skin applies at any size.
bool want_list(const eph_ctx *c) {
  // with the df64 pair sums (whose pass 2 no longer hides the bin search) the
  // lists pay at every size from 2^15 atoms on (measured on GB300, step time
  // bin search -> lists: 131,072 atoms 0.543 -> 0.482 ms, 500,000 atoms
  // 1.447 -> 1.112 ms, 1,000,188 atoms 2.663 -> 2.007 ms, 2,048,000 atoms
  // 5.133 -> 3.849 ms)
  const bool size_ok = c->lskin_user || (c->n >= (1 << 15) && (c->n <= (1 << 20) || c->pair_arith == EPH_PAIRS_DF64));
  if (c->mode != EPH_MODE_FAST || c->lskin <= 0.0 || c->list_block || c->eam || c->n <= 0 ||
      !(c->tpa == 1 || c->n >= 16384) || !fused_friction(c) || !size_ok)
    return false;
  for (int k = 0; k < 3; ++k)
    if ((int)(c->prd[k] / ((c->beta.r_cutoff + c->lskin) * (1.0 + 5e-5))) < 3) return false;
  return true;
}

void drop_list(eph_ctx *c) {
  c->reuse = false;
  c->lcap = 0;
  c->cl.free();
  c->cl_n.free();
  c->state.free();
  c->rb.free();
  c->flist.free();
  c->xref.free();
}

int configure_list(eph_ctx *c) {
  const bool want = want_list(c);
  if (!want && !c->reuse) return EPH_OK;
  const double rc = c->beta.r_cutoff;
  const int nbins_was = c->nbins, bcap_was = c->bcap;
  int r = set_bin_geometry(c, want ? rc + c->lskin : rc);
  if (r) return r;
  if (!c->bcap_user) c->bcap = auto_bcap(c);
  c->P.bcap = c->bcap;
  if (c->nbins != nbins_was || c->bcap != bcap_was || !c->bins.p) {
    CUDA_TRY(c, c->bins.alloc((size_t)c->nbins * c->bcap));
    CUDA_TRY(c, c->bin_count.alloc((size_t)c->nbins));
    CUDA_TRY(c, cudaMemsetAsync(c->bin_count.p, 0, sizeof(int) * (size_t)c->nbins, c->stream));
  }
  c->buf_gen += 1;
  drop_graph(c);
  if (!want) {
    drop_list(c);
    return EPH_OK;
  }
  const size_t N = (size_t)c->n;
  const double rl = rc + c->lskin, rm = rc + 0.5 * c->lskin;
  const double dens = c->n / (c->prd[0] * c->prd[1] * c->prd[2]);
  const int lcap = std::min(256, ((int)std::ceil(2.0 * dens * 4.18879020478639 * rl * rl * rl + 24.0) + 7) / 8 * 8);
  if (lcap != c->lcap || c->cl.n != (size_t)lcap * N) CUDA_TRY(c, c->cl.alloc((size_t)lcap * N));
  c->lcap = lcap;
  for (DevBuf<int> *b : {&c->cl_n, &c->state})
    if (b->n != N) CUDA_TRY(c, b->alloc(N));
  if (c->xref.n != N) CUDA_TRY(c, c->xref.alloc(N));
  if (!c->rb.p) CUDA_TRY(c, c->rb.alloc(4));
  if (!c->flist.p) CUDA_TRY(c, c->flist.alloc(LIST_FMAX));
  CUDA_TRY(c, cudaMemsetAsync(c->rb.p, 0, 4 * sizeof(int), c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->rb.p, 0x01, 1, c->stream));  // rb[0] = 1: the next step builds
  c->P.lcap = lcap;
  c->P.rl2_band = (float)(rl * rl * (1.0 + 1e-4));
  c->P.rmark2_band = (float)(rm * rm * (1.0 + 1e-4));
  c->P.lslow2 = 0.25 * c->lskin * c->lskin;
  for (int k = 0; k < 3; ++k) {
    c->P.half_prd[k] = 0.5 * c->prd[k];
    c->P.half_prdf[k] = (float)c->P.half_prd[k];
  }
  c->reuse = true;
  return EPH_OK;
}

// stage 1 as its own sweep: EXACT mode (FAST mode folds it into the density sweep)
void launch_friction_w(eph_ctx *c) {
  k_friction_w<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->P, c->mask.p, c->v.p, c->pj.p, c->pe.p, c->pg.p,
                                                       c->nshort.p, c->A.p, c->Bw.p);
}

template <bool FAST, bool FRIC, bool RAND>
void launch_ttm_t(eph_ctx *c) {
  k_forces_ttm<FAST, FRIC, RAND><<<nblocks(c->n), BLOCK, 0, c->stream>>>(
      c->P, c->mask.p, c->x.p, c->v.p, c->A.p, c->Bw.p, c->rho.p, c->beta_i.p, c->Te_i.p, c->f.p, c->f_eph.p,
      c->f_rng.p, c->d_err.p);
}

template <bool FAST>
void launch_ttm(eph_ctx *c) {
  const bool fr = c->P.flags & FLAG_FRICTION, ra = c->P.flags & FLAG_RANDOM;
  if (fr && ra) launch_ttm_t<FAST, true, true>(c);
  else if (fr) launch_ttm_t<FAST, true, false>(c);
  else if (ra) launch_ttm_t<FAST, false, true>(c);
  else launch_ttm_t<FAST, false, false>(c);
}

template <bool FAST, bool MULTI>
void launch_forces_m(eph_ctx *c) {
  const bool fr = c->P.flags & FLAG_FRICTION, ra = c->P.flags & FLAG_RANDOM;
  if (fr && ra) launch_forces_t<FAST, MULTI, true, true>(c);
  else if (fr) launch_forces_t<FAST, MULTI, true, false>(c);
  else if (ra) launch_forces_t<FAST, MULTI, false, true>(c);
  else launch_forces_t<FAST, MULTI, false, false>(c);
}

// post_force: bins, density, friction pre-vector, forces
int launch_post_force(eph_ctx *c, int xi_mode) {
  int r = launch_bin(c);
  if (r) return r;
  return launch_pair_sweeps(c, xi_mode);
}

int launch_bin(eph_ctx *c) {
  const int nb = nblocks(c->n);
  PhaseScope ps(c, EPH_PHASE_BIN);
  if (c->reuse) {
    // the engine's wrap and the displacements since the list build; a build
    // step (decided on the device) bins and sorts as below, any other step
    // flags the atoms near moved ones and leaves the bins as they are
    int *rb = c->rb.p;
    CUDA_TRY(c, cudaMemsetAsync(rb + 1, 0, sizeof(int), c->stream));
    const bool df = df_active(c);
    k_list_check<<<nb, BLOCK, 0, c->stream>>>(c->P, c->x.p, c->xhold.p, c->wrapflag.p, c->xref.p, c->state.p, rb,
                                              c->flist.p, c->counters.p, df ? c->dfrec.p : nullptr,
                                              df ? c->dfvrec.p : nullptr, c->v.p);
    k_list_decide<<<1, 32, 0, c->stream>>>(rb, c->flist.p, c->counters.p);
    k_list_mark<<<LIST_FMAX, BLOCK, 0, c->stream>>>(c->P, c->x.p, rb, c->flist.p, c->bin_count.p, c->bins.p,
                                                    c->state.p);
    k_zero_if<<<nblocks(c->nbins), BLOCK, 0, c->stream>>>(c->bin_count.p, c->nbins, rb + 2);
    k_bin<<<nb, BLOCK, 0, c->stream>>>(c->P, c->x.p, c->xhold.p, c->wrapflag.p, c->bin_count.p, c->bins.p,
                                       c->atom_bin.p, c->atom_off.p, c->d_err.p, c->counters.p, 0, rb + 2,
                                       c->xref.p);
    if (c->bcap <= 64 && c->nbins < 32768)
      k_bin_sort_warp<<<nblocks((long)c->nbins * 32), BLOCK, 0, c->stream>>>(c->nbins, c->bcap, c->bin_count.p,
                                                                              c->bins.p, rb + 2);
    else
      k_bin_sort<<<nblocks(c->nbins), BLOCK, 0, c->stream>>>(c->nbins, c->bcap, c->bin_count.p, c->bins.p, rb + 2);
    ps.launched(6);
    CUDA_TRY(c, cudaGetLastError());
    return EPH_OK;
  }
  ps.launched();
  CUDA_TRY(c, cudaMemsetAsync(c->bin_count.p, 0, sizeof(int) * (size_t)c->nbins, c->stream));
  const bool df = df_active(c);
  k_bin<<<nb, BLOCK, 0, c->stream>>>(c->P, c->x.p, c->xhold.p, c->wrapflag.p, c->bin_count.p, c->bins.p,
                                     c->atom_bin.p, c->atom_off.p, c->d_err.p, c->counters.p, 1, nullptr, nullptr,
                                     df ? c->dfrec.p : nullptr, df ? c->dfvrec.p : nullptr, c->v.p);
  ps.launched();
  // a warp per bin where the bins are few (the sort's latency shows), a
  // thread per bin where they are many (measured on GB300: 343 bins 20 ->
  // ~2 µs; 226,981 bins 0.06 ms by thread, 0.10 ms by warp)
  if (c->bcap <= 64 && c->nbins < 32768)
    k_bin_sort_warp<<<nblocks((long)c->nbins * 32), BLOCK, 0, c->stream>>>(c->nbins, c->bcap, c->bin_count.p,
                                                                            c->bins.p);
  else
    k_bin_sort<<<nblocks(c->nbins), BLOCK, 0, c->stream>>>(c->nbins, c->bcap, c->bin_count.p, c->bins.p);
  CUDA_TRY(c, cudaGetLastError());
  return EPH_OK;
}

int launch_pair_sweeps(eph_ctx *c, int xi_mode) {
  const bool fast = c->mode == EPH_MODE_FAST;
  {
    PhaseScope ps(c, EPH_PHASE_DENSITY);
    ps.launched();
    if (fast) {
      if (c->multi) launch_density_t<true, true>(c, xi_mode);
      else launch_density_t<true, false>(c, xi_mode);
    } else {
      if (c->multi) launch_density_t<false, true>(c, xi_mode);
      else launch_density_t<false, false>(c, xi_mode);
    }
    c->eam_list_fresh = false;  // read (or not) by this step's density sweep only
  }
  // eph_post_force_host: the engine's force, uploaded while the density
  // sweep ran, goes into f before the force sweeps add to it
  if (c->f_pending) {
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->f_ready, 0));
    k_pack3<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->n, c->hstage.p + 3 * (size_t)c->n, c->f.p);
    c->f_pending = false;
    c->launches += 1;
  }
  if (c->args.model == 1) {  // force_ttm: per-atom, no pair sums
    PhaseScope ps(c, EPH_PHASE_FORCES);
    ps.launched();
    if (fast) launch_ttm<true>(c);
    else launch_ttm<false>(c);
    CUDA_TRY(c, cudaGetLastError());
    return EPH_OK;
  }
  if ((c->P.flags & FLAG_FRICTION) && !fused_friction(c)) {
    PhaseScope ps(c, EPH_PHASE_FRICTION_W);
    ps.launched();
    launch_friction_w(c);
  }
  {
    PhaseScope ps(c, EPH_PHASE_FORCES);
    ps.launched();
    if (fast) {
      if (c->multi) launch_forces_m<true, true>(c);
      else launch_forces_m<true, false>(c);
    } else {
      if (c->multi) launch_forces_m<false, true>(c);
      else launch_forces_m<false, false>(c);
    }
  }
  CUDA_TRY(c, cudaGetLastError());
  return EPH_OK;
}

template <bool FRIC, bool RAND, bool GRID>
void launch_deposit_t(eph_ctx *c) {
  k_deposit<FRIC, RAND, GRID><<<nblocks(c->n, 256), 256, 0, c->stream>>>(
      c->P, c->mask.p, c->v.p, c->f_eph.p, c->f_rng.p, c->cell.p, c->acc.p, c->part.p, c->d_err.p);
}

// end_of_step: deposits, FDM substeps, energy total
int launch_end_of_step(eph_ctx *c) {
  const bool fr = c->P.flags & FLAG_FRICTION, ra = c->P.flags & FLAG_RANDOM, gr = c->P.flags & FLAG_FDM;
  if (fr || ra) {
    PhaseScope ps(c, EPH_PHASE_DEPOSIT);
    ps.launched(2);
    if (fr && ra) {
      if (gr) launch_deposit_t<true, true, true>(c);
      else launch_deposit_t<true, true, false>(c);
    } else if (fr) {
      if (gr) launch_deposit_t<true, false, true>(c);
      else launch_deposit_t<true, false, false>(c);
    } else {
      if (gr) launch_deposit_t<false, true, true>(c);
      else launch_deposit_t<false, true, false>(c);
    }
    k_energy_total<<<1, 1024, 0, c->stream>>>(c->part.p, nblocks(c->n, 256), c->scal.p + 1, c->scal.p + 0);
  }
  if (gr) {
    PhaseScope ps(c, EPH_PHASE_FDM);
    const Grid &g = c->grid;
    if (c->td.tdyn) {
      // eph_fdm.h:280-313: T-dependent C_e, kappa_e, then this step's substeps
      k_fdm_tdyn_params<<<nblocks(g.ntotal, 128), 128, 0, c->stream>>>(g.ntotal, c->td, c->T0.p, c->gC.p,
                                                                       c->kappa.p, c->rhoC.p, c->d_err.p);
      k_fdm_bounds<<<1, 256, 0, c->stream>>>(g.ntotal, c->gC.p, c->grho.p, c->kappa.p, c->gflag.p, c->bounds.p);
      CUDA_TRY(c, cudaMemcpyAsync(c->h_bounds, c->bounds.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      c->nsub = g.substeps_from(c->h_bounds[0], c->h_bounds[1], c->h_bounds[2], &c->inner_dt);
      ps.launched(2);
    }
    const double3 ih2 = make_double3(1.0 / (g.dx * g.dx), 1.0 / (g.dy * g.dy), 1.0 / (g.dz * g.dz));
    double *src = c->T0.p, *dst = c->T1.p;
    if (!c->td.tdyn && c->fdm_cluster && c->nsub > 1 && g.ntotal <= 2048) {
      // a small grid: every substep in one launch of one thread-block cluster,
      // the cells spread evenly over its blocks (measured on GB300: 10^3
      // cells, 17 substeps, 0.178 -> 0.169 ms per step; 16^3 cells, 11
      // substeps, 35 us per step slower than the per-substep launches, whose
      // FP64 work then spreads over more SMs)
      ps.launched(1);
      const long per_block = ((g.ntotal + FDM_CLUSTER - 1) / FDM_CLUSTER + 31) / 32 * 32;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(FDM_CLUSTER);
      cfg.blockDim = dim3((unsigned)per_block);
      cfg.stream = c->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = FDM_CLUSTER;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      double *rec = c->fdm_rec;
      if (c->mode == EPH_MODE_FAST)
        CUDA_TRY(c, cudaLaunchKernelEx(&cfg, k_fdm_cluster<true>, (long)g.nx, (long)g.ny, (long)g.nz, g.dx, g.dy,
                                       g.dz, c->inner_dt, c->nsub, c->T0.p, c->T1.p, rec, (const double *)c->kappa.p,
                                       (const double *)c->rhoC.p, (const double *)c->S.p,
                                       (const signed char *)c->gflag.p, c->dT.p, c->acc.p, c->counters.p, c->td, ih2,
                                       (const double *)c->irhoC.p));
      else
        CUDA_TRY(c, cudaLaunchKernelEx(&cfg, k_fdm_cluster<false>, (long)g.nx, (long)g.ny, (long)g.nz, g.dx, g.dy,
                                       g.dz, c->inner_dt, c->nsub, c->T0.p, c->T1.p, rec, (const double *)c->kappa.p,
                                       (const double *)c->rhoC.p, (const double *)c->S.p,
                                       (const signed char *)c->gflag.p, c->dT.p, c->acc.p, c->counters.p, c->td, ih2,
                                       (const double *)c->irhoC.p));
      // where the last substep wrote, as with the per-substep launches below
      if (rec) src = rec + (size_t)(c->nsub - 1) * (size_t)g.ntotal;
      else if (c->nsub % 2) src = c->T1.p;
      if (src != c->T0.p)
        CUDA_TRY(c, cudaMemcpyAsync(c->T0.p, src, sizeof(double) * (size_t)g.ntotal, cudaMemcpyDeviceToDevice,
                                    c->stream));
      CUDA_TRY(c, cudaGetLastError());
      return EPH_OK;
    }
    ps.launched((int)c->nsub);
    for (unsigned s = 0; s < c->nsub; ++s) {
      if (c->fdm_rec) dst = c->fdm_rec + (size_t)s * (size_t)g.ntotal;
      // each substep a programmatic dependent of the one before (the kernel
      // waits for it before touching memory; its launch overlaps that tail)
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(nblocks(g.ntotal, 64));
      cfg.blockDim = dim3(64);
      cfg.stream = c->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      at[0].val.programmaticStreamSerializationAllowed = s > 0 ? 1 : 0;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      const double *csrc = src;
      const int first = s == 0;
      if (c->mode == EPH_MODE_FAST)
        CUDA_TRY(c, cudaLaunchKernelEx(&cfg, k_fdm_substep<true>, (long)g.nx, (long)g.ny, (long)g.nz, g.dx, g.dy, g.dz,
                                       c->inner_dt, csrc, dst, (const double *)c->kappa.p, (const double *)c->rhoC.p,
                                       (const double *)c->S.p, (const signed char *)c->gflag.p, c->dT.p, c->acc.p,
                                       first, c->counters.p, c->td, ih2, (const double *)c->irhoC.p));
      else
        CUDA_TRY(c, cudaLaunchKernelEx(&cfg, k_fdm_substep<false>, (long)g.nx, (long)g.ny, (long)g.nz, g.dx, g.dy,
                                       g.dz, c->inner_dt, csrc, dst, (const double *)c->kappa.p,
                                       (const double *)c->rhoC.p, (const double *)c->S.p,
                                       (const signed char *)c->gflag.p, c->dT.p, c->acc.p, first, c->counters.p,
                                       c->td, ih2, (const double *)c->irhoC.p));
      if (c->fdm_rec) src = dst;
      else std::swap(src, dst);
    }
    if (src != c->T0.p)
      CUDA_TRY(c, cudaMemcpyAsync(c->T0.p, src, sizeof(double) * (size_t)g.ntotal, cudaMemcpyDeviceToDevice,
                                  c->stream));
  }
  CUDA_TRY(c, cudaGetLastError());
  return EPH_OK;
}

int download_grid(eph_ctx *c) {
  CUDA_TRY(c, cudaMemcpyAsync(c->grid.T.data(), c->T0.p, sizeof(double) * (size_t)c->grid.ntotal,
                              cudaMemcpyDeviceToHost, c->stream));
  if (c->td.tdyn) {  // C_e and kappa_e follow T in these cells
    CUDA_TRY(c, cudaMemcpyAsync(c->grid.C.data(), c->gC.p, sizeof(double) * (size_t)c->grid.ntotal,
                                cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->grid.kappa.data(), c->kappa.p, sizeof(double) * (size_t)c->grid.ntotal,
                                cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return EPH_OK;
}

int write_T_output(eph_ctx *c) {
  // end_of_step (fix_eph.cpp:397-399): every T_freq steps
  if (c->args.T_freq > 0 && (c->ntimestep % c->args.T_freq) == 0) {
    int r = download_grid(c);
    if (r) return r;
    if (c->grid.save_temperature(c->args.T_out.c_str(), (int)(c->ntimestep / c->args.T_freq)))
      return fail(c, EPH_ERR_FILE, "cannot write " + c->args.T_out);
  }
  return EPH_OK;
}

// One engine step (Verlet::run order) issued on the context's stream; the
// same sequence is executed directly or captured into a graph.
int record_step(eph_ctx *c, int xi_mode) {
  int r;
  if ((r = launch_initial(c, 1))) return r;
  if (c->eam) {
    // the engine's pair force on this step's positions (Verlet: after the
    // wrap and the neighbour bins, before post_force)
    if ((r = launch_bin(c)) || (r = launch_eam(c)) || (r = launch_pair_sweeps(c, xi_mode))) return r;
  } else {
    // force clear + the external (pair) force
    if (c->have_fext)
      CUDA_TRY(c, cudaMemcpyAsync(c->f.p, c->fext.p, sizeof(D4) * (size_t)c->n, cudaMemcpyDeviceToDevice, c->stream));
    else
      CUDA_TRY(c, cudaMemsetAsync(c->f.p, 0, sizeof(D4) * (size_t)c->n, c->stream));
    if ((r = launch_post_force(c, xi_mode))) return r;
  }
  if ((r = launch_final(c))) return r;
  return launch_end_of_step(c);
}

void drop_graph(eph_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
  c->graph_xi = -1;
}

// Capture one step into c->gexec (replays must not change host-side state:
// the random-number counter and the wrap flag live on the device).
int capture_step(eph_ctx *c, int xi_mode) {
  drop_graph(c);
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  const long before = c->launches;
  const int r = record_step(c, xi_mode);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->graph_launches = c->launches - before;
  c->launches = before;
  if (r || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();  // a failed capture leaves its error behind for the next caller
    return r ? r : fail(c, EPH_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
  }
  c->graph = g;
  CUDA_TRY(c, cudaGraphInstantiate(&c->gexec, g, 0));
  c->graph_xi = xi_mode;
  return EPH_OK;
}

}  // namespace ctxi
}  // namespace ephgb

using namespace ephgb::ctxi;

// =================================================================== C ABI

extern "C" {

const char *eph_status_string(int s) {
  switch (s) {
    case EPH_OK: return "ok";
    case EPH_ERR_ARG: return "bad argument";
    case EPH_ERR_FILE: return "file error";
    case EPH_ERR_UNSUPPORTED_MODEL: return "unsupported model";
    case EPH_ERR_CAPACITY: return "capacity exceeded";
    case EPH_ERR_TIMEOUT: return "device wait timed out";
    case EPH_ERR_CUDA: return "CUDA error";
    case EPH_ERR_STATE: return "call out of order";
    case EPH_ERR_RANGE: return "input out of range";
    default: return "unknown status";
  }
}

const char *eph_last_error(const eph_ctx *c) { return c ? c->err.c_str() : "null context"; }

int eph_create(int narg, const char *const *arg, const eph_md *md, eph_ctx **out) {
  if (!out || !md || !arg) return EPH_ERR_ARG;
  *out = nullptr;
  eph_ctx *c = new (std::nothrow) eph_ctx();
  if (!c) return EPH_ERR_ARG;
  std::string why;
  int r = parse_fix_args(narg, arg, &c->args, &why);
  if (r) {
    *out = c;
    return fail(c, r, why);
  }
  *out = c;
  if (c->args.model != 4 && c->args.model != 1)
    return fail(c, EPH_ERR_UNSUPPORTED_MODEL, "models 1 (TTM) and 4 (PRL 120, 185501) run on the GPU path");
  if (md->ntypes < 1 || md->ntypes > 64 || !md->mass) return fail(c, EPH_ERR_ARG, "ntypes must be 1..64 with masses");
  if (!(md->dt > 0)) return fail(c, EPH_ERR_ARG, "dt must be positive");
  c->ntypes = md->ntypes;
  c->mass.assign(md->mass, md->mass + md->ntypes + 1);
  for (int k = 0; k < 3; ++k) {
    c->boxlo[k] = md->boxlo[k];
    c->boxhi[k] = md->boxhi[k];
    c->prd[k] = md->boxhi[k] - md->boxlo[k];
    if (!(c->prd[k] > 0)) return fail(c, EPH_ERR_ARG, "empty box");
  }
  c->dt = md->dt;
  c->boltz = md->boltz;
  c->ftm2v = md->ftm2v;
  c->skin = md->skin;
  c->groupbit = md->groupbit;
  c->device = md->device;
  c->mode = md->mode == EPH_MODE_EXACT ? EPH_MODE_EXACT : EPH_MODE_FAST;
  // grid (fix_eph.cpp:131-161)
  if (c->args.T_infile == "NULL") {
    c->grid.create(c->args.nx, c->args.ny, c->args.nz, c->boxlo[0], c->boxhi[0], c->boxlo[1], c->boxhi[1],
                   c->boxlo[2], c->boxhi[2], c->args.T_e, c->args.C_e, c->args.rho_e, c->args.kappa_e);
  } else {
    std::string e = c->grid.load(c->args.T_infile.c_str());
    if (!e.empty()) return fail(c, EPH_ERR_FILE, e);
  }
  // element map (fix_eph.cpp:168-198), including its check type_map > types
  if (c->ntypes > narg - 17) return fail(c, EPH_ERR_ARG, "Fix eph: number of types larger than provided in fix");
  {
    std::string e = c->beta.load(c->args.beta_file.c_str());
    if (!e.empty()) return fail(c, EPH_ERR_FILE, e);
  }
  c->type_map.assign(c->ntypes + 1, 0);
  for (int t = 0; t < c->ntypes; ++t) {
    long m = 2147483647L;
    for (int j = 0; j < c->beta.n_elements; ++j)
      if (c->beta.names[j] == c->args.elements[t]) m = j;
    if (m > c->ntypes) return fail(c, EPH_ERR_ARG, "Fix eph: elements not found in input file");
    c->type_map[t + 1] = (int)m;
  }
  int used[64] = {0}, nused = 0;
  for (int t = 1; t <= c->ntypes; ++t)
    if (!used[c->type_map[t]]) used[c->type_map[t]] = 1, ++nused;
  c->multi = nused > 1;
  // device
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->own_stream = true;
  {  // can a cluster of the small-grid solve be resident (a query; nothing is launched)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(FDM_CLUSTER);
    cfg.blockDim = dim3(1024);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = FDM_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n1 = 0, n2 = 0;
    c->fdm_cluster = cudaOccupancyMaxActiveClusters(&n1, k_fdm_cluster<true>, &cfg) == cudaSuccess &&
                     cudaOccupancyMaxActiveClusters(&n2, k_fdm_cluster<false>, &cfg) == cudaSuccess && n1 >= 1 &&
                     n2 >= 1;
    cudaGetLastError();
  }
  CUDA_TRY(c, cudaMallocHost(&c->h_err, sizeof(unsigned)));
  CUDA_TRY(c, c->d_err.alloc(1));
  CUDA_TRY(c, c->counters.alloc(NCOUNTERS));
  CUDA_TRY(c, c->wrapflag.alloc(1));
  CUDA_TRY(c, c->step_ctr.alloc(1));
  CUDA_TRY(c, cudaMemset(c->step_ctr.p, 0, sizeof(unsigned long long)));
  CUDA_TRY(c, c->scal.alloc(4));
  CUDA_TRY(c, c->gsum.alloc(1));
  CUDA_TRY(c, cudaMemset(c->d_err.p, 0, sizeof(unsigned)));
  CUDA_TRY(c, cudaMemset(c->counters.p, 0, sizeof(unsigned long long) * NCOUNTERS));
  CUDA_TRY(c, cudaMemset(c->wrapflag.p, 0, sizeof(int)));
  CUDA_TRY(c, cudaMemset(c->scal.p, 0, sizeof(double) * 4));
  r = upload_tables(c);
  if (r) return r;
  r = upload_grid(c);
  if (r) return r;
  // step constants
  StepParams &P = c->P;
  P.flags = c->args.flags;
  P.groupbit = c->groupbit;
  P.nelem = c->beta.n_elements;
  for (int k = 0; k < 3; ++k) {
    P.lo[k] = c->boxlo[k];
    P.hi[k] = c->boxhi[k];
    P.prd[k] = c->prd[k];
    P.prd_hi[k] = (float)P.prd[k];
    P.prd_lo[k] = (float)(P.prd[k] - (double)P.prd_hi[k]);
  }
  P.rc2 = c->beta.r_cutoff_sq;
  P.rc2_band = (float)(c->beta.r_cutoff_sq * (1.0 + 1e-4));
  P.rc2_hi = (float)P.rc2;
  P.rc2_lo = (float)(P.rc2 - (double)P.rc2_hi);
  P.tab_rho_r_sq = c->tab_rho_r_sq.p;
  P.tab_beta = c->tab_beta.p;
  P.tab_alpha = c->tab_alpha.p;
  P.inv_dr_sq = c->beta.rho_r_sq[0].inv_dx;
  P.inv_drho = c->beta.beta[0].inv_dx;
  P.n_rho = (int)c->beta.n_rho;
  P.n_beta = (int)c->beta.n_beta;
  P.rho_cutoff = c->beta.rho_cutoff;
  P.triggersq = 0.25 * c->skin * c->skin;
  for (int t = 0; t <= 64; ++t) P.type_map[t] = t <= c->ntypes ? c->type_map[t] : 0;
  const Grid &g = c->grid;
  P.gnx = g.nx;
  P.gny = g.ny;
  P.gnz = g.nz;
  P.ncells = g.ntotal;
  P.gx0 = g.x0;
  P.gy0 = g.y0;
  P.gz0 = g.z0;
  P.gdx = g.dx;
  P.gdy = g.dy;
  P.gdz = g.dz;
  P.seed = (unsigned)c->args.seed;
  P.coloured = c->args.coloured ? 1 : 0;
  P.step = c->step_ctr.p;
  set_time_params(c);
  // bins: edge >= rc (1 + 5e-5), at least 3 per axis
  if ((r = set_bin_geometry(c, c->beta.r_cutoff))) return r;
  CUDA_TRY(c, cudaDeviceSynchronize());  // the set-up copies and memsets above ran on the default stream
  return EPH_OK;
}

void eph_destroy(eph_ctx *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  collect_marks(c);
  for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
  for (cudaStream_t s : {c->s_in, c->s_out, c->s_arr})
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  for (cudaEvent_t e : c->xev) cudaEventDestroy(e);
  if (c->f_ready) cudaEventDestroy(c->f_ready);
  if (c->arr_done) cudaEventDestroy(c->arr_done);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->h_bounds) cudaFreeHost(c->h_bounds);
  eam_free(c);
  delete c;
}

int eph_set_capacity(eph_ctx *c, int bin_capacity, int pair_capacity) {
  if (!c) return EPH_ERR_ARG;
  drop_graph(c);
  if (pair_capacity > KMAX) return fail(c, EPH_ERR_ARG, "pair capacity above the compiled maximum");
  c->buf_gen += 1;
  if (bin_capacity > 0) c->bcap = bin_capacity, c->bcap_user = true;
  if (pair_capacity > 0) c->kcap = pair_capacity;
  if (c->n > 0) {
    c->P.bcap = c->bcap;
    c->P.kcap = c->kcap;
    CUDA_TRY(c, c->bins.alloc((size_t)c->nbins * c->bcap));
    CUDA_TRY(c, c->pj.alloc((size_t)c->kcap * c->n));
    CUDA_TRY(c, c->pe.alloc((size_t)c->kcap * c->n));
    CUDA_TRY(c, alloc_pg(c));
  }
  return EPH_OK;
}

int eph_set_threads_per_atom(eph_ctx *c, int tpa) {
  if (!c) return EPH_ERR_ARG;
  if (tpa != 0 && tpa != 1 && tpa != 2 && tpa != 4 && tpa != 8)
    return fail(c, EPH_ERR_ARG, "lanes per atom: 0 (automatic), 1, 2, 4 or 8");
  drop_graph(c);
  c->buf_gen += 1;  // graphs captured elsewhere hold the old launch shape
  c->tpa_auto = tpa == 0;
  c->tpa = tpa == 0 ? auto_tpa(c->n) : tpa;
  return c->n > 0 ? configure_list(c) : EPH_OK;
}

int eph_set_pair_arithmetic(eph_ctx *c, int which) {
  if (!c) return EPH_ERR_ARG;
  if (which != EPH_PAIRS_FP64 && which != EPH_PAIRS_DF64)
    return fail(c, EPH_ERR_ARG, "pair arithmetic: EPH_PAIRS_FP64 or EPH_PAIRS_DF64");
  drop_graph(c);
  c->buf_gen += 1;  // graphs captured elsewhere hold the old kernels
  c->pair_arith = which;
  return c->n > 0 ? configure_list(c) : EPH_OK;  // the lists' default range depends on it
}

namespace {
// the list skin and whether it was the caller's choice (a caller's skin
// applies at any size), then the bins and lists of the new radius
int apply_list_skin(eph_ctx *c, double skin, bool user) {
  drop_graph(c);
  c->lskin = skin;
  c->lskin_user = user;
  if (c->n <= 0) return EPH_OK;
  const bool was = c->reuse;
  if (was) drop_list(c);  // a new radius: new bins and lists
  int r = configure_list(c);
  if (r) return r;
  if (was && !c->reuse) {  // back to the cutoff's bins
    if ((r = set_bin_geometry(c, c->beta.r_cutoff))) return r;
    if (!c->bcap_user) c->bcap = auto_bcap(c);
    c->P.bcap = c->bcap;
    CUDA_TRY(c, c->bins.alloc((size_t)c->nbins * c->bcap));
    CUDA_TRY(c, c->bin_count.alloc((size_t)c->nbins));
    c->buf_gen += 1;
  }
  return EPH_OK;
}
}  // namespace

int eph_set_list_skin(eph_ctx *c, double skin) {
  if (!c || !(skin >= 0.0)) return EPH_ERR_ARG;
  return apply_list_skin(c, skin, true);
}

int eph_get_list_skin(eph_ctx *c, double *skin, int *active) {
  if (!c) return EPH_ERR_ARG;
  if (skin) *skin = c->lskin;
  if (active) *active = c->reuse ? 1 : 0;
  return EPH_OK;
}

int eph_get_threads_per_atom(eph_ctx *c, int *tpa) {
  if (!c || !tpa) return EPH_ERR_ARG;
  *tpa = c->mode == EPH_MODE_FAST ? c->tpa : 1;
  return EPH_OK;
}

int eph_autotune(eph_ctx *c, int *chosen) {
  if (!c) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  if (c->mode != EPH_MODE_FAST || c->args.model != 4) {
    if (chosen) *chosen = 1;
    return EPH_OK;  // EXACT keeps the reference's order: one lane per atom
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  // the sweeps need a step's pairs
  unsigned long long steps = 0;
  CUDA_TRY(c, cudaMemcpy(&steps, c->step_ctr.p, sizeof(steps), cudaMemcpyDeviceToHost));
  if (steps == 0) return fail(c, EPH_ERR_STATE, "autotune needs one step (or post_force) first");
  const size_t N = (size_t)c->n;
  DevBuf<D4> save[5];
  DevBuf<D4> *bufs[5] = {&c->f, &c->f_eph, &c->f_rng, &c->f_dis, &c->f_sto};
  for (int k = 0; k < 5; ++k) {
    CUDA_TRY(c, save[k].alloc(N));
    CUDA_TRY(c, cudaMemcpyAsync(save[k].p, bufs[k]->p, sizeof(D4) * N, cudaMemcpyDeviceToDevice, c->stream));
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CUDA_TRY(c, cudaEventCreate(&e0));
  CUDA_TRY(c, cudaEventCreate(&e1));
  const bool prof = c->profiling;
  c->profiling = false;
  const int keep = c->tpa;
  int best = 1;
  float best_ms = 1e30f;
  for (int tpa : {1, 2, 4, 8}) {
    c->tpa = tpa;
    float total = 0.f;
    for (int rep = 0; rep < 7; ++rep) {
      CUDA_TRY(c, cudaMemcpyAsync(c->f.p, save[0].p, sizeof(D4) * N, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(c, cudaEventRecord(e0, c->stream));
      // with stage 1 folded into the density sweep only the force sweep has lanes
      if ((c->P.flags & FLAG_FRICTION) && !fused_friction(c)) launch_friction_w(c);
      if (c->multi) launch_forces_m<true, true>(c);
      else launch_forces_m<true, false>(c);
      CUDA_TRY(c, cudaEventRecord(e1, c->stream));
      CUDA_TRY(c, cudaEventSynchronize(e1));
      float ms = 0.f;
      CUDA_TRY(c, cudaEventElapsedTime(&ms, e0, e1));
      if (rep >= 2) total += ms;  // two warm-up runs
    }
    if (total < best_ms) {
      best_ms = total;
      best = tpa;
    }
  }
  c->tpa = keep;
  c->profiling = prof;
  for (int k = 0; k < 5; ++k)
    CUDA_TRY(c, cudaMemcpyAsync(bufs[k]->p, save[k].p, sizeof(D4) * N, cudaMemcpyDeviceToDevice, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  r = eph_set_threads_per_atom(c, best);
  if (r) return r;
  if (chosen) *chosen = best;
  return EPH_OK;
}

int eph_autotune_list_skin(eph_ctx *c, const double *skins, int nskins, int steps, double *chosen) {
  if (!c || !skins || nskins < 1 || steps < 1) return EPH_ERR_ARG;
  for (int k = 0; k < nskins; ++k)
    if (!(skins[k] >= 0.0)) return fail(c, EPH_ERR_ARG, "list skin must be >= 0");
  int r = require_atoms(c);
  if (r) return r;
  // where no skin can turn the lists on (EXACT, model 1, several lanes per
  // atom below 16,384 atoms, the EAM engine, an adjoint, a box narrower
  // than three list radii for every candidate) nothing runs
  bool applies = false;
  {
    const double keep_s = c->lskin;
    const bool keep_u = c->lskin_user;
    c->lskin_user = true;
    for (int k = 0; k < nskins && !applies; ++k) {
      c->lskin = skins[k];
      applies = skins[k] > 0.0 && want_list(c);
    }
    c->lskin = keep_s;
    c->lskin_user = keep_u;
  }
  if (!applies) {
    if (chosen) *chosen = c->lskin;
    return EPH_OK;
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  unsigned long long calls = 0;
  CUDA_TRY(c, cudaMemcpy(&calls, c->step_ctr.p, sizeof(calls), cudaMemcpyDeviceToHost));
  if (calls == 0) return fail(c, EPH_ERR_STATE, "list-skin autotune needs one step (or post_force) first");
  // the state a step reads or a caller may read back afterwards
  const size_t N = (size_t)c->n, NC = (size_t)c->grid.ntotal;
  DevBuf<D4> *d4[] = {&c->x, &c->v, &c->f, &c->xhold, &c->f_eph, &c->f_rng, &c->f_dis, &c->f_sto, &c->xi, &c->A, &c->Bw};
  const int ND4 = (int)(sizeof(d4) / sizeof(d4[0]));
  DevBuf<D4> s_d4[ND4];
  DevBuf<double> s_rho, s_beta, s_tei, s_T, s_scal;
  DevBuf<unsigned long long> s_cnt, s_step;
  DevBuf<int> s_wrap, s_cell;
  for (int k = 0; k < ND4; ++k) CUDA_TRY(c, s_d4[k].alloc(N));
  CUDA_TRY(c, s_rho.alloc(N));
  CUDA_TRY(c, s_beta.alloc(N));
  CUDA_TRY(c, s_tei.alloc(N));
  CUDA_TRY(c, s_cell.alloc(N));
  CUDA_TRY(c, s_T.alloc(NC));
  CUDA_TRY(c, s_scal.alloc(4));
  CUDA_TRY(c, s_cnt.alloc(NCOUNTERS));
  CUDA_TRY(c, s_step.alloc(1));
  CUDA_TRY(c, s_wrap.alloc(1));
  auto copy_all = [&](bool save) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    auto cp = [&](void *dst, const void *src, size_t bytes) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, c->stream);
    };
    auto pair = [&](void *live, void *kept, size_t bytes) { save ? cp(kept, live, bytes) : cp(live, kept, bytes); };
    for (int k = 0; k < ND4; ++k) pair(d4[k]->p, s_d4[k].p, sizeof(D4) * N);
    pair(c->rho.p, s_rho.p, sizeof(double) * N);
    pair(c->beta_i.p, s_beta.p, sizeof(double) * N);
    // the atoms' grid cells and T_e there: between post_force and
    // end_of_step (an engine's hooks) the deposition still reads them
    pair(c->Te_i.p, s_tei.p, sizeof(double) * N);
    pair(c->cell.p, s_cell.p, sizeof(int) * N);
    pair(c->T0.p, s_T.p, sizeof(double) * NC);
    pair(c->scal.p, s_scal.p, sizeof(double) * 4);
    pair(c->counters.p, s_cnt.p, sizeof(unsigned long long) * NCOUNTERS);
    pair(c->step_ctr.p, s_step.p, sizeof(unsigned long long));
    pair(c->wrapflag.p, s_wrap.p, sizeof(int));
    return e;
  };
  CUDA_TRY(c, copy_all(true));
  const long keep_ts = c->ntimestep, keep_launches = c->launches;
  const int keep_freq = c->args.T_freq;
  const bool keep_prof = c->profiling;
  const double keep_skin = c->lskin;
  const bool keep_user = c->lskin_user;
  c->args.T_freq = 0;  // no temperature files from trial steps
  c->profiling = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CUDA_TRY(c, cudaEventCreate(&e0));
  CUDA_TRY(c, cudaEventCreate(&e1));
  const int xi_mode = 0;  // device deviates: timing only
  double best = keep_skin;
  float best_ms = 1e30f;
  int status = EPH_OK;
  for (int k = 0; k < nskins && status == EPH_OK; ++k) {
    // each window starts from the saved state with a list build, as a run
    // does after eph_set_list_skin; one untimed window first settles the
    // allocations of the new radius
    for (int rep = 0; rep < 2 && status == EPH_OK; ++rep) {
      if (copy_all(false) != cudaSuccess) {
        status = fail(c, EPH_ERR_CUDA, "restoring the state");
        break;
      }
      if ((status = apply_list_skin(c, skins[k], true)) != EPH_OK) break;
      if (cudaEventRecord(e0, c->stream) != cudaSuccess) {
        status = fail(c, EPH_ERR_CUDA, "event");
        break;
      }
      for (int s = 0; s < steps && status == EPH_OK; ++s) {
        c->ntimestep += 1;
        status = record_step(c, xi_mode);
      }
      if (status != EPH_OK) break;
      float ms = 0.f;
      if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        status = fail(c, EPH_ERR_CUDA, "timing a trial window");
        break;
      }
      if ((status = check_device(c)) == EPH_ERR_CAPACITY) {
        status = EPH_OK;  // this radius overflows the bins or pair rows: not a candidate
        break;
      }
      if (status != EPH_OK) break;
      if (rep == 1 && ms < best_ms) {
        best_ms = ms;
        best = skins[k];
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->args.T_freq = keep_freq;
  c->profiling = keep_prof;
  c->ntimestep = keep_ts;
  c->launches = keep_launches;
  if (copy_all(false) != cudaSuccess && status == EPH_OK) status = fail(c, EPH_ERR_CUDA, "restoring the state");
  if (status != EPH_OK) {
    apply_list_skin(c, keep_skin, keep_user);  // as it was (the lists rebuild on the next step)
    return status;
  }
  if (!(best_ms < 1e30f)) {
    apply_list_skin(c, keep_skin, keep_user);
    return fail(c, EPH_ERR_CAPACITY, "every candidate list skin overflows the bins or pair rows");
  }
  if ((r = apply_list_skin(c, best, true))) return r;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (chosen) *chosen = best;
  return EPH_OK;
}

int eph_set_atoms(eph_ctx *c, int n, const double *hx, const double *hv, const int *htype, const int *hmask) {
  if (!c) return EPH_ERR_ARG;
  drop_graph(c);
  if (n < 1) return fail(c, EPH_ERR_ARG, "fix_eph: error no atoms in simulation");
  if ((unsigned)n > IDX_MASK) return fail(c, EPH_ERR_ARG, "too many atoms for one context");
  if (!hx || !hv || !htype) return fail(c, EPH_ERR_ARG, "null atom buffer");
  for (int i = 0; i < n; ++i)
    if (htype[i] < 1 || htype[i] > c->ntypes) return fail(c, EPH_ERR_ARG, "atom type outside 1..ntypes");
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const size_t N = (size_t)n;
  int r0;
  if (n != c->n) {  // (re)allocate the per-atom storage
    c->buf_gen += 1;
    c->n = n;
    c->P.n = n;
    if (c->tpa_auto) c->tpa = auto_tpa(n);
    for (DevBuf<D4> *b : {&c->x, &c->v, &c->f, &c->xhold, &c->f_eph, &c->f_rng, &c->xi, &c->A, &c->Bw, &c->f_dis,
                          &c->f_sto})
      CUDA_TRY(c, b->alloc(N));
    // the coloured-noise memory starts at zero (fix_eph_coloured_exp.cpp:229-230) and
    // follows the atom index afterwards
    CUDA_TRY(c, cudaMemsetAsync(c->f_dis.p, 0, sizeof(D4) * N, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->f_sto.p, 0, sizeof(D4) * N, c->stream));
    CUDA_TRY(c, c->Mm.alloc(2 * N));
    CUDA_TRY(c, c->G.alloc(2 * N));
    CUDA_TRY(c, c->type.alloc(N));
    CUDA_TRY(c, c->mask.alloc(N));
    CUDA_TRY(c, c->nshort.alloc(N));
    CUDA_TRY(c, c->cell.alloc(N));
    CUDA_TRY(c, c->rho.alloc(N));
    CUDA_TRY(c, c->beta_i.alloc(N));
    CUDA_TRY(c, c->Te_i.alloc(N));
    CUDA_TRY(c, c->stage.alloc(8 * N));
    CUDA_TRY(c, c->atom_bin.alloc(N));
    CUDA_TRY(c, c->atom_off.alloc(N));
    CUDA_TRY(c, c->dfrec.alloc(2 * N));
    CUDA_TRY(c, c->dfvrec.alloc(2 * N));
    CUDA_TRY(c, c->part.alloc((size_t)nblocks(n, 256)));
    if (c->fext.p) CUDA_TRY(c, c->fext.alloc(N));
    // capacities from the number density: a bin holds ~density*w^3 atoms, the
    // cutoff sphere ~density*4/3 pi rc^3
    const double vol = c->prd[0] * c->prd[1] * c->prd[2];
    const double dens = n / vol;
    const double per_bin = dens * c->P.w[0] * c->P.w[1] * c->P.w[2];
    const double rc = c->beta.r_cutoff;
    const double per_sphere = dens * 4.18879020478639 * rc * rc * rc;
    if (c->bcap <= 0) c->bcap = ((int)std::ceil(2.0 * per_bin + 16.0) + 7) / 8 * 8;
    if (c->kcap <= 0) c->kcap = std::min(KMAX, ((int)std::ceil(2.0 * per_sphere + 24.0) + 7) / 8 * 8);
    c->P.bcap = c->bcap;
    c->P.kcap = c->kcap;
    CUDA_TRY(c, c->bins.alloc((size_t)c->nbins * c->bcap));
    CUDA_TRY(c, c->pj.alloc((size_t)c->kcap * N));
    CUDA_TRY(c, c->pe.alloc((size_t)c->kcap * N));
    CUDA_TRY(c, alloc_pg(c));
  }
  if ((r0 = eam_resize(c))) return r0;
  if (!c->tmap.p) CUDA_TRY(c, c->tmap.alloc(65));
  if (!c->bin_count.p) CUDA_TRY(c, c->bin_count.alloc((size_t)c->nbins));
  // atoms
  std::vector<int> m(N, 1);
  if (hmask) std::memcpy(m.data(), hmask, sizeof(int) * N);
  CUDA_TRY(c, cudaMemcpy(c->type.p, htype, sizeof(int) * N, cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->mask.p, m.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->tmap.p, c->P.type_map, sizeof(int) * 65, cudaMemcpyHostToDevice));
  for (DevBuf<D4> *b : {&c->x, &c->v, &c->f, &c->xhold, &c->f_eph, &c->f_rng, &c->xi, &c->A, &c->Bw})
    CUDA_TRY(c, cudaMemsetAsync(b->p, 0, sizeof(D4) * N, c->stream));
  int r = eph_put(c, EPH_FIELD_X, hx, EPH_HOST);
  if (r) return r;
  r = eph_put(c, EPH_FIELD_V, hv, EPH_HOST);
  if (r) return r;
  k_set_elem<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->type.p, c->tmap.p, c->x.p);
  CUDA_TRY(c, cudaMemcpyAsync(c->xhold.p, c->x.p, sizeof(D4) * N, cudaMemcpyDeviceToDevice, c->stream));
  // the engine wraps positions at set-up (Verlet::setup)
  CUDA_TRY(c, cudaMemsetAsync(c->wrapflag.p, 0xff, sizeof(int), c->stream));
  // list reuse as the settings allow (may change the bins); the next step builds
  if ((r = configure_list(c))) return r;
  CUDA_TRY(c, cudaMemsetAsync(c->bin_count.p, 0, sizeof(int) * (size_t)c->nbins, c->stream));
  k_bin<<<nblocks(n), BLOCK, 0, c->stream>>>(c->P, c->x.p, c->xhold.p, c->wrapflag.p, c->bin_count.p, c->bins.p,
                                             c->atom_bin.p, c->atom_off.p, c->d_err.p, c->counters.p, 0);
  CUDA_TRY(c, cudaMemsetAsync(c->wrapflag.p, 0, sizeof(int), c->stream));
  c->have_fext = false;
  CUDA_TRY(c, cudaGetLastError());
  return check_device(c);
}

int eph_put(eph_ctx *c, int field, const double *src, int where) {
  if (!c || !src) return EPH_ERR_ARG;
  if (field == EPH_FIELD_T_E) {
    const size_t nc = (size_t)c->grid.ntotal;
    CUDA_TRY(c, cudaMemcpyAsync(c->T0.p, src, nc * 8,
                                where == EPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
    if (where == EPH_HOST) CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return EPH_OK;
  }
  int r = require_atoms(c);
  if (r) return r;
  DevBuf<D4> *dst = nullptr;
  switch (field) {
    case EPH_FIELD_X: dst = &c->x; break;
    case EPH_FIELD_V: dst = &c->v; break;
    case EPH_FIELD_F: dst = &c->f; break;
    case EPH_FIELD_XI: dst = &c->xi; c->have_xi = true; break;
    case EPH_FIELD_F_EXT:
      if (!c->fext.p) {
        c->buf_gen += 1;
        CUDA_TRY(c, c->fext.alloc((size_t)c->n));
      }
      dst = &c->fext;
      if (!c->have_fext) drop_graph(c);  // the captured step cleared f instead of copying it
      c->have_fext = true;
      break;
    default: return fail(c, EPH_ERR_ARG, "field cannot be written");
  }
  const double *s = src;
  const bool host = where == EPH_HOST || where == EPH_HOST_ASYNC;
  if (host) {
    CUDA_TRY(c, cudaMemcpyAsync(c->stage.p, src, sizeof(double) * 3 * (size_t)c->n, cudaMemcpyHostToDevice,
                                c->stream));
    s = c->stage.p;
  }
  k_pack3<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->n, s, dst->p);
  CUDA_TRY(c, cudaGetLastError());
  if (where == EPH_HOST) CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // src may be reused at return
  return EPH_OK;
}

int eph_get(eph_ctx *c, int field, double *dst, int where) {
  if (!c || !dst) return EPH_ERR_ARG;
  if (field == EPH_FIELD_T_E) {
    CUDA_TRY(c, cudaMemcpyAsync(dst, c->T0.p, sizeof(double) * (size_t)c->grid.ntotal,
                                where == EPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
  }
  int r = require_atoms(c);
  if (r) return r;
  const int n = c->n;
  const bool host = where == EPH_HOST || where == EPH_HOST_ASYNC;
  double *d = host ? c->stage.p : dst;
  size_t count = 3 * (size_t)n;
  switch (field) {
    case EPH_FIELD_X: k_unpack3<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->x.p, d); break;
    case EPH_FIELD_V: k_unpack3<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->v.p, d); break;
    case EPH_FIELD_F: k_unpack3<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->f.p, d); break;
    case EPH_FIELD_XI: k_get_xi<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->A.p, c->Bw.p, d); break;
    case EPH_FIELD_F_EPH: k_unpack3<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->f_eph.p, d); break;
    case EPH_FIELD_F_RNG: k_unpack3<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->f_rng.p, d); break;
    case EPH_FIELD_W: k_get_w<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->Bw.p, d); break;
    case EPH_FIELD_RHO:
      count = (size_t)n;
      CUDA_TRY(c, cudaMemcpyAsync(d, c->rho.p, sizeof(double) * count, cudaMemcpyDeviceToDevice, c->stream));
      break;
    case EPH_FIELD_PERATOM:
      count = 8 * (size_t)n;
      k_peratom<<<nblocks(n), BLOCK, 0, c->stream>>>(n, c->groupbit, c->mask.p, c->rho.p, c->beta_i.p, c->f_eph.p,
                                                     c->f_rng.p, d);
      break;
    default: return fail(c, EPH_ERR_ARG, "field cannot be read");
  }
  CUDA_TRY(c, cudaGetLastError());
  if (host) CUDA_TRY(c, cudaMemcpyAsync(dst, c->stage.p, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
  if (where == EPH_HOST_ASYNC) return EPH_OK;  // complete (and checked) at the next synchronising call
  return check_device(c);
}

int eph_initial_integrate(eph_ctx *c) {
  if (!c) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  return launch_initial(c, 0);
}

int eph_post_force(eph_ctx *c, int xi_source) {
  if (!c) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  if (xi_source == EPH_XI_GIVEN && !c->have_xi && (c->P.flags & FLAG_RANDOM))
    return fail(c, EPH_ERR_STATE, "EPH_XI_GIVEN without eph_put(EPH_FIELD_XI)");
  r = launch_post_force(c, xi_source == EPH_XI_GIVEN ? 1 : 0);
  if (r) return r;
  return EPH_OK;
}

int eph_final_integrate(eph_ctx *c) {
  if (!c) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  return launch_final(c);
}

int eph_end_of_step(eph_ctx *c) {
  if (!c) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  r = launch_end_of_step(c);
  if (r) return r;
  if (c->arr_pending) {  // the per-atom array eph_post_force_host sent out
    CUDA_TRY(c, cudaEventSynchronize(c->arr_done));
    c->arr_pending = false;
  }
  return write_T_output(c);
}

}  // extern "C"

namespace {

constexpr int HOST_CHUNKS = 8;          // chunks of a pipelined host exchange
constexpr int HOST_CHUNK_MIN = 1 << 16;  // atoms per chunk at least

// the copy streams, chunk events and staging rows of the host-array hooks
int host_io_ready(eph_ctx *c) {
  for (cudaStream_t *s : {&c->s_in, &c->s_out, &c->s_arr})
    if (!*s) CUDA_TRY(c, cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));
  while (c->xev.size() < 2 * HOST_CHUNKS + 2) {
    cudaEvent_t e;
    CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->xev.push_back(e);
  }
  if (!c->f_ready) CUDA_TRY(c, cudaEventCreateWithFlags(&c->f_ready, cudaEventDisableTiming));
  if (!c->arr_done) CUDA_TRY(c, cudaEventCreateWithFlags(&c->arr_done, cudaEventDisableTiming));
  const size_t need = 20 * (size_t)c->n;
  if (c->hstage.n != need) {
    if (c->arr_pending) CUDA_TRY(c, cudaEventSynchronize(c->arr_done));
    c->arr_pending = false;
    CUDA_TRY(c, c->hstage.alloc(need));
  }
  return EPH_OK;
}

// the per-atom array copied out by eph_post_force_host: written before the
// host reads it or its staging is reused
int host_array_wait(eph_ctx *c) {
  if (c->arr_pending) {
    CUDA_TRY(c, cudaEventSynchronize(c->arr_done));
    c->arr_pending = false;
  }
  return EPH_OK;
}

// Chunk k of n atoms in `chunks` pieces: [base, base + count)
void chunk_range(int n, int chunks, int k, int &base, int &count) {
  const long b = (long)n * k / chunks, e = (long)n * (k + 1) / chunks;
  base = (int)b;
  count = (int)(e - b);
}

// A hook with the engine's host arrays, pipelined over chunks of atoms: the
// rows of `in` (n x 3 doubles each) go up on the copy-in stream, `kernel`
// (the fused pack + hook + unpack of one chunk) runs on the context's
// stream, and the rows it staged for `out` come back on the copy-out
// stream, so that the copies of one chunk overlap those of its neighbours in
// both directions of the host link.  Returns when `out` is written.
template <class Kernel>
int host_pipeline(eph_ctx *c, const double *const *in, int nin, double *const *out, int nout, Kernel kernel) {
  const size_t N = (size_t)c->n;
  const int chunks = std::max(1, std::min(HOST_CHUNKS, c->n / HOST_CHUNK_MIN));
  double *sin = c->hstage.p, *sout = c->hstage.p + 3 * N * (size_t)nin;
  for (int k = 0; k < chunks; ++k) {
    int base, count;
    chunk_range(c->n, chunks, k, base, count);
    const size_t off = 3 * (size_t)base, bytes = 3 * sizeof(double) * (size_t)count;
    for (int q = 0; q < nin; ++q)
      CUDA_TRY(c, cudaMemcpyAsync(sin + 3 * N * q + off, in[q] + off, bytes, cudaMemcpyHostToDevice, c->s_in));
    cudaEvent_t e_in = c->xev[2 * k], e_done = c->xev[2 * k + 1];
    CUDA_TRY(c, cudaEventRecord(e_in, c->s_in));
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, e_in, 0));
    kernel(base, count, sin + off, sout + off);
    c->launches += 1;
    CUDA_TRY(c, cudaGetLastError());
    CUDA_TRY(c, cudaEventRecord(e_done, c->stream));
    CUDA_TRY(c, cudaStreamWaitEvent(c->s_out, e_done, 0));
    for (int q = 0; q < nout; ++q)
      CUDA_TRY(c, cudaMemcpyAsync(out[q] + off, sout + 3 * N * q + off, bytes, cudaMemcpyDeviceToHost, c->s_out));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->s_out));
  return EPH_OK;
}

}  // namespace

extern "C" {

int eph_initial_integrate_host(eph_ctx *c, double *x, double *v) {
  if (!c || !x || !v) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r || (r = host_io_ready(c))) return r;
  const size_t N = (size_t)c->n;
  const double *in[2] = {x, v};
  double *out[2] = {x, v};
  PhaseScope ps(c, EPH_PHASE_INTEGRATE);
  return host_pipeline(c, in, 2, out, 2, [&](int base, int count, const double *s, double *o) {
    StepParams P = c->P;
    const int nb = nblocks(count);
    const size_t b = (size_t)base;
    if (c->mode == EPH_MODE_FAST)
      k_initial_host<true><<<nb, BLOCK, 0, c->stream>>>(P, count, s, s + 3 * N, c->x.p + b, c->v.p + b, c->f.p + b,
                                                        c->type.p + b, c->mask.p + b, o, o + 3 * N);
    else
      k_initial_host<false><<<nb, BLOCK, 0, c->stream>>>(P, count, s, s + 3 * N, c->x.p + b, c->v.p + b, c->f.p + b,
                                                         c->type.p + b, c->mask.p + b, o, o + 3 * N);
  });
}

int eph_final_integrate_host(eph_ctx *c, const double *f, double *v) {
  if (!c || !f || !v) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r || (r = host_io_ready(c))) return r;
  const double *in[1] = {f};
  double *out[1] = {v};
  PhaseScope ps(c, EPH_PHASE_INTEGRATE);
  return host_pipeline(c, in, 1, out, 1, [&](int base, int count, const double *s, double *o) {
    const int nb = nblocks(count);
    const size_t b = (size_t)base;
    if (c->mode == EPH_MODE_FAST)
      k_final_host<true><<<nb, BLOCK, 0, c->stream>>>(c->P, count, s, c->f.p + b, c->v.p + b, c->type.p + b,
                                                      c->mask.p + b, o);
    else
      k_final_host<false><<<nb, BLOCK, 0, c->stream>>>(c->P, count, s, c->f.p + b, c->v.p + b, c->type.p + b,
                                                       c->mask.p + b, o);
  });
}

int eph_pin(void *p, size_t bytes) {
  if (!p || !bytes) return EPH_ERR_ARG;
  if (cudaHostRegister(p, bytes, cudaHostRegisterDefault) == cudaSuccess) return EPH_OK;
  cudaGetLastError();  // not sticky: the copies then run from pageable memory
  return EPH_ERR_CUDA;
}

int eph_unpin(void *p) {
  if (!p) return EPH_ERR_ARG;
  if (cudaHostUnregister(p) == cudaSuccess) return EPH_OK;
  cudaGetLastError();
  return EPH_ERR_CUDA;
}

int eph_post_force_host(eph_ctx *c, const double *x, const double *f_in, double *f_out, double *array,
                        int xi_source) {
  if (!c || !f_in || !f_out) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r || (r = host_io_ready(c)) || (r = host_array_wait(c))) return r;
  if (xi_source == EPH_XI_GIVEN && !c->have_xi && (c->P.flags & FLAG_RANDOM))
    return fail(c, EPH_ERR_STATE, "EPH_XI_GIVEN without eph_put(EPH_FIELD_XI)");
  const size_t N = (size_t)c->n;
  double *sx = c->hstage.p, *sf = c->hstage.p + 3 * N, *so = c->hstage.p + 6 * N, *sa = c->hstage.p + 12 * N;
  // positions first (the bins need them), then the engine's force, which
  // the force sweep waits for: its copy overlaps the binning and the density
  // sweep
  if (x) {
    CUDA_TRY(c, cudaMemcpyAsync(sx, x, 3 * sizeof(double) * N, cudaMemcpyHostToDevice, c->s_in));
    CUDA_TRY(c, cudaEventRecord(c->xev[0], c->s_in));
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->xev[0], 0));
    k_pack3<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->n, sx, c->x.p);
    c->launches += 1;
  }
  CUDA_TRY(c, cudaMemcpyAsync(sf, f_in, 3 * sizeof(double) * N, cudaMemcpyHostToDevice, c->s_in));
  CUDA_TRY(c, cudaEventRecord(c->f_ready, c->s_in));
  c->f_pending = true;
  r = launch_post_force(c, xi_source == EPH_XI_GIVEN ? 1 : 0);
  if (c->f_pending) {  // no force sweep ran (no pair sweeps): f as the engine gave it
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->f_ready, 0));
    k_pack3<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->n, sf, c->f.p);
    c->f_pending = false;
  }
  if (r) return r;
  k_unpack3<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->n, c->f.p, so);
  c->launches += 1;
  CUDA_TRY(c, cudaEventRecord(c->xev[1], c->stream));
  if (array) {
    // the per-atom array (fix_eph.cpp:406-428) is final here; it leaves on
    // its own stream while the next hooks run and is waited for by
    // eph_end_of_step (or any call that synchronises the context)
    k_peratom<<<nblocks(c->n), BLOCK, 0, c->stream>>>(c->n, c->groupbit, c->mask.p, c->rho.p, c->beta_i.p,
                                                      c->f_eph.p, c->f_rng.p, sa);
    c->launches += 1;
    CUDA_TRY(c, cudaEventRecord(c->xev[2], c->stream));
    CUDA_TRY(c, cudaStreamWaitEvent(c->s_arr, c->xev[2], 0));
    CUDA_TRY(c, cudaMemcpyAsync(array, sa, 8 * sizeof(double) * N, cudaMemcpyDeviceToHost, c->s_arr));
    CUDA_TRY(c, cudaEventRecord(c->arr_done, c->s_arr));
    c->arr_pending = true;
  }
  CUDA_TRY(c, cudaStreamWaitEvent(c->s_out, c->xev[1], 0));
  CUDA_TRY(c, cudaMemcpyAsync(f_out, so, 3 * sizeof(double) * N, cudaMemcpyDeviceToHost, c->s_out));
  CUDA_TRY(c, cudaStreamSynchronize(c->s_out));
  return check_device(c);
}

int eph_step(eph_ctx *c, int nsteps, int xi_source) {
  if (!c || nsteps < 0) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  if (xi_source == EPH_XI_GIVEN && !c->have_xi && (c->P.flags & FLAG_RANDOM))
    return fail(c, EPH_ERR_STATE, "EPH_XI_GIVEN without eph_put(EPH_FIELD_XI)");
  const int xi_mode = xi_source == EPH_XI_GIVEN ? 1 : 0;
  // a T-dependent grid decides its substep count on the host every step
  const bool graph = c->use_graph && !c->profiling && !c->td.tdyn;
  if (graph && (!c->gexec || c->graph_xi != xi_mode) && (r = capture_step(c, xi_mode))) return r;
  for (int s = 0; s < nsteps; ++s) {
    c->ntimestep += 1;
    if (graph) {
      CUDA_TRY(c, cudaGraphLaunch(c->gexec, c->stream));
      c->launches += c->graph_launches;
    } else if ((r = record_step(c, xi_mode))) {
      return r;
    }
    if ((r = write_T_output(c))) return r;
  }
  return EPH_OK;
}

int eph_set_graph(eph_ctx *c, int on) {
  if (!c) return EPH_ERR_ARG;
  c->use_graph = on != 0;
  if (!c->use_graph) drop_graph(c);
  return EPH_OK;
}

int eph_synchronize(eph_ctx *c) {
  if (!c) return EPH_ERR_ARG;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (c->arr_pending) {
    CUDA_TRY(c, cudaEventSynchronize(c->arr_done));
    c->arr_pending = false;
  }
  return check_device(c);
}

int eph_compute_vector(eph_ctx *c, int i, double *out) {
  if (!c || !out) return EPH_ERR_ARG;
  if (i == 1) {
    CUDA_TRY(c, cudaMemsetAsync(c->gsum.p, 0, sizeof(U128), c->stream));
    k_grid_sum<<<std::min(nblocks(c->grid.ntotal, 256), 1024), 256, 0, c->stream>>>(c->T0.p, c->grid.ntotal,
                                                                                    c->gsum.p, c->d_err.p);
    k_from_fixed<<<1, 1, 0, c->stream>>>(c->gsum.p, c->scal.p + 2);
    double s;
    CUDA_TRY(c, cudaMemcpyAsync(&s, c->scal.p + 2, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int r = check_device(c);
    if (r) return r;
    *out = s / (double)(size_t)c->grid.ntotal;
    return EPH_OK;
  }
  CUDA_TRY(c, cudaMemcpyAsync(out, c->scal.p + 0, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return check_device(c);
}

int eph_reset_dt(eph_ctx *c, double dt) {
  if (!c || !(dt > 0)) return EPH_ERR_ARG;
  drop_graph(c);
  c->dt = dt;
  set_time_params(c);
  return EPH_OK;
}

int eph_save_state(eph_ctx *c, const char *path) {
  if (!c || !path) return EPH_ERR_ARG;
  int r = download_grid(c);
  if (r) return r;
  if (c->grid.save_state(path)) return fail(c, EPH_ERR_FILE, std::string("cannot write ") + path);
  return EPH_OK;
}

int eph_save_temperature(eph_ctx *c, const char *path, int n) {
  if (!c || !path) return EPH_ERR_ARG;
  int r = download_grid(c);
  if (r) return r;
  if (c->grid.save_temperature(path, n)) return fail(c, EPH_ERR_FILE, std::string("cannot write ") + path);
  return EPH_OK;
}

int eph_post_run(eph_ctx *c) {
  if (!c) return EPH_ERR_ARG;
  return eph_save_state(c, c->args.T_state.c_str());
}

int eph_set_timestep(eph_ctx *c, long ntimestep) {
  if (!c) return EPH_ERR_ARG;
  c->ntimestep = ntimestep;
  return EPH_OK;
}

int eph_set_stream(eph_ctx *c, void *stream) {
  if (!c) return EPH_ERR_ARG;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->own_stream = false;
  c->stream = (cudaStream_t)stream;
  return EPH_OK;
}

int eph_set_profiling(eph_ctx *c, int on) {
  if (!c) return EPH_ERR_ARG;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  collect_marks(c);
  for (int k = 0; k < EPH_NPHASES; ++k) {
    c->phase_ms[k] = 0.0;
    c->phase_launches[k] = 0;
  }
  c->launches = 0;
  c->profiling = on != 0;
  return EPH_OK;
}

int eph_phase_times(eph_ctx *c, double *ms, long *launches) {
  if (!c) return EPH_ERR_ARG;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  collect_marks(c);
  for (int k = 0; k < EPH_NPHASES; ++k) {
    if (ms) ms[k] = c->phase_ms[k];
    if (launches) launches[k] = c->phase_launches[k];
  }
  return EPH_OK;
}

int eph_launch_count(eph_ctx *c, long *out) {
  if (!c || !out) return EPH_ERR_ARG;
  *out = c->launches;
  return EPH_OK;
}

int eph_pair_count(eph_ctx *c, long *out) {
  if (!c || !out) return EPH_ERR_ARG;
  int r = require_atoms(c);
  if (r) return r;
  std::vector<int> h((size_t)c->n);
  CUDA_TRY(c, cudaMemcpyAsync(h.data(), c->nshort.p, sizeof(int) * h.size(), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  long t = 0;
  for (int v : h) t += v;
  *out = t;
  return EPH_OK;
}

int eph_get_counter(eph_ctx *c, int which, long *out) {
  if (!c || !out || which < 0 || which >= NCOUNTERS) return EPH_ERR_ARG;
  unsigned long long v = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&v, c->counters.p + which, sizeof(v), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *out = (long)v;
  return EPH_OK;
}

// ------------------------------------------------------ batched replicas

struct eph_batch {
  std::vector<eph_ctx *> reps;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long launches_per_step = 0;
  std::string err;
};

static void batch_drop_graph(eph_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
}

int eph_batch_create(int nrep, const int *narg, const char *const *const *arg, const eph_md *md, eph_batch **out) {
  if (!out || nrep < 1 || !narg || !arg || !md) return EPH_ERR_ARG;
  *out = nullptr;
  eph_batch *b = new (std::nothrow) eph_batch();
  if (!b) return EPH_ERR_ARG;
  *out = b;
  for (int r = 0; r < nrep; ++r) {
    eph_ctx *c = nullptr;
    const int rc = eph_create(narg[r], arg[r], &md[r], &c);
    b->reps.push_back(c);
    if (rc) {
      b->err = "replica " + std::to_string(r) + ": " + eph_last_error(c);
      return rc;
    }
    if (md[r].device != md[0].device) {
      b->err = "all replicas of a batch run on one device";
      return EPH_ERR_ARG;
    }
  }
  if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    b->err = "cannot create the batch stream";
    return EPH_ERR_CUDA;
  }
  b->joins.assign(nrep, nullptr);
  for (auto &e : b->joins)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return EPH_ERR_CUDA;
  return EPH_OK;
}

void eph_batch_destroy(eph_batch *b) {
  if (!b) return;
  if (b->main) cudaStreamSynchronize(b->main);
  batch_drop_graph(b);
  for (eph_ctx *c : b->reps) eph_destroy(c);
  for (auto e : b->joins)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->main) cudaStreamDestroy(b->main);
  delete b;
}

const char *eph_batch_last_error(const eph_batch *b) { return b ? b->err.c_str() : "null batch"; }

eph_ctx *eph_batch_context(eph_batch *b, int rep) {
  if (!b || rep < 0 || rep >= (int)b->reps.size()) return nullptr;
  return b->reps[rep];
}

int eph_batch_set_atoms(eph_batch *b, int rep, int n, const double *x, const double *v, const int *type,
                        const int *mask) {
  eph_ctx *c = eph_batch_context(b, rep);
  if (!c) return EPH_ERR_ARG;
  batch_drop_graph(b);
  return eph_set_atoms(c, n, x, v, type, mask);
}

// Capture one step of every replica as parallel branches of one graph.
static int batch_capture(eph_batch *b) {
  batch_drop_graph(b);
  for (eph_ctx *c : b->reps) {
    if (c->n <= 0) {
      b->err = "a replica has no atoms";
      return EPH_ERR_STATE;
    }
    if (c->td.tdyn) {
      b->err = "replicas with temperature-dependent grid cells cannot be captured (substeps decided per step)";
      return EPH_ERR_STATE;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return EPH_ERR_CUDA;
  }
  if (cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return EPH_ERR_CUDA;
  int rc = EPH_OK;
  long launches = 0;
  if (cudaEventRecord(b->fork, b->main) != cudaSuccess) rc = EPH_ERR_CUDA;
  for (size_t r = 0; r < b->reps.size() && !rc; ++r) {
    eph_ctx *c = b->reps[r];
    if (cudaStreamWaitEvent(c->stream, b->fork, 0) != cudaSuccess) {
      rc = EPH_ERR_CUDA;
      break;
    }
    const long before = c->launches;
    rc = record_step(c, 0);
    launches += c->launches - before;
    c->launches = before;
    if (rc) {
      b->err = "replica " + std::to_string(r) + ": " + c->err;
      break;
    }
    if (cudaEventRecord(b->joins[r], c->stream) != cudaSuccess || cudaStreamWaitEvent(b->main, b->joins[r], 0) != cudaSuccess)
      rc = EPH_ERR_CUDA;
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->main, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (!rc) b->err = std::string("batch capture: ") + cudaGetErrorString(e);
    return rc ? rc : EPH_ERR_CUDA;
  }
  b->graph = g;
  if (cudaGraphInstantiate(&b->gexec, g, 0) != cudaSuccess) {
    b->err = "cannot instantiate the batch graph";
    return EPH_ERR_CUDA;
  }
  b->launches_per_step = launches;
  return EPH_OK;
}

int eph_batch_step(eph_batch *b, int nsteps) {
  if (!b || nsteps < 0) return EPH_ERR_ARG;
  int rc;
  if (!b->gexec && (rc = batch_capture(b))) return rc;
  for (int s = 0; s < nsteps; ++s) {
    if (cudaGraphLaunch(b->gexec, b->main) != cudaSuccess) {
      b->err = "graph launch failed";
      return EPH_ERR_CUDA;
    }
    for (eph_ctx *c : b->reps) {
      c->ntimestep += 1;
      if (c->args.T_freq > 0) {
        if (cudaStreamSynchronize(b->main) != cudaSuccess) return EPH_ERR_CUDA;
        if ((rc = write_T_output(c))) return rc;
      }
    }
  }
  return EPH_OK;
}

int eph_batch_synchronize(eph_batch *b) {
  if (!b) return EPH_ERR_ARG;
  if (cudaStreamSynchronize(b->main) != cudaSuccess) return EPH_ERR_CUDA;
  for (size_t r = 0; r < b->reps.size(); ++r) {
    const int rc = eph_synchronize(b->reps[r]);
    if (rc) {
      b->err = "replica " + std::to_string(r) + ": " + b->reps[r]->err;
      return rc;
    }
  }
  return EPH_OK;
}

int eph_batch_launch_count(eph_batch *b, long *per_step) {
  if (!b || !per_step) return EPH_ERR_ARG;
  *per_step = b->launches_per_step;
  return EPH_OK;
}

// ------------------------------------------------------ host-side helpers

struct eph_beta {
  Beta b;
};

int eph_beta_load(const char *path, eph_beta **out) {
  if (!path || !out) return EPH_ERR_ARG;
  eph_beta *b = new (std::nothrow) eph_beta();
  if (!b) return EPH_ERR_ARG;
  if (!b->b.load(path).empty()) {
    delete b;
    *out = nullptr;
    return EPH_ERR_FILE;
  }
  *out = b;
  return EPH_OK;
}

void eph_beta_free(eph_beta *b) { delete b; }

int eph_beta_info(const eph_beta *b, int *n_elements, double *r_cutoff, double *rho_cutoff) {
  if (!b) return EPH_ERR_ARG;
  if (n_elements) *n_elements = b->b.n_elements;
  if (r_cutoff) *r_cutoff = b->b.r_cutoff;
  if (rho_cutoff) *rho_cutoff = b->b.rho_cutoff;
  return EPH_OK;
}

double eph_beta_eval(const eph_beta *b, int which, int elem, double x) {
  if (!b || elem < 0 || elem >= b->b.n_elements) return NAN;
  return b->b.table(which, elem)(x);
}

long eph_beta_table(const eph_beta *b, int which, int elem, double *out) {
  if (!b || elem < 0 || elem >= b->b.n_elements) return -1;
  const Spline &s = b->b.table(which, elem);
  if (out) std::memcpy(out, s.c.data(), sizeof(double) * 4 * (size_t)s.n);
  return s.n;
}

int eph_beta_set_knots(eph_beta *b, int elem, const double *rho_knots, long n_rho, const double *beta_knots,
                       long n_beta) {
  if (!b || !rho_knots || !beta_knots) return EPH_ERR_ARG;
  return b->b.set_knots(elem, rho_knots, n_rho, beta_knots, n_beta).empty() ? EPH_OK : EPH_ERR_ARG;
}

int eph_beta_knot_gradient(const eph_beta *b, int elem, const double *g_rho_r_sq, const double *g_alpha,
                           double *g_rho, double *g_beta) {
  if (!b || elem < 0 || elem >= b->b.n_elements || !g_rho_r_sq || !g_alpha || !g_rho || !g_beta)
    return EPH_ERR_ARG;
  b->b.knot_gradient(elem, g_rho_r_sq, g_alpha, g_rho, g_beta);
  return EPH_OK;
}

int eph_set_beta_knots(eph_ctx *c, int elem, const double *rho_knots, long n_rho, const double *beta_knots,
                       long n_beta) {
  if (!c || !rho_knots || !beta_knots) return EPH_ERR_ARG;
  std::string e = c->beta.set_knots(elem, rho_knots, n_rho, beta_knots, n_beta);
  if (!e.empty()) return fail(c, EPH_ERR_ARG, e);
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // no kernel of the stream reads the tables meanwhile
  return upload_tables(c);
}

int eph_set_grid_constants(eph_ctx *c, double C_e, double kappa_e) {
  if (!c) return EPH_ERR_ARG;
  if (c->args.T_infile != "NULL")
    return fail(c, EPH_ERR_STATE, "the grid was read from a file: its cells keep their own C_e and kappa_e");
  if (!(C_e > 0) || !(kappa_e >= 0)) return fail(c, EPH_ERR_ARG, "C_e must be positive and kappa_e non-negative");
  Grid &g = c->grid;
  const size_t nc = (size_t)g.ntotal;
  c->args.C_e = C_e;
  c->args.kappa_e = kappa_e;
  g.C.assign(nc, C_e);
  g.kappa.assign(nc, kappa_e);
  std::vector<double> rc(nc);
  for (size_t i = 0; i < nc; ++i) rc[i] = g.rho[i] * g.C[i];
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  CUDA_TRY(c, cudaMemcpy(c->rhoC.p, rc.data(), nc * 8, cudaMemcpyHostToDevice));
  CUDA_TRY(c, upload_inverse(c, rc));
  CUDA_TRY(c, cudaMemcpy(c->kappa.p, g.kappa.data(), nc * 8, cudaMemcpyHostToDevice));
  drop_graph(c);  // the substep count may change
  set_time_params(c);
  return EPH_OK;
}

struct eph_grid {
  Grid g;
};

int eph_grid_create(long nx, long ny, long nz, const double *lo, const double *hi, double T_e, double C_e,
                    double rho_e, double kappa_e, eph_grid **out) {
  if (!out || !lo || !hi || nx < 1 || ny < 1 || nz < 1) return EPH_ERR_ARG;
  eph_grid *g = new (std::nothrow) eph_grid();
  if (!g) return EPH_ERR_ARG;
  g->g.create(nx, ny, nz, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], T_e, C_e, rho_e, kappa_e);
  *out = g;
  return EPH_OK;
}

int eph_grid_load(const char *path, eph_grid **out) {
  if (!path || !out) return EPH_ERR_ARG;
  eph_grid *g = new (std::nothrow) eph_grid();
  if (!g) return EPH_ERR_ARG;
  if (!g->g.load(path).empty()) {
    delete g;
    *out = nullptr;
    return EPH_ERR_FILE;
  }
  *out = g;
  return EPH_OK;
}

void eph_grid_free(eph_grid *g) { delete g; }
long eph_grid_ncells(const eph_grid *g) { return g ? g->g.ntotal : -1; }

unsigned eph_grid_substeps(const eph_grid *g, double dt, double *inner_dt) {
  if (!g) return 0;
  Grid t = g->g;
  t.dt = dt;
  double idt = 0;
  const unsigned s = t.substeps(&idt);
  if (inner_dt) *inner_dt = idt;
  return s;
}

int eph_grid_save_state(const eph_grid *g, const char *path) {
  if (!g || !path) return EPH_ERR_ARG;
  return g->g.save_state(path) ? EPH_ERR_FILE : EPH_OK;
}

int eph_grid_save_temperature(const eph_grid *g, const char *path, int n) {
  if (!g || !path) return EPH_ERR_ARG;
  return g->g.save_temperature(path, n) ? EPH_ERR_FILE : EPH_OK;
}

}  // extern "C"
