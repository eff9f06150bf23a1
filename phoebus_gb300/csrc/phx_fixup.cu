// phx_fixup.cu -- fixup::ConservedToPrimitiveFixup (fixup_c2p.cpp:170-353) and
// fixup::ApplyFloors (fixup.cpp:370-540), fluid parts.
//
// The c2p fixup replaces the primitives of a failed zone by the average of
// its non-failed face neighbours (or by near-zero floors) and recomputes its
// conserved variables.  It works in place like the reference: a failed zone
// only writes itself and reads neighbours weighted by their fail flags, so a
// failed neighbour contributes 0 * value whether it was already fixed or not
// (the result equals a pre-fixup snapshot whenever failed zones hold finite
// primitives, which con2prim guarantees).
//
// ApplyFloors injects the mass and energy the floors (and the MHD ceilings on
// b^2/rho, b^2/u) require, at rest in the normal-observer frame, re-inverts
// the zone with the robust con2prim (through the same warp-vote root find as
// k_c2p, so lanes of zones without floors just vote "done"), falls back to the
// floor state if that inversion fails, and applies the gamma / energy
// ceilings with the reference's velocity rescale.
#include "phx_kernels.cuh"

namespace phx {

// t runs over the interior zones.
template <bool MINK>
__device__ __forceinline__ void c2p_fixup_at(const Par &p, const BView &b, long long t) {
  const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1;
  const int i = b.ng + (int)(t % ni);
  const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
  const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
  const long long id = b.idx(k, j, i);
  if (b.fail[id] != 0.0) return;
  const long long vs = b.vs;
  const long long di = 1, dj = b.n1t, dk = (long long)b.n1t * b.n2t;
  const double *F = b.fail;
  double *P = b.prim;
  auto fixv = [&](int iv, double inv_mask_sum) {
    const double *q = P + iv * vs;
    double s = F[id - di] * q[id - di] + F[id + di] * q[id + di];
    if (b.ndim > 1) {
      s += F[id - dj] * q[id - dj] + F[id + dj] * q[id + dj];
      if (b.ndim == 3) s += F[id - dk] * q[id - dk] + F[id + dk] * q[id + dk];
    }
    return inv_mask_sum * s;
  };
  double num_valid = F[id - di] + F[id + di];
  if (b.ndim > 1) num_valid += F[id - dj] + F[id + dj];
  if (b.ndim == 3) num_valid += F[id - dk] + F[id + dk];
  double rho, u, vp[3];
  if (num_valid > 0.5 && !p.strategy_floors) {
    const double norm = 1.0 / num_valid;
    rho = fixv(PHX_PRHO, norm);
    for (int d = 0; d < 3; d++) vp[d] = fixv(PHX_PVEL + d, norm);
    u = fixv(PHX_PENG, norm);
    rho = rmax(rho, 100. * kSMALL);
    u = rmax(u, 100. * kSMALL);
  } else {
    rho = 100. * kSMALL;
    u = 100. * kSMALL;
    vp[0] = vp[1] = vp[2] = 0.;
  }
  Pt g{};
  if constexpr (!MINK) load_pt(b, 0, j, i, g);
  const double gamma_max = p.g0;
  double W = lorentz<MINK>(g, vp);
  if (W > gamma_max) {
    const double rescale = sqrt(gamma_max * gamma_max - 1.) / (W * W - 1.);
    for (int d = 0; d < 3; d++) vp[d] *= rescale;
    W = gamma_max;
  }
  const double T = eos_T_rho_sie(p, rho, ratio(u, rho));
  const double Pr = eos_P_rho_T(p, rho, T);
  const double g1 = ratio(eos_bmod_rho_T(p, rho, T), Pr);
  double bp[3] = {0.0, 0.0, 0.0};
  if (p.mhd)
    for (int d = 0; d < 3; d++) bp[d] = P[(PHX_PB + d) * vs + id];
  double D, tau, S[3], bc[3], sig[3];
  p2c<MINK>(rho, vp, bp, u, Pr, g1, g, MINK ? 1.0 : g.detgam, D, S, bc, tau, sig);
  P[PHX_PRHO * vs + id] = rho;
  for (int d = 0; d < 3; d++) P[(PHX_PVEL + d) * vs + id] = vp[d];
  P[PHX_PENG * vs + id] = u;
  P[PHX_PTMP * vs + id] = T;
  P[PHX_PPRS * vs + id] = Pr;
  P[PHX_PGM1 * vs + id] = g1;
  b.cons[PHX_CRHO * vs + id] = D;
  b.cons[PHX_CENG * vs + id] = tau;
  for (int d = 0; d < 3; d++) b.cons[(PHX_CMOM + d) * vs + id] = S[d];
  for (int d = 0; d < b.ndim; d++) b.cell_sig[d * vs + id] = sig[d];
}

template <bool MINK>
__global__ void __launch_bounds__(128) k_c2p_fixup(Par p, BView b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) c2p_fixup_at<MINK>(p, b, t);
}

void launch_c2p_fixup(const Par &p, const BView &b, cudaStream_t s) {
  if (!p.c2p_fixup) return;
  const long long n = (long long)b.nx1 * (b.ndim >= 2 ? b.nx2 : 1) * (b.ndim >= 3 ? b.nx3 : 1);
  const int T = 128;
  if (b.fmks)
    k_c2p_fixup<false><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(p, b, n);
  else
    k_c2p_fixup<true><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(p, b, n);
}

// ------------------------------------------------------------ floors
// Zone t of the index box r (valid: this lane owns a zone).  Every lane of a
// warp must call it together (the re-inversion's root find votes).  flag
// (optional, [N]): 1 where floors or ceilings acted, else 0 (the radiation
// part of ApplyFloors redoes the closure inversion there).
template <bool MINK>
__device__ __forceinline__ void floors_at(const Par &p, const BView &b, const Range3 &r, long long t, bool valid,
                                          DevStats *stats, unsigned int *err, double *flag = nullptr) {
  int k = 0, j = 0, i = 0;
  if (valid) {
    const int ni = r.ie - r.is + 1, nj = r.je - r.js + 1;
    i = r.is + (int)(t % ni);
    const long long q = t / ni;
    j = r.js + (int)(q % nj);
    k = r.ks + (int)(q / nj);
  }
  const long long id = b.idx(k, j, i);
  const long long vs = b.vs;
  Pt g{};
  if constexpr (!MINK) {
    if (valid) load_pt(b, 0, j, i, g);
  }
  double pr[PHX_NPRIM], U[PHX_NCONS];
  bool floor_applied = false;
  double drho = 0.0, du = 0.0, dprs = 0.0, dgm1 = 0.0, bp[3] = {0.0, 0.0, 0.0};
  double x1 = 0.0, x2 = 0.0, x3 = 0.0;
  if (valid) {
    for (int v = 0; v < PHX_NPRIM; v++) pr[v] = b.prim[v * vs + id];
    for (int m = 0; m < PHX_NCONS; m++) U[m] = b.cons[m * vs + id];
    x1 = b.Xc(0, i);
    x2 = b.Xc(1, j);
    x3 = b.Xc(2, k);
    double rho_floor, sie_floor;
    get_floors(p, x1, x2, x3, rho_floor, sie_floor);
    const double e_max = p.smax0;
    double rho_floor_max = rho_floor;
    double u_floor_max = rho_floor * sie_floor;
    if (p.enable_mhd_floors) {
      const double vp[3] = {pr[PHX_PVEL], pr[PHX_PVEL + 1], pr[PHX_PVEL + 2]};
      const double bb[3] = {pr[PHX_PB], pr[PHX_PB + 1], pr[PHX_PB + 2]};
      const double W = lorentz<MINK>(g, vp);
      const double iW = rcp_p(W);
      double Bsq, Bdotv;
      if constexpr (MINK) {
        Bsq = bb[0] * bb[0] + bb[1] * bb[1] + bb[2] * bb[2];
        Bdotv = bb[0] * vp[0] + bb[1] * vp[1] + bb[2] * vp[2];
      } else {
        Bsq = 0.0;
        Bdotv = 0.0;
        for (int ii = 0; ii < 3; ii++)
          for (int jj = 0; jj < 3; jj++) {
            Bsq += g.gcov[ii + 1][jj + 1] * bb[ii] * bb[jj];
            Bdotv += g.gcov[ii + 1][jj + 1] * bb[ii] * vp[jj];
          }
      }
      const double alpha = MINK ? 1.0 : g.alpha;
      const double bcon0 = div_p(W * Bdotv, alpha);
      const double bsq = (Bsq + alpha * alpha * bcon0 * bcon0) * iW * iW;
      rho_floor_max = rmax(rho_floor_max, div_p(bsq, p.bsqorho0));
      u_floor_max = rmax(u_floor_max, div_p(bsq, p.bsqou0));
      rho_floor_max = rmax(rho_floor_max, div_p(rmax(pr[PHX_PENG], u_floor_max), e_max));
    }
    drho = rho_floor_max - pr[PHX_PRHO];
    du = u_floor_max - pr[PHX_PENG];
    if (drho > 0. || du > 0.) {
      floor_applied = true;
      drho = rmax(drho, du / sie_floor);
      du = rmax(du, sie_floor * drho);
    }
    if (p.mhd)
      for (int d = 0; d < 3; d++) bp[d] = pr[PHX_PB + d];
    if (floor_applied) {
      const double vz[3] = {0.0, 0.0, 0.0};
      dprs = eos_P_rho_sie(p, drho, ratio(du, drho));
      dgm1 = ratio(fmax(0.0, (p.gm1 + 1) * p.gm1 * drho * ratio(du, drho)), dprs);
      double dcrho, dS[3], dB[3], dtau;
      p2c<MINK>(drho, vz, bp, du, dprs, dgm1, g, MINK ? 1.0 : g.detgam, dcrho, dS, dB, dtau, nullptr);
      U[PHX_CRHO] += dcrho;
      for (int d = 0; d < 3; d++) U[PHX_CMOM + d] += dS[d];
      U[PHX_CENG] += dtau;
    }
  }
  // re-inversion of the floored zones (con2prim_robust.hpp:299-453)
  Residual res;
  double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0;
  bool setup_ok = false;
  if (valid && floor_applied) setup_ok = c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
  C2POut out{0, 0, false, true, false};
  const double mu = regula_falsi_warp(p, res, setup_ok, 0.0, 1.0, valid ? pr[PHX_PMU] : 0.0, out);
  if (!valid) return;
  if (floor_applied) {
    bool success = false;
    if (setup_ok) {
      double sig[3];
      bool used_bounds;
      double np[PHX_NPRIM];
      c2p_finish<MINK>(p, g, res, mu, rcon, bu, Bprim, bdotr, np, U, sig, used_bounds);
      for (int v = 0; v < PHX_NPRIM; v++) {
        if (v >= PHX_PB && v < PHX_PB + 3 && !p.mhd) continue;
        pr[v] = np[v];
      }
      for (int d = 0; d < b.ndim; d++) b.cell_sig[d * vs + id] = sig[d];
      const int num_nans = isnan(U[PHX_CRHO]) + isnan(U[PHX_CMOM]) + isnan(U[PHX_CENG]);
      success = out.bracketed && num_nans == 0;
      if (p.fail_on_floors && (res.used_density_floor || res.used_energy_floor)) success = false;
      if (p.fail_on_ceilings && res.used_gamma_max) success = false;
      if (!out.bracketed) atomicOr(err, ERR_UNBRACKETED);
    }
    if (stats && !success) atomicAdd(&stats->failures, 1ull);
    if (!success) {
      const double vz[3] = {0.0, 0.0, 0.0};
      pr[PHX_PRHO] = drho;
      for (int d = 0; d < 3; d++) pr[PHX_PVEL + d] = 0.0;
      pr[PHX_PENG] = du;
      pr[PHX_PTMP] = eos_T_rho_sie(p, pr[PHX_PRHO], pr[PHX_PENG] / pr[PHX_PRHO]);
      double Dn, taun, dS[3], dB[3];
      p2c<MINK>(drho, vz, bp, du, dprs, dgm1, g, MINK ? 1.0 : g.detgam, Dn, dS, dB, taun, nullptr);
      U[PHX_CRHO] = Dn;
      U[PHX_CENG] = taun;
      for (int d = 0; d < 3; d++) U[PHX_CMOM + d] = dS[d];
    }
  }
  const double gamma_max = p.g0, e_max = p.smax0;
  double vpcon[3] = {pr[PHX_PVEL], pr[PHX_PVEL + 1], pr[PHX_PVEL + 2]};
  const double W = lorentz<MINK>(g, vpcon);
  const bool ceiling_applied = (W > gamma_max || div_p(pr[PHX_PENG], pr[PHX_PRHO]) > e_max);
  if (ceiling_applied) {
    const double rescale = sqrt(gamma_max * gamma_max - 1.) / (W * W - 1.);
    for (int d = 0; d < 3; d++) {
      vpcon[d] *= rescale;
      pr[PHX_PVEL + d] = vpcon[d];
    }
    double Dn, taun, dS[3], dB[3];
    p2c<MINK>(pr[PHX_PRHO], vpcon, bp, pr[PHX_PENG], pr[PHX_PPRS], pr[PHX_PGM1], g, MINK ? 1.0 : g.detgam, Dn, dS,
              dB, taun, nullptr);
    U[PHX_CRHO] = Dn;
    U[PHX_CENG] = taun;
    for (int d = 0; d < 3; d++) U[PHX_CMOM + d] = dS[d];
  }
  if (flag) flag[id] = (floor_applied || ceiling_applied) ? 1.0 : 0.0;
  if (floor_applied || ceiling_applied) {
    pr[PHX_PTMP] = eos_T_rho_sie(p, pr[PHX_PRHO], ratio(pr[PHX_PENG], pr[PHX_PRHO]));
    pr[PHX_PPRS] = eos_P_rho_T(p, pr[PHX_PRHO], pr[PHX_PTMP]);
    pr[PHX_PGM1] = ratio(eos_bmod_rho_T(p, pr[PHX_PRHO], pr[PHX_PTMP]), pr[PHX_PPRS]);
    for (int v = 0; v < PHX_NPRIM; v++) {
      if (v >= PHX_PB && v < PHX_PB + 3 && !p.mhd) continue;
      b.prim[v * vs + id] = pr[v];
    }
    for (int m = 0; m < 5; m++) b.cons[m * vs + id] = U[m];
  }
}

template <bool MINK>
__global__ void __launch_bounds__(128) k_floors(Par p, BView b, Range3 r, long long ntot, DevStats *stats,
                                                unsigned int *err, double *flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  floors_at<MINK>(p, b, r, t, t < ntot, stats, err, flag);
}

void launch_floors(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err, cudaStream_t s,
                   double *flag) {
  if (!p.enable_floors) return;
  const long long n = (long long)(r.ie - r.is + 1) * (r.je - r.js + 1) * (r.ke - r.ks + 1);
  if (n <= 0) return;
  const int T = 128;
  if (b.fmks)
    k_floors<false><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(p, b, r, n, stats, err, flag);
  else
    k_floors<true><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(p, b, r, n, stats, err, flag);
}

// ------------------------------------------------------------- batched
template <bool MINK>
__global__ void __launch_bounds__(128) kb_c2p_fixup(Par p, const BView *views, const WorkItem *items, int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) c2p_fixup_at<MINK>(p, views[w.block], t);
  }
}
template <bool MINK>
__global__ void __launch_bounds__(128) kb_floors(Par p, const BView *views, const WorkItem *items, int nitems,
                                                 DevStats *stats, unsigned int *err) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const BView &b = views[w.block];
    const Range3 r{0, b.n1t - 1, 0, b.n2t - 1, 0, b.n3t - 1};
    const long long t = w.first + threadIdx.x;
    floors_at<MINK>(p, b, r, t, t < w.last, stats, err);
  }
}

void launch_c2p_fixup_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems,
                              cudaStream_t s) {
  if (!p.c2p_fixup || nitems <= 0) return;
  if (mink)
    kb_c2p_fixup<true><<<persistent_grid(kb_c2p_fixup<true>, 128, 0, nitems, 0), 128, 0, s>>>(p, views, items, nitems);
  else
    kb_c2p_fixup<false><<<persistent_grid(kb_c2p_fixup<false>, 128, 0, nitems, 0), 128, 0, s>>>(p, views, items,
                                                                                                 nitems);
}
void launch_floors_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems,
                           DevStats *stats, unsigned int *err, cudaStream_t s) {
  if (!p.enable_floors || nitems <= 0) return;
  if (mink)
    kb_floors<true><<<persistent_grid(kb_floors<true>, 128, 0, nitems, 0), 128, 0, s>>>(p, views, items, nitems,
                                                                                         stats, err);
  else
    kb_floors<false><<<persistent_grid(kb_floors<false>, 128, 0, nitems, 0), 128, 0, s>>>(p, views, items, nitems,
                                                                                           stats, err);
}

}  // namespace phx
