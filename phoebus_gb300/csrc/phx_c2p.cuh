// phx_c2p.cuh -- robust con2prim for one zone on the device
// (con2prim_robust.hpp:46-453, root_find.hpp:27-167).
//
// The regula-falsi loop is warp-synchronous: every lane stays in the loop
// until the warp's vote (__any_sync) says no lane is still iterating, so all
// 32 lanes re-enter each iteration together and reconverge after it.
// In the production build the residual's divisions use the Newton-refined
// hardware reciprocal (rcp_p / ratio_p); the exact build divides as the
// reference does.
#pragma once
#include "phx_device.cuh"

namespace phx {

struct Residual {
  double D, q, bsq, bsq_rpsq, rsq, rbsq, v0sq;
  FloorPt fl;  // floor_point of the zone: every evaluation's floors come from it
  double rho_floor, gam_max, e_max;
  bool used_density_floor, used_energy_floor, used_energy_max, used_gamma_max;

  __device__ __forceinline__ void init(const Par &p) {
    double garbage = 0.0;
    rho_floor = 0.0;
    floors_from(p, fl, rho_floor, garbage);
    gam_max = p.g0;
    e_max = p.smax0;
    rho_floor *= p.fsf;
    used_density_floor = used_energy_floor = used_energy_max = used_gamma_max = false;
  }
  __device__ __forceinline__ double x_mu(double mu) const { return ratio_p(1.0, 1.0 + mu * bsq); }
  __device__ __forceinline__ double rbarsq_mu(double mu, double x) const {
    return x * (x * rsq + mu * (1.0 + x) * rbsq);
  }
  __device__ __forceinline__ double qbar_mu(double mu, double x) const {
    const double mux = mu * x;
    return q - 0.5 * (bsq + mux * mux * bsq_rpsq);
  }
  __device__ __forceinline__ double vhatsq_mu(double mu, double rbarsq) {
    const double vsq_trial = mu * mu * rbarsq;
    if (vsq_trial > v0sq) {
      used_gamma_max = true;
      return v0sq;
    }
    used_gamma_max = false;
    return vsq_trial;
  }
  __device__ __forceinline__ double iWhat_mu(double vhatsq) const { return sqrt(1.0 - vhatsq); }
  __device__ __forceinline__ double rhohat_mu(double iWhat) {
    const double rho_trial = D * iWhat;
    if (rho_trial <= rho_floor) {
      used_density_floor = true;
      return rho_floor;
    }
    used_density_floor = false;
    return rho_trial;
  }
  __device__ __forceinline__ double ehat_mu(const Par &p, double mu, double qbar, double rbarsq,
                                            double vhatsq, double What) {
    double rho = rhohat_mu(ratio_p(1.0, What));
    double e_floor;
    floors_from(p, fl, rho, e_floor);
    e_floor *= p.fsf;
    const double ehat_trial = What * (qbar - mu * rbarsq) + vhatsq * What * ratio_p(What, 1.0 + What);
    used_energy_floor = false;
    used_energy_max = false;
    if (ehat_trial <= e_floor) {
      used_energy_floor = true;
      return e_floor;
    } else if (ehat_trial > e_max) {
      used_energy_max = true;
      return e_max;
    }
    return ehat_trial;
  }
  // ehat_mu with the density from a known 1/W (production build)
  __device__ __forceinline__ double ehat_mu_iw(const Par &p, double mu, double qbar, double rbarsq, double vhatsq,
                                               double What, double iWhat) {
    double rho = rhohat_mu(iWhat);
    double e_floor;
    floors_from(p, fl, rho, e_floor);
    e_floor *= p.fsf;
    // What = 1 / sqrt(1 - vhatsq): vhatsq What^2 / (1 + What) = What - 1
    const double ehat_trial = fma(What, qbar - mu * rbarsq, What - 1.0);
    used_energy_floor = false;
    used_energy_max = false;
    if (ehat_trial <= e_floor) {
      used_energy_floor = true;
      return e_floor;
    } else if (ehat_trial > e_max) {
      used_energy_max = true;
      return e_max;
    }
    return ehat_trial;
  }
  __device__ __forceinline__ double operator()(const Par &p, double mu) {
    const double x = x_mu(mu);
    const double rbarsq = rbarsq_mu(mu, x);
    const double qbar = qbar_mu(mu, x);
    const double vhatsq = vhatsq_mu(mu, rbarsq);
#ifdef PHX_EXACT
    const double iWhat = iWhat_mu(vhatsq);
    const double What = ratio_p(1.0, iWhat);
    const double rhohat = rhohat_mu(iWhat);
    const double ehat = ehat_mu(p, mu, qbar, rbarsq, vhatsq, What);
#else
    // production build: W and 1/W from one rsqrt; the density inside ehat
    // reuses 1/W instead of inverting W again
    const double What = rsqrt_p(1.0 - vhatsq);
    const double iWhat = (1.0 - vhatsq) * What;
    const double rhohat = rhohat_mu(iWhat);
    const double ehat = ehat_mu_iw(p, mu, qbar, rbarsq, vhatsq, What, iWhat);
#endif
    const double Phat = eos_P_rho_sie(p, rhohat, ehat);
    const double hhat = rhohat * (1.0 + ehat) + Phat;
    // Both builds keep the reference's two reciprocals: muhat = 1 / (nuhat +
    // mu rbarsq) with nuhat >= 1 stays <= 1 under rounding, so f(1) >= 0 holds
    // where the root sits at the end of [0, 1] (cold gas); a single merged
    // reciprocal den / (c M + ...) loses that and can leave the root unbracketed.
    const double ahat = div_p(Phat, make_positive(hhat - Phat));
    const double nua = (1.0 + ahat) * (1.0 + ehat) * iWhat;
    const double nub = (1.0 + ahat) * (1.0 + qbar - mu * rbarsq);
    const double nuhat = rmax(nua, nub);
    const double muhat = rcp_p(nuhat + mu * rbarsq);
    return mu - muhat;
  }
  __device__ __forceinline__ bool used_bounds() const {
    return used_density_floor || used_energy_floor || used_energy_max || used_gamma_max;
  }
};

// Outcome of one zone (written back by the caller).
struct C2POut {
  int iterations;
  int evals;
  bool success;
  bool bracketed;
  bool nan_input;
  bool learned;  // the learned start was accepted
};

// Setup of the inversion (con2prim_robust.hpp:303-366).  Returns false when
// the input is NaN (the reference returns failure before touching prims).
template <bool MINK>
__device__ __forceinline__ bool c2p_setup(const Par &p, const Pt &g, const double U[PHX_NCONS],
                                          double x1, double x2, double x3, Residual &res,
                                          double rcon[3], double rcov[3], double bu[3],
                                          double Bprim[3], double &bdotr) {
  const int num_nans = isnan(U[PHX_CRHO]) + isnan(U[PHX_CMOM]) + isnan(U[PHX_CENG]);
  if (num_nans > 0) return false;
  const double gdet = MINK ? 1.0 : g.detgam;
  const double igdet = MINK ? 1.0 : rcp_p(gdet);  // 1 / 1 = 1 in both builds
  double rhoflr = 0.0, epsflr;
  const FloorPt fl = floor_point(p, x1, x2, x3);
  floors_from(p, fl, rhoflr, epsflr);
  rhoflr *= p.fsf;
  const double gam_max = p.g0;
  const double D = U[PHX_CRHO] * igdet;
  const double tau = U[PHX_CENG] * igdet;
  double bsq = 0.0, bsq_rpsq = 0.0, rbsq = 0.0, rsq;
  bdotr = 0.0;
#ifdef PHX_EXACT
  const double q = ratio_p(tau, D);
  rcov[0] = ratio(U[PHX_CMOM], U[PHX_CRHO]);
  rcov[1] = ratio(U[PHX_CMOM + 1], U[PHX_CRHO]);
  rcov[2] = ratio(U[PHX_CMOM + 2], U[PHX_CRHO]);
#else
  // tau / D = U_tau / U_D: one reciprocal serves q and the three r_i
  const double ic = ratio_p(1.0, U[PHX_CRHO]);
  const double q = U[PHX_CENG] * ic;
  rcov[0] = U[PHX_CMOM] * ic;
  rcov[1] = U[PHX_CMOM + 1] * ic;
  rcov[2] = U[PHX_CMOM + 2] * ic;
#endif
  if constexpr (MINK) {
    rcon[0] = rcov[0];
    rcon[1] = rcov[1];
    rcon[2] = rcov[2];
    rsq = rcon[0] * rcov[0] + rcon[1] * rcov[1] + rcon[2] * rcov[2];
  } else {
    rsq = 0.0;
#pragma unroll
    for (int ii = 0; ii < 3; ii++) {
      rcon[ii] = 0.0;
#pragma unroll
      for (int jj = 0; jj < 3; jj++) rcon[ii] += g.gamcon[ii][jj] * rcov[jj];
      rsq += rcon[ii] * rcov[ii];
    }
  }
  bu[0] = bu[1] = bu[2] = 0.0;
  if (p.mhd) {
#pragma unroll
    for (int ii = 0; ii < 3; ii++) Bprim[ii] = U[PHX_CB + ii] * igdet;
#ifdef PHX_EXACT
    const double sD = rcp_p(sqrt(rmax(D, rhoflr)));
#else
    const double sD = rsqrt_p(rmax(D, rhoflr));
#endif
#pragma unroll
    for (int ii = 0; ii < 3; ii++) {
      bu[ii] = Bprim[ii] * sD;
      bdotr += bu[ii] * rcov[ii];
    }
    bsq = dot_sp<MINK>(g, bu, bu);
    bsq = fmax(0.0, bsq);
    rbsq = bdotr * bdotr;
    bsq_rpsq = bsq * rsq - rbsq;
  }
  const double zsq = rsq / 1.0;  // h0sq_ = 1
#ifdef PHX_EXACT
  const double v0sq = rmin(div_p(zsq, 1.0 + zsq), 1.0 - rcp_p(gam_max * gam_max));
#else
  const double v0sq = rmin(div_p(zsq, 1.0 + zsq), p.vsq_max);  // 1 - 1 / gam_max^2, formed on the host
#endif
  res.D = D;
  res.q = q;
  res.bsq = bsq;
  res.bsq_rpsq = bsq_rpsq;
  res.rsq = rsq;
  res.rbsq = rbsq;
  res.v0sq = v0sq;
  res.fl = fl;
  res.init(p);
  return true;
}

// Inputs of the learned con2prim start (no reference counterpart): scale-free
// invariants of the inversion from the setup quantities, mapped to O(1) in
// FP32: log10 q / 4, log10 r^2 / 4, log10 b^2 / 4, (b.r)^2 / (b^2 r^2),
// v0^2, log10 D / 8 (log10 arguments bounded below by 1e-12, 1e-30).
__device__ __forceinline__ void c2p_features(const Residual &r, float f[6]) {
  f[0] = log10f((float)fmax(r.q, 1e-12)) * 0.25f;
  f[1] = log10f((float)fmax(r.rsq, 1e-12)) * 0.25f;
  f[2] = log10f((float)fmax(r.bsq, 1e-12)) * 0.25f;
  f[3] = (float)r.rbsq / fmaxf((float)r.bsq * (float)r.rsq, 1e-30f);
  f[4] = (float)r.v0sq;
  f[5] = log10f((float)fmax(r.D, 1e-30)) * 0.125f;
}

// The same six invariants for inference, in FP32 arithmetic from the
// conserved variables and the metric (GB300 issues FP32 at 64x its FP64 rate;
// the invariants agree with c2p_setup's FP64 ones to FP32 rounding, far
// below the network's own error).  Returns false for NaN input, as
// c2p_setup does.
template <bool MINK>
__device__ __forceinline__ bool c2p_features_fp32(const Par &p, const Pt &g, const double U[PHX_NCONS], double x1,
                                                  double x2, double x3, float f[6]) {
  if (isnan(U[PHX_CRHO]) || isnan(U[PHX_CMOM]) || isnan(U[PHX_CENG])) return false;
  double rhoflr_d = 0.0, epsflr;
  get_floors(p, x1, x2, x3, rhoflr_d, epsflr);
  const float rhoflr = (float)(rhoflr_d * p.fsf);
  const float igdet = MINK ? 1.0f : 1.0f / (float)g.detgam;
  const float D = (float)U[PHX_CRHO] * igdet;
  const float q = (float)U[PHX_CENG] * igdet / D;
  const float ic = 1.0f / (float)U[PHX_CRHO];
  float rcov[3], rcon[3];
#pragma unroll
  for (int ii = 0; ii < 3; ii++) rcov[ii] = (float)U[PHX_CMOM + ii] * ic;
  float rsq = 0.0f;
#pragma unroll
  for (int ii = 0; ii < 3; ii++) {
    if constexpr (MINK) {
      rcon[ii] = rcov[ii];
    } else {
      rcon[ii] = 0.0f;
#pragma unroll
      for (int jj = 0; jj < 3; jj++) rcon[ii] += (float)g.gamcon[ii][jj] * rcov[jj];
    }
    rsq += rcon[ii] * rcov[ii];
  }
  float bsq = 0.0f, rbsq = 0.0f;
  if (p.mhd) {
    const float sD = rsqrtf(fmaxf(D, rhoflr));
    float bu[3], bdotr = 0.0f;
#pragma unroll
    for (int ii = 0; ii < 3; ii++) {
      bu[ii] = (float)U[PHX_CB + ii] * igdet * sD;
      bdotr += bu[ii] * rcov[ii];
    }
#pragma unroll
    for (int m = 0; m < 3; m++)
#pragma unroll
      for (int n = 0; n < 3; n++) bsq += (MINK ? (m == n ? 1.0f : 0.0f) : (float)g.gcov[m + 1][n + 1]) * bu[m] * bu[n];
    bsq = fmaxf(0.0f, bsq);
    rbsq = bdotr * bdotr;
  }
  const float v0sq = fminf(rsq / (1.0f + rsq), (float)p.vsq_max);
  f[0] = log10f(fmaxf(q, 1e-12f)) * 0.25f;
  f[1] = log10f(fmaxf(rsq, 1e-12f)) * 0.25f;
  f[2] = log10f(fmaxf(bsq, 1e-12f)) * 0.25f;
  f[3] = rbsq / fmaxf(bsq * rsq, 1e-30f);
  f[4] = v0sq;
  f[5] = log10f(fmaxf(D, 1e-30f)) * 0.125f;
  return true;
}

// State of one zone's regula falsi (root_find.hpp:110-167) between
// iterations: the bracket [a, b] with sign-normalised end values, the Illinois
// counters, and the tallies.  Saving and restoring it resumes the same
// sequence of operations.
struct RFState {
  double a, b, ya, yb, sign;
  int it, evals, b1, b2;
  bool bracketed, learned;
};

// Start: refine_bracket + check_bracket (root_find.hpp:42-58, 110-119) from
// [a, b] and guess.  LEARNED: lb = (m, lo, hi), a predicted root and bracket
// in [0, 1]; f(m) picks the half that should hold the root (f < 0 below it,
// > 0 above), one more evaluation checks that half's sign change; when it
// holds, the iterations start from that half, otherwise from the reference's
// own start.  The learned start is only tried for a cold zone (guess = 0, no
// previous solution): a previous mu is the better start (measured: about 1.5
// iterations from it).  A bracket that is not ordered inside [0, 1] (e.g.
// NaN) is not tried.
template <bool LEARNED>
__device__ __forceinline__ void rf_start(const Par &p, Residual &res, bool valid, double a, double b, double guess,
                                         const double *lb, RFState &s) {
  double ya = 0.0, yb = 0.0;
  int evals = 0;
  bool bracketed = true;
  bool started = false;
  s.learned = false;
  if constexpr (LEARNED) {
    if (valid && !(guess > 0.0) && lb[1] >= 0.0 && lb[1] <= lb[0] && lb[0] <= lb[2] && lb[2] <= 1.0) {
      double la, lbb, lya, lyb;
      const double ym = res(p, lb[0]);
      if (ym > 0.0) {
        la = lb[1];
        lbb = lb[0];
        lyb = ym;
        lya = res(p, la);
      } else {
        la = lb[0];
        lbb = lb[2];
        lya = ym;
        lyb = res(p, lbb);
      }
      evals += 2;
      if (lya * lyb <= 0.0) {
        a = la;
        b = lbb;
        ya = lya;
        yb = lyb;
        started = true;
        s.learned = true;
      }
    }
  }
  if (valid && !started) {
    if (a <= guess && b >= guess) {
      ya = res(p, guess);
      yb = res(p, b);
      evals += 2;
      if (ya * yb > 0.0) {
        yb = ya;
        b = guess;
        ya = res(p, a);
        evals++;
      } else {
        a = guess;
      }
    } else {
      ya = res(p, a);
      yb = res(p, b);
      evals += 2;
    }
    bracketed = !(ya * yb > 0.0);
  }
  s.sign = (ya < 0 ? 1.0 : -1.0);
  s.a = a;
  s.b = b;
  s.ya = ya * s.sign;
  s.yb = yb * s.sign;
  s.it = 0;
  s.b1 = s.b2 = 0;
  s.evals = evals;
  s.bracketed = bracketed;
}

// True while the zone still iterates (root_find.hpp:120 loop condition).
__device__ __forceinline__ bool rf_running(const Par &p, const RFState &s) {
  return s.bracketed && (s.b - s.a > 2.0 * p.c2p_tol) && (s.it < p.c2p_max_iter);
}

// The Illinois iterations (root_find.hpp:120-166), warp-synchronous: every
// lane stays in the loop until the warp's vote says none is still
// iterating.  A lane stops after cap iterations in total even if it has not
// converged (rf_running stays true: the caller resumes it later).  WARP =
// false: the lane loops on its own (for callers whose lanes may have left;
// the arithmetic is the same).
template <bool WARP = true>
__device__ __forceinline__ void rf_iterate(const Par &p, Residual &res, bool valid, RFState &s, int cap) {
  const double tol = p.c2p_tol;
  const int max_iter = p.c2p_max_iter;
  double a = s.a, b = s.b, ya = s.ya, yb = s.yb;
  const double sign = s.sign;
  int it = s.it, b1 = s.b1, b2 = s.b2, evals = s.evals;
  bool active = valid && s.bracketed && (b - a > 2.0 * tol) && (it < max_iter) && (it < cap);
  while (WARP ? __any_sync(0xffffffffu, active) : active) {
    if (active) {
      const double c = div_p(a * yb - b * ya, yb - ya);
      if (c == a) {
        b = a;
      } else if (c == b) {
        a = b;
      } else {
        const double yc = sign * res(p, c);
        evals++;
        if (yc > 0.0) {
          b = c;
          yb = yc;
          b1++;
          ya *= (b1 > 1 ? 0.5 : 1.0);
          b2 = 0;
        } else if (yc < 0.0) {
          a = c;
          ya = yc;
          b2++;
          yb *= (b2 > 1 ? 0.5 : 1.0);
          b1 = 0;
        } else {
          a = c;
          b = c;
        }
      }
      it++;
      active = (b - a > 2.0 * tol) && (it < max_iter) && (it < cap);
    }
  }
  s.a = a;
  s.b = b;
  s.ya = ya;
  s.yb = yb;
  s.it = it;
  s.b1 = b1;
  s.b2 = b2;
  s.evals = evals;
}

__device__ __forceinline__ double rf_result(const RFState &s, double guess, C2POut &out) {
  out.iterations = s.it;
  out.evals = s.evals;
  out.bracketed = s.bracketed;
  out.learned = s.learned;
  if (!s.bracketed) return guess;
  return 0.5 * (s.a + s.b);
}

// refine_bracket + regula_falsi (root_find.hpp:42-58, 110-167) in one call.
// valid = this lane owns a zone.  Returns mu; iterations/evals/bracketed
// through out.  a/b: starting bracket ([0, 1] in the reference).
template <bool LEARNED = false>
__device__ __forceinline__ double regula_falsi_warp(const Par &p, Residual &res, bool valid, double a, double b,
                                                   double guess, C2POut &out, const double *lb = nullptr) {
  RFState s;
  rf_start<LEARNED>(p, res, valid, a, b, guess, lb, s);
  rf_iterate(p, res, valid, s, p.c2p_max_iter);
  return rf_result(s, guess, out);
}

// Unwrap mu into primitives (con2prim_robust.hpp:381-452).
// prim[] receives PHX_NPRIM values (B slots only when mhd), U[] may be
// rewritten by p2c when bounds were used; sig[3] receives signal speeds.
template <bool MINK>
__device__ __forceinline__ void c2p_finish(const Par &p, const Pt &g, Residual &res, double mu,
                                           const double rcon[3], const double bu_in[3],
                                           const double Bprim[3], double bdotr,
                                           double prim[PHX_NPRIM], double U[PHX_NCONS],
                                           double sig[3], bool &used_bounds_out) {
  prim[PHX_PMU] = mu;
  const double x = res.x_mu(mu);
  const double rbarsq = res.rbarsq_mu(mu, x);
  const double vsq = res.vhatsq_mu(mu, rbarsq);
#ifdef PHX_EXACT
  const double iW = res.iWhat_mu(vsq);
  const double W = rcp_p(iW);
#else
  // W and 1/W from one reciprocal square root, as in the residual
  const double W = rsqrt_p(1.0 - vsq);
  const double iW = (1.0 - vsq) * W;
#endif
  prim[PHX_PRHO] = res.rhohat_mu(iW);
  const double qbar = res.qbar_mu(mu, x);
#ifdef PHX_EXACT
  double eng = res.ehat_mu(p, mu, qbar, rbarsq, vsq, W);
#else
  double eng = res.ehat_mu_iw(p, mu, qbar, rbarsq, vsq, W, iW);  // 1/W known
#endif
  prim[PHX_PTMP] = eos_T_rho_sie(p, prim[PHX_PRHO], eng);
  eng *= prim[PHX_PRHO];
  prim[PHX_PENG] = eng;
  prim[PHX_PPRS] = eos_P_rho_T(p, prim[PHX_PRHO], prim[PHX_PTMP]);
#ifdef PHX_EXACT
  prim[PHX_PGM1] = div_p(eos_bmod_rho_T(p, prim[PHX_PRHO], prim[PHX_PTMP]), prim[PHX_PPRS]);
#else
  // production build: bmod / P of the ideal gas is Gamma wherever P > 0 (the
  // quotient, NaN for P = 0, elsewhere)
  prim[PHX_PGM1] = prim[PHX_PPRS] > 0.0
                       ? p.gm1 + 1.0
                       : div_p(eos_bmod_rho_T(p, prim[PHX_PRHO], prim[PHX_PTMP]), prim[PHX_PPRS]);
#endif
  double vel[3];
#pragma unroll
  for (int ii = 0; ii < 3; ii++) {
    vel[ii] = W * mu * x * (rcon[ii] + mu * bdotr * bu_in[ii]);
    prim[PHX_PVEL + ii] = vel[ii];
  }
  double bu[3] = {0.0, 0.0, 0.0};
  if (p.mhd) {
#pragma unroll
    for (int ii = 0; ii < 3; ii++) {
      prim[PHX_PB + ii] = Bprim[ii];
      bu[ii] = Bprim[ii];
    }
  }
  used_bounds_out = res.used_bounds();
  if (used_bounds_out) {
    double S[3], bcons[3], Dn, taun;
    const double gdet = MINK ? 1.0 : g.detgam;
    p2c<MINK>(prim[PHX_PRHO], vel, bu, prim[PHX_PENG], prim[PHX_PPRS], prim[PHX_PGM1], g, gdet,
              Dn, S, bcons, taun, sig);
    U[PHX_CRHO] = Dn;
    U[PHX_CENG] = taun;
#pragma unroll
    for (int ii = 0; ii < 3; ii++) U[PHX_CMOM + ii] = S[ii];
  } else {
#pragma unroll
    for (int m = 0; m < 3; m++) vel[m] *= iW;
    double bsq = 0.0;
    if (p.mhd) {
      double bdotv;
      if constexpr (MINK) {
        bsq = bu[0] * bu[0] + bu[1] * bu[1] + bu[2] * bu[2];
        bdotv = bu[0] * vel[0] + bu[1] * vel[1] + bu[2] * vel[2];
      } else {
#ifdef PHX_EXACT
        bdotv = 0.0;
#pragma unroll
        for (int m = 0; m < 3; m++)
#pragma unroll
          for (int n = 0; n < 3; n++) {
            bsq += bu[m] * bu[n] * g.gcov[m + 1][n + 1];
            bdotv += bu[m] * vel[n] * g.gcov[m + 1][n + 1];
          }
#else
        double blo[3];  // lowered B serves both contractions
        lower_sp(g, bu, blo);
        bsq = dot3(bu, blo);
        bdotv = dot3(vel, blo);
#endif
      }
      bsq = iW * iW * bsq + bdotv * bdotv;
    }
    signal_speeds<MINK>(prim[PHX_PRHO], prim[PHX_PENG], prim[PHX_PPRS], bsq, vel, vsq,
                        prim[PHX_PGM1], g, sig);
  }
}

}  // namespace phx
