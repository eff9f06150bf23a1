// phx_fmks.cuh -- the FMKS coordinate system on the device:
// Modified<SphericalKerrSchild, McKinneyGammieRyan> (fmks.hpp:44) at a point.
//
// exp, sin, cos and pow are phx_math.h's; the translation units that include
// this header are compiled without contraction in both library builds, so a
// point evaluation here equals the oracle's bit for bit.
#pragma once
#include "phx_kernels.cuh"
#include "phx_math.h"

namespace phx {

struct FmksDev {
  double a, a2, h, xt, alpha, x0, smooth, norm, hexp_br, hexp_nsq, hexp_csq;
  double epsfd;  // finite-difference step scale eps^(1/3) (geometry_utils.hpp:153)
  int derefine_poles;

  // ---- McKinneyGammieRyan (mckinney_gammie_ryan.hpp:64-198)
  __device__ double r_(double X1) const {
    const double hexp_dr = X1 - hexp_br;
    return phx_math::exp(X1 + (hexp_dr > 0.) * hexp_csq * phx_math::pow(hexp_dr, hexp_nsq));
  }
  __device__ double thG_(double X2) const {
    return M_PI * X2 + ((1. - h) / 2.) * phx_math::sin(2. * M_PI * X2);
  }
  __device__ void thJ_(double X2, double &y, double &thJ) const {
    y = 2. * X2 - 1.;
    thJ = norm * y * (1. + phx_math::pow(y / xt, alpha) / (alpha + 1.)) + 0.5 * M_PI;
  }
  __device__ void th_(double X1, double X2, double &y, double &th) const {
    const double thG = thG_(X2);
    if (derefine_poles) {
      double thJ;
      thJ_(X2, y, thJ);
      const double fac = x0 - X1;
      th = thG + phx_math::exp(smooth * fac) * (thJ - thG);
    } else {
      y = 0;
      th = thG;
    }
    constexpr double SINGSMALL = 1.e-20;
    if (fabs(th) < SINGSMALL) th = th >= 0. ? SINGSMALL : -SINGSMALL;
    if (fabs(M_PI - th) < SINGSMALL) th = th >= M_PI ? M_PI + SINGSMALL : M_PI - SINGSMALL;
  }
  __device__ void transform(double X1, double X2, double C[3], double Jcov[3][3], double Jcon[3][3]) const {
    double y, th, thJ;
    const double r = r_(X1);
    th_(X1, X2, y, th);
    C[0] = r;
    C[1] = th;
    C[2] = 0.0;
    const double hexp_dr = X1 - hexp_br;
    const double drdX1 = phx_math::exp(X1 + (hexp_dr > 0.) * hexp_csq * phx_math::pow(hexp_dr, hexp_nsq)) *
                         (1. + (hexp_dr > 0.) * hexp_csq * hexp_nsq * phx_math::pow(hexp_dr, hexp_nsq - 1.));
    const double dthGdX2 = M_PI + M_PI * (1 - h) * phx_math::cos(2 * M_PI * X2);
    double dthdX1, dthdX2;
    if (derefine_poles) {
      thJ_(X2, y, thJ);
      const double thG = thG_(X2);
      const double dydX2 = 2.;
      const double dthJdy = norm * (1 + phx_math::pow(y / xt, alpha));
      const double dthJdX2 = dthJdy * dydX2;
      const double fac = x0 - X1;
      dthdX1 = -smooth * (thJ - thG) * phx_math::exp(smooth * fac);
      dthdX2 = dthGdX2 + phx_math::exp(smooth * fac) * (dthJdX2 - dthGdX2);
    } else {
      dthdX1 = 0.0;
      dthdX2 = dthGdX2;
    }
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Jcov[i][j] = Jcon[i][j] = 0;
    Jcov[0][0] = drdX1;
    Jcov[1][0] = dthdX1;
    Jcov[1][1] = dthdX2;
    Jcov[2][2] = 1.;
    Jcon[0][0] = ratio(1., drdX1);
    Jcon[1][0] = -ratio(dthdX1, drdX1 * dthdX2);
    Jcon[1][1] = ratio(1., dthdX2);
    Jcon[2][2] = 1.;
  }
  // ---- SphericalKerrSchild (spherical_kerr_schild.hpp:48-243)
  __device__ double rho2_(double r, double cth) const { return r * r + a2 * cth * cth; }
  __device__ double ks_lapse(double X1, double X2) const {
    const double r = fabs(X1), cth = phx_math::cos(X2), rho2 = rho2_(r, cth);
    return sqrt(ratio(rho2, 2 * r + rho2));
  }
  __device__ void ks_gcov(double X1, double X2, double g[4][4]) const {
    const double r = fabs(X1), th = X2, cth = phx_math::cos(th), sth = phx_math::sin(th), sth2 = sth * sth;
    const double rho2 = rho2_(r, cth);
    for (int m = 0; m < 4; m++)
      for (int n = 0; n < 4; n++) g[m][n] = 0;
    g[0][1] = g[1][0] = ratio(2 * r, rho2);
    g[0][0] = -1 + g[0][1];
    g[0][3] = g[3][0] = -ratio(2 * a * r * sth2, rho2);
    g[1][1] = 1 + g[0][1];
    g[1][3] = g[3][1] = -a * (1 + g[0][1]) * sth2;
    g[2][2] = rho2;
    g[3][3] = (rho2 + a2 * (1 + g[0][1]) * sth2) * sth2;
  }
  __device__ void ks_gamcon(double X1, double X2, double g[3][3]) const {
    const double r = fabs(X1), th = X2, cth = phx_math::cos(th), sth = phx_math::sin(th), sth2 = sth * sth;
    const double rho2 = rho2_(r, cth);
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) g[m][n] = 0;
    g[0][0] = ratio(rho2, 2 * r + rho2) + ratio(a2 * sth2, rho2);
    g[0][2] = g[2][0] = ratio(a, rho2);
    g[1][1] = ratio(1, rho2);
    g[2][2] = ratio(1, rho2 * sth2);
  }
  __device__ double ks_detgam(double X1, double X2) const {
    const double r = fabs(X1), th = X2, cth = phx_math::cos(th), sth = phx_math::sin(th), sth2 = sth * sth;
    const double rho2 = rho2_(r, cth);
    return sqrt(fabs(rho2 * (2 * r + rho2) * sth2));
  }
  __device__ static double s2st(const double A[3][3], int mu, int nu) {
    if (mu == 0 || nu == 0) return (mu == nu) ? 1 : 0;
    return A[mu - 1][nu - 1];
  }
  // ---- Modified<> (modified_system.hpp:65-200)
  __device__ double Lapse(double X1, double X2) const {
    double C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, C, Jcov, Jcon);
    return ks_lapse(C[0], C[1]);
  }
  __device__ void Shift(double X1, double X2, double beta[3]) const {
    double C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, C, Jcov, Jcon);
    const double r = fabs(C[0]), cth = phx_math::cos(C[1]), rho2 = rho2_(r, cth);
    const double beta0[3] = {ratio(2 * r, 2 * r + rho2), 0, 0};
    for (int i = 0; i < 3; i++) {
      double s = 0;
      for (int j = 0; j < 3; j++) s += Jcon[i][j] * beta0[j];
      beta[i] = s;
    }
  }
  __device__ void SpacetimeMetric(double X1, double X2, double g[4][4]) const {
    double g0[4][4], C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, C, Jcov, Jcon);
    ks_gcov(C[0], C[1], g0);
    for (int mu = 0; mu < 4; mu++)
      for (int nu = 0; nu < 4; nu++) {
        double s = 0;
        for (int lam = 0; lam < 4; lam++)
          for (int kap = 0; kap < 4; kap++) s += g0[lam][kap] * s2st(Jcov, lam, mu) * s2st(Jcov, kap, nu);
        g[mu][nu] = s;
      }
  }
  __device__ void point(double X1, double X2, double *out, long long pitch) const {
    double C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, C, Jcov, Jcon);
    out[PHX_G_ALPHA * pitch] = ks_lapse(C[0], C[1]);
    // sqrt(gamma) |det J|  (linear_algebra.hpp:48-54 determinant)
    const double detJ = (Jcov[0][0] * Jcov[1][1] * Jcov[2][2] + Jcov[0][1] * Jcov[1][2] * Jcov[2][0] +
                         Jcov[0][2] * Jcov[1][0] * Jcov[2][1] - Jcov[0][2] * Jcov[1][1] * Jcov[2][0] -
                         Jcov[0][1] * Jcov[1][0] * Jcov[2][2] - Jcov[0][0] * Jcov[1][2] * Jcov[2][1]);
    out[PHX_G_DETGAM * pitch] = fabs(ks_detgam(C[0], C[1]) * detJ);
    {  // shift: beta^i = Jcon^i_j beta0^j
      const double r = fabs(C[0]), cth = phx_math::cos(C[1]), rho2 = rho2_(r, cth);
      const double beta0[3] = {ratio(2 * r, 2 * r + rho2), 0, 0};
      for (int i = 0; i < 3; i++) {
        double s = 0;
        for (int j = 0; j < 3; j++) s += Jcon[i][j] * beta0[j];
        out[(PHX_G_BETA + i) * pitch] = s;
      }
    }
    {
      double g0[4][4];
      ks_gcov(C[0], C[1], g0);
      for (int mu = 0; mu < 4; mu++)
        for (int nu = mu; nu < 4; nu++) {
          double s = 0;
          for (int lam = 0; lam < 4; lam++)
            for (int kap = 0; kap < 4; kap++) s += g0[lam][kap] * s2st(Jcov, lam, mu) * s2st(Jcov, kap, nu);
          out[(PHX_G_GCOV + flat2(mu, nu)) * pitch] = s;
        }
    }
    {
      double g0[3][3];
      ks_gamcon(C[0], C[1], g0);
      for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
          double s = 0;
          for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) s += g0[k][l] * Jcon[i][k] * Jcon[j][l];
          out[(PHX_G_GAMCON + flat2(i, j)) * pitch] = s;
        }
    }
  }
};

inline FmksDev make_fmks(const phx_geometry &g) {
  FmksDev f;
  f.a = g.a;
  f.a2 = g.a * g.a;
  f.h = g.hslope;
  f.xt = g.poly_xt;
  f.alpha = g.poly_alpha;
  f.x0 = g.x0;
  f.smooth = g.smooth;
  f.hexp_br = g.hexp_br;
  f.hexp_nsq = g.hexp_nsq;
  f.hexp_csq = g.hexp_csq;
  f.derefine_poles = g.derefine_poles;
  f.norm = 0.5 * M_PI * 1. / (1. + 1. / (f.alpha + 1.) * 1. / phx_math::pow(f.xt, f.alpha));
  f.epsfd = phx_math::pow(2.220446049250313e-16, 1.0 / 3.0);
  return f;
}

}  // namespace phx
