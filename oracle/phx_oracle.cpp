// phx_oracle.cpp -- CPU restatement of the phoebus GRMHD fluid hot path.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is checked
// against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg load it.  Nothing in the product links or calls it.
//
// It restates, function by function and in the reference's floating-point
// operation order, the per-zone algorithms of phoebus (paths relative to the
// phoebus source tree):
//   robust.hpp:10-40, root_find.hpp:27-167, relativity_utils.hpp:38-58,
//   prim2con.hpp:25-102, con2prim_robust.hpp:46-453, reconstruction.hpp:101-244,
//   riemann.hpp:32-301, fluid.cpp:359-944, tmunu.hpp:36-137,
//   geometry_utils.hpp:72-187, minkowski.hpp:35-115,
//   spherical_kerr_schild.hpp:42-243, mckinney_gammie_ryan.hpp:64-198,
//   modified_system.hpp:52-248, cached_system.hpp:86-640, fixup.hpp:72-327,
//   fixup_c2p.cpp:44-356, fixup.cpp:285-687.
// Third-party semantics restated from their definitions (not in the phoebus
// tree): singularity-eos IdealGas (P = (Gamma-1) rho eps, T = eps / Cv,
// bulk modulus = Gamma P), Parthenon UniformCartesian coordinates,
// FluxDivergence, SumData, Average/UpdateIndependentData, the rk2
// LowStorageIntegrator coefficients and periodic ghost exchange.
//
// Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -fPIC -shared.
// -ffp-contract=off keeps every multiply and add separately rounded, so the
// CUDA exact build (nvcc -fmad=false) can be compared bit for bit.
//
// Transcendentals: the reference calls std::exp, std::sin, std::cos and
// std::pow in the FMKS geometry and the floors.  Those calls go to the
// library's written-out exp, sin, cos and pow (phoebus_gb300/csrc/phx_math.h,
// series restated from the mathematics and measured within 2 ulp of the C
// library's), which the CUDA kernels also evaluate: a libm choice, like
// glibc's, that makes the geometry tables and the exponential floors
// comparable bit for bit.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "../include/phx_fluid.h"
#include "../include/phx_radiation.h"
#include "../phoebus_gb300/csrc/phx_math.h"

namespace orc {

using Real = double;
constexpr int NDSPACE = 3;
constexpr int NDFULL = 4;

// ---------------------------------------------------------------- robust.hpp
constexpr Real SMALL = 10 * std::numeric_limits<Real>::min();
constexpr Real EPS = 10 * std::numeric_limits<Real>::epsilon();
inline Real make_positive(Real v) { return std::max(v, EPS); }
inline Real make_bounded(Real v, Real vmin, Real vmax) {
  return std::min(std::max(v, vmin + EPS), vmax * (1.0 - EPS));
}
inline Real ratio(Real a, Real b) {
  const Real sgn = b >= 0 ? 1 : -1;
  return a / (b + sgn * SMALL);
}

// ------------------------------------------------ singularity-eos IdealGas
struct EOS {
  Real gm1, Cv;
  Real PressureFromDensityInternalEnergy(Real rho, Real sie) const {
    return std::max(0.0, gm1 * rho * sie);
  }
  Real TemperatureFromDensityInternalEnergy(Real rho, Real sie) const {
    return std::max(0.0, sie / Cv);
  }
  Real PressureFromDensityTemperature(Real rho, Real T) const {
    return std::max(0.0, gm1 * rho * Cv * T);
  }
  Real BulkModulusFromDensityTemperature(Real rho, Real T) const {
    return std::max(0.0, (gm1 + 1) * gm1 * rho * Cv * T);
  }
  Real BulkModulusFromDensityInternalEnergy(Real rho, Real sie) const {
    return std::max(0.0, gm1 * (gm1 + 1) * rho * sie);
  }
};

// ------------------------------------------------------------- fixup.hpp
struct Bounds {
  int floor_type;
  Real r0, s0, ralpha, salpha, rho_min_eos, sie_min_eos;
  Real g0, smax0;          // ceilings
  Real bsqorho0, bsqou0;   // MHD ceilings
  explicit Bounds(const phx_params &p) {
    // fixup.cpp:124-133: c2p fixup and MHD floors force floors on
    if (p.enable_floors || p.enable_c2p_fixup || (p.enable_mhd_floors && p.mhd)) {
      floor_type = p.floor_type;
      r0 = p.rho0_floor;
      s0 = p.sie0_floor;
      ralpha = p.rho_exp_floor;
      salpha = p.sie_exp_floor;
    } else {  // Floors() default: ConstantRhoSie with -max (fixup.hpp:75-78)
      floor_type = PHX_FLOOR_CONSTANT_RHO_SIE;
      r0 = -std::numeric_limits<Real>::max();
      s0 = -std::numeric_limits<Real>::max();
      ralpha = salpha = 0.0;
    }
    rho_min_eos = p.rho_min_eos;
    sie_min_eos = p.sie_min_eos;
    if (p.enable_ceilings) {
      g0 = p.gam0_ceiling;
      smax0 = p.sie0_ceiling;
    } else {
      g0 = std::numeric_limits<Real>::max();
      smax0 = std::numeric_limits<Real>::max();
    }
    if (p.enable_mhd_floors && p.mhd) {
      bsqorho0 = p.bsqorho0_ceiling;
      bsqou0 = p.bsqou0_ceiling;
    } else {
      bsqorho0 = std::numeric_limits<Real>::max();
      bsqou0 = std::numeric_limits<Real>::max();
    }
  }
  // fixup.hpp:94-134
  void GetFloors(Real x1, Real x2, Real x3, Real &rflr, Real &sflr) const {
    switch (floor_type) {
    case PHX_FLOOR_CONSTANT_RHO_SIE:
      rflr = r0;
      sflr = s0;
      break;
    case PHX_FLOOR_EXPX1_RHO_SIE:
      rflr = r0 * phx_math::exp(ralpha * x1);
      sflr = s0 * phx_math::exp(salpha * x1);
      break;
    case PHX_FLOOR_EXPX1_RHO_U: {
      Real scratch = r0 * phx_math::exp(ralpha * x1);
      sflr = s0 * phx_math::exp(salpha * x1) / std::max(rflr, scratch);
      rflr = scratch;
    } break;
    case PHX_FLOOR_X1_RHO_SIE:
      rflr = r0 * std::min(1.0, phx_math::pow(x1, ralpha));
      sflr = s0 * std::min(1.0, phx_math::pow(x1, salpha));
      break;
    default: {  // PHX_FLOOR_R_RHO_SIE
      Real r = std::sqrt(x1 * x1 + x2 * x2 + x3 * x3);
      rflr = r0 * std::min(1.0, phx_math::pow(r, ralpha));
      sflr = s0 * std::min(1.0, phx_math::pow(r, salpha));
    } break;
    }
    rflr = std::max(rflr, rho_min_eos);
    sflr = std::max(sflr, sie_min_eos);
  }
  void GetCeilings(Real, Real, Real, Real &gmax, Real &smax) const {
    gmax = g0;
    smax = smax0;
  }
  void GetMHDCeilings(Real, Real, Real, Real &bsqorho, Real &bsqou) const {
    bsqorho = bsqorho0;
    bsqou = bsqou0;
  }
};

// ------------------------------------------------- block indexing helpers
struct Blk {
  const phx_block *b;
  int n1t, n2t, n3t;
  long long N, vs;
  int ndim, ng;
  explicit Blk(const phx_block *blk) : b(blk) {
    ndim = blk->ndim;
    ng = blk->ng;
    n1t = blk->nx1 + 2 * ng;
    n2t = ndim >= 2 ? blk->nx2 + 2 * ng : 1;
    n3t = ndim >= 3 ? blk->nx3 + 2 * ng : 1;
    N = (long long)n1t * n2t * n3t;
    vs = blk->var_stride ? blk->var_stride : N;
  }
  long long idx(int k, int j, int i) const { return ((long long)k * n2t + j) * n1t + i; }
  Real &P(int v, int k, int j, int i) const { return b->prim[v * vs + idx(k, j, i)]; }
  Real &U(int v, int k, int j, int i) const { return b->cons[v * vs + idx(k, j, i)]; }
  Real &F(int d, int m, int k, int j, int i) const {
    return b->flux[((long long)d * PHX_NCONS + m) * vs + idx(k, j, i)];
  }
  // Parthenon UniformCartesian (restated): ghost origin then uniform spacing
  Real x0(int d) const {
    const Real xmin = d == 1 ? b->x1min : (d == 2 ? b->x2min : b->x3min);
    const Real dx = d == 1 ? b->dx1 : (d == 2 ? b->dx2 : b->dx3);
    return d <= ndim ? xmin - ng * dx : xmin;
  }
  Real dx(int d) const { return d == 1 ? b->dx1 : (d == 2 ? b->dx2 : b->dx3); }
  Real Xc(int d, int idx) const { return x0(d) + (idx + 0.5) * dx(d); }
  Real Xf(int d, int idx) const { return x0(d) + idx * dx(d); }
  int is() const { return ng; }
  int ie() const { return ng + b->nx1 - 1; }
  int js() const { return ndim >= 2 ? ng : 0; }
  int je() const { return ndim >= 2 ? ng + b->nx2 - 1 : 0; }
  int ks() const { return ndim >= 3 ? ng : 0; }
  int ke() const { return ndim >= 3 ? ng + b->nx3 - 1 : 0; }
};

// ------------------------------------------------------------ geometry
enum Loc { CENT = 0, FACE1 = 1, FACE2 = 2, FACE3 = 3 };

inline int flatten2(int m, int n) {  // geometry_utils.hpp:180-185
  static const int ind[4][4] = {{0, 1, 3, 6}, {1, 2, 4, 7}, {3, 4, 5, 8}, {6, 7, 8, 9}};
  return ind[m][n];
}
inline int flatten2s(int m, int n) {  // 3x3 symmetric, same table
  static const int ind[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
  return ind[m][n];
}

// Analytic FMKS: Modified<SphericalKerrSchild, McKinneyGammieRyan>.
struct FMKS {
  Real a, a2;
  bool derefine_poles;
  Real h, xt, alpha, x0, smooth, norm, hexp_br, hexp_nsq, hexp_csq;
  Real dxfd;
  explicit FMKS(const phx_geometry &g)
      : a(g.a), a2(g.a * g.a), derefine_poles(g.derefine_poles != 0), h(g.hslope),
        xt(g.poly_xt), alpha(g.poly_alpha), x0(g.x0), smooth(g.smooth),
        hexp_br(g.hexp_br), hexp_nsq(g.hexp_nsq), hexp_csq(g.hexp_csq), dxfd(1e-8) {
    // mckinney_gammie_ryan.hpp:188-190 GetNorm_
    norm = 0.5 * M_PI * 1. / (1. + 1. / (alpha + 1.) * 1. / phx_math::pow(xt, alpha));
  }
  // ---- McKinneyGammieRyan (mckinney_gammie_ryan.hpp:64-198)
  Real r_(Real X1) const {
    const Real hexp_dr = X1 - hexp_br;
    return phx_math::exp(X1 + (hexp_dr > 0.) * hexp_csq * phx_math::pow(hexp_dr, hexp_nsq));
  }
  Real thG_(Real X2) const { return M_PI * X2 + ((1. - h) / 2.) * phx_math::sin(2. * M_PI * X2); }
  void thJ_(Real X2, Real &y, Real &thJ) const {
    y = 2. * X2 - 1.;
    thJ = norm * y * (1. + phx_math::pow(y / xt, alpha) / (alpha + 1.)) + 0.5 * M_PI;
  }
  void th_(Real X1, Real X2, Real &y, Real &th) const {
    Real thG = thG_(X2);
    if (derefine_poles) {
      Real thJ;
      thJ_(X2, y, thJ);
      const Real fac = x0 - X1;
      th = thG + phx_math::exp(smooth * fac) * (thJ - thG);
    } else {
      y = 0;
      th = thG;
    }
    constexpr Real SINGSMALL = 1.e-20;
    if (std::fabs(th) < SINGSMALL) {
      if (th >= 0.)
        th = SINGSMALL;
      else if (th < 0)
        th = -SINGSMALL;
    }
    if (std::fabs(M_PI - th) < SINGSMALL) {
      if (th >= M_PI)
        th = M_PI + SINGSMALL;
      else if (th < M_PI)
        th = M_PI - SINGSMALL;
    }
  }
  void transform(Real X1, Real X2, Real X3, Real C[3], Real Jcov[3][3],
                 Real Jcon[3][3]) const {
    Real y, th, thJ;
    const Real r = r_(X1);
    th_(X1, X2, y, th);
    C[0] = r;
    C[1] = th;
    C[2] = X3;
    const Real hexp_dr = X1 - hexp_br;
    const Real drdX1 =
        phx_math::exp(X1 + (hexp_dr > 0.) * hexp_csq * phx_math::pow(hexp_dr, hexp_nsq)) *
        (1. + (hexp_dr > 0.) * hexp_csq * hexp_nsq * phx_math::pow(hexp_dr, hexp_nsq - 1.));
    const Real dthGdX2 = M_PI + M_PI * (1 - h) * phx_math::cos(2 * M_PI * X2);
    Real dthdX1, dthdX2;
    if (derefine_poles) {
      thJ_(X2, y, thJ);
      const Real thG = thG_(X2);
      const Real dydX2 = 2.;
      const Real dthJdy = norm * (1 + phx_math::pow(y / xt, alpha));
      const Real dthJdX2 = dthJdy * dydX2;
      const Real fac = x0 - X1;
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
  Real rho2_(Real r, Real cth) const { return r * r + a2 * cth * cth; }
  void vars_(Real X1, Real X2, Real &r, Real &th, Real &cth, Real &sth, Real &sth2,
             Real &rho2) const {
    r = std::abs(X1);
    th = X2;
    cth = phx_math::cos(th);
    sth = phx_math::sin(th);
    sth2 = sth * sth;
    rho2 = rho2_(r, cth);
  }
  Real ks_lapse(Real X1, Real X2) const {
    const Real r = std::abs(X1);
    const Real cth = phx_math::cos(X2);
    const Real rho2 = rho2_(r, cth);
    return std::sqrt(ratio(rho2, 2 * r + rho2));
  }
  void ks_shift(Real X1, Real X2, Real beta[3]) const {
    Real r = std::abs(X1);
    Real cth = phx_math::cos(X2);
    const Real rho2 = rho2_(r, cth);
    beta[0] = ratio(2 * r, 2 * r + rho2);
    beta[1] = 0;
    beta[2] = 0;
  }
  void ks_gcov(Real X1, Real X2, Real g[4][4]) const {
    Real r, th, cth, sth, sth2, rho2;
    vars_(X1, X2, r, th, cth, sth, sth2, rho2);
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
  void ks_gamcon(Real X1, Real X2, Real g[3][3]) const {
    Real r, th, cth, sth, sth2, rho2;
    vars_(X1, X2, r, th, cth, sth, sth2, rho2);
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) g[m][n] = 0;
    g[0][0] = ratio(rho2, 2 * r + rho2) + ratio(a2 * sth2, rho2);
    g[0][2] = g[2][0] = ratio(a, rho2);
    g[1][1] = ratio(1, rho2);
    g[2][2] = ratio(1, rho2 * sth2);
  }
  Real ks_detgam(Real X1, Real X2) const {
    Real r, th, cth, sth, sth2, rho2;
    vars_(X1, X2, r, th, cth, sth, sth2, rho2);
    return std::sqrt(std::abs(rho2 * (2 * r + rho2) * sth2));
  }
  static Real s2st(const Real A[3][3], int mu, int nu) {
    if (mu == 0 || nu == 0) return (mu == nu) ? 1 : 0;
    return A[mu - 1][nu - 1];
  }
  static Real det3(const Real A[3][3]) {  // linear_algebra.hpp:48-54
    return (A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] +
            A[0][2] * A[1][0] * A[2][1] - A[0][2] * A[1][1] * A[2][0] -
            A[0][1] * A[1][0] * A[2][2] - A[0][0] * A[1][2] * A[2][1]);
  }
  // ---- Modified<> (modified_system.hpp:65-200)
  Real Lapse(Real X1, Real X2, Real X3) const {
    Real C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, X3, C, Jcov, Jcon);
    return ks_lapse(C[0], C[1]);
  }
  void Shift(Real X1, Real X2, Real X3, Real beta[3]) const {
    Real beta0[3], C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, X3, C, Jcov, Jcon);
    ks_shift(C[0], C[1], beta0);
    for (int i = 0; i < 3; i++) {
      beta[i] = 0;
      for (int j = 0; j < 3; j++) beta[i] += Jcon[i][j] * beta0[j];
    }
  }
  void SpacetimeMetric(Real X1, Real X2, Real X3, Real g[4][4]) const {
    Real g0[4][4], C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, X3, C, Jcov, Jcon);
    ks_gcov(C[0], C[1], g0);
    for (int mu = 0; mu < 4; mu++)
      for (int nu = 0; nu < 4; nu++) {
        g[mu][nu] = 0;
        for (int lam = 0; lam < 4; lam++)
          for (int kap = 0; kap < 4; kap++)
            g[mu][nu] += g0[lam][kap] * s2st(Jcov, lam, mu) * s2st(Jcov, kap, nu);
      }
  }
  void MetricInverse(Real X1, Real X2, Real X3, Real g[3][3]) const {
    Real g0[3][3], C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, X3, C, Jcov, Jcon);
    ks_gamcon(C[0], C[1], g0);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        g[i][j] = 0;
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) g[i][j] += g0[k][l] * Jcon[i][k] * Jcon[j][l];
      }
  }
  Real DetGamma(Real X1, Real X2, Real X3) const {
    Real C[3], Jcov[3][3], Jcon[3][3];
    transform(X1, X2, X3, C, Jcov, Jcon);
    Real detJ = det3(Jcov);
    return std::abs(ks_detgam(C[0], C[1]) * detJ);
  }
  // geometry_utils.hpp:149-178 SetMetricGradientByFD (dx argument unused)
  void MetricDerivative(Real X1, Real X2, Real X3, Real dg[4][4][4]) const {
    Real EPSFD = phx_math::pow(2.220446049250313e-16, 1.0 / 3.0);
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++)
        for (int c = 0; c < 4; c++) dg[a][b][c] = 0;
    Real gl[4][4], gr[4][4];
    Real dx = dxfd;
    for (int d = 1; d < 4; ++d) {
      Real X1L = X1, X2L = X2, X3L = X3, X1R = X1, X2R = X2, X3R = X3;
      if (d == 1) {
        dx = std::max(std::abs(X1), 1.0) * EPSFD;
        X1L -= dx;
        X1R += dx;
      }
      if (d == 2) {
        dx = std::max(std::abs(X2), 1.0) * EPSFD;
        X2L -= dx;
        X2R += dx;
      }
      if (d == 3) {
        dx = std::max(std::abs(X3), 1.0) * EPSFD;
        X3L -= dx;
        X3R += dx;
      }
      SpacetimeMetric(X1R, X2R, X3R, gr);
      SpacetimeMetric(X1L, X2L, X3L, gl);
      for (int mu = 0; mu < 4; mu++)
        for (int nu = 0; nu < 4; nu++)
          dg[mu][nu][d] = ratio(gr[mu][nu] - gl[mu][nu], 2 * dx);
    }
  }
  // geometry_utils.hpp:89-119 SetGradLnAlphaByFD
  void GradLnAlpha(Real X1, Real X2, Real X3, Real da[4]) const {
    Real EPSFD = phx_math::pow(2.220446049250313e-16, 1.0 / 3.0);
    for (int m = 0; m < 4; m++) da[m] = 0;
    Real dx = dxfd;
    for (int d = 1; d < 4; ++d) {
      Real X1p = X1, X1m = X1, X2p = X2, X2m = X2, X3p = X3, X3m = X3;
      if (d == 1) {
        dx = std::max(std::abs(X1), 1.0) * EPSFD;
        X1p += dx;
        X1m -= dx;
      } else if (d == 2) {
        dx = std::max(std::abs(X2), 1.0) * EPSFD;
        X2p += dx;
        X2m -= dx;
      } else if (d == 3) {
        dx = std::max(std::abs(X3), 1.0) * EPSFD;
        X3p += dx;
        X3m -= dx;
      }
      Real alpham = Lapse(X1m, X2m, X3m);
      Real alphap = Lapse(X1p, X2p, X3p);
      da[d] = ratio(alphap - alpham, dx * (alpham + alphap));
    }
  }
};

// Geometry at a point, as read by the fluid kernels.  For Minkowski these are
// the analytic constants; for FMKS they come from the cached tables.
struct GeomPt {
  Real alpha, beta[3], gcov[4][4], gamcon[3][3], detgam;
};

struct Geom {
  const phx_geometry *g;  // NULL = Minkowski
  const Blk *B;
  Geom(const phx_geometry *gg, const Blk *bb) : g(gg), B(bb) {}
  bool mink() const { return g == nullptr || g->kind == PHX_GEOM_MINKOWSKI; }
  const double *table(Loc loc, long long &pitch, int j, int i, long long &off) const {
    if (loc == FACE1) {
      pitch = (long long)B->n2t * (B->n1t + 1);
      off = (long long)j * (B->n1t + 1) + i;
      return g->face1;
    } else if (loc == FACE2) {
      pitch = (long long)(B->n2t + 1) * B->n1t;
      off = (long long)j * B->n1t + i;
      return g->face2;
    }
    pitch = (long long)B->n2t * B->n1t;
    off = (long long)j * B->n1t + i;
    return g->cent;
  }
  void at(Loc loc, int k, int j, int i, GeomPt &p) const {
    if (mink()) {  // minkowski.hpp:37-83
      p.alpha = 1.;
      for (int d = 0; d < 3; d++) p.beta[d] = 0;
      for (int mu = 0; mu < 4; mu++)
        for (int nu = 0; nu < 4; nu++) p.gcov[mu][nu] = (mu == nu) ? (mu == 0 ? -1 : 1) : 0;
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) p.gamcon[a][b] = (a == b ? 1 : 0);
      p.detgam = 1.;
      return;
    }
    long long pitch, off;
    const double *t = table(loc, pitch, j, i, off);
    p.alpha = t[PHX_G_ALPHA * pitch + off];
    for (int d = 0; d < 3; d++) p.beta[d] = t[(PHX_G_BETA + d) * pitch + off];
    for (int mu = 0; mu < 4; mu++)
      for (int nu = 0; nu < 4; nu++)
        p.gcov[mu][nu] = t[(PHX_G_GCOV + flatten2(mu, nu)) * pitch + off];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++)
        p.gamcon[a][b] = t[(PHX_G_GAMCON + flatten2s(a, b)) * pitch + off];
    p.detgam = t[PHX_G_DETGAM * pitch + off];
  }
  // DetG: analytic Minkowski = 1; cached = Lapse * DetGamma (cached_system.hpp:325)
  Real DetG(const GeomPt &p) const { return mink() ? 1. : p.alpha * p.detgam; }
  void MetricDerivative(int k, int j, int i, Real dg[4][4][4]) const {
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++)
        for (int c = 0; c < 4; c++) dg[a][b][c] = 0;
    if (mink()) return;
    const long long pitch = (long long)B->n2t * B->n1t, off = (long long)j * B->n1t + i;
    for (int mu = 0; mu < 4; mu++)
      for (int nu = 0; nu < 4; nu++) {
        dg[mu][nu][0] = 0.0;
        for (int s = 1; s < 4; s++)
          dg[mu][nu][s] = g->deriv[(PHX_GD_DG + 3 * flatten2(mu, nu) + s - 1) * pitch + off];
      }
  }
  void GradLnAlpha(int k, int j, int i, Real da[4]) const {
    for (int m = 0; m < 4; m++) da[m] = 0;
    if (mink()) return;
    const long long pitch = (long long)B->n2t * B->n1t, off = (long long)j * B->n1t + i;
    for (int d = 1; d < 4; d++) da[d] = g->deriv[(PHX_GD_DALPHA + d - 1) * pitch + off];
  }
  // cached_system.hpp:282-299
  void SpacetimeMetricInverse(const GeomPt &p, Real gi[4][4]) const {
    if (mink()) {
      for (int mu = 0; mu < 4; mu++)
        for (int nu = 0; nu < 4; nu++) gi[mu][nu] = (mu == nu) ? (mu == 0 ? -1 : 1) : 0;
      return;
    }
    Real alpha2 = p.alpha;
    alpha2 *= alpha2;
    gi[0][0] = -ratio(1, alpha2);
    for (int mu = 0; mu < 3; mu++) gi[mu + 1][0] = gi[0][mu + 1] = ratio(p.beta[mu], alpha2);
    for (int mu = 0; mu < 3; mu++)
      for (int nu = 0; nu < 3; nu++) {
        gi[mu + 1][nu + 1] = p.gamcon[mu][nu];
        gi[mu + 1][nu + 1] -= gi[0][mu + 1] * gi[0][nu + 1] * alpha2;
      }
  }
};

// --------------------------------------------------- relativity_utils.hpp
inline Real GetLorentzFactor(const Real v[3], const Real gcov[4][4]) {
  Real vsq = 0.;
  for (int ii = 0; ii < 3; ii++)
    for (int jj = 0; jj < 3; jj++) vsq += gcov[ii + 1][jj + 1] * v[ii] * v[jj];
  return std::sqrt(1. + vsq);
}

// ------------------------------------------------------------ prim2con.hpp
void signal_speeds(Real rho, Real u, Real p, Real bsq, const Real v[], Real vsq,
                   Real gam1, Real alpha, const Real beta[], const Real gcon[3][3],
                   Real *sig) {
  const Real rho_rel = rho + u + p;
  const Real vasq = bsq / (rho_rel + bsq);
  Real cssq = gam1 * p / rho_rel;
  cssq += vasq - cssq * vasq;
  const Real vcoff = alpha / (1.0 - vsq * cssq);
  for (int m = 0; m < 3; m++) {
    const Real vpm = std::sqrt(cssq * (1.0 - vsq) *
                               (gcon[m][m] * (1.0 - vsq * cssq) - v[m] * v[m] * (1.0 - cssq)));
    const Real vp = vcoff * (v[m] * (1.0 - cssq) + vpm) - beta[m];
    const Real vm = vcoff * (v[m] * (1.0 - cssq) - vpm) - beta[m];
    sig[m] = std::max(std::fabs(vp), std::fabs(vm));
  }
}

void p2c(Real rho, const Real vp[], const Real b[], Real u, Real p, Real gam1,
         const Real gcov[4][4], const Real gcon[3][3], const Real beta[], Real alpha,
         Real gdet, Real &D, Real S[], Real bcons[], Real &tau, Real *sig) {
  Real vsq = 0.0, Bsq = 0.0, Bdotv = 0.0;
  const Real W = GetLorentzFactor(vp, gcov);
  const Real iW = 1.0 / W;
  Real v[3] = {vp[0] * iW, vp[1] * iW, vp[2] * iW};
  for (int ii = 0; ii < 3; ii++)
    for (int jj = 0; jj < 3; jj++) {
      vsq += gcov[ii + 1][jj + 1] * v[ii] * v[jj];
      Bsq += gcov[ii + 1][jj + 1] * b[ii] * b[jj];
      Bdotv += gcov[ii + 1][jj + 1] * b[ii] * v[jj];
    }
  const Real b0 = W * Bdotv;
  Real bcon[] = {W * Bdotv / alpha, 0.0, 0.0, 0.0};
  for (int m = 0; m < 3; m++) bcon[m + 1] = b[m] * iW + Bdotv * W * (v[m] - beta[m] / alpha);
  const Real bsq = Bsq * iW * iW + Bdotv * Bdotv;
  Real bcov[3] = {0.0, 0.0, 0.0};
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 4; n++) bcov[m] += gcov[m + 1][n] * bcon[n];
  D = gdet * rho * W;
  const Real rho_rel = (rho + u + p + bsq) * W * W;
  for (int m = 0; m < 3; m++) {
    Real vcov = 0.0;
    for (int n = 0; n < 3; n++) vcov += gcov[m + 1][n + 1] * v[n];
    S[m] = gdet * (rho_rel * vcov - b0 * bcov[m]);
    bcons[m] = gdet * b[m];
  }
  tau = gdet * (rho_rel - (p + 0.5 * bsq) - b0 * b0) - D;  // USE_VALENCIA
  if (sig != nullptr) signal_speeds(rho, u, p, bsq, v, vsq, gam1, alpha, beta, gcon, sig);
}

// ------------------------------------------------------- root_find.hpp
struct RootFind {
  int iteration_count = 0, max_iter;
  int evals = 0;
  explicit RootFind(int mi) : max_iter(mi) {}
  template <typename F>
  void refine_bracket(F &func, Real guess, Real &a, Real &b, Real &ya, Real &yb) {
    if (a <= guess && b >= guess) {
      ya = func(guess);
      yb = func(b);
      evals += 2;
      if (ya * yb > 0.0) {
        yb = ya;
        b = guess;
        ya = func(a);
        evals++;
      } else {
        a = guess;
      }
    } else {
      ya = func(a);
      yb = func(b);
      evals += 2;
    }
  }
  // returns false when unbracketed (the reference aborts; we return guess)
  template <typename F>
  Real regula_falsi(F &func, Real a, Real b, Real tol, Real guess, bool &bracketed) {
    Real ya, yb;
    refine_bracket(func, guess, a, b, ya, yb);
    bracketed = !(ya * yb > 0.0);
    if (!bracketed) return guess;
    return iterate(func, a, b, ya, yb, tol);
  }
  // The Illinois iterations of regula_falsi (root_find.hpp:120-166) from a
  // sign-changing bracket [a, b] with f(a) = ya, f(b) = yb.
  template <typename F>
  Real iterate(F &func, Real a, Real b, Real ya, Real yb, Real tol) {
    Real sign = (ya < 0 ? 1.0 : -1.0);
    ya *= sign;
    yb *= sign;
    int b1 = 0, b2 = 0;
    while (b - a > 2.0 * tol && iteration_count < max_iter) {
      Real c = (a * yb - b * ya) / (yb - ya);
      if (c == a) {
        b = a;
        iteration_count++;
        continue;
      } else if (c == b) {
        a = b;
        iteration_count++;
        continue;
      }
      Real yc = sign * func(c);
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
      iteration_count++;
    }
    return 0.5 * (a + b);
  }
  // Learned starting bracket (no reference counterpart).  m: predicted root
  // in [lo, hi] (all in [0, 1]).  f(m) picks the half that should hold the
  // root (f < 0 below the root, > 0 above it); one more evaluation at that
  // half's outer end checks the sign change.  Accepted: the same Illinois
  // iterations from that half.  Rejected: the reference's own start from
  // [0, 1] refined by guess.  Only cold zones (guess = 0) try it.
  template <typename F>
  Real regula_falsi_learned(F &func, Real m, Real lo, Real hi, Real tol, Real guess, bool &bracketed,
                            bool &accepted) {
    accepted = false;
    if (guess > 0.0 || !(lo >= 0.0 && lo <= m && m <= hi && hi <= 1.0))  // warm zone, or no usable bracket
      return regula_falsi(func, 0.0, 1.0, tol, guess, bracketed);
    Real a, b, ya, yb;
    const Real ym = func(m);
    if (ym > 0.0) {
      a = lo;
      b = m;
      yb = ym;
      ya = func(lo);
    } else {
      a = m;
      b = hi;
      ya = ym;
      yb = func(hi);
    }
    evals += 2;
    accepted = ya * yb <= 0.0;
    if (!accepted) return regula_falsi(func, 0.0, 1.0, tol, guess, bracketed);
    bracketed = true;
    return iterate(func, a, b, ya, yb, tol);
  }
};

// -------------------------------------------------- con2prim_robust.hpp
struct Residual {
  Real D_, q_, bsq_, bsq_rpsq_, rsq_, rbsq_, v0sq_;
  const EOS &eos_;
  const Bounds &bounds_;
  Real x1_, x2_, x3_, floor_scale_fac_;
  Real rho_floor_ = 0.0, e_floor_ = 0.0, gam_max_ = 0.0, e_max_ = 0.0;
  bool used_density_floor_ = false, used_energy_floor_ = false, used_energy_max_ = false,
       used_gamma_max_ = false;
  Residual(Real D, Real q, Real bsq, Real bsq_rpsq, Real rsq, Real rbsq, Real v0sq,
           const EOS &eos, const Bounds &bnds, Real x1, Real x2, Real x3, Real fsf)
      : D_(D), q_(q), bsq_(bsq), bsq_rpsq_(bsq_rpsq), rsq_(rsq), rbsq_(rbsq), v0sq_(v0sq),
        eos_(eos), bounds_(bnds), x1_(x1), x2_(x2), x3_(x3), floor_scale_fac_(fsf) {
    Real garbage = 0.0;
    bounds_.GetFloors(x1_, x2_, x3_, rho_floor_, garbage);
    bounds_.GetCeilings(x1_, x2_, x3_, gam_max_, e_max_);
    rho_floor_ *= floor_scale_fac_;
  }
  Real x_mu(Real mu) const { return ratio(1.0, 1.0 + mu * bsq_); }
  Real rbarsq_mu(Real mu, Real x) const { return x * (x * rsq_ + mu * (1.0 + x) * rbsq_); }
  Real qbar_mu(Real mu, Real x) const {
    const Real mux = mu * x;
    return q_ - 0.5 * (bsq_ + mux * mux * bsq_rpsq_);
  }
  Real vhatsq_mu(Real mu, Real rbarsq) {
    const Real vsq_trial = mu * mu * rbarsq;
    if (vsq_trial > v0sq_) {
      used_gamma_max_ = true;
      return v0sq_;
    }
    used_gamma_max_ = false;
    return vsq_trial;
  }
  Real iWhat_mu(Real vhatsq) const { return std::sqrt(1.0 - vhatsq); }
  Real rhohat_mu(Real iWhat) {
    const Real rho_trial = D_ * iWhat;
    if (rho_trial <= rho_floor_) {
      used_density_floor_ = true;
      return rho_floor_;
    }
    used_density_floor_ = false;
    return rho_trial;
  }
  Real ehat_mu(Real mu, Real qbar, Real rbarsq, Real vhatsq, Real What) {
    Real rho = rhohat_mu(ratio(1.0, What));
    bounds_.GetFloors(x1_, x2_, x3_, rho, e_floor_);
    e_floor_ *= floor_scale_fac_;
    const Real ehat_trial = What * (qbar - mu * rbarsq) + vhatsq * What * ratio(What, 1.0 + What);
    used_energy_floor_ = false;
    used_energy_max_ = false;
    if (ehat_trial <= e_floor_) {
      used_energy_floor_ = true;
      return e_floor_;
    } else if (ehat_trial > e_max_) {
      used_energy_max_ = true;
      return e_max_;
    }
    return ehat_trial;
  }
  Real operator()(Real mu) {
    const Real x = x_mu(mu);
    const Real rbarsq = rbarsq_mu(mu, x);
    const Real qbar = qbar_mu(mu, x);
    const Real vhatsq = vhatsq_mu(mu, rbarsq);
    const Real iWhat = iWhat_mu(vhatsq);
    const Real What = ratio(1.0, iWhat);
    Real rhohat = rhohat_mu(iWhat);
    Real ehat = ehat_mu(mu, qbar, rbarsq, vhatsq, What);
    const Real Phat = eos_.PressureFromDensityInternalEnergy(rhohat, ehat);
    Real hhat = rhohat * (1.0 + ehat) + Phat;
    const Real ahat = Phat / make_positive(hhat - Phat);
    const Real nua = (1.0 + ahat) * (1.0 + ehat) * iWhat;
    const Real nub = (1.0 + ahat) * (1.0 + qbar - mu * rbarsq);
    const Real nuhat = std::max(nua, nub);
    const Real muhat = 1.0 / (nuhat + mu * rbarsq);
    return mu - muhat;
  }
  bool used_bounds() const {
    return used_density_floor_ || used_energy_floor_ || used_energy_max_ || used_gamma_max_;
  }
};

struct C2PResult {
  bool success;
  bool bracketed;
  int iterations;
  int evals;
  bool learned_accepted;
};

// Inputs of the learned con2prim start (no reference counterpart): scale-free
// invariants of the inversion, each mapped to O(1).  log10 arguments are
// bounded below so that zero momentum or field give finite values.
// The arithmetic after the FP64 setup is FP32, as on the device.
inline void c2p_features(Real D, Real q, Real rsq, Real bsq, Real rbsq, Real v0sq, float f[PHX_MLP_IN]) {
  f[0] = std::log10((float)std::max(q, 1e-12)) * 0.25f;
  f[1] = std::log10((float)std::max(rsq, 1e-12)) * 0.25f;
  f[2] = std::log10((float)std::max(bsq, 1e-12)) * 0.25f;
  f[3] = (float)rbsq / std::max((float)bsq * (float)rsq, 1e-30f);
  f[4] = (float)v0sq;
  f[5] = std::log10((float)std::max(D, 1e-30)) * 0.125f;
}

// One zone's primitive and conserved values: P[v * vs], U[v * vs].
struct ZoneRef {
  Real *Pz, *Uz;
  long long vs;
  Real &P(int v) const { return Pz[v * vs]; }
  Real &U(int v) const { return Uz[v * vs]; }
};

// con2prim_robust.hpp:299-453 for one zone, given its metric g and its
// cell-centre coordinates x1..x3 (used by the floors).  guess: the starting
// value of the regula-falsi (the stored c2p_mu in the reference).  sig gets
// the three cell signal speeds.
// fixed_mu (not the reference's): skip the root find and finish at *fixed_mu
// (the tests use it to evaluate the reference's finish at another build's root).
C2PResult con2prim_core(const GeomPt &g, const EOS &eos, const Bounds &bounds, const phx_params &par,
                        Real x1, Real x2, Real x3, const ZoneRef &z, Real guess, Real sig[3],
                        const Real *learned = nullptr, const Real *fixed_mu = nullptr) {
  C2PResult res{false, true, 0, 0, false};
  auto P = [&](int v) -> Real & { return z.P(v); };
  auto U = [&](int v) -> Real & { return z.U(v); };
  sig[0] = sig[1] = sig[2] = 0.0;
  const Real gdet = g.detgam, lapse = g.alpha;
  const bool mhd = par.mhd != 0;

  int num_nans = std::isnan(U(PHX_CRHO)) + std::isnan(U(PHX_CMOM)) + std::isnan(U(PHX_CENG));
  if (num_nans > 0) return res;
  const Real igdet = 1.0 / gdet;
  Real rhoflr = 0.0, epsflr;
  bounds.GetFloors(x1, x2, x3, rhoflr, epsflr);
  rhoflr *= par.c2p_floor_scale_fac;
  epsflr *= par.c2p_floor_scale_fac;
  Real gam_max, eps_max;
  bounds.GetCeilings(x1, x2, x3, gam_max, eps_max);
  const Real D = U(PHX_CRHO) * igdet;
  const Real tau = U(PHX_CENG) * igdet;
  const Real q = ratio(tau, D);

  Real bsq = 0.0, bsq_rpsq = 0.0, rbsq = 0.0, rsq = 0.0, bdotr = 0.0;
  Real rcon[3];
  Real rcov[] = {ratio(U(PHX_CMOM), U(PHX_CRHO)), ratio(U(PHX_CMOM + 1), U(PHX_CRHO)),
                 ratio(U(PHX_CMOM + 2), U(PHX_CRHO))};
  for (int ii = 0; ii < 3; ii++) {
    rcon[ii] = 0.0;
    for (int jj = 0; jj < 3; jj++) rcon[ii] += g.gamcon[ii][jj] * rcov[jj];
    rsq += rcon[ii] * rcov[ii];
  }
  Real bu[] = {0.0, 0.0, 0.0};
  if (mhd) {
    for (int ii = 0; ii < 3; ii++) P(PHX_PB + ii) = U(PHX_CB + ii) * igdet;
    const Real sD = 1.0 / std::sqrt(std::max(D, rhoflr));
    for (int ii = 0; ii < 3; ii++) {
      bu[ii] = P(PHX_PB + ii) * sD;
      bdotr += bu[ii] * rcov[ii];
    }
    for (int ii = 0; ii < 3; ii++)
      for (int jj = 0; jj < 3; jj++) bsq += g.gcov[ii + 1][jj + 1] * bu[ii] * bu[jj];
    bsq = std::max(0.0, bsq);
    rbsq = bdotr * bdotr;
    bsq_rpsq = bsq * rsq - rbsq;
  }
  const Real h0sq_ = 1.0;
  const Real zsq = rsq / h0sq_;
  Real v0sq = std::min(zsq / (1.0 + zsq), 1.0 - 1.0 / (gam_max * gam_max));
  Residual resid(D, q, bsq, bsq_rpsq, rsq, rbsq, v0sq, eos, bounds, x1, x2, x3,
                 par.c2p_floor_scale_fac);
  Real mu;
  if (fixed_mu) {
    mu = *fixed_mu;
    res.bracketed = true;
    res.iterations = 0;
    res.evals = 1;
  } else {
    RootFind root(par.c2p_max_iter);
    bool bracketed = true;
    mu = learned ? root.regula_falsi_learned(resid, learned[0], learned[1], learned[2], par.c2p_tol, guess,
                                             bracketed, res.learned_accepted)
                 : root.regula_falsi(resid, 0.0, 1.0, par.c2p_tol, guess, bracketed);
    res.bracketed = bracketed;
    res.iterations = root.iteration_count;
    res.evals = root.evals;
  }
  P(PHX_PMU) = mu;

  const Real x = resid.x_mu(mu);
  const Real rbarsq = resid.rbarsq_mu(mu, x);
  Real vsq = resid.vhatsq_mu(mu, rbarsq);
  Real iW = resid.iWhat_mu(vsq);
  P(PHX_PRHO) = resid.rhohat_mu(iW);
  const Real qbar = resid.qbar_mu(mu, x);
  Real W = 1.0 / iW;
  P(PHX_PENG) = resid.ehat_mu(mu, qbar, rbarsq, vsq, W);
  P(PHX_PTMP) = eos.TemperatureFromDensityInternalEnergy(P(PHX_PRHO), P(PHX_PENG));
  P(PHX_PENG) *= P(PHX_PRHO);
  P(PHX_PPRS) = eos.PressureFromDensityTemperature(P(PHX_PRHO), P(PHX_PTMP));
  P(PHX_PGM1) = eos.BulkModulusFromDensityTemperature(P(PHX_PRHO), P(PHX_PTMP)) / P(PHX_PPRS);

  Real vel[3];
  for (int ii = 0; ii < 3; ii++) {
    vel[ii] = W * mu * x * (rcon[ii] + mu * bdotr * bu[ii]);
    P(PHX_PVEL + ii) = vel[ii];
  }
  if (mhd)
    for (int ii = 0; ii < 3; ii++) bu[ii] = P(PHX_PB + ii);

  if (resid.used_bounds()) {
    Real S[3], bcons[3];
    Real Dn, taun;
    p2c(P(PHX_PRHO), vel, bu, P(PHX_PENG), P(PHX_PPRS), P(PHX_PGM1), g.gcov, g.gamcon,
        g.beta, g.alpha, gdet, Dn, S, bcons, taun, sig);
    U(PHX_CRHO) = Dn;
    U(PHX_CENG) = taun;
    for (int ii = 0; ii < 3; ii++) U(PHX_CMOM + ii) = S[ii];
  } else {
    for (int m = 0; m < 3; m++) vel[m] *= iW;
    bsq = 0.0;
    if (mhd) {
      Real bdotv = 0.0;
      for (int m = 0; m < 3; m++)
        for (int n = 0; n < 3; n++) {
          bsq += bu[m] * bu[n] * g.gcov[m + 1][n + 1];
          bdotv += bu[m] * vel[n] * g.gcov[m + 1][n + 1];
        }
      bsq = iW * iW * bsq + bdotv * bdotv;
    }
    signal_speeds(P(PHX_PRHO), P(PHX_PENG), P(PHX_PPRS), bsq, vel, vsq, P(PHX_PGM1), lapse,
                  g.beta, g.gamcon, sig);
  }
  num_nans = std::isnan(U(PHX_CRHO)) + std::isnan(U(PHX_CMOM)) + std::isnan(U(PHX_CENG));
  if (!res.bracketed) return res;
  if (num_nans > 0) return res;
  if (par.c2p_fail_on_floors && (resid.used_density_floor_ || resid.used_energy_floor_))
    return res;
  if (par.c2p_fail_on_ceilings && resid.used_gamma_max_) return res;
  res.success = true;
  return res;
}

// The zone (k, j, i) of a block: metric from the block's geometry, the
// floors at the cell centre, cell_sig for the active dimensions.
C2PResult con2prim_zone(const Blk &B, const Geom &G, const EOS &eos, const Bounds &bounds,
                        const phx_params &par, int k, int j, int i, Real guess_override,
                        bool use_override) {
  GeomPt g;
  G.at(CENT, k, j, i, g);
  const long long id = B.idx(k, j, i);
  const ZoneRef z{B.b->prim + id, B.b->cons + id, B.vs};
  const Real guess = use_override ? guess_override : z.P(PHX_PMU);
  Real sig[3];
  C2PResult r = con2prim_core(g, eos, bounds, par, B.Xc(1, i), B.Xc(2, j), B.Xc(3, k), z, guess, sig);
  if (r.evals == 0) return r;  // NaN input: nothing written (con2prim_robust.hpp:308-309)
  for (int d = 0; d < B.ndim; d++) B.b->cell_sig[d * B.vs + id] = sig[d];
  return r;
}

// ------------------------------------------------- reconstruction.hpp
inline Real mc(Real dm, Real dp, Real alpha) {
  const Real dc = (dm * dp > 0.0) * 0.5 * (dm + dp);
  return std::copysign(std::min(std::fabs(dc), alpha * std::min(std::fabs(dm), std::fabs(dp))),
                       dc);
}
inline void PiecewiseLinear(Real qm, Real q0, Real qp, Real &ql, Real &qr) {
  Real dq = qp - q0;
  dq = mc(q0 - qm, dq, 1.5);
  ql = q0 + 0.5 * dq;
  qr = q0 - 0.5 * dq;
}
inline void WENO5Z(Real q0, Real q1, Real q2, Real q3, Real q4, Real &ql, Real &qr) {
  constexpr Real w5alpha[3][3] = {{1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0},
                                  {-1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0},
                                  {1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0}};
  constexpr Real w5gamma[3] = {0.1, 0.6, 0.3};
  constexpr Real eps = 1e-100;
  constexpr Real thirteen_thirds = 13.0 / 3.0;
  Real a = q0 - 2 * q1 + q2;
  Real b = q0 - 4.0 * q1 + 3.0 * q2;
  Real beta0 = thirteen_thirds * a * a + b * b + eps;
  a = q1 - 2.0 * q2 + q3;
  b = q3 - q1;
  Real beta1 = thirteen_thirds * a * a + b * b + eps;
  a = q2 - 2.0 * q3 + q4;
  b = q4 - 4.0 * q3 + 3.0 * q2;
  Real beta2 = thirteen_thirds * a * a + b * b + eps;
  const Real tau5 = std::fabs(beta2 - beta0);
  beta0 = (beta0 + tau5) / beta0;
  beta1 = (beta1 + tau5) / beta1;
  beta2 = (beta2 + tau5) / beta2;
  Real w0 = w5gamma[0] * beta0 + eps;
  Real w1 = w5gamma[1] * beta1 + eps;
  Real w2 = w5gamma[2] * beta2 + eps;
  Real wsum = 1.0 / (w0 + w1 + w2);
  ql = w0 * (w5alpha[0][0] * q0 + w5alpha[0][1] * q1 + w5alpha[0][2] * q2);
  ql += w1 * (w5alpha[1][0] * q1 + w5alpha[1][1] * q2 + w5alpha[1][2] * q3);
  ql += w2 * (w5alpha[2][0] * q2 + w5alpha[2][1] * q3 + w5alpha[2][2] * q4);
  ql *= wsum;
  const Real alpha_l =
      3.0 * wsum * w0 * w1 * w2 /
          (w5gamma[2] * w0 * w1 + w5gamma[1] * w0 * w2 + w5gamma[0] * w1 * w2) +
      eps;
  w0 = w5gamma[0] * beta2 + eps;
  w1 = w5gamma[1] * beta1 + eps;
  w2 = w5gamma[2] * beta0 + eps;
  wsum = 1.0 / (w0 + w1 + w2);
  qr = w0 * (w5alpha[0][0] * q4 + w5alpha[0][1] * q3 + w5alpha[0][2] * q2);
  qr += w1 * (w5alpha[1][0] * q3 + w5alpha[1][1] * q2 + w5alpha[1][2] * q1);
  qr += w2 * (w5alpha[2][0] * q2 + w5alpha[2][1] * q1 + w5alpha[2][2] * q0);
  qr *= wsum;
  const Real alpha_r =
      3.0 * wsum * w0 * w1 * w2 /
          (w5gamma[2] * w0 * w1 + w5gamma[1] * w0 * w2 + w5gamma[0] * w1 * w2) +
      eps;
  Real dq = q3 - q2;
  dq = mc(q2 - q1, dq, 2.0);
  const Real alpha_lin = 2.0 * alpha_l * alpha_r / (alpha_l + alpha_r);
  ql = alpha_lin * ql + (1.0 - alpha_lin) * (q2 + 0.5 * dq);
  qr = alpha_lin * qr + (1.0 - alpha_lin) * (q2 - 0.5 * dq);
}
inline Real MINMOD(Real a, Real b) { return a * b > 0.0 ? (std::fabs(a) < std::fabs(b) ? a : b) : 0.0; }
inline Real Median(Real a, Real b, Real c) { return a + MINMOD(b - a, c - a); }
inline Real mp5_subcalc(Real Fjm2, Real Fjm1, Real Fj, Real Fjp1, Real Fjp2) {
  Real f, d2, d2p, d2m, dMMm, dMMp, scrh1, scrh2, Fmin, Fmax, fAV, fMD, fLC, fUL, fMP;
  constexpr Real alpha = 4.0, epsm = 1.e-12;
  f = 2.0 * Fjm2 - 13.0 * Fjm1 + 47.0 * Fj + 27.0 * Fjp1 - 3.0 * Fjp2;
  f /= 60.0;
  fMP = Fj + MINMOD(Fjp1 - Fj, alpha * (Fj - Fjm1));
  if ((f - Fj) * (f - fMP) <= epsm) return f;
  d2m = Fjm2 + Fj - 2.0 * Fjm1;
  d2 = Fjm1 + Fjp1 - 2.0 * Fj;
  d2p = Fj + Fjp2 - 2.0 * Fjp1;
  scrh1 = MINMOD(4.0 * d2 - d2p, 4.0 * d2p - d2);
  scrh2 = MINMOD(d2, d2p);
  dMMp = MINMOD(scrh1, scrh2);
  scrh1 = MINMOD(4.0 * d2m - d2, 4.0 * d2 - d2m);
  scrh2 = MINMOD(d2, d2m);
  dMMm = MINMOD(scrh1, scrh2);
  fUL = Fj + alpha * (Fj - Fjm1);
  fAV = 0.5 * (Fj + Fjp1);
  fMD = fAV - 0.5 * dMMp;
  fLC = 0.5 * (3.0 * Fj - Fjm1) + 4.0 / 3.0 * dMMm;
  scrh1 = std::fmin(Fj, Fjp1);
  scrh1 = std::fmin(scrh1, fMD);
  scrh2 = std::fmin(Fj, fUL);
  scrh2 = std::fmin(scrh2, fLC);
  Fmin = std::fmax(scrh1, scrh2);
  scrh1 = std::fmax(Fj, Fjp1);
  scrh1 = std::fmax(scrh1, fMD);
  scrh2 = std::fmax(Fj, fUL);
  scrh2 = std::fmax(scrh2, fLC);
  Fmax = std::fmin(scrh1, scrh2);
  f = Median(f, Fmin, Fmax);
  return f;
}
inline void MP5(Real q0, Real q1, Real q2, Real q3, Real q4, Real &ql, Real &qr) {
  ql = mp5_subcalc(q0, q1, q2, q3, q4);
  qr = mp5_subcalc(q4, q3, q2, q1, q0);
}

// --------------------------------------------------------- riemann.hpp
struct FaceGeom {
  Real alpha, gdet, gammadet, gcov[4][4], beta[3], gdd, X[4];
};
void face_geom(const Blk &B, const Geom &G, int d, int k, int j, int i, FaceGeom &fg) {
  const Loc loc = (Loc)d;
  GeomPt p;
  G.at(loc, k, j, i, p);
  fg.alpha = p.alpha;
  fg.gdet = G.DetG(p);
  fg.gammadet = p.detgam;
  fg.gdd = p.gamcon[d - 1][d - 1];
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) fg.gcov[mu][nu] = p.gcov[mu][nu];
  for (int m = 0; m < 3; m++) fg.beta[m] = p.beta[m];
  fg.X[1] = (d == 1 ? B.Xf(1, i) : B.Xc(1, i));
  fg.X[2] = (d == 2 ? B.Xf(2, j) : B.Xc(2, j));
  fg.X[3] = (d == 3 ? B.Xf(3, k) : B.Xc(3, k));
}

// riemann.hpp:88-209; q[] = the PHX_NRECON face values
void prim_to_flux(int d, const FaceGeom &g, const Real q[], const Bounds &bounds, bool mhd,
                  Real &vm, Real &vp, Real *U, Real *F, Real sie_max, Real gam_max) {
  const int dir = d - 1;
  Real rho_floor = q[PHX_PRHO];
  Real sie_floor;
  bounds.GetFloors(g.X[1], g.X[2], g.X[3], rho_floor, sie_floor);
  const Real rho = std::max(q[PHX_PRHO], rho_floor);
  Real vpcon[] = {q[PHX_PVEL], q[PHX_PVEL + 1], q[PHX_PVEL + 2]};
  Real W = GetLorentzFactor(vpcon, g.gcov);
  if (W > gam_max) {
    const Real rescale = std::sqrt((gam_max * gam_max - 1.) / (W * W - 1.));
    for (int ii = 0; ii < 3; ii++) vpcon[ii] *= rescale;
  }
  Real vcon[] = {vpcon[0] / W, vpcon[1] / W, vpcon[2] / W};
  const Real &vel = vcon[dir];
  Real Bcon[] = {0.0, 0.0, 0.0};
  const Real u = (q[PHX_PENG] / rho > sie_floor
                      ? (q[PHX_PENG] / rho > sie_max ? rho * sie_max : q[PHX_PENG])
                      : rho * sie_floor);
  const Real P = std::max(q[PHX_PPRS], 0.0);
  const Real gamma1 = q[PHX_PGM1];
  if (mhd)
    for (int m = 0; m < 3; m++) Bcon[m] = q[PHX_PB + m];
  Real BdotB = 0.0, Bdotv = 0.0, vsq = 0.0;
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++) {
      vsq += g.gcov[m + 1][n + 1] * vcon[m] * vcon[n];
      Bdotv += g.gcov[m + 1][n + 1] * Bcon[m] * vcon[n];
      BdotB += g.gcov[m + 1][n + 1] * Bcon[m] * Bcon[n];
    }
  const Real vsq_max = 1.0 - 1.0 / (gam_max * gam_max);
  if (vsq > vsq_max) {
    Real scale = vsq_max / vsq;
    vsq *= scale;
    scale = std::sqrt(scale);
    Bdotv *= scale;
    for (int m = 0; m < 3; m++) vcon[m] *= scale;
  }
  W = 1.0 / std::sqrt(1 - vsq);
  const Real vtil = vel - g.beta[dir] / g.alpha;
  U[PHX_CRHO] = rho * W;
  F[PHX_CRHO] = U[PHX_CRHO] * vtil;
  Real b0 = W * Bdotv;
  const Real bsq = (BdotB + b0 * b0) / (W * W);
  const Real rhohWsq = (rho + u + P) * W * W;
  const Real bsqWsq = bsq * W * W;
  for (int m = 0; m < 3; m++) {
    Real bcovm = g.gcov[m + 1][0] * b0 / g.alpha;
    Real vcovm = 0.0;
    for (int n = 1; n < 4; n++) {
      bcovm += g.gcov[m + 1][n] * (Bcon[n - 1] / W + b0 * (vcon[n - 1] - g.beta[n - 1] / g.alpha));
      vcovm += g.gcov[m + 1][n] * vcon[n - 1];
    }
    U[PHX_CMOM + m] = (rhohWsq + bsqWsq) * vcovm - b0 * bcovm;
    F[PHX_CMOM + m] = U[PHX_CMOM + m] * vtil + (P + 0.5 * bsq) * (dir == m) - bcovm * Bcon[dir] / W;
  }
  U[PHX_CENG] = rhohWsq + bsqWsq - (P + 0.5 * bsq) - b0 * b0 - U[PHX_CRHO];
  F[PHX_CENG] = U[PHX_CENG] * vtil + (P + 0.5 * bsq) * vel - Bdotv * Bcon[dir];
  if (mhd)
    for (int m = 0; m < 3; m++) {
      U[PHX_CB + m] = Bcon[m];
      F[PHX_CB + m] = U[PHX_CB + m] * vtil - Bcon[dir] * (vcon[m] - g.beta[m] / g.alpha);
    }
  const Real vasq = bsqWsq / make_positive(rhohWsq + bsqWsq);
  const Real cssq = make_bounded(gamma1 * P * W * W / make_positive(rhohWsq), 0.0, 1.0);
  Real cmsq = make_bounded(cssq + vasq * (1.0 - cssq), 0.0, 1.0);
  const Real vcoff = g.alpha / (1.0 - vsq * cmsq);
  const Real v0 = vel * (1.0 - cmsq);
  const Real vpm = std::sqrt(make_positive(cmsq * (1.0 - vsq) * (g.gdd * (1.0 - vsq * cmsq) - vel * v0)));
  vp = vcoff * (v0 + vpm) - g.beta[dir];
  vm = vcoff * (v0 - vpm) - g.beta[dir];
}

// ---------------------------------------------------------- fluid.cpp
// CalculateFluxes (fluid.cpp:659-773): the reference's two loops, verbatim
// in structure, with the ql/qr arrays as scratch.
void calculate_fluxes(const phx_params &par, const phx_block *blk) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  Bounds bounds(par);
  const int ndim = B.ndim;
  const int dk = (ndim == 3 ? 1 : 0), dj = (ndim > 1 ? 1 : 0);
  const long long N = B.N;
  const int nrecon = PHX_NRECON;
  std::vector<Real> ql((size_t)ndim * nrecon * N, 0.0), qr((size_t)ndim * nrecon * N, 0.0);
  auto QL = [&](int d, int n, long long id) -> Real & { return ql[((size_t)d * nrecon + n) * N + id]; };
  auto QR = [&](int d, int n, long long id) -> Real & { return qr[((size_t)d * nrecon + n) * N + id]; };
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
  const int nvr = par.mhd ? nrecon : nrecon;  // B slots are present either way
#pragma omp parallel for collapse(2) schedule(static)
  for (int n = 0; n < nvr; n++)
    for (int k = ks - dk; k <= ke + dk; k++)
      for (int j = js - dj; j <= je + dj; j++)
        for (int i = is - 1; i <= ie + 1; i++) {
          auto v = [&](int kk, int jj, int ii) { return B.P(n, kk, jj, ii); };
          Real l, r;
          for (int d = 0; d < ndim; d++) {
            const int di = d == 0, djj = d == 1, dkk = d == 2;
            const Real qm2 = v(k - 2 * dkk, j - 2 * djj, i - 2 * di);
            const Real qm1 = v(k - dkk, j - djj, i - di);
            const Real q0 = v(k, j, i);
            const Real qp1 = v(k + dkk, j + djj, i + di);
            const Real qp2 = v(k + 2 * dkk, j + 2 * djj, i + 2 * di);
            switch (par.recon) {
            case PHX_RECON_WENO5Z: WENO5Z(qm2, qm1, q0, qp1, qp2, l, r); break;
            case PHX_RECON_MP5: MP5(qm2, qm1, q0, qp1, qp2, l, r); break;
            case PHX_RECON_LINEAR: PiecewiseLinear(qm1, q0, qp1, l, r); break;
            default: l = r = q0; break;
            }
            // ql at the face above the cell, qr at the face of the cell
            QL(d, n, B.idx(k + dkk, j + djj, i + di)) = l;
            QR(d, n, B.idx(k, j, i)) = r;
          }
        }
#pragma omp parallel for collapse(2) schedule(static)
  for (int d = 1; d <= ndim; d++)
    for (int k = ks - dk; k <= ke + dk; k++)
      for (int j = js - dj; j <= je + dj; j++)
        for (int i = is - 1; i <= ie + 1; i++) {
          const long long id = B.idx(k, j, i);
          FaceGeom fg;
          face_geom(B, G, d, k, j, i, fg);
          Real gam_max, sie_max;
          bounds.GetCeilings(fg.X[1], fg.X[2], fg.X[3], gam_max, sie_max);
          Real qlv[PHX_NRECON], qrv[PHX_NRECON];
          for (int n = 0; n < nrecon; n++) {
            qlv[n] = QL(d - 1, n, id);
            qrv[n] = QR(d - 1, n, id);
          }
          Real Ul[PHX_NCONS] = {0}, Ur[PHX_NCONS] = {0}, Fl[PHX_NCONS] = {0}, Fr[PHX_NCONS] = {0};
          Real vml, vpl, vmr, vpr;
          prim_to_flux(d, fg, qlv, bounds, par.mhd != 0, vml, vpl, Ul, Fl, sie_max, gam_max);
          prim_to_flux(d, fg, qrv, bounds, par.mhd != 0, vmr, vpr, Ur, Fr, sie_max, gam_max);
          const int ncons = par.mhd ? PHX_NCONS : 5;
          Real sigv;
          if (par.riemann == PHX_RIEMANN_LLF) {
            const Real cmax = std::max(std::max(-vml, vpl), std::max(-vmr, vpr));
            for (int m = 0; m < ncons; m++)
              B.F(d - 1, m, k, j, i) = 0.5 * ((Fl[m] + Fr[m]) * fg.gdet - cmax * ((Ur[m] - Ul[m]) * fg.gammadet));
            sigv = cmax;
          } else {
            const Real cl = std::min(std::min(vml, vmr), 0.0);
            const Real cr = std::max(std::max(vpl, vpr), 0.0);
            const Real crcl = cr * cl;
            const Real inv_cr_cl = ratio(1.0, cr - cl);
            for (int m = 0; m < ncons; m++)
              B.F(d - 1, m, k, j, i) =
                  ((cr * Fl[m] - cl * Fr[m]) * fg.gdet + crcl * (Ur[m] - Ul[m]) * fg.gammadet) * inv_cr_cl;
            sigv = std::max(-cl, cr);
          }
          blk->face_sig[(d - 1) * B.vs + id] = sigv;
        }
}

// FluxCT (fluid.cpp:775-841)
void flux_ct(const phx_block *blk) {
  Blk B(blk);
  const int ndim = B.ndim;
  if (ndim == 1) return;
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
  auto emf = [&](int c, int k, int j, int i) -> Real & { return blk->emf[c * B.vs + B.idx(k, j, i)]; };
  auto F = [&](int d, int m, int k, int j, int i) -> Real & { return B.F(d, PHX_CB + m, k, j, i); };
  if (ndim == 2) {
    for (int k = ks; k <= ke; k++)
      for (int j = js; j <= je + 1; j++)
        for (int i = is; i <= ie + 1; i++)
          emf(0, k, j, i) = 0.25 * (F(0, 1, k, j, i) + F(0, 1, k, j - 1, i) - F(1, 0, k, j, i) - F(1, 0, k, j, i - 1));
    for (int k = ks; k <= ke; k++)
      for (int j = js; j <= je + 1; j++)
        for (int i = is; i <= ie + 1; i++) {
          F(0, 0, k, j, i) = 0.0;
          F(0, 1, k, j, i) = 0.5 * (emf(0, k, j, i) + emf(0, k, j + 1, i));
          F(1, 0, k, j, i) = -0.5 * (emf(0, k, j, i) + emf(0, k, j, i + 1));
          F(1, 1, k, j, i) = 0.0;
        }
  } else {
#pragma omp parallel for schedule(static)
    for (int k = ks; k <= ke + 1; k++)
      for (int j = js; j <= je + 1; j++)
        for (int i = is; i <= ie + 1; i++) {
          emf(0, k, j, i) = 0.25 * (F(1, 2, k, j, i) + F(1, 2, k - 1, j, i) - F(2, 1, k, j, i) - F(2, 1, k, j - 1, i));
          emf(1, k, j, i) = -0.25 * (F(0, 2, k, j, i) + F(0, 2, k - 1, j, i) - F(2, 0, k, j, i) - F(2, 0, k, j, i - 1));
          emf(2, k, j, i) = 0.25 * (F(0, 1, k, j, i) + F(0, 1, k, j - 1, i) - F(1, 0, k, j, i) - F(1, 0, k, j, i - 1));
        }
#pragma omp parallel for schedule(static)
    for (int k = ks; k <= ke + 1; k++)
      for (int j = js; j <= je + 1; j++)
        for (int i = is; i <= ie + 1; i++) {
          F(0, 0, k, j, i) = 0.0;
          F(0, 1, k, j, i) = 0.5 * (emf(2, k, j, i) + emf(2, k, j + 1, i));
          F(0, 2, k, j, i) = -0.5 * (emf(1, k, j, i) + emf(1, k + 1, j, i));
          F(1, 0, k, j, i) = -0.5 * (emf(2, k, j, i) + emf(2, k, j, i + 1));
          F(1, 1, k, j, i) = 0.0;
          F(1, 2, k, j, i) = 0.5 * (emf(0, k, j, i) + emf(0, k + 1, j, i));
          F(2, 0, k, j, i) = 0.5 * (emf(1, k, j, i) + emf(1, k, j, i + 1));
          F(2, 1, k, j, i) = -0.5 * (emf(0, k, j, i) + emf(0, k, j + 1, i));
          F(2, 2, k, j, i) = 0.0;
        }
  }
}

// tmunu.hpp:62-131 (StressEnergyTensorCon::operator()) + fluid.cpp:593-654
void sources(const phx_params &par, const phx_block *blk) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
  const bool mhd = par.mhd != 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
        GeomPt p;
        G.at(CENT, k, j, i, p);
        // GetTmunuTerms_: gammacov = spatial part of gcov
        Real gam[3][3];
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) gam[a][b] = p.gcov[a + 1][b + 1];
        Real vp[3] = {B.P(PHX_PVEL, k, j, i), B.P(PHX_PVEL + 1, k, j, i), B.P(PHX_PVEL + 2, k, j, i)};
        Real vsqw = 0.;
        for (int ii = 0; ii < 3; ii++)
          for (int jj = 0; jj < 3; jj++) vsqw += gam[ii][jj] * vp[ii] * vp[jj];
        const Real W = std::sqrt(1. + vsqw);
        auto bfield = [&](int l) { return mhd ? B.P(PHX_PB + l - 1, k, j, i) : 0.0; };
        Real Bdotv = 0.0, Bsq = 0.0;
        for (int ii = 0; ii < 3; ii++)
          for (int jj = 0; jj < 3; jj++) {
            const Real bi = bfield(ii + 1), bj = bfield(jj + 1);
            Bdotv += bi * (vp[jj] / W) * gam[ii][jj];
            Bsq += bi * bj * gam[ii][jj];
          }
        const Real iW = ratio(1., W);
        const Real alpha = p.alpha;
        Real u[4], bb[4];
        u[0] = ratio(W, std::abs(alpha));
        bb[0] = u[0] * Bdotv;
        for (int l = 1; l < 4; ++l) {
          u[l] = vp[l - 1] - u[0] * p.beta[l - 1];
          bb[l] = iW * (bfield(l) + alpha * bb[0] * u[l]);
        }
        const Real bsq = Bsq * iW * iW + Bdotv * Bdotv;
        Real gi[4][4];
        G.SpacetimeMetricInverse(p, gi);
        const Real rho = B.P(PHX_PRHO, k, j, i), uu = B.P(PHX_PENG, k, j, i), P = B.P(PHX_PPRS, k, j, i);
        const Real A = rho + uu + P + bsq;
        const Real Bt = P + 0.5 * bsq;
        Real T[4][4];
        for (int mu = 0; mu < 4; mu++)
          for (int nu = 0; nu < 4; nu++) T[mu][nu] = A * u[mu] * u[nu] + Bt * gi[mu][nu] - bb[mu] * bb[nu];
        const Real gdet = G.DetG(p);
        Real dg[4][4][4], gm[4][4][4];
        G.MetricDerivative(k, j, i, dg);
        for (int a = 0; a < 4; a++)  // geometry_utils.hpp:72-78
          for (int b = 0; b < 4; b++)
            for (int c = 0; c < 4; c++) gm[a][b][c] = 0.5 * (dg[b][a][c] + dg[c][a][b] - dg[b][c][a]);
        for (int l = 0; l < 3; l++) {
          Real src_mom = 0.0;
          for (int m = 0; m < 4; m++)
            for (int n = 0; n < 4; n++) src_mom += T[m][n] * (dg[n][l + 1][m] - gm[l + 1][n][m]);
          blk->src[l * B.vs + B.idx(k, j, i)] = gdet * src_mom;
        }
        Real TGam = 0.0;
        const Real inv_alpha2 = ratio(1, alpha * alpha);
        Real gcon0[4] = {-inv_alpha2, inv_alpha2 * p.beta[0], inv_alpha2 * p.beta[1], inv_alpha2 * p.beta[2]};
        for (int m = 0; m < 4; m++)
          for (int n = 0; n < 4; n++) {
            Real gam0 = 0;
            for (int r = 0; r < 4; r++) gam0 += gcon0[r] * gm[r][m][n];
            TGam += T[m][n] * gam0;
          }
        Real Ta = 0.0, da[4];
        G.GradLnAlpha(k, j, i, da);
        for (int m = 0; m < 4; m++) Ta += T[m][0] * da[m];
        blk->src[3 * B.vs + B.idx(k, j, i)] = gdet * alpha * (Ta - TGam);
      }
}


// fixup_c2p.cpp:170-353 (ConservedToPrimitiveFixupImpl, fluid part) on the
// interior.  Neighbour prims are read from a snapshot taken before the loop,
// so the result does not depend on the order zones are fixed in.
void c2p_fixup(const phx_params &par, const phx_block *blk) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  Bounds bounds(par);
  EOS eos{par.gm1, par.Cv};
  if (!par.enable_c2p_fixup) return;
  const int ndim = B.ndim;
  const bool mhd = par.mhd != 0;
  std::vector<double> snap(blk->prim, blk->prim + (size_t)PHX_NPRIM * B.vs);
  auto S = [&](int v, int k, int j, int i) { return snap[v * B.vs + B.idx(k, j, i)]; };
  auto fl = [&](int k, int j, int i) { return blk->fail[B.idx(k, j, i)]; };
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
        if (fl(k, j, i) != 0.0) continue;
        Real gamma_max, e_max;
        bounds.GetCeilings(B.Xc(1, i), B.Xc(2, j), B.Xc(3, k), gamma_max, e_max);
        auto fixv = [&](int iv, Real inv_mask_sum) {
          Real s = fl(k, j, i - 1) * S(iv, k, j, i - 1) + fl(k, j, i + 1) * S(iv, k, j, i + 1);
          if (ndim > 1) {
            s += fl(k, j - 1, i) * S(iv, k, j - 1, i) + fl(k, j + 1, i) * S(iv, k, j + 1, i);
            if (ndim == 3) s += fl(k - 1, j, i) * S(iv, k - 1, j, i) + fl(k + 1, j, i) * S(iv, k + 1, j, i);
          }
          return inv_mask_sum * s;
        };
        Real num_valid = fl(k, j, i - 1) + fl(k, j, i + 1);
        if (ndim > 1) num_valid += fl(k, j - 1, i) + fl(k, j + 1, i);
        if (ndim == 3) num_valid += fl(k - 1, j, i) + fl(k + 1, j, i);
        if (num_valid > 0.5 && !par.c2p_failure_strategy_floors) {
          const Real norm = 1.0 / num_valid;
          B.P(PHX_PRHO, k, j, i) = fixv(PHX_PRHO, norm);
          for (int pv = 0; pv < 3; pv++) B.P(PHX_PVEL + pv, k, j, i) = fixv(PHX_PVEL + pv, norm);
          B.P(PHX_PENG, k, j, i) = fixv(PHX_PENG, norm);
          B.P(PHX_PRHO, k, j, i) = std::max<Real>(B.P(PHX_PRHO, k, j, i), 100. * SMALL);
          B.P(PHX_PENG, k, j, i) = std::max<Real>(B.P(PHX_PENG, k, j, i), 100. * SMALL);
        } else {
          B.P(PHX_PRHO, k, j, i) = 100. * SMALL;
          B.P(PHX_PENG, k, j, i) = 100. * SMALL;
          for (int ii = 0; ii < 3; ii++) B.P(PHX_PVEL + ii, k, j, i) = 0.;
        }
        GeomPt g;
        G.at(CENT, k, j, i, g);
        Real vpcon[3] = {B.P(PHX_PVEL, k, j, i), B.P(PHX_PVEL + 1, k, j, i), B.P(PHX_PVEL + 2, k, j, i)};
        Real W = GetLorentzFactor(vpcon, g.gcov);
        if (W > gamma_max) {
          const Real rescale = std::sqrt(gamma_max * gamma_max - 1.) / (W * W - 1.);
          for (int ii = 0; ii < 3; ii++) vpcon[ii] *= rescale;
          for (int ii = 0; ii < 3; ii++) B.P(PHX_PVEL + ii, k, j, i) = vpcon[ii];
          W = gamma_max;
        }
        Real &rho = B.P(PHX_PRHO, k, j, i);
        B.P(PHX_PTMP, k, j, i) = eos.TemperatureFromDensityInternalEnergy(rho, ratio(B.P(PHX_PENG, k, j, i), rho));
        B.P(PHX_PPRS, k, j, i) = eos.PressureFromDensityTemperature(rho, B.P(PHX_PTMP, k, j, i));
        B.P(PHX_PGM1, k, j, i) =
            ratio(eos.BulkModulusFromDensityTemperature(rho, B.P(PHX_PTMP, k, j, i)), B.P(PHX_PPRS, k, j, i));
        Real bp[3] = {0.0, 0.0, 0.0};
        if (mhd)
          for (int ii = 0; ii < 3; ii++) bp[ii] = B.P(PHX_PB + ii, k, j, i);
        Real Sv[3], bc[3], sig[3], D, tau;
        p2c(rho, vpcon, bp, B.P(PHX_PENG, k, j, i), B.P(PHX_PPRS, k, j, i), B.P(PHX_PGM1, k, j, i), g.gcov,
            g.gamcon, g.beta, g.alpha, g.detgam, D, Sv, bc, tau, sig);
        B.U(PHX_CRHO, k, j, i) = D;
        B.U(PHX_CENG, k, j, i) = tau;
        for (int ii = 0; ii < 3; ii++) B.U(PHX_CMOM + ii, k, j, i) = Sv[ii];
        for (int d = 0; d < ndim; d++) blk->cell_sig[d * B.vs + B.idx(k, j, i)] = sig[d];
      }
}

// fixup.cpp:370-540 (ApplyFloorsImpl, fluid part) over the given range.
// Returns the number of zones whose re-inversion failed (set to floors).
// flag (optional, [N]): 1 where floors or ceilings acted, else 0.
long long apply_floors(const phx_params &par, const phx_block *blk, phx_range ib, phx_range jb, phx_range kb,
                       double *flag = nullptr) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  Bounds bounds(par);
  EOS eos{par.gm1, par.Cv};
  if (!(par.enable_floors || par.enable_c2p_fixup || (par.enable_mhd_floors && par.mhd))) return 0;
  const bool mhd_floors = par.enable_mhd_floors && par.mhd;
  const bool mhd = par.mhd != 0;
  long long nfail = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) reduction(+ : nfail)
  for (int k = kb.s; k <= kb.e; k++)
    for (int j = jb.s; j <= jb.e; j++)
      for (int i = ib.s; i <= ib.e; i++) {
        auto P = [&](int v) -> Real & { return B.P(v, k, j, i); };
        auto U = [&](int v) -> Real & { return B.U(v, k, j, i); };
        const Real x1 = B.Xc(1, i), x2 = B.Xc(2, j), x3 = B.Xc(3, k);
        Real rho_floor, sie_floor;
        bounds.GetFloors(x1, x2, x3, rho_floor, sie_floor);
        Real gamma_max, e_max;
        bounds.GetCeilings(x1, x2, x3, gamma_max, e_max);
        Real bsqorho_max, bsqou_max;
        bounds.GetMHDCeilings(x1, x2, x3, bsqorho_max, bsqou_max);
        Real rho_floor_max = rho_floor;
        Real u_floor_max = rho_floor * sie_floor;
        bool floor_applied = false, ceiling_applied = false;
        GeomPt g;
        G.at(CENT, k, j, i, g);
        if (mhd_floors) {
          Real Bsq = 0.0, Bdotv = 0.0;
          const Real vp[3] = {P(PHX_PVEL), P(PHX_PVEL + 1), P(PHX_PVEL + 2)};
          const Real bp[3] = {P(PHX_PB), P(PHX_PB + 1), P(PHX_PB + 2)};
          const Real W = GetLorentzFactor(vp, g.gcov);
          const Real iW = 1.0 / W;
          for (int ii = 0; ii < 3; ii++)
            for (int jj = 0; jj < 3; jj++) {
              Bsq += g.gcov[ii + 1][jj + 1] * bp[ii] * bp[jj];
              Bdotv += g.gcov[ii + 1][jj + 1] * bp[ii] * vp[jj];
            }
          Real bcon0 = W * Bdotv / g.alpha;
          const Real bsq = (Bsq + g.alpha * g.alpha * bcon0 * bcon0) * iW * iW;
          rho_floor_max = std::max<Real>(rho_floor_max, bsq / bsqorho_max);
          u_floor_max = std::max<Real>(u_floor_max, bsq / bsqou_max);
          rho_floor_max = std::max<Real>(rho_floor_max, std::max<Real>(P(PHX_PENG), u_floor_max) / e_max);
        }
        Real drho = rho_floor_max - P(PHX_PRHO);
        Real du = u_floor_max - P(PHX_PENG);
        if (drho > 0. || du > 0.) {
          floor_applied = true;
          drho = std::max<Real>(drho, du / sie_floor);
          du = std::max<Real>(du, sie_floor * drho);
        }
        Real bp[3] = {0, 0, 0};
        if (mhd)
          for (int ii = 0; ii < 3; ii++) bp[ii] = P(PHX_PB + ii);
        Real dS[3], dB[3], dcrho, dtau;
        if (floor_applied) {
          Real vp_normalobs[3] = {0, 0, 0};
          Real dprs = eos.PressureFromDensityInternalEnergy(drho, ratio(du, drho));
          // BulkModulusFromDensityInternalEnergy = (gm1 + 1) gm1 rho sie
          Real dgm1 = ratio(std::max(0.0, (eos.gm1 + 1) * eos.gm1 * drho * ratio(du, drho)), dprs);
          p2c(drho, vp_normalobs, bp, du, dprs, dgm1, g.gcov, g.gamcon, g.beta, g.alpha, g.detgam, dcrho, dS, dB,
              dtau, nullptr);
          U(PHX_CRHO) += dcrho;
          for (int ii = 0; ii < 3; ii++) U(PHX_CMOM + ii) += dS[ii];
          U(PHX_CENG) += dtau;
          C2PResult r = con2prim_zone(B, G, eos, bounds, par, k, j, i, 0.0, false);
          if (!r.success) {
            nfail++;
            P(PHX_PRHO) = drho;
            for (int ii = 0; ii < 3; ii++) P(PHX_PVEL + ii) = vp_normalobs[ii];
            P(PHX_PENG) = du;
            P(PHX_PTMP) = eos.TemperatureFromDensityInternalEnergy(P(PHX_PRHO), P(PHX_PENG) / P(PHX_PRHO));
            Real Dn, taun;
            p2c(drho, vp_normalobs, bp, du, dprs, dgm1, g.gcov, g.gamcon, g.beta, g.alpha, g.detgam, Dn, dS, dB,
                taun, nullptr);
            U(PHX_CRHO) = Dn;
            U(PHX_CENG) = taun;
            for (int ii = 0; ii < 3; ii++) U(PHX_CMOM + ii) = dS[ii];
          }
        }
        Real vpcon[3] = {P(PHX_PVEL), P(PHX_PVEL + 1), P(PHX_PVEL + 2)};
        const Real W = GetLorentzFactor(vpcon, g.gcov);
        if (W > gamma_max || P(PHX_PENG) / P(PHX_PRHO) > e_max) ceiling_applied = true;
        if (ceiling_applied) {
          const Real rescale = std::sqrt(gamma_max * gamma_max - 1.) / (W * W - 1.);
          for (int ii = 0; ii < 3; ii++) vpcon[ii] *= rescale;
          for (int ii = 0; ii < 3; ii++) P(PHX_PVEL + ii) = vpcon[ii];
          Real Dn, taun;
          p2c(P(PHX_PRHO), vpcon, bp, P(PHX_PENG), P(PHX_PPRS), P(PHX_PGM1), g.gcov, g.gamcon, g.beta, g.alpha,
              g.detgam, Dn, dS, dB, taun, nullptr);
          U(PHX_CRHO) = Dn;
          U(PHX_CENG) = taun;
          for (int ii = 0; ii < 3; ii++) U(PHX_CMOM + ii) = dS[ii];
        }
        if (flag) flag[B.idx(k, j, i)] = (floor_applied || ceiling_applied) ? 1.0 : 0.0;
        if (floor_applied || ceiling_applied) {
          P(PHX_PTMP) = eos.TemperatureFromDensityInternalEnergy(P(PHX_PRHO), ratio(P(PHX_PENG), P(PHX_PRHO)));
          P(PHX_PPRS) = eos.PressureFromDensityTemperature(P(PHX_PRHO), P(PHX_PTMP));
          P(PHX_PGM1) = ratio(eos.BulkModulusFromDensityTemperature(P(PHX_PRHO), P(PHX_PTMP)), P(PHX_PPRS));
        }
      }
  return nfail;
}
}  // namespace orc

using namespace orc;

extern "C" {

int orc_abi_version() { return PHX_ABI_VERSION; }

// fluid.cpp:368-449 PrimitiveToConservedRegion
void orc_prim_to_con(const phx_params *par, const phx_block *blk, phx_range ib, phx_range jb,
                     phx_range kb) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  const bool mhd = par->mhd != 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = kb.s; k <= kb.e; k++)
    for (int j = jb.s; j <= jb.e; j++)
      for (int i = ib.s; i <= ib.e; i++) {
        GeomPt g;
        G.at(CENT, k, j, i, g);
        Real S[3], bcons[3], sig[3];
        const Real vel[] = {B.P(PHX_PVEL, k, j, i), B.P(PHX_PVEL + 1, k, j, i), B.P(PHX_PVEL + 2, k, j, i)};
        Real bp[3] = {0.0, 0.0, 0.0};
        if (mhd)
          for (int d = 0; d < 3; ++d) bp[d] = B.P(PHX_PB + d, k, j, i);
        Real D, tau;
        p2c(B.P(PHX_PRHO, k, j, i), vel, bp, B.P(PHX_PENG, k, j, i), B.P(PHX_PPRS, k, j, i),
            B.P(PHX_PGM1, k, j, i), g.gcov, g.gamcon, g.beta, g.alpha, g.detgam, D, S, bcons,
            tau, sig);
        B.U(PHX_CRHO, k, j, i) = D;
        B.U(PHX_CENG, k, j, i) = tau;
        for (int d = 0; d < 3; ++d) B.U(PHX_CMOM + d, k, j, i) = S[d];
        if (mhd)
          for (int d = 0; d < 3; ++d) B.U(PHX_CB + d, k, j, i) = bcons[d];
        for (int d = 0; d < B.ndim; d++) blk->cell_sig[d * B.vs + B.idx(k, j, i)] = sig[d];
      }
}

// fluid.cpp:477-517 ConservedToPrimitiveRobust.  iters (optional, [N]) gets
// the root-find iteration count per zone; guess (optional, [N]) replaces the
// c2p_mu warm start.  Returns the number of unbracketed zones.
long long orc_con_to_prim(const phx_params *par, const phx_block *blk, phx_range ib,
                          phx_range jb, phx_range kb, int *iters, const double *guess,
                          long long *evals_total) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  Bounds bounds(*par);
  EOS eos{par->gm1, par->Cv};
  long long unbr = 0, ev = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) reduction(+ : unbr, ev)
  for (int k = kb.s; k <= kb.e; k++)
    for (int j = jb.s; j <= jb.e; j++)
      for (int i = ib.s; i <= ib.e; i++) {
        const long long id = B.idx(k, j, i);
        C2PResult r = con2prim_zone(B, G, eos, bounds, *par, k, j, i, guess ? guess[id] : 0.0,
                                    guess != nullptr);
        blk->fail[id] = r.success ? 1.0 : 0.0;
        if (iters) iters[id] = r.iterations;
        if (!r.bracketed) unbr++;
        ev += r.evals;
      }
  if (evals_total) *evals_total = ev;
  return unbr;
}

// Point geometry of zone q from geom [21][n] (null = Minkowski).
static void zone_geom(const double *geom, long long n, long long q, GeomPt &g) {
  if (!geom) {
    Geom(nullptr, nullptr).at(CENT, 0, 0, 0, g);
    return;
  }
  g.alpha = geom[PHX_G_ALPHA * n + q];
  for (int d = 0; d < 3; d++) g.beta[d] = geom[(PHX_G_BETA + d) * n + q];
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) g.gcov[mu][nu] = geom[(PHX_G_GCOV + flatten2(mu, nu)) * n + q];
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) g.gamcon[a][b] = geom[(PHX_G_GAMCON + flatten2s(a, b)) * n + q];
  g.detgam = geom[PHX_G_DETGAM * n + q];
}

// prim2con.hpp:25-102 over n independent zones (prim [12][n] -> cons [8][n]).
void orc_prim_to_con_zones(const phx_params *par, long long n, const double *prim, const double *geom,
                           double *cons, double *cell_sig) {
  const bool mhd = par->mhd != 0;
#pragma omp parallel for schedule(static)
  for (long long q = 0; q < n; q++) {
    GeomPt g;
    zone_geom(geom, n, q, g);
    auto P = [&](int v) { return prim[v * n + q]; };
    Real S[3], bcons[3], sig[3];
    const Real vel[] = {P(PHX_PVEL), P(PHX_PVEL + 1), P(PHX_PVEL + 2)};
    Real bp[3] = {0.0, 0.0, 0.0};
    if (mhd)
      for (int d = 0; d < 3; ++d) bp[d] = P(PHX_PB + d);
    Real D, tau;
    p2c(P(PHX_PRHO), vel, bp, P(PHX_PENG), P(PHX_PPRS), P(PHX_PGM1), g.gcov, g.gamcon, g.beta, g.alpha, g.detgam,
        D, S, bcons, tau, sig);
    cons[PHX_CRHO * n + q] = D;
    cons[PHX_CENG * n + q] = tau;
    for (int d = 0; d < 3; ++d) cons[(PHX_CMOM + d) * n + q] = S[d];
    if (mhd)
      for (int d = 0; d < 3; ++d) cons[(PHX_CB + d) * n + q] = bcons[d];
    if (cell_sig)
      for (int d = 0; d < 3; d++) cell_sig[d * n + q] = sig[d];
  }
}

// con2prim over n independent zones: cons/prim [var][n], geom [21][n] per
// zone (null = Minkowski), coords [3][n] (null = 0; used by the floors),
// fail [n], cell_sig [3][n] (null = not written).  The same per-zone
// inversion as a block zone.  bracket [3][n] (optional): a learned start
// (m, lo, hi) per zone for RootFind::regula_falsi_learned.
// con2prim of independent zones finished at the given roots mu[n] (no root
// find): the reference's finish arithmetic at another build's roots.
void orc_con_to_prim_zones_at_mu(const phx_params *par, long long n, double *cons, double *prim,
                                 const double *geom, const double *mu, double *fail) {
  Bounds bounds(*par);
  EOS eos{par->gm1, par->Cv};
#pragma omp parallel for schedule(static)
  for (long long q = 0; q < n; q++) {
    GeomPt g;
    zone_geom(geom, n, q, g);
    const ZoneRef z{prim + q, cons + q, n};
    Real sig[3];
    const Real m = mu[q];
    C2PResult r = con2prim_core(g, eos, bounds, *par, 0.0, 0.0, 0.0, z, m, sig, nullptr, &m);
    if (fail) fail[q] = r.success ? 1.0 : 0.0;
  }
}

long long orc_con_to_prim_zones(const phx_params *par, long long n, double *cons, double *prim,
                                const double *geom, double *fail, double *cell_sig,
                                const double *coords, int *iters, const double *guess,
                                const double *bracket, long long *evals_total, long long *accepted_total) {
  Bounds bounds(*par);
  EOS eos{par->gm1, par->Cv};
  long long unbr = 0, ev = 0, acc = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : unbr, ev, acc)
  for (long long q = 0; q < n; q++) {
    GeomPt g;
    zone_geom(geom, n, q, g);
    const ZoneRef z{prim + q, cons + q, n};
    const Real x1 = coords ? coords[q] : 0.0, x2 = coords ? coords[n + q] : 0.0,
               x3 = coords ? coords[2 * n + q] : 0.0;
    Real sig[3];
    Real lb[3];
    if (bracket)
      for (int c = 0; c < 3; c++) lb[c] = bracket[c * n + q];
    C2PResult r = con2prim_core(g, eos, bounds, *par, x1, x2, x3, z, guess ? guess[q] : z.P(PHX_PMU), sig,
                                bracket ? lb : nullptr);
    acc += r.learned_accepted;
    if (r.evals > 0 && cell_sig)
      for (int d = 0; d < 3; d++) cell_sig[d * n + q] = sig[d];
    fail[q] = r.success ? 1.0 : 0.0;
    if (iters) iters[q] = r.iterations;
    if (!r.bracketed) unbr++;
    ev += r.evals;
  }
  if (evals_total) *evals_total = ev;
  if (accepted_total) *accepted_total = acc;
  return unbr;
}

void orc_fmks_point(const phx_geometry *g, double X1, double X2, double X3, double *out21);

// The 6 FP32 inputs of the learned con2prim start, from the same setup
// quantities as con2prim_robust.hpp:303-366 (D, q, r^2, b^2, (b.r)^2, v0^2).
// Mirrors c2p_features on the device; no reference counterpart.
void orc_c2p_features_zones(const phx_params *par, long long n, const double *cons, const double *geom,
                            const double *coords, float *x) {
  Bounds bounds(*par);
#pragma omp parallel for schedule(static)
  for (long long q = 0; q < n; q++) {
    GeomPt g;
    zone_geom(geom, n, q, g);
    auto U = [&](int v) { return cons[v * n + q]; };
    const Real x1 = coords ? coords[q] : 0.0, x2 = coords ? coords[n + q] : 0.0,
               x3 = coords ? coords[2 * n + q] : 0.0;
    const Real igdet = 1.0 / g.detgam;
    Real rhoflr = 0.0, epsflr;
    bounds.GetFloors(x1, x2, x3, rhoflr, epsflr);
    rhoflr *= par->c2p_floor_scale_fac;
    Real gam_max, eps_max;
    bounds.GetCeilings(x1, x2, x3, gam_max, eps_max);
    const Real D = U(PHX_CRHO) * igdet;
    const Real qq = ratio(U(PHX_CENG) * igdet, D);
    Real rcov[] = {ratio(U(PHX_CMOM), U(PHX_CRHO)), ratio(U(PHX_CMOM + 1), U(PHX_CRHO)),
                   ratio(U(PHX_CMOM + 2), U(PHX_CRHO))};
    Real rsq = 0.0, bsq = 0.0, bdotr = 0.0;
    for (int ii = 0; ii < 3; ii++) {
      Real rc = 0.0;
      for (int jj = 0; jj < 3; jj++) rc += g.gamcon[ii][jj] * rcov[jj];
      rsq += rc * rcov[ii];
    }
    if (par->mhd) {
      Real bu[3];
      const Real sD = 1.0 / std::sqrt(std::max(D, rhoflr));
      for (int ii = 0; ii < 3; ii++) {
        bu[ii] = U(PHX_CB + ii) * igdet * sD;
        bdotr += bu[ii] * rcov[ii];
      }
      for (int ii = 0; ii < 3; ii++)
        for (int jj = 0; jj < 3; jj++) bsq += g.gcov[ii + 1][jj + 1] * bu[ii] * bu[jj];
      bsq = std::max(0.0, bsq);
    }
    const Real v0sq = std::min(rsq / (1.0 + rsq), 1.0 - 1.0 / (gam_max * gam_max));
    float f[PHX_MLP_IN];
    c2p_features(D, qq, rsq, bsq, bdotr * bdotr, v0sq, f);
    for (int c = 0; c < PHX_MLP_IN; c++) x[c * n + q] = f[c];
  }
}

// FMKS metric at n points (X1[q], X2[q]) into geom [21][n].
void orc_fmks_points(const phx_geometry *g, long long n, const double *x1, const double *x2, double *geom) {
#pragma omp parallel for schedule(static)
  for (long long q = 0; q < n; q++) {
    double out[PHX_GEOM_NLOC];
    orc_fmks_point(g, x1[q], x2[q], 0.0, out);
    for (int v = 0; v < PHX_GEOM_NLOC; v++) geom[v * n + q] = out[v];
  }
}

void orc_calculate_fluxes(const phx_params *par, const phx_block *blk) {
  calculate_fluxes(*par, blk);
}
void orc_flux_ct(const phx_block *blk) { flux_ct(blk); }
void orc_sources(const phx_params *par, const phx_block *blk) { sources(*par, blk); }

// Parthenon FluxDivergence on UniformCartesian + SumData(dudt, src):
// dudt = -(A1 (F1(i+1) - F1(i)) + A2 (...) + A3 (...)) / V + src
void orc_flux_divergence(const phx_params *par, const phx_block *blk) {
  Blk B(blk);
  const int ndim = B.ndim;
  const Real dx1 = blk->dx1, dx2 = blk->dx2, dx3 = blk->dx3;
  const Real A1 = dx2 * dx3, A2 = dx1 * dx3, A3 = dx1 * dx2, V = dx1 * dx2 * dx3;
  const int ncons = par->mhd ? PHX_NCONS : 5;
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
#pragma omp parallel for collapse(2) schedule(static)
  for (int m = 0; m < ncons; m++)
    for (int k = ks; k <= ke; k++)
      for (int j = js; j <= je; j++)
        for (int i = is; i <= ie; i++) {
          Real du = (A1 * B.F(0, m, k, j, i + 1) - A1 * B.F(0, m, k, j, i));
          if (ndim >= 2) du += A2 * B.F(1, m, k, j + 1, i) - A2 * B.F(1, m, k, j, i);
          if (ndim == 3) du += A3 * B.F(2, m, k + 1, j, i) - A3 * B.F(2, m, k, j, i);
          Real r = -du / V;
          if (m >= 1 && m <= 4) r = r + blk->src[(m - 1) * B.vs + B.idx(k, j, i)];
          blk->dudt[m * B.vs + B.idx(k, j, i)] = r;
        }
}

// AverageIndependentData + UpdateIndependentData (interior)
void orc_update(const phx_params *par, const phx_block *blk, const double *base, double *out,
                double beta, double dt) {
  Blk B(blk);
  const int ncons = par->mhd ? PHX_NCONS : 5;
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
  const Real bdt = beta * dt;
#pragma omp parallel for collapse(2) schedule(static)
  for (int m = 0; m < ncons; m++)
    for (int k = ks; k <= ke; k++)
      for (int j = js; j <= je; j++)
        for (int i = is; i <= ie; i++) {
          const long long id = m * B.vs + B.idx(k, j, i);
          Real u0 = blk->cons[id];
          u0 = beta * u0 + (1 - beta) * base[id];
          blk->cons[id] = u0;
          out[id] = u0 + bdt * blk->dudt[id];
        }
}

// Periodic ghost fill of nvar variables (applied x1, then x2, then x3 so
// edges and corners take the periodic image).
void orc_fill_ghosts_periodic(const phx_block *blk, double *field, int nvar) {
  Blk B(blk);
  const int ng = B.ng;
  for (int v = 0; v < nvar; v++) {
    double *f = field + v * B.vs;
    const int nx1 = blk->nx1, nx2 = blk->nx2, nx3 = blk->nx3;
    for (int k = 0; k < B.n3t; k++)
      for (int j = 0; j < B.n2t; j++)
        for (int g = 0; g < ng; g++) {
          f[B.idx(k, j, g)] = f[B.idx(k, j, g + nx1)];
          f[B.idx(k, j, ng + nx1 + g)] = f[B.idx(k, j, ng + g)];
        }
    if (B.ndim >= 2)
      for (int k = 0; k < B.n3t; k++)
        for (int g = 0; g < ng; g++)
          for (int i = 0; i < B.n1t; i++) {
            f[B.idx(k, g, i)] = f[B.idx(k, g + nx2, i)];
            f[B.idx(k, ng + nx2 + g, i)] = f[B.idx(k, ng + g, i)];
          }
    if (B.ndim >= 3)
      for (int g = 0; g < ng; g++)
        for (int j = 0; j < B.n2t; j++)
          for (int i = 0; i < B.n1t; i++) {
            f[B.idx(g, j, i)] = f[B.idx(g + nx3, j, i)];
            f[B.idx(ng + nx3 + g, j, i)] = f[B.idx(ng + g, j, i)];
          }
  }
}

// fluid.cpp:899-944 EstimateTimestepBlock
double orc_estimate_timestep(const phx_params *par, const phx_block *blk, int use_face) {
  Blk B(blk);
  const int ndim = B.ndim;
  const int is = B.is(), ie = B.ie(), js = B.js(), je = B.je(), ks = B.ks(), ke = B.ke();
  Real min_dt = std::numeric_limits<Real>::max();
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
        Real ldt = 0.0;
        for (int d = 0; d < ndim; d++) {
          const Real w = B.dx(d + 1);
          const long long id = d * B.vs + B.idx(k, j, i);
          Real ms = blk->cell_sig[id];
          if (use_face) {
            const long long idp = d * B.vs + B.idx(k + (d == 2), j + (d == 1), i + (d == 0));
            ms = std::max(blk->cell_sig[id], std::max(blk->face_sig[id], blk->face_sig[idp]));
          }
          ldt += ms / w;
        }
        min_dt = std::min(min_dt, 1.0 / (ldt + 1.e-50));
      }
  return par->cfl * min_dt;
}

// Fill FMKS tables on the host (cached_system.hpp:560-640, analytic branch).
void orc_geometry_fill_fmks(const phx_geometry *g, const phx_block *blk) {
  Blk B(blk);
  FMKS f(*g);
  const Real X3c = B.Xc(3, 0);
  auto fill_loc = [&](double *t, int nj, int ni, int locd) {
    const long long pitch = (long long)nj * ni;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nj; j++)
      for (int i = 0; i < ni; i++) {
        const Real X1 = (locd == 1 ? B.Xf(1, i) : B.Xc(1, i));
        const Real X2 = (locd == 2 ? B.Xf(2, j) : B.Xc(2, j));
        const long long off = (long long)j * ni + i;
        t[PHX_G_ALPHA * pitch + off] = f.Lapse(X1, X2, X3c);
        t[PHX_G_DETGAM * pitch + off] = f.DetGamma(X1, X2, X3c);
        Real beta[3];
        f.Shift(X1, X2, X3c, beta);
        for (int d = 0; d < 3; d++) t[(PHX_G_BETA + d) * pitch + off] = beta[d];
        Real gc[4][4];
        f.SpacetimeMetric(X1, X2, X3c, gc);
        for (int mu = 0; mu < 4; mu++)
          for (int nu = mu; nu < 4; nu++) t[(PHX_G_GCOV + flatten2(mu, nu)) * pitch + off] = gc[mu][nu];
        Real gi[3][3];
        f.MetricInverse(X1, X2, X3c, gi);
        for (int a = 0; a < 3; a++)
          for (int b = a; b < 3; b++) t[(PHX_G_GAMCON + flatten2s(a, b)) * pitch + off] = gi[a][b];
      }
  };
  fill_loc(g->cent, B.n2t, B.n1t, 0);
  fill_loc(g->face1, B.n2t, B.n1t + 1, 1);
  fill_loc(g->face2, B.n2t + 1, B.n1t, 2);
  const long long pitch = (long long)B.n2t * B.n1t;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < B.n2t; j++)
    for (int i = 0; i < B.n1t; i++) {
      const Real X1 = B.Xc(1, i), X2 = B.Xc(2, j);
      const long long off = (long long)j * B.n1t + i;
      Real da[4];
      f.GradLnAlpha(X1, X2, X3c, da);
      for (int d = 1; d < 4; d++) g->deriv[(PHX_GD_DALPHA + d - 1) * pitch + off] = da[d];
      Real dg[4][4][4];
      f.MetricDerivative(X1, X2, X3c, dg);
      for (int s = 1; s < 4; s++)
        for (int mu = 0; mu < 4; mu++)
          for (int nu = mu; nu < 4; nu++)
            g->deriv[(PHX_GD_DG + 3 * flatten2(mu, nu) + s - 1) * pitch + off] = dg[mu][nu][s];
    }
}

// Analytic FMKS point evaluation, for tests of the tables.
void orc_fmks_point(const phx_geometry *g, double X1, double X2, double X3, double *out21) {
  FMKS f(*g);
  out21[PHX_G_ALPHA] = f.Lapse(X1, X2, X3);
  Real beta[3];
  f.Shift(X1, X2, X3, beta);
  for (int d = 0; d < 3; d++) out21[PHX_G_BETA + d] = beta[d];
  Real gc[4][4];
  f.SpacetimeMetric(X1, X2, X3, gc);
  for (int mu = 0; mu < 4; mu++)
    for (int nu = mu; nu < 4; nu++) out21[PHX_G_GCOV + flatten2(mu, nu)] = gc[mu][nu];
  Real gi[3][3];
  f.MetricInverse(X1, X2, X3, gi);
  for (int a = 0; a < 3; a++)
    for (int b = a; b < 3; b++) out21[PHX_G_GAMCON + flatten2s(a, b)] = gi[a][b];
  out21[PHX_G_DETGAM] = f.DetGamma(X1, X2, X3);
}

void orc_c2p_fixup(const phx_params *par, const phx_block *blk) { c2p_fixup(*par, blk); }

long long orc_apply_floors(const phx_params *par, const phx_block *blk, phx_range ib, phx_range jb, phx_range kb) {
  return apply_floors(*par, blk, ib, jb, kb);
}

}  // extern "C"

// ---------------------------------------------------------------------
// The magnetised Fishbone-Moncrief torus (pgen/torus.cpp, ideal gas, nsub =
// 1, no radiation, no tracers), restated from the reference's loops.
namespace torus {

// torus.cpp:743-754
Real lfish_calc(Real r, Real a) {
  using phx_math::pow;
  return (((pow(a, 2) - 2. * a * std::sqrt(r) + pow(r, 2)) *
           ((-2. * a * r * (pow(a, 2) - 2. * a * std::sqrt(r) + pow(r, 2))) /
                std::sqrt(2. * a * std::sqrt(r) + (-3. + r) * r) +
            ((a + (-2. + r) * std::sqrt(r)) * (pow(r, 3) + pow(a, 2) * (2. + r))) /
                std::sqrt(1 + (2. * a) / pow(r, 1.5) - 3. / r))) /
          (pow(r, 3) * std::sqrt(2. * a * std::sqrt(r) + (-3. + r) * r) * (pow(a, 2) + (-2. + r) * r)));
}

// torus.cpp:756-793
Real log_enthalpy(Real r, Real th, Real a, Real rin, Real l, Real &uphi) {
  const Real sth = phx_math::sin(th);
  const Real cth = phx_math::cos(th);
  const Real DD = r * r - 2. * r + a * a;
  const Real AA = (r * r + a * a) * (r * r + a * a) - DD * a * a * sth * sth;
  const Real SS = r * r + a * a * cth * cth;
  const Real thin = M_PI / 2.;
  const Real sthin = phx_math::sin(thin);
  const Real cthin = phx_math::cos(thin);
  const Real DDin = rin * rin - 2. * rin + a * a;
  const Real AAin = (rin * rin + a * a) * (rin * rin + a * a) - DDin * a * a * sthin * sthin;
  const Real SSin = rin * rin + a * a * cthin * cthin;
  uphi = 0.0;
  const Real lnh =
      0.5 * phx_math::log((1. + std::sqrt(1. + 4. * (l * l * SS * SS) * DD / (AA * AA * sth * sth))) /
                          (SS * DD / AA)) -
      0.5 * std::sqrt(1. + 4. * (l * l * SS * SS) * DD / (AA * AA * sth * sth)) - 2. * a * r * l / AA -
      (0.5 * phx_math::log((1. + std::sqrt(1. + 4. * (l * l * SSin * SSin) * DDin /
                                                (AAin * AAin * sthin * sthin))) /
                           (SSin * DDin / AAin)) -
       0.5 * std::sqrt(1. + 4. * (l * l * SSin * SSin) * DDin / (AAin * AAin * sthin * sthin)) -
       2. * a * rin * l / AAin);
  if (lnh > 0.0) {
    Real expm2chi = SS * SS * DD / (AA * AA * sth * sth);
    Real up1 = std::sqrt((-1. + std::sqrt(1. + 4. * l * l * expm2chi)) / 2.);
    uphi = 2. * a * r * std::sqrt(1. + up1 * up1) / std::sqrt(AA * SS * DD) + std::sqrt(SS / AA) * up1 / sth;
  }
  return lnh;
}

// torus.cpp:799-829, the IdealGas branch
void GetStateFromEnthalpy(Real hm1, Real kappa, Real gam, Real rho_rmax, Real &rho_out, Real &u_out) {
  rho_out = phx_math::pow(hm1 * (gam - 1.) / (kappa * gam), 1. / (gam - 1.));
  u_out = kappa * phx_math::pow(rho_out, gam) / (gam - 1.) / rho_rmax;
  rho_out /= rho_rmax;
}

// torus.cpp:831-843
Real ucon_norm(Real ucon[4], Real gcov[4][4]) {
  Real AA = gcov[0][0];
  Real BB = 2. * (gcov[0][1] * ucon[1] + gcov[0][2] * ucon[2] + gcov[0][3] * ucon[3]);
  Real CC = 1. + gcov[1][1] * ucon[1] * ucon[1] + gcov[2][2] * ucon[2] * ucon[2] +
            gcov[3][3] * ucon[3] * ucon[3] +
            2. * (gcov[1][2] * ucon[1] * ucon[2] + gcov[1][3] * ucon[1] * ucon[3] + gcov[2][3] * ucon[2] * ucon[3]);
  Real discr = BB * BB - 4. * AA * CC;
  return (-BB - std::sqrt(discr)) / (2. * AA);
}

// Geometry::BoyerLindquist::SpacetimeMetric (boyer_lindquist.hpp:77-95, 262-280)
void bl_spacetime_metric(Real a_, Real X1, Real X2, Real g[4][4]) {
  const Real a2_ = a_ * a_;
  const Real r = std::abs(X1);
  const Real th = X2;
  const Real sth = phx_math::sin(th);
  const Real cth = phx_math::cos(th);
  const Real r2 = r * r;
  const Real r3 = r2 * r;
  const Real DD = 1. - ratio(2., r) + ratio(a2_, r2);
  const Real mu = 1. + ratio(a2_ * cth * cth, r2);
  const Real sth2 = sth * sth;
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) g[m][n] = 0;
  g[0][0] = -(1.0 - ratio(2.0, r * mu));
  g[0][3] = g[3][0] = -ratio(2.0 * a_ * sth2, r * mu);
  g[1][1] = mu / DD;
  g[2][2] = r2 * mu;
  g[3][3] = r2 * sth2 * (1.0 + ratio(a2_, r2) + ratio(2.0 * a2_ * sth2, r3 * mu));
}

// McKinneyGammieRyan::bl_to_ks, bl_to_fmks (mckinney_gammie_ryan.hpp:119-151)
void bl_to_fmks(const FMKS &f, Real x1, Real x2, Real x3, Real a, Real *ucon_bl, Real *ucon_fmks) {
  Real trans[4][4];
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) trans[m][n] = 0;
  const Real r = f.r_(x1);
  const Real idenom = 1.0 / (r * r - 2.0 * r + a * a);
  trans[0][0] = 1.0;
  trans[0][1] = 2.0 * r * idenom;
  trans[1][1] = 1.0;
  trans[2][2] = 1.0;
  trans[3][1] = a * idenom;
  trans[3][3] = 1.0;
  Real ucon_ks[4] = {0, 0, 0, 0};
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) ucon_ks[mu] += trans[mu][nu] * ucon_bl[nu];
  Real c[3], Jcov[3][3], Jcon[3][3];
  f.transform(x1, x2, x3, c, Jcov, Jcon);
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) trans[m][n] = 0;
  trans[0][0] = 1.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) trans[i + 1][j + 1] = Jcon[i][j];
  for (int mu = 0; mu < 4; mu++) ucon_fmks[mu] = 0;
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) ucon_fmks[mu] += trans[mu][nu] * ucon_ks[nu];
}

// The noise U: SplitMix64 of the counter (seed, stream 0, idx), 53 bits
Real uniform(unsigned long long seed, unsigned long long idx) {
  uint64_t z = (uint64_t)seed * 0x100000001B3ull;
  z += (uint64_t)(idx + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (Real)(z >> 11) * (1.0 / 9007199254740992.0);
}

// ProblemGenerator (torus.cpp:130-474) for one block; noise0 = the counter of
// its first zone
void ProblemGenerator(const phx_params &par, const phx_torus_params &tp, const phx_block *blk,
                      unsigned long long noise0) {
  Blk B(blk);
  Geom G(blk->geom, &B);
  FMKS tr(*blk->geom);
  EOS eos{par.gm1, par.Cv};
  Bounds floor(par);
  const Real gam = par.gm1 + 1.0, Cv = par.Cv;
  const Real rin = tp.rin, rmax = tp.rmax, kappa = tp.kappa, u_jitter = tp.u_jitter;
  const Real a = blk->geom->a;
  const int nsub = 1;
  const Real angular_mom = lfish_calc(rmax, a);
  Real uphi_rmax;
  const Real hm1_rmax = phx_math::exp(log_enthalpy(rmax, 0.5 * M_PI, a, rin, angular_mom, uphi_rmax)) - 1.0;
  Real rho_rmax, u_rmax;
  GetStateFromEnthalpy(hm1_rmax, kappa, gam, 1.0, rho_rmax, u_rmax);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < B.n3t; k++)
    for (int j = 0; j < B.n2t; j++)
      for (int i = 0; i < B.n1t; i++) {
        const Real dx_sub = B.dx(1) / nsub;
        const Real dy_sub = B.dx(2) / nsub;
        B.P(PHX_PRHO, k, j, i) = 0.0;
        B.P(PHX_PENG, k, j, i) = 0.0;
        for (int d = 0; d < 3; d++) B.P(PHX_PVEL + d, k, j, i) = 0.0;
        const Real x3 = B.Xc(3, k);
        for (int m = 0; m < nsub; m++) {
          for (int n = 0; n < nsub; n++) {
            const Real x1 = B.Xf(1, i) + (m + 0.5) * dx_sub;
            const Real x2 = B.Xf(2, j) + (n + 0.5) * dy_sub;
            Real r = tr.r_(x1);
            Real yy, th;
            tr.th_(x1, x2, yy, th);
            Real lnh = -1.0;
            Real uphi;
            if (r > rin) lnh = log_enthalpy(r, th, a, rin, angular_mom, uphi);
            if (lnh > 0.0) {
              Real hm1 = phx_math::exp(lnh) - 1.;
              Real rho, u;
              GetStateFromEnthalpy(hm1, kappa, gam, rho_rmax, rho, u);
              Real ucon_bl[] = {0.0, 0.0, 0.0, uphi};
              Real gcov[4][4];
              bl_spacetime_metric(a, r, th, gcov);
              ucon_bl[0] = ucon_norm(ucon_bl, gcov);
              Real ucon[4];
              bl_to_fmks(tr, x1, x2, x3, a, ucon_bl, ucon);
              const Real lapse = tr.Lapse(x1, x2, x3);
              Real beta[3];
              tr.Shift(x1, x2, x3, beta);
              tr.SpacetimeMetric(x1, x2, x3, gcov);
              ucon[0] = ucon_norm(ucon, gcov);
              const Real W = lapse * ucon[0];
              Real vcon[] = {ucon[1] / W + beta[0] / lapse, ucon[2] / W + beta[1] / lapse,
                             ucon[3] / W + beta[2] / lapse};
              B.P(PHX_PRHO, k, j, i) += rho / (nsub * nsub);
              B.P(PHX_PENG, k, j, i) += u / (nsub * nsub);
              for (int d = 0; d < 3; d++) B.P(PHX_PVEL + d, k, j, i) += W * vcon[d] / (nsub * nsub);
            }
          }
        }
        const Real x1v = B.Xc(1, i);
        const Real x2v = B.Xc(2, j);
        B.P(PHX_PENG, k, j, i) *= (1. + u_jitter * (uniform(tp.seed, noise0 + (unsigned long long)B.idx(k, j, i)) - 0.5));
        Real rhoflr = 0;
        Real epsflr;
        floor.GetFloors(x1v, x2v, x3, rhoflr, epsflr);
        B.P(PHX_PRHO, k, j, i) = B.P(PHX_PRHO, k, j, i) < rhoflr ? rhoflr : B.P(PHX_PRHO, k, j, i);
        B.P(PHX_PENG, k, j, i) = B.P(PHX_PENG, k, j, i) / B.P(PHX_PRHO, k, j, i) < epsflr
                                     ? B.P(PHX_PRHO, k, j, i) * epsflr
                                     : B.P(PHX_PENG, k, j, i);
        B.P(PHX_PTMP, k, j, i) =
            eos.TemperatureFromDensityInternalEnergy(B.P(PHX_PRHO, k, j, i), B.P(PHX_PENG, k, j, i) / B.P(PHX_PRHO, k, j, i));
        B.P(PHX_PPRS, k, j, i) = eos.PressureFromDensityTemperature(B.P(PHX_PRHO, k, j, i), B.P(PHX_PTMP, k, j, i));
        B.P(PHX_PGM1, k, j, i) =
            eos.BulkModulusFromDensityTemperature(B.P(PHX_PRHO, k, j, i), B.P(PHX_PTMP, k, j, i)) /
            B.P(PHX_PPRS, k, j, i);
        for (int d = 0; d < 3; d++) B.P(PHX_PB + d, k, j, i) = 0.0;  // Parthenon's zero-initialised field
        B.P(PHX_PMU, k, j, i) = 0.0;
      }
  (void)Cv;
  // the vector potential at the corners (torus.cpp:452-470), from the k = kb.s plane
  std::vector<Real> A((size_t)B.n2t * B.n1t, 0.0);
  for (int j = 1; j <= B.n2t - 1; j++)
    for (int i = 1; i <= B.n1t - 1; i++) {
      const Real rho_av = 0.25 * (B.P(PHX_PRHO, 0, j, i) + B.P(PHX_PRHO, 0, j, i - 1) + B.P(PHX_PRHO, 0, j - 1, i) +
                                  B.P(PHX_PRHO, 0, j - 1, i - 1));
      const Real q = rho_av - 0.2;
      A[(size_t)j * B.n1t + i] = (q > 0 ? q : 0.0);
    }
  auto Aij = [&](int j, int i) { return A[(size_t)j * B.n1t + i]; };
  // the poloidal field (torus.cpp:472-488)
  for (int k = 0; k < B.n3t; k++)
    for (int j = 0; j <= B.n2t - 2; j++)
      for (int i = 0; i <= B.n1t - 2; i++) {
        GeomPt g;
        G.at(CENT, k, j, i, g);
        const Real gamdet = g.detgam;
        B.P(PHX_PB, k, j, i) =
            -(Aij(j, i) - Aij(j + 1, i) + Aij(j, i + 1) - Aij(j + 1, i + 1)) / (2.0 * B.dx(2) * gamdet);
        B.P(PHX_PB + 1, k, j, i) =
            (Aij(j, i) + Aij(j + 1, i) - Aij(j, i + 1) - Aij(j + 1, i + 1)) / (2.0 * B.dx(1) * gamdet);
        B.P(PHX_PB + 2, k, j, i) = 0.0;
      }
}

}  // namespace torus

extern "C" {

// ProblemGenerator on every block, then PostInitializationModifier's
// HARM-style normalisation (torus.cpp:525-740, ComputeBetas :844-924).
void orc_torus_init(const phx_params *par, const phx_torus_params *tp, phx_block *blocks, int nblocks,
                    double *field_factor) {
  unsigned long long noise0 = 0;
  for (int q = 0; q < nblocks; q++) {
    Blk B(&blocks[q]);
    torus::ProblemGenerator(*par, *tp, &blocks[q], noise0);
    const phx_range ib{0, B.n1t - 1}, jb{0, B.n2t - 1}, kb{0, B.n3t - 1};
    orc_prim_to_con(par, &blocks[q], ib, jb, kb);
    apply_floors(*par, &blocks[q], ib, jb, kb);
    noise0 += (unsigned long long)B.N;
  }
  Real bsq_max = -std::numeric_limits<Real>::infinity();
  Real press_max = -std::numeric_limits<Real>::infinity();
  for (int q = 0; q < nblocks; q++) {
    Blk B(&blocks[q]);
    Geom G(blocks[q].geom, &B);
    for (int k = B.ks(); k <= B.ke(); k++)
      for (int j = B.js(); j <= B.je(); j++)
        for (int i = B.is(); i <= B.ie(); i++) {
          GeomPt g;
          G.at(CENT, k, j, i, g);
          Real gcov[3][3];
          for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) gcov[m][n] = g.gcov[m + 1][n + 1];
          const Real vp[] = {B.P(PHX_PVEL, k, j, i), B.P(PHX_PVEL + 1, k, j, i), B.P(PHX_PVEL + 2, k, j, i)};
          const Real Bp[] = {B.P(PHX_PB, k, j, i), B.P(PHX_PB + 1, k, j, i), B.P(PHX_PB + 2, k, j, i)};
          // GetLorentzFactor and GetMagneticFieldSquared (relativity_utils.hpp:38-43, 131-164)
          Real vsq = 0.;
          for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) vsq += gcov[m][n] * vp[m] * vp[n];
          const Real W = std::sqrt(1. + vsq);
          Real Bsq = 0, Bdotv = 0;
          for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) {
              Bdotv += gcov[m][n] * ratio(vp[m], W) * Bp[n];
              Bsq += gcov[m][n] * Bp[m] * Bp[n];
            }
          const Real bsq = ratio(Bsq, W * W) + Bdotv * Bdotv;
          bsq_max = std::max(bsq, bsq_max);
          press_max = std::max(B.P(PHX_PPRS, k, j, i), press_max);
        }
  }
  const Real beta_pmax = ratio(press_max, 0.5 * bsq_max);
  const Real B_field_fac = tp->magnetized ? std::sqrt(beta_pmax / tp->target_beta) : 0;
  for (int q = 0; q < nblocks; q++) {
    Blk B(&blocks[q]);
    for (int k = B.ks(); k <= B.ke(); k++)
      for (int j = B.js(); j <= B.je(); j++)
        for (int i = B.is(); i <= B.ie(); i++)
          for (int d = 0; d < 3; d++) B.P(PHX_PB + d, k, j, i) *= B_field_fac;
    orc_prim_to_con(par, &blocks[q], phx_range{0, B.n1t - 1}, phx_range{0, B.n2t - 1}, phx_range{0, B.n3t - 1});
  }
  if (field_factor) *field_factor = B_field_fac;
}

}  // extern "C"

// =====================================================================
// Radiation moments (M1 and Eddington closures), one species, on Minkowski
// or FMKS blocks.  Restates radiation/closure.hpp:49-352,
// closure_m1.hpp:31-372, local_three_geometry.hpp:123-185, moments.cpp:61-995
// (with CalculateGeometricSourceImpl, moments.cpp:764-885),
// moments_source.cpp:152-965 (oned solver, both update_fluid settings),
// radiation.cpp:585-648, linear_algebra.hpp:58-96 and root_find.hpp:20-160.
// Minkowski: the spatial metric is the identity, lapse 1, shift 0.  Each
// contraction keeps the reference's order over its non-zero terms; for finite
// values the zero terms of the full 3x3 sums change no rounding.  FMKS: the
// cached tables' values at the cell centre or face, and the closures'
// LocalThreeGeometry (gamma^ij from matrixInverse3x3, full 3x3 sums).
// Third-party semantics restated from their definitions: gray opacities
// (kappaJ = rho kappa_a, kappaH = kappaJ + rho kappa_s, JBB = a T^4; the
// Rosseland means of a gray opacity are the gray values) and the
// singularity-eos IdealGas energy sie = Cv T.
// std::pow(x, 2) and std::pow(x, 3) are written as products; tanh is the
// restatement below (the same algorithm as the device's).
// =====================================================================
namespace orc {
namespace rad {

// std::min / std::max semantics (NaN handling matters for bitwise parity)
inline Real smin(Real a, Real b) { return (b < a) ? b : a; }
inline Real smax(Real a, Real b) { return (a < b) ? b : a; }
inline Real sgn(Real v) { return (Real)((0.0 <= v) - (v < 0.0)); }  // robust.hpp sgn

// tanh from exp and expm1 written out: Cody-Waite reduction
// y = n ln2 + r (ln2 split into a 32-bit head and a tail so n * head is
// exact), Taylor series of e^r to degree 13 (|r| <= ln2 / 2: truncation below
// 5e-18), e^y - 1 by its own Taylor series to degree 14 for |y| < 1/4, and
// tanh(x) = -m / (2 + m) with m = e^{-2|x|} - 1.  Host and device evaluate
// the same operations in the same order.
constexpr Real LN2_HI = 0.693147180369123816490;   // 2977044471 / 2^32
constexpr Real LN2_LO = 1.9082149292705877000e-10; // ln 2 - LN2_HI
constexpr Real INV_LN2 = 1.4426950408889634074;
inline Real exp_taylor(Real r) {
  Real p = 1.0 / 6227020800.0;  // 1/13!
  p = p * r + 1.0 / 479001600.0;
  p = p * r + 1.0 / 39916800.0;
  p = p * r + 1.0 / 3628800.0;
  p = p * r + 1.0 / 362880.0;
  p = p * r + 1.0 / 40320.0;
  p = p * r + 1.0 / 5040.0;
  p = p * r + 1.0 / 720.0;
  p = p * r + 1.0 / 120.0;
  p = p * r + 1.0 / 24.0;
  p = p * r + 1.0 / 6.0;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  return p;
}
inline Real expm1_small(Real y) {  // |y| < 1/4
  Real p = 1.0 / 87178291200.0;  // 1/14!
  p = p * y + 1.0 / 6227020800.0;
  p = p * y + 1.0 / 479001600.0;
  p = p * y + 1.0 / 39916800.0;
  p = p * y + 1.0 / 3628800.0;
  p = p * y + 1.0 / 362880.0;
  p = p * y + 1.0 / 40320.0;
  p = p * y + 1.0 / 5040.0;
  p = p * y + 1.0 / 720.0;
  p = p * y + 1.0 / 120.0;
  p = p * y + 1.0 / 24.0;
  p = p * y + 1.0 / 6.0;
  p = p * y + 0.5;
  p = p * y + 1.0;
  return p * y;
}
// e^y for -46 <= y <= 0
inline Real exp_neg(Real y) {
  const Real n = std::floor(y * INV_LN2 + 0.5);
  const Real r = (y - n * LN2_HI) - n * LN2_LO;
  return std::ldexp(exp_taylor(r), (int)n);
}
inline Real tanh_r(Real x) {
  const Real ax = std::fabs(x);
  Real t;
  if (ax > 22.0) {
    t = 1.0;
  } else {
    const Real y = -2.0 * ax;
    const Real m = (y > -0.25) ? expm1_small(y) : exp_neg(y) - 1.0;
    t = -m / (2.0 + m);
  }
  return std::copysign(t, x);
}

struct V3 {
  Real d[3];
  Real &operator()(int i) { return d[i]; }
  const Real &operator()(int i) const { return d[i]; }
};
struct T2 {
  Real d[3][3];
  Real &operator()(int i, int j) { return d[i][j]; }
  const Real &operator()(int i, int j) const { return d[i][j]; }
};

// local_three_geometry.hpp:150-185 with gamma_ij = delta_ij
inline void lower3(const V3 &a, V3 &o) {
  for (int i = 0; i < 3; i++) o(i) = 0.0 + a(i);
}
inline void raise3(const V3 &a, V3 &o) {
  for (int i = 0; i < 3; i++) o(i) = 0.0 + a(i);
}
inline Real ccov(const V3 &a, const V3 &b) {  // contractCov3Vectors
  Real s = 0.0;
  for (int i = 0; i < 3; i++) s += a(i) * b(i);
  return s;
}
inline Real cconcov(const V3 &a, const V3 &b) {  // contractConCov3Vectors
  Real s = 0.0;
  for (int i = 0; i < 3; i++) s += a(i) * b(i);
  return s;
}
inline Real gdelta(int i, int j) { return i == j ? 1.0 : 0.0; }

// linear_algebra.hpp:58-96
inline Real DifferenceOfProducts(Real a, Real b, Real c, Real d) {
  const Real cd = c * d;
  const Real err = std::fma(-c, d, cd);
  const Real dop = std::fma(a, b, -cd);
  return dop + err;
}
inline void SolveAxb2x2(Real A[2][2], Real b[2], Real x[2]) {
  const Real invDet = 1.0 / DifferenceOfProducts(A[0][0], A[1][1], A[0][1], A[1][0]);
  x[0] = invDet * DifferenceOfProducts(A[1][1], b[0], A[0][1], b[1]);
  x[1] = invDet * DifferenceOfProducts(A[0][0], b[1], A[1][0], b[0]);
}
// linear_algebra.hpp:67-89: the adjugate over the determinant, each entry
// a DifferenceOfProducts, the determinant expanded along the first column.
inline Real matrixInverse3x3(const Real A[3][3], Real Ainv[3][3]) {
  Ainv[0][0] = DifferenceOfProducts(A[1][1], A[2][2], A[1][2], A[2][1]);
  Ainv[1][0] = -DifferenceOfProducts(A[1][0], A[2][2], A[1][2], A[2][0]);
  Ainv[2][0] = DifferenceOfProducts(A[1][0], A[2][1], A[1][1], A[2][0]);
  Ainv[0][1] = -DifferenceOfProducts(A[0][1], A[2][2], A[0][2], A[2][1]);
  Ainv[1][1] = DifferenceOfProducts(A[0][0], A[2][2], A[0][2], A[2][0]);
  Ainv[2][1] = -DifferenceOfProducts(A[0][0], A[2][1], A[0][1], A[2][0]);
  Ainv[0][2] = DifferenceOfProducts(A[0][1], A[1][2], A[0][2], A[1][1]);
  Ainv[1][2] = -DifferenceOfProducts(A[0][0], A[1][2], A[0][2], A[1][0]);
  Ainv[2][2] = DifferenceOfProducts(A[0][0], A[1][1], A[0][1], A[1][0]);
  const Real det = std::fma(A[0][0], Ainv[0][0], DifferenceOfProducts(A[2][0], Ainv[2][0], A[1][0], -Ainv[1][0]));
  const Real invDet = 1.0 / det;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ainv[i][j] *= invDet;
  return det;
}

// LocalThreeGeometry (local_three_geometry.hpp:123-185) off Minkowski:
// gamma_ij of the location, gamma^ij from matrixInverse3x3 of it (not the
// table's inverse), the lapse.  Contractions keep the reference's loop order.
struct G3 {
  Real cov[3][3], con[3][3], alpha;
  G3() = default;
  explicit G3(const GeomPt &p) {
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) cov[a][b] = p.gcov[a + 1][b + 1];
    matrixInverse3x3(cov, con);
    alpha = p.alpha;
  }
  void lower(const V3 &a, V3 &o) const {
    for (int i = 0; i < 3; i++) o(i) = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) o(i) += a(j) * cov[i][j];
  }
  void raise(const V3 &a, V3 &o) const {
    for (int i = 0; i < 3; i++) o(i) = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) o(i) += a(j) * con[i][j];
  }
  Real contract_cov(const V3 &a, const V3 &b) const {  // contractCov3Vectors
    Real s(0.0);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) s += con[i][j] * a(i) * b(j);
    return s;
  }
};

// relativity_utils.hpp:38-43 (GetLorentzFactor with gamma_ij)
inline Real lorentz_g(const Real vp[3], const G3 &g) {
  Real vsq = 0.;
  for (int ii = 0; ii < 3; ii++)
    for (int jj = 0; jj < 3; jj++) vsq += g.cov[ii][jj] * vp[ii] * vp[jj];
  return std::sqrt(1. + vsq);
}

// relativity_utils.hpp:38-43 with the spatial metric
inline Real lorentz3(const Real vp[3]) {
  Real vsq = 0.;
  for (int i = 0; i < 3; i++) vsq += vp[i] * vp[i];
  return std::sqrt(1. + vsq);
}

enum Status { SUCCESS = 0, FAILURE = 1, MODIFIED = 2 };
constexpr Real PI = 3.141592653589793;
constexpr Real SIN_PI = 1.2246467991473532e-16;  // sin of the double nearest pi

// ClosureEdd (closure.hpp:49-352) and ClosureM1 (closure_m1.hpp:31-372),
// energy-conserving settings.
struct Closure {
  bool m1, robust;
  const G3 *geo;  // null: Minkowski (gamma_ij = delta_ij)
  V3 con_v, cov_v;
  Real v2, W, W2;
  void lower(const V3 &a, V3 &o) const {
    if (geo)
      geo->lower(a, o);
    else
      lower3(a, o);
  }
  void raise(const V3 &a, V3 &o) const {
    if (geo)
      geo->raise(a, o);
    else
      raise3(a, o);
  }
  Real ccv(const V3 &a, const V3 &b) const { return geo ? geo->contract_cov(a, b) : ccov(a, b); }
  Real gcon(int i, int j) const { return geo ? geo->con[i][j] : gdelta(i, j); }
  Closure(const V3 &cv, bool m1_, bool robust_, const G3 *g_ = nullptr) : m1(m1_), robust(robust_), geo(g_) {
    con_v = cv;
    lower(con_v, cov_v);
    v2 = 0.0;
    for (int i = 0; i < 3; i++) v2 += con_v(i) * cov_v(i);
    v2 = smin(v2, 0.9999);
    W = 1 / std::sqrt(1 - v2);
    W2 = W * W;
  }
  void TilPiContractions(const T2 &Pi, V3 &cov_vPi, Real &vvPi) const {
    V3 con_vPi;
    vvPi = 0.0;
    for (int i = 0; i < 3; i++) {
      con_vPi(i) = 0.0;
      for (int j = 0; j < 3; j++) con_vPi(i) += cov_v(j) * Pi(i, j);
      vvPi += cov_v(i) * con_vPi(i);
    }
    lower(con_vPi, cov_vPi);
  }
  void LinearSourceUpdate(Real Estar, const V3 &cov_Fstar, const T2 &Pi, Real JBB, Real tauJ, Real tauH,
                          Real &dE, V3 &cov_dF) const {
    Real vvPi;
    V3 cov_vPi;
    TilPiContractions(Pi, cov_vPi, vvPi);
    Real A[2][2], x[2], b[2];
    A[0][0] = (4 * W2 - 1) / 3 + W2 * vvPi + W * tauJ;
    A[0][1] = 2 * W + tauH;
    A[1][0] = A[0][0] - 1 - tauJ / W;
    A[1][1] = A[0][1] - 1 / W;
    const Real vFstar = cconcov(con_v, cov_Fstar);
    b[0] = Estar + W * tauJ * JBB;
    b[1] = vFstar + (W2 - 1) / W * tauJ * JBB;
    SolveAxb2x2(A, b, x);
    const Real J = x[0], zeta = x[1];
    dE = (4 * W2 - 1 + 3 * W2 * vvPi) / 3 * J + 2 * W * zeta - Estar;
    for (int i = 0; i < 3; i++)
      cov_dF(i) = (cov_v(i) * tauH * (4 * W2 / 3 * J + W * zeta) + tauH * cov_vPi(i) * J +
                   tauJ * W2 * cov_v(i) * (JBB - J) + W * cov_Fstar(i)) /
                      (W + tauH) -
                  cov_Fstar(i);
  }
  void ConCovP(Real J, const V3 &cov_H, const T2 &Pi, T2 &P) const {
    V3 con_H;
    T2 ccPi;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        if (geo) {
          ccPi(i, j) = 0.0;
          for (int k = 0; k < 3; k++) ccPi(i, j) += Pi(i, k) * geo->cov[k][j];
        } else {
          ccPi(i, j) = 0.0 + Pi(i, j);
        }
      }
    raise(cov_H, con_H);
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++)
        P(i, j) = 4.0 / 3.0 * W2 * con_v(i) * cov_v(j) * J + W * (con_v(i) * cov_H(j) + cov_v(j) * con_H(i)) +
                  J * ccPi(i, j);
      P(i, i) += J / 3.0;
    }
  }
  void ConP(Real J, const V3 &cov_H, const T2 &Pi, T2 &P) const {
    V3 con_H;
    raise(cov_H, con_H);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        P(i, j) = 4.0 / 3.0 * W2 * con_v(i) * con_v(j) * J + W * (con_v(i) * con_H(j) + con_v(j) * con_H(i)) +
                  J * Pi(i, j) + J / 3.0 * gcon(i, j);
  }
  void Prim2Con(Real J, const V3 &cov_H, const T2 &Pi, Real &E, V3 &cov_F) const {
    Real vvPi;
    V3 cov_vPi;
    TilPiContractions(Pi, cov_vPi, vvPi);
    Real vH = 0.0;
    for (int i = 0; i < 3; i++) vH += con_v(i) * cov_H(i);
    E = (4 * W2 - 1 + 3 * W2 * vvPi) / 3 * J + 2 * W * vH;
    for (int i = 0; i < 3; i++)
      cov_F(i) = 4 * W2 / 3 * cov_v(i) * J + W * cov_v(i) * vH + W * cov_H(i) + J * cov_vPi(i);
  }
  // getFluxesFromPrim (on Minkowski the lapse scalings by 1 are exact)
  void FluxesFromPrim(Real J, const V3 &cov_H, const T2 &Pi, V3 &con_F, T2 &P) const {
    ConCovP(J, cov_H, Pi, P);
    Real E;
    V3 cov_F;
    Prim2Con(J, cov_H, Pi, E, cov_F);
    raise(cov_F, con_F);
    if (geo) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) P(i, j) *= geo->alpha;
      for (int i = 0; i < 3; i++) con_F(i) *= geo->alpha;
    }
  }
  Status Con2Prim(Real E, const V3 &cov_F, const T2 &Pi, Real &J, V3 &cov_H) const {
    Real vvPi;
    V3 cov_vPi;
    TilPiContractions(Pi, cov_vPi, vvPi);
    double vF = 0.0;
    for (int i = 0; i < 3; i++) vF += con_v(i) * cov_F(i);
    const Real lam = (2.0 * W2 + 1.0) / 3.0 + (2.0 * W2 - 3.0) * W2 * vvPi;
    const Real a = ratio(W2, lam) * ((4 * W2 / 3 - vvPi) * E - ((4 * W2 + 1) / 3 - W2 * vvPi) * vF);
    J = ratio((2 * W2 - 1) * E - 2 * W2 * vF, lam);
    for (int i = 0; i < 3; i++) cov_H(i) = (cov_F(i) - J * cov_vPi(i) - cov_v(i) * a) / W;
    const Real vh = cconcov(con_v, cov_H);
    const Real xi = std::sqrt(ccv(cov_H, cov_H) - vh * vh) / J;
    if (std::isnan(xi) || std::isnan(J)) return FAILURE;
    if (J < 0. || xi >= 1.0) {
      if (robust) {
        if (J < 0.) J = smin(J, 10. * SMALL);
        if (xi >= 1.0)
          for (int i = 0; i < 3; i++) cov_H(i) *= 0.999 / xi;
        return MODIFIED;
      }
      return FAILURE;
    }
    return SUCCESS;
  }
  static Real closure_fn(Real xi) { return (1.0 - 2 * (xi * xi) + 4 * (xi * xi * xi)) / 3.0; }
  // M1FluidPressureTensor from J and H (closure_m1.hpp:274-299)
  void PressureFromPrim(Real J, const V3 &cov_H, T2 &Pi, V3 &con_f) const {
    V3 con_H;
    raise(cov_H, con_H);
    Real H = 0.0, vH = 0.0;
    for (int i = 0; i < 3; i++) H += cov_H(i) * con_H(i);
    for (int i = 0; i < 3; i++) vH += cov_H(i) * con_v(i);
    H = std::sqrt(H - vH * vH);
    for (int i = 0; i < 3; i++) con_f(i) = ratio(con_H(i), H);
    const Real xi = smax(smin(1.0, ratio(H, J)), 0.0);
    const Real athin = 0.5 * (3 * closure_fn(xi) - 1);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        Pi(i, j) = con_f(i) * con_f(j) - (W2 * con_v(i) * con_v(j) + gcon(i, j)) / 3;
        Pi(i, j) *= athin;
      }
  }
  // M1FluidPressureTensor from xi, phi and the basis (closure_m1.hpp:301-324)
  void PressureFromAngles(Real xi, Real phi, const V3 &g, const V3 &dd, T2 &Pi, V3 &con_f) const {
    Real s, c;
    if (phi == PI) {
      s = SIN_PI;
      c = -1.0;
    } else {
      s = std::sin(phi);
      c = std::cos(phi);
    }
    for (int i = 0; i < 3; i++) con_f(i) = -c * g(i) + s * dd(i);
    const Real athin = 0.5 * (3 * closure_fn(xi) - 1);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        Pi(i, j) = con_f(i) * con_f(j) - (W2 * con_v(i) * con_v(j) + gcon(i, j)) / 3;
        Pi(i, j) *= athin;
      }
  }
  // closure_m1.hpp:326-372
  void BasisVectors(const V3 &cov_F, V3 &g, V3 &dd) const {
    V3 con_F;
    raise(cov_F, con_F);
    Real Fmag = 0.0, vl = 0.0, vv = 0.0;
    for (int i = 0; i < 3; i++) Fmag += cov_F(i) * con_F(i);
    Fmag = std::sqrt(Fmag);
    for (int i = 0; i < 3; i++) vl += cov_F(i) * con_v(i);
    vl = ratio(vl, Fmag);
    for (int i = 0; i < 3; i++) vv += cov_v(i) * con_v(i);
    const Real lam = ratio(1.0, W * (1 - vl));
    const Real aa = std::sqrt(vv * (1 + 10 * std::numeric_limits<Real>::epsilon()) - vl * vl);
    for (int i = 0; i < 3; i++) {
      g(i) = ratio(con_F(i) * lam, Fmag) - W * con_v(i);
      dd(i) = ratio(ratio(con_F(i), Fmag) * (1 - lam / W) + con_v(i), aa);
    }
  }
  void Residuals(Real E, const V3 &cov_F, Real xi, Real phi, const V3 &g, const V3 &dd, Real &fXi,
                 Real &fPhi) const {
    T2 Pi;
    V3 con_f;
    PressureFromAngles(xi, phi, g, dd, Pi, con_f);
    Real J;
    V3 cov_H;
    Con2Prim(E, cov_F, Pi, J, cov_H);
    Real H(0.0), vH(0.0), Hf(0.0), vf(0.0);
    if (geo) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) H += cov_H(i) * cov_H(j) * geo->con[i][j];
    } else {
      for (int i = 0; i < 3; i++) H += cov_H(i) * cov_H(i);
    }
    for (int i = 0; i < 3; i++) vH += con_v(i) * cov_H(i);
    for (int i = 0; i < 3; i++) Hf += cov_H(i) * con_f(i);
    for (int i = 0; i < 3; i++) vf += cov_v(i) * con_f(i);
    Hf -= vf * vH;
    H = std::sqrt(H - vH * vH);
    fXi = xi - ratio(H, J);
    fPhi = Hf - H;
  }
  // SolveClosure (closure_m1.hpp:178-258).  The reference holds phi at pi
  // (its "first two updates" test is true for every iteration) and drops the
  // 2x2 solve; the two phi-perturbed residuals only feed that solve and are
  // not evaluated here.  Returns the iteration count; *failed on NaN or the
  // iteration cap.
  int SolveClosure(Real E, V3 cov_F, Real &xi_out, Real &phi_out, Real xi_guess, bool &failed) const {
    const int max_iter = 30;
    const Real tol = 1.e6 * std::numeric_limits<Real>::epsilon();
    const Real eps = std::sqrt(10 * std::numeric_limits<Real>::epsilon());
    const Real delta = 20 * std::numeric_limits<Real>::epsilon();
    for (int i = 0; i < 3; i++)
      cov_F(i) = ratio(cov_F(i), E) + 1.e3 * sgn(cov_F(i)) * std::numeric_limits<Real>::min();
    E = 1.0;
    V3 g, dd;
    BasisVectors(cov_F, g, dd);
    int iter = 0;
    Real fXi = 1.e3, fPhi = 1.e3;
    Real xi = xi_guess;
    Real phi = PI;
    do {
      Real fXi_up, fXi_lo, fPhi_up, fPhi_lo;
      const Real xi_up = smin(xi * (1.0 + eps) + delta, 1.0);
      const Real xi_lo = smax(xi * (1.0 - eps) - delta, 0.0);
      Residuals(E, cov_F, xi_up, phi, g, dd, fXi_up, fPhi_up);
      Residuals(E, cov_F, xi_lo, phi, g, dd, fXi_lo, fPhi_lo);
      const Real J00 = (fXi_up - fXi_lo) / (xi_up - xi_lo);
      Residuals(E, cov_F, xi, phi, g, dd, fXi, fPhi);
      const Real dx0 = fXi / J00, dx1 = 0.0;
      fPhi = 0.0;
      Real cdx = smin(dx0, xi - delta * xi);
      cdx = smax(cdx, xi - (1 - delta * (1 - xi)));
      Real alpha = ratio(cdx, dx0);
      alpha = smin(alpha, 0.5 * 3.14159 / std::fabs(dx1));
      xi -= alpha * dx0;
      phi -= alpha * dx1;
      ++iter;
    } while (iter < max_iter && (std::fabs(fXi) > tol || std::fabs(fPhi) > tol));
    xi_out = xi;
    phi_out = phi;
    failed = std::isnan(xi) || iter >= max_iter;
    return iter;
  }
  // GetConTilPiFromCon: M1 solves the closure from the xi guess; Eddington
  // returns pi = 0, xi = 0, phi = pi.
  void TilPiFromCon(Real E, const V3 &cov_F, Real &xi, Real &phi, T2 &Pi) const {
    if (!m1) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Pi(i, j) = 0.0;
      xi = 0.0;
      phi = PI;
      return;
    }
    bool failed;
    SolveClosure(E, cov_F, xi, phi, xi, failed);
    V3 g, dd, con_f;
    BasisVectors(cov_F, g, dd);
    PressureFromAngles(xi, phi, g, dd, Pi, con_f);
  }
  void TilPiFromPrim(Real J, const V3 &cov_H, T2 &Pi) const {
    if (!m1) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Pi(i, j) = 0.0;
      return;
    }
    V3 con_f;
    PressureFromPrim(J, cov_H, Pi, con_f);
  }
};

struct RBlk {
  Blk B;
  const phx_rad_block *r;
  long long rvs;
  explicit RBlk(const phx_block *fb, const phx_rad_block *rb) : B(fb), r(rb) {
    rvs = rb->var_stride ? rb->var_stride : B.N;
  }
  Real &U(int v, long long id) const { return r->cons[v * rvs + id]; }
  Real &Q(int v, long long id) const { return r->prim[v * rvs + id]; }
  Real &F(int d, int m, long long id) const { return r->flux[((long long)d * PHX_RNCONS + m) * rvs + id]; }
  Real fp(int v, long long id) const { return B.b->prim[v * B.vs + id]; }
  V3 con_v(long long id, Real *Wout = nullptr) const {
    const Real vp[3] = {fp(PHX_PVEL, id), fp(PHX_PVEL + 1, id), fp(PHX_PVEL + 2, id)};
    const Real W = lorentz3(vp);
    if (Wout) *Wout = W;
    return V3{{vp[0] / W, vp[1] / W, vp[2] / W}};
  }
};

struct RPar {
  bool m1, robust, bounds;
  int recon;
  Real cfl, tol, kappa_a, kappa_s, jbb;
  int maxiter, oned_fixup;
  bool update_fluid, fixup_floors;
  bool fourd, oned_backup;  // src_solver fourd; src_use_oned_backup
  Real fd_eps;              // src_rootfind_eps
  bool floor_expx1;         // rad_floor_type ExpX1J
  Real J_alpha;             // J_exp_floor
  Real J_floor, xi_ceiling, tau_max, W_ceiling, Cv;
  RPar(const phx_rad_params &rp, const phx_params &p) {
    update_fluid = rp.update_fluid != 0;
    fixup_floors = rp.rad_c2p_failure_floors != 0;
    fourd = rp.src_solver == PHX_RAD_SRC_FOURD;
    oned_backup = rp.src_use_oned_backup != 0;
    fd_eps = rp.src_rootfind_eps;
    m1 = rp.method == PHX_RAD_M1;
    robust = !rp.closure_frail;
    bounds = rp.recon_fixup_bounds != 0;
    recon = rp.recon;
    cfl = rp.cfl;
    tol = rp.src_rootfind_tol;
    maxiter = rp.src_rootfind_maxiter;
    oned_fixup = rp.oned_fixup_strategy;
    kappa_a = rp.kappa_a;
    kappa_s = rp.kappa_s;
    jbb = rp.jbb_coeff;
    J_floor = rp.enable_rad_floors ? rp.J0_floor : -std::numeric_limits<Real>::max();
    floor_expx1 = rp.enable_rad_floors && rp.rad_floor_type == PHX_RAD_FLOOR_EXPX1_J;
    J_alpha = rp.J_exp_floor;
    xi_ceiling = rp.enable_rad_ceilings ? rp.xi0_ceiling : std::numeric_limits<Real>::max();
    tau_max = rp.enable_rad_ceilings ? rp.tau0_ceiling : std::numeric_limits<Real>::max();
    W_ceiling = p.enable_ceilings ? p.gam0_ceiling : std::numeric_limits<Real>::max();
    Cv = p.Cv;
  }
  // RadiationFloors::GetRadiationFloors (fixup.hpp:166-177) at X1 = x1
  Real JFloor(Real x1) const { return floor_expx1 ? J_floor * phx_math::exp(J_alpha * x1) : J_floor; }
  Real kappaJ(Real rho, Real T) const { return rho * kappa_a; }
  Real kappaS(Real rho, Real T) const { return rho * kappa_s; }
  Real JBB(Real T) const { return jbb * (T * T) * (T * T); }
};

// The geometry a moment task reads at one location (loc at k, j, i): the
// tables' lapse, shift, gamma_ij, gamma^ij (MetricInverse) and sqrt(gamma),
// and off Minkowski the LocalThreeGeometry built from them.
struct RGeo {
  GeomPt p;
  G3 g3;
  bool mink;
  RGeo(const RBlk &R, Loc loc, int k, int j, int i) {
    const Geom G(R.B.b->geom, &R.B);
    G.at(loc, k, j, i, p);
    mink = G.mink();
    if (!mink) g3 = G3(p);
  }
  const G3 *g() const { return mink ? nullptr : &g3; }
  Real cov(int a, int b) const { return p.gcov[a + 1][b + 1]; }
  Real con(int a, int b) const { return p.gamcon[a][b]; }
};
// con_v = (W v^i) / W, W from gamma_ij (relativity_utils.hpp:38-43)
inline V3 con_v_at(const RBlk &R, long long id, const RGeo &G, Real *Wout = nullptr) {
  if (G.mink) return R.con_v(id, Wout);
  const Real vp[3] = {R.fp(PHX_PVEL, id), R.fp(PHX_PVEL + 1, id), R.fp(PHX_PVEL + 2, id)};
  const Real W = lorentz_g(vp, G.g3);
  if (Wout) *Wout = W;
  return V3{{vp[0] / W, vp[1] / W, vp[2] / W}};
}

// MomentPrim2Con (moments.cpp:198-256)
void prim_to_con(const RPar &rp, const RBlk &R, int k, int j, int i) {
  const long long id = R.B.idx(k, j, i);
  const RGeo G(R, CENT, k, j, i);
  const Closure c(con_v_at(R, id, G), rp.m1, true, G.g());
  const Real J = R.Q(PHX_RJ, id);
  const V3 covH{{R.Q(PHX_RH, id) * J, R.Q(PHX_RH + 1, id) * J, R.Q(PHX_RH + 2, id) * J}};
  T2 Pi;
  c.TilPiFromPrim(J, covH, Pi);
  Real E;
  V3 covF;
  c.Prim2Con(J, covH, Pi, E, covF);
  const Real sdetgam = G.p.detgam;
  R.U(PHX_RE, id) = sdetgam * E;
  for (int d = 0; d < 3; d++) R.U(PHX_RF + d, id) = sdetgam * covF(d);
}

// MomentCon2PrimImpl (moments.cpp:61-159)
void con_to_prim(const RPar &rp, const RBlk &R, int k, int j, int i) {
  const long long id = R.B.idx(k, j, i);
  const RGeo G(R, CENT, k, j, i);
  const Real isdetgam = 1.0 / G.p.detgam;
  const Closure c(con_v_at(R, id, G), rp.m1, rp.robust, G.g());
  Real J;
  V3 covH;
  T2 Pi;
  Real E = R.U(PHX_RE, id) * isdetgam;
  V3 covF{{R.U(PHX_RF, id) * isdetgam, R.U(PHX_RF + 1, id) * isdetgam, R.U(PHX_RF + 2, id) * isdetgam}};
  Real xi = 0.0, phi = PI;
  if (rp.m1) {
    xi = R.Q(PHX_RXI, id);
    phi = 1.0001 * R.Q(PHX_RPHI, id);
  }
  c.TilPiFromCon(E, covF, xi, phi, Pi);
  if (rp.m1) {
    R.Q(PHX_RXI, id) = xi;
    R.Q(PHX_RPHI, id) = phi;
  }
  Status st = c.Con2Prim(E, covF, Pi, J, covH);
  if (st == MODIFIED) {
    c.Prim2Con(J, covH, Pi, E, covF);
    R.U(PHX_RE, id) = E / isdetgam;
    for (int d = 0; d < 3; d++) R.U(PHX_RF + d, id) = covF(d) / isdetgam;
    st = SUCCESS;
  }
  R.Q(PHX_RJ, id) = J;
  for (int d = 0; d < 3; d++) R.Q(PHX_RH + d, id) = ratio(covH(d), J);
  R.Q(PHX_RFAIL, id) = st == SUCCESS ? 1.0 : 0.0;
}

// MomentCalculateOpacities (moments.cpp:960-991)
void opacities(const RPar &rp, const RBlk &R, long long id) {
  const Real rho = R.fp(PHX_PRHO, id), T = R.fp(PHX_PTMP, id);
  const Real kJ = rp.kappaJ(rho, T);
  const Real kH = kJ + rp.kappaS(rho, T);
  R.Q(PHX_RJBB, id) = rp.JBB(T);
  R.Q(PHX_RKAPPAJ, id) = kJ;
  R.Q(PHX_RKAPPAH, id) = kH;
}

inline void recon5(int recon, Real qm2, Real qm1, Real q0, Real qp1, Real qp2, Real &ql, Real &qr) {
  switch (recon) {
  case PHX_RECON_WENO5Z: WENO5Z(qm2, qm1, q0, qp1, qp2, ql, qr); break;
  case PHX_RECON_MP5: MP5(qm2, qm1, q0, qp1, qp2, ql, qr); break;
  case PHX_RECON_LINEAR: PiecewiseLinear(qm1, q0, qp1, ql, qr); break;
  default: ql = q0; qr = q0;
  }
}

// One face of CalculateFluxesImpl (moments.cpp:548-722): direction d, the
// face between cells (k, j, i) - e_d and (k, j, i).  Left and right states
// come from the reconstruction of the two cells (ReconstructEdgeStates,
// moments.cpp:282-458: ql of a face = the upper value of the cell below,
// qr = the lower value of the cell above), dJ from its face formulas.
void face_flux(const RPar &rp, const RBlk &R, int d, int k, int j, int i) {
  const Blk &B = R.B;
  const int ndim = B.ndim;
  const int dj = ndim > 1 ? 1 : 0, dk = ndim > 2 ? 1 : 0;
  const long long st = d == 0 ? 1 : (d == 1 ? (long long)B.n1t : (long long)B.n1t * B.n2t);
  const long long id = B.idx(k, j, i), idm = id - st;
  // reconstructed J, H/J (4 values) and velocity (3): left from cell idm, right from id
  Real ql[7], qr[7];
  for (int n = 0; n < 7; n++) {
    auto val = [&](long long c) { return n < 4 ? R.Q(PHX_RJ + n, c) : R.fp(PHX_PVEL + n - 4, c); };
    Real a, b;
    recon5(rp.recon, val(idm - 2 * st), val(idm - st), val(idm), val(idm + st), val(idm + 2 * st), ql[n], a);
    recon5(rp.recon, val(id - 2 * st), val(id - st), val(id), val(id + st), val(id + 2 * st), b, qr[n]);
  }
  // dJ at this face (moments.cpp:412-455)
  auto Jat = [&](int kk, int jj, int ii) { return R.Q(PHX_RJ, B.idx(kk, jj, ii)); };
  const Real idx = 1.0 / B.dx(1), idx4 = 0.25 * idx;
  const Real idy = 1.0 / B.dx(2), idy4 = 0.25 * idy;
  const Real idz = 1.0 / B.dx(3), idz4 = 0.25 * idz;
  V3 cov_dJ;
  if (d == 0) {
    cov_dJ(0) = (Jat(k, j, i) - Jat(k, j, i - 1)) * idx;
    cov_dJ(1) = (Jat(k, j + dj, i) + Jat(k, j + dj, i - 1) - Jat(k, j - dj, i) - Jat(k, j - dj, i - 1)) * idy4;
    cov_dJ(2) = (Jat(k + dk, j, i) + Jat(k + dk, j, i - 1) - Jat(k - dk, j, i) - Jat(k - dk, j, i - 1)) * idz4;
  } else if (d == 1) {
    cov_dJ(0) = (Jat(k, j, i + 1) + Jat(k, j - dj, i + 1) - Jat(k, j, i - 1) - Jat(k, j - dj, i - 1)) * idx4;
    cov_dJ(1) = (Jat(k, j, i) - Jat(k, j - dj, i)) * idy;
    cov_dJ(2) = (Jat(k + dk, j, i) + Jat(k + dk, j - dj, i) - Jat(k - dk, j, i) - Jat(k - dk, j - dj, i)) * idz4;
  } else {
    cov_dJ(0) = (Jat(k, j, i + 1) + Jat(k - dk, j, i + 1) - Jat(k, j, i - 1) - Jat(k - dk, j, i - 1)) * idx4;
    cov_dJ(1) = (Jat(k, j + dj, i) + Jat(k - dk, j + dj, i) - Jat(k, j - dj, i) - Jat(k - dk, j - dj, i)) * idy4;
    cov_dJ(2) = (Jat(k, j, i) - Jat(k - dk, j, i)) * idz;
  }
  const RGeo G(R, d == 0 ? FACE1 : (d == 1 ? FACE2 : CENT), k, j, i);  // X3 faces: the centre table
  const Real dx = B.dx(d + 1) * std::sqrt(G.cov(d, d));
  Real vpl[3] = {ql[4], ql[5], ql[6]}, vpr[3] = {qr[4], qr[5], qr[6]};
  Real Wl = G.mink ? lorentz3(vpl) : lorentz_g(vpl, G.g3), Wr = G.mink ? lorentz3(vpr) : lorentz_g(vpr, G.g3);
  if (rp.bounds) {
    if (Wl > rp.W_ceiling) {
      const Real rescale = std::sqrt(rp.W_ceiling * rp.W_ceiling - 1.) / (Wl * Wl - 1.);
      for (int a = 0; a < 3; a++) vpl[a] *= rescale;
      Wl = rp.W_ceiling;
    }
    if (Wr > rp.W_ceiling) {
      const Real rescale = std::sqrt(rp.W_ceiling * rp.W_ceiling - 1.) / (Wr * Wr - 1.);
      for (int a = 0; a < 3; a++) vpr[a] *= rescale;
      Wr = rp.W_ceiling;
    }
  }
  const V3 vl{{vpl[0] / Wl, vpl[1] / Wl, vpl[2] / Wl}}, vr{{vpr[0] / Wr, vpr[1] / Wr, vpr[2] / Wr}};
  const Real alpha = G.p.alpha, beta_d = G.p.beta[d];
  const Real sigp = alpha * std::sqrt(G.con(d, d)) - beta_d;
  const Real sigm = -alpha * std::sqrt(G.con(d, d)) - beta_d;
  const Real asym_sigl = alpha * vl(d) - beta_d;
  const Real asym_sigr = alpha * vr(d) - beta_d;

  Real Jl = ql[0], Jr = qr[0];
  if (rp.bounds) {
    // at the face's X1 (moments.cpp:562-575)
    const Real Jf = rp.JFloor(d == 0 ? R.B.Xf(1, i) : R.B.Xc(1, i));
    Jl = smax(Jl, Jf);
    Jr = smax(Jr, Jf);
  }
  V3 Hl{{Jl * ql[1], Jl * ql[2], Jl * ql[3]}}, Hr{{Jr * qr[1], Jr * qr[2], Jr * qr[3]}};
  if (rp.bounds) {
    const Real vhl = cconcov(vl, Hl), vhr = cconcov(vr, Hr);
    const Real hhl = G.mink ? ccov(Hl, Hl) : G.g3.contract_cov(Hl, Hl);
    const Real hhr = G.mink ? ccov(Hr, Hr) : G.g3.contract_cov(Hr, Hr);
    const Real xil = std::sqrt(hhl - vhl * vhl) / Jl;
    const Real xir = std::sqrt(hhr - vhr * vhr) / Jr;
    if (xil > rp.xi_ceiling)
      for (int a = 0; a < 3; a++) Hl(a) *= rp.xi_ceiling / xil;
    if (xir > rp.xi_ceiling)
      for (int a = 0; a < 3; a++) Hr(a) *= rp.xi_ceiling / xir;
  }
  const Real kappaH = std::sqrt(R.Q(PHX_RKAPPAH, id) * R.Q(PHX_RKAPPAH, idm));
  const Real a = tanh_r(ratio(1.0, std::fabs(kappaH * dx)));
  const Real kappaH_min = 1.e-20;
  V3 HasymL;
  for (int c = 0; c < 3; c++) HasymL(c) = ratio(-cov_dJ(c), 3 * kappaH + 3 * kappaH_min);
  const V3 HasymR = HasymL;
  const Closure cl(vl, rp.m1, true, G.g()), cr(vr, rp.m1, true, G.g());
  T2 Pil, Pir, Pl, Pr, Pl_asym, Pr_asym;
  V3 conFl, conFr, conFl_asym, conFr_asym, covFl, covFr;
  Real El, Er;
  cl.TilPiFromPrim(Jl, HasymL, Pil);
  cr.TilPiFromPrim(Jr, HasymR, Pir);
  cl.FluxesFromPrim(Jl, HasymL, Pil, conFl_asym, Pl_asym);
  cr.FluxesFromPrim(Jr, HasymR, Pir, conFr_asym, Pr_asym);
  cl.TilPiFromPrim(Jl, Hl, Pil);
  cr.TilPiFromPrim(Jr, Hr, Pir);
  cl.FluxesFromPrim(Jl, Hl, Pil, conFl, Pl);
  cr.FluxesFromPrim(Jr, Hr, Pir, conFr, Pr);
  cl.Prim2Con(Jl, Hl, Pil, El, covFl);
  cr.Prim2Con(Jr, Hr, Pir, Er, covFr);
  for (int c = 0; c < 3; c++) {
    conFl(c) = a * conFl(c) + (1 - a) * conFl_asym(c);
    conFr(c) = a * conFr(c) + (1 - a) * conFr_asym(c);
  }
  for (int p = 0; p < 3; p++)
    for (int q = 0; q < 3; q++) {
      Pl(p, q) = a * Pl(p, q) + (1 - a) * Pl_asym(p, q);
      Pr(p, q) = a * Pr(p, q) + (1 - a) * Pr_asym(p, q);
    }
  const Real rad_sigspeed = smax(std::fabs(sigm), std::fabs(sigp));
  const Real asym_sigspeed = smax(std::fabs(asym_sigl), std::fabs(asym_sigr));
  const Real sigspeed = a * rad_sigspeed + (1. - a) * asym_sigspeed;
  conFl(d) -= beta_d * El;
  conFr(d) -= beta_d * Er;
  for (int c = 0; c < 3; c++) {
    Pl(d, c) -= beta_d * covFl(c);
    Pr(d, c) -= beta_d * covFr(c);
  }
  const Real sdetgam = G.p.detgam;
  R.F(d, PHX_RE, id) = 0.5 * sdetgam * (conFl(d) + conFr(d) + sigspeed * (El - Er));
  for (int c = 0; c < 3; c++)
    R.F(d, PHX_RF + c, id) = 0.5 * sdetgam * (Pl(d, c) + Pr(d, c) + sigspeed * (covFl(c) - covFr(c)));
  if (sdetgam < SMALL) {
    R.F(d, PHX_RE, id) = 0.0;
    for (int c = 0; c < 3; c++) R.F(d, PHX_RF + c, id) = 0.0;
  }
}

// CalculateGeometricSourceImpl (moments.cpp:764-885) of one zone off
// Minkowski: the radiation stress tensor T^{mu nu} from E, F^i (stage input)
// and P^{ij} of J, H_i (the stored primitives), contracted with the
// connection coefficients 0.5 (dg_{b a, c} + dg_{c a, b} - dg_{b c, a}) of the
// derivative table, g^{0 r} and d ln(alpha).  src: E, F_1..3 (densitised).
void geometric_source(bool m1, const RBlk &R, int k, int j, int i, Real src[4]) {
  const long long id = R.B.idx(k, j, i);
  const Geom Gm(R.B.b->geom, &R.B);
  const RGeo G(R, CENT, k, j, i);
  const V3 con_v = con_v_at(R, id, G);
  const Closure c(con_v, m1, true, G.g());
  const Real alp = G.p.alpha, sdetgam = G.p.detgam;
  const Real *con_beta = G.p.beta;
  Real con_g[4][4];
  Gm.SpacetimeMetricInverse(G.p, con_g);
  Real dlnalp[4], dg[4][4][4], Gamma[4][4][4];
  Gm.GradLnAlpha(k, j, i, dlnalp);
  Gm.MetricDerivative(k, j, i, dg);
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++)
      for (int cc = 0; cc < 4; cc++) Gamma[a][b][cc] = 0.5 * (dg[b][a][cc] + dg[cc][a][b] - dg[b][cc][a]);
  const Real con_n[4] = {1. / alp, -con_beta[0] / alp, -con_beta[1] / alp, -con_beta[2] / alp};
  const Real E = R.U(PHX_RE, id) / sdetgam;
  const Real J = R.Q(PHX_RJ, id);
  const V3 covF{{R.U(PHX_RF, id) / sdetgam, R.U(PHX_RF + 1, id) / sdetgam, R.U(PHX_RF + 2, id) / sdetgam}};
  const V3 covH{{J * R.Q(PHX_RH, id), J * R.Q(PHX_RH + 1, id), J * R.Q(PHX_RH + 2, id)}};
  T2 conTilPi, conP;
  c.TilPiFromPrim(J, covH, conTilPi);
  c.ConP(J, covH, conTilPi, conP);
  V3 conF;
  G.g3.raise(covF, conF);
  Real con_T[4][4];
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) con_T[mu][nu] = 0;
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) con_T[mu][nu] += con_n[mu] * con_n[nu] * E;
  for (int mu = 0; mu < 4; mu++)
    for (int ii = 0; ii < 3; ii++) {
      con_T[mu][ii + 1] += con_n[mu] * conF(ii);
      con_T[ii + 1][mu] += con_n[mu] * conF(ii);
    }
  for (int ii = 0; ii < 3; ii++)
    for (int jj = 0; jj < 3; jj++) con_T[ii + 1][jj + 1] += conP(ii, jj);
  Real TGam = 0.0;
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) {
      Real gam0 = 0.;
      for (int r = 0; r < 4; r++) gam0 += con_g[0][r] * Gamma[r][m][n];
      TGam += con_T[m][n] * gam0;
    }
  Real Ta = 0.0;
  for (int m = 0; m < 4; m++) Ta += con_T[m][0] * dlnalp[m];
  src[0] = sdetgam * alp * alp * (Ta - TGam);
  for (int l = 0; l < 3; l++) {
    Real src_mom = 0.0;
    for (int m = 0; m < 4; m++)
      for (int n = 0; n < 4; n++) src_mom += con_T[m][n] * (dg[n][l + 1][m] - Gamma[l + 1][n][m]);
    src[1 + l] = alp * sdetgam * src_mom;
  }
}

// The temperature residual of the oned solver (moments_source.cpp:152-196)
struct TResidual {
  const RPar &rp;
  Real rho, ug0, J0, dtau, alpha_max;
  Real operator()(Real T) const {
    Real kappa = rp.kappaJ(rho, T);
    kappa = smin(kappa, alpha_max);
    const Real JBB = rp.JBB(T);
    const Real dJ = (J0 + dtau * kappa * JBB) / (1. + dtau * kappa) - J0;
    const Real ug1 = rho * (rp.Cv * T);
    return ((ug1 - ug0) + dJ) / (ug0 + J0);
  }
};
// RootFind::regula_falsi with a status (root_find.hpp:111-160); the object
// (and its iteration count) persists across the re-bracketing attempts.
struct RF {
  int iteration_count = 0, max_iter;
  explicit RF(int m) : max_iter(m) {}
  template <typename Fn>
  Real regula_falsi(const Fn &func, Real a, Real b, Real tol, Real guess, bool &ok) {
    Real ya, yb;
    if (a <= guess && b >= guess) {
      ya = func(guess);
      yb = func(b);
      if (ya * yb > 0.0) {
        yb = ya;
        b = guess;
        ya = func(a);
      } else {
        a = guess;
      }
    } else {
      ya = func(a);
      yb = func(b);
    }
    if (ya * yb > 0.0) {
      ok = false;
      return guess;
    }
    const Real sign = (ya < 0 ? 1.0 : -1.0);
    ya *= sign;
    yb *= sign;
    int b1 = 0, b2 = 0;
    while (b - a > 2.0 * tol && iteration_count < max_iter) {
      const Real c = (a * yb - b * ya) / (yb - ya);
      if (c == a) {
        b = a;
        iteration_count++;
        continue;
      } else if (c == b) {
        a = b;
        iteration_count++;
        continue;
      }
      const Real yc = sign * func(c);
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
      iteration_count++;
    }
    ok = iteration_count != max_iter;
    return 0.5 * (a + b);
  }
};

// The fluid inversion of MomentFluidSourceImpl (ConToPrimSetup with
// c2p_fail_on_floors and c2p_fail_on_ceilings true, moments_source.cpp:286-295):
// con2prim_robust's solve of zone (k, j, i) from its stored mu, writing
// prims, cell speeds and (bounds used) conserved variables.  fp carries the
// two failure flags set.  True on success.
bool fluid_invert(const phx_params &fp, const Blk &B, int k, int j, int i) {
  GeomPt g;
  Geom(B.b->geom, &B).at(CENT, k, j, i, g);
  const EOS eos{fp.gm1, fp.Cv};
  const Bounds bounds(fp);
  const long long id = B.idx(k, j, i);
  const ZoneRef z{B.b->prim + id, B.b->cons + id, B.vs};
  Real sig[3];
  const C2PResult r = con2prim_core(g, eos, bounds, fp, B.Xc(1, i), B.Xc(2, j), B.Xc(3, k), z, z.P(PHX_PMU), sig);
  if (r.evals == 0) return false;  // NaN input: nothing written
  for (int d = 0; d < B.ndim; d++) B.b->cell_sig[d * B.vs + id] = sig[d];
  return r.success;
}

// update_fluid = true (moments_source.cpp:807-965): the fluid loses what the
// radiation gained (dE, cov_dF: the solve's last values, whether or not the
// radiation kept them), is inverted, and the closure inversion runs with the
// new fluid velocity (frail strategy).  On failure of either inversion the
// fluid is reset to rho = u = 10 SMALL at rest (P, T and the bulk modulus in
// the gamma1 slot, prim2con into D, S, tau) and the radiation to J = SMALL,
// H = 0 through the closure of the reset fluid, with the tilde-pressure
// tensor as the failed inversion left it (zero if the fluid failed).  B
// primitives enter that prim2con as stored (zero without MHD).
void update_fluid_zone(const RPar &rp, const phx_params &fp, const RBlk &R, const RGeo &G, int k, int j, int i,
                       long long id, Real dE, const V3 &cov_dF) {
  const Real sdetgam = G.p.detgam;
  const Blk &B = R.B;
  auto FU = [&](int v) -> Real & { return B.b->cons[v * B.vs + id]; };
  auto FP = [&](int v) -> Real & { return B.b->prim[v * B.vs + id]; };
  FU(PHX_CENG) -= sdetgam * dE;
  for (int a = 0; a < 3; a++) FU(PHX_CMOM + a) -= sdetgam * cov_dF(a);
  T2 Pi;
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 3; c++) Pi(a, c) = 0.0;
  Real E = R.U(PHX_RE, id) / sdetgam;
  V3 covF, covH;
  Real J;
  if (fluid_invert(fp, B, k, j, i)) {
    Real W;
    const V3 cv = con_v_at(R, id, G, &W);
    const Closure c(cv, rp.m1, false, G.g());
    for (int a = 0; a < 3; a++) covF(a) = R.U(PHX_RF + a, id) / sdetgam;
    Real xi = 0.0, phi = PI;
    c.TilPiFromCon(E, covF, xi, phi, Pi);
    if (c.Con2Prim(E, covF, Pi, J, covH) == SUCCESS) {
      R.Q(PHX_RJ, id) = J;
      for (int a = 0; a < 3; a++) R.Q(PHX_RH + a, id) = covH(a) / J;
      return;
    }
  }
  const EOS eos{fp.gm1, fp.Cv};
  FP(PHX_PRHO) = 10. * SMALL;
  FP(PHX_PENG) = 10. * SMALL;
  for (int a = 0; a < 3; a++) FP(PHX_PVEL + a) = 0.;
  FP(PHX_PPRS) = eos.PressureFromDensityInternalEnergy(FP(PHX_PRHO), ratio(FP(PHX_PENG), FP(PHX_PRHO)));
  FP(PHX_PTMP) = eos.TemperatureFromDensityInternalEnergy(FP(PHX_PRHO), ratio(FP(PHX_PENG), FP(PHX_PRHO)));
  FP(PHX_PGM1) = eos.BulkModulusFromDensityTemperature(FP(PHX_PRHO), FP(PHX_PTMP));
  const Real vp[3] = {FP(PHX_PVEL), FP(PHX_PVEL + 1), FP(PHX_PVEL + 2)};
  Real bp[3] = {0.0, 0.0, 0.0};
  if (fp.mhd)
    for (int a = 0; a < 3; a++) bp[a] = FP(PHX_PB + a);
  const GeomPt &g = G.p;
  Real D, tau, S[3], bcons[3], sig[3];
  p2c(FP(PHX_PRHO), vp, bp, FP(PHX_PENG), FP(PHX_PPRS), FP(PHX_PGM1), g.gcov, g.gamcon, g.beta, g.alpha, sdetgam, D,
      S, bcons, tau, sig);
  FU(PHX_CRHO) = D;
  for (int a = 0; a < 3; a++) FU(PHX_CMOM + a) = S[a];
  FU(PHX_CENG) = tau;
  Real Wc;
  const V3 cv2 = con_v_at(R, id, G, &Wc);
  const Closure c(cv2, rp.m1, false, G.g());
  R.Q(PHX_RJ, id) = SMALL;
  J = R.Q(PHX_RJ, id);
  for (int a = 0; a < 3; a++) {
    R.Q(PHX_RH + a, id) = 0.;
    covH(a) = R.Q(PHX_RH + a, id) * J;
  }
  c.Prim2Con(J, covH, Pi, E, covF);
  R.U(PHX_RE, id) = E * sdetgam;
  for (int a = 0; a < 3; a++) R.U(PHX_RF + a, id) = covF(a) * sdetgam;
}

// The fourd source solver's residual pieces (moments_source.cpp:39-150) for
// one zone.  Properties of the reference kept as they are: the fluid state
// enters prim2con with B = 0 (MomentFluidSourceImpl declares the B array a
// second time inside the block that reads it, moments_source.cpp:324-328, so
// the array it hands on stays zero); kappaH is the absorption coefficient
// added twice (:106-109), both capped at 1e5 before the source; the closure's
// xi guess, an uninitialised local there (:94-96), is SolveClosure's
// declared default 0.5 here.
struct SourceResidual4 {
  const RPar &rp;
  const EOS &eos;
  const RGeo &G;
  Real rho, sdetgam, alpha;
  Real U_mhd_0[4], U_rad_0[4];
  void MHDConserved(const Real P_mhd[4], Real U_mhd[4]) const {
    const Real Pg = eos.PressureFromDensityInternalEnergy(rho, P_mhd[0] / rho);
    const Real gam1 = eos.BulkModulusFromDensityInternalEnergy(rho, P_mhd[0] / rho) / Pg;
    const Real bprim[3] = {0.0, 0.0, 0.0};
    Real D, bcons[3], sig[3];
    p2c(rho, &P_mhd[1], bprim, P_mhd[0], Pg, gam1, G.p.gcov, G.p.gamcon, G.p.beta, G.p.alpha, sdetgam, D, &U_mhd[1],
        bcons, U_mhd[0], sig);
  }
  void RadConserved(const Real U_mhd[4], Real U_rad[4]) const {
    for (int n = 0; n < 4; n++) U_rad[n] = U_rad_0[n] - (U_mhd[n] - U_mhd_0[n]);
  }
  Real W_of(const Real P_mhd[4]) const {
    Real W = 0.;
    for (int ii = 0; ii < 3; ii++)
      for (int jj = 0; jj < 3; jj++) W += G.p.gcov[ii + 1][jj + 1] * P_mhd[ii + 1] * P_mhd[jj + 1];
    return std::sqrt(1. + W);
  }
  Status RadPrimitive(const Real P_mhd[4], const Real U_rad[4], Real P_rad[4]) const {
    const Real E = U_rad[0] / sdetgam;
    const V3 cov_F{{U_rad[1] / sdetgam, U_rad[2] / sdetgam, U_rad[3] / sdetgam}};
    const Real W = W_of(P_mhd);
    const V3 con_v{{P_mhd[1] / W, P_mhd[2] / W, P_mhd[3] / W}};
    const Closure c(con_v, rp.m1, true, G.g());
    Real xi = 0.5, phi = PI;
    T2 Pi;
    c.TilPiFromCon(E, cov_F, xi, phi, Pi);
    V3 cov_H;
    const Status st = c.Con2Prim(E, cov_F, Pi, P_rad[0], cov_H);
    for (int ii = 0; ii < 3; ii++) P_rad[ii + 1] = cov_H(ii);
    return st;
  }
  void Source(const Real P_mhd[4], const Real P_rad[4], Real S[4]) const {
    const Real Tg = eos.TemperatureFromDensityInternalEnergy(rho, P_mhd[0] / rho);
    const Real JBB = rp.JBB(Tg);
    Real kappaJ = rp.kappaJ(rho, Tg);
    Real kappaH = kappaJ + rp.kappaJ(rho, Tg);
    kappaH = smin(kappaH, 1.e5);
    kappaJ = smin(kappaJ, 1.e5);
    const Real W = W_of(P_mhd);
    Real cov_v[3] = {0.0, 0.0, 0.0};
    for (int ii = 0; ii < 3; ii++)
      for (int jj = 0; jj < 3; jj++) cov_v[ii] += G.p.gcov[ii + 1][jj + 1] * P_mhd[jj + 1] / W;
    Real vdH = 0.;
    for (int ii = 0; ii < 3; ii++) vdH += P_mhd[ii + 1] / W * P_rad[ii + 1];
    S[0] = alpha * sdetgam * (kappaJ * W * (JBB - P_rad[0]) - kappaH * vdH);
    for (int ii = 0; ii < 3; ii++)
      S[ii + 1] = alpha * sdetgam * (kappaJ * W * cov_v[ii] * (JBB - P_rad[0]) - kappaH * P_rad[1 + ii]);
  }
  // U_mhd, U_rad, P_rad and the source at P_mhd; the closure inversion's status
  Status eval(const Real P_mhd[4], Real U_mhd[4], Real U_rad[4], Real P_rad[4], Real S[4]) const {
    MHDConserved(P_mhd, U_mhd);
    RadConserved(U_mhd, U_rad);
    const Status st = RadPrimitive(P_mhd, U_rad, P_rad);
    Source(P_mhd, P_rad, S);
    return st;
  }
};

// LinearAlgebra::matrixInverse4x4 (linear_algebra.hpp:90-147): the adjugate
// from 3x3 minors (cofactor expansion), divided by the determinant expanded
// along the first row.
inline Real minor3(const Real m[16], int r0, int r1, int r2, int c0, int c1, int c2) {
  return m[4 * r0 + c0] * (m[4 * r1 + c1] * m[4 * r2 + c2] - m[4 * r2 + c1] * m[4 * r1 + c2]) -
         m[4 * r0 + c1] * (m[4 * r1 + c0] * m[4 * r2 + c2] - m[4 * r2 + c0] * m[4 * r1 + c2]) +
         m[4 * r0 + c2] * (m[4 * r1 + c0] * m[4 * r2 + c1] - m[4 * r2 + c0] * m[4 * r1 + c1]);
}
void inverse4x4(const Real a[4][4], Real inv[4][4]) {
  const Real *m = &a[0][0];
  Real *o = &inv[0][0];
  // column c of the adjugate holds the cofactors of row c
  static const int R[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  for (int col = 0; col < 4; col++)      // adjugate column = matrix row left out
    for (int row = 0; row < 4; row++) {  // adjugate row = matrix column left out
      const Real mn = minor3(m, R[col][0], R[col][1], R[col][2], R[row][0], R[row][1], R[row][2]);
      o[4 * row + col] = ((row + col) % 2 == 0) ? mn : -mn;
    }
  const Real det = m[0] * minor3(m, 1, 2, 3, 1, 2, 3) - m[1] * minor3(m, 1, 2, 3, 0, 2, 3) +
                   m[2] * minor3(m, 1, 2, 3, 0, 1, 3) - m[3] * minor3(m, 1, 2, 3, 0, 1, 2);
  for (int i = 0; i < 16; i++) o[i] /= det;
}

// The fourd solver (moments_source.cpp:489-786): Newton's method over
// P_mhd = (u, W v^i) for U_mhd(P) - U_mhd_0 + dt S = 0.  Each step: the
// Jacobian from centred differences of step eps max(min_m |P_m| over the
// nonzero P_m, |P_m|) (one-sided from the current guess when the closure
// inversion fails at one support point, failure at both), the update
// P -= J^-1 r, and after a failed inversion at the new guess the reference's
// step rescaling (its factor test admits only factors >= 1).  Converged when
// max_n |r_n| / max_n(|U_mhd_n| + |U_mhd_0,n| + |dt S_n|) <= tol; success
// also needs finite U_rad and fewer than maxiter iterations.  dE, cov_dF (the
// radiation's change, per sdetgam) are written only on success.
bool fourd_zone(const RPar &rp, const phx_params &fp, const RBlk &R, const RGeo &G, long long id, Real dt, Real &dE,
                V3 &cov_dF) {
  const EOS eos{fp.gm1, fp.Cv};
  const Real sdetgam = G.p.detgam;
  const Real rho = R.fp(PHX_PRHO, id), ug = R.fp(PHX_PENG, id);
  Real P[4] = {ug, R.fp(PHX_PVEL, id), R.fp(PHX_PVEL + 1, id), R.fp(PHX_PVEL + 2, id)};
  SourceResidual4 srm{rp, eos, G, rho, sdetgam, G.p.alpha, {}, {}};
  srm.MHDConserved(P, srm.U_mhd_0);
  for (int n = 0; n < 4; n++) srm.U_rad_0[n] = R.U(PHX_RE + n, id);
  const Real eps = rp.fd_eps, xi_max = rp.xi_ceiling;
  Real U_mhd[4], U_rad[4], P_rad[4], dS[4], resid[4];
  Status status = srm.eval(P, U_mhd, U_rad, P_rad, dS);
  for (int n = 0; n < 4; n++) resid[n] = U_mhd[n] - srm.U_mhd_0[n] + dt * dS[n];
  Real err = 1.e100;
  int niter = 0;
  bool bad_guess = false;
  do {
    Real jac[4][4] = {{0}};
    Real mag_min = std::numeric_limits<Real>::max();
    for (int m = 0; m < 4; m++)
      if (std::fabs(P[m]) > 0.) mag_min = smin(mag_min, std::fabs(P[m]));
    bool bad_m = false, bad_p = false;
    for (int m = 0; m < 4; m++) {
      Real Pm[4] = {P[0], P[1], P[2], P[3]}, Pp[4] = {P[0], P[1], P[2], P[3]};
      const Real step = smax(eps * mag_min, eps * std::fabs(P[m]));
      Pm[m] -= step;
      Pp[m] += step;
      Real Um[4], Urm[4], Prm[4], dSm[4], Up[4], Urp[4], Prp[4], dSp[4];
      if (srm.eval(Pm, Um, Urm, Prm, dSm) == FAILURE) bad_m = true;
      if (srm.eval(Pp, Up, Urp, Prp, dSp) == FAILURE) bad_p = true;
      for (int n = 0; n < 4; n++) {
        const Real fpl = Up[n] - srm.U_mhd_0[n] + dt * dSp[n];
        const Real fmi = Um[n] - srm.U_mhd_0[n] + dt * dSm[n];
        jac[n][m] = (fpl - fmi) / (Pp[m] - Pm[m]);
      }
    }
    if (bad_m && bad_p) {
      bad_guess = true;
      break;
    } else if (bad_m || bad_p) {  // one-sided from the guess, on the good side
      const Real side = bad_m ? 1.0 : -1.0;
      for (int m = 0; m < 4; m++) {
        Real Ps[4] = {P[0], P[1], P[2], P[3]};
        Ps[m] += side * smax(eps * mag_min, eps * std::fabs(Ps[m]));
        Real Us[4], Urs[4], Prs[4], dSs[4];
        srm.eval(Ps, Us, Urs, Prs, dSs);
        for (int n = 0; n < 4; n++) {
          const Real fs = Us[n] - srm.U_mhd_0[n] + dt * dSs[n];
          const Real fg = U_mhd[n] - srm.U_mhd_0[n] + dt * dS[n];
          jac[n][m] = bad_m ? (fs - fg) / (Ps[m] - P[m]) : (fg - fs) / (P[m] - Ps[m]);
        }
      }
    }
    Real jinv[4][4];
    inverse4x4(jac, jinv);
    if (!bad_guess) {
      const Real ug0 = P[0], ur0 = P_rad[0];
      for (int m = 0; m < 4; m++)
        for (int n = 0; n < 4; n++) P[m] -= jinv[m][n] * resid[n];
      status = srm.eval(P, U_mhd, U_rad, P_rad, dS);
      if (status == FAILURE) bad_guess = true;
      if (bad_guess) {
        const V3 cov_H{{P_rad[1] / P_rad[0], P_rad[2] / P_rad[0], P_rad[3] / P_rad[0]}};
        const V3 con_v{{P[1], P[2], P[3]}};
        const Real J = P_rad[0];
        Real hh, vh;
        if (G.mink) {
          hh = 0.0;
          for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) hh += (a == b ? 1.0 : 0.0) * cov_H(a) * cov_H(b);
        } else {
          hh = G.g3.contract_cov(cov_H, cov_H);
        }
        vh = 0.0;
        for (int a = 0; a < 3; a++) vh += con_v(a) * cov_H(a);
        const Real xi = std::sqrt(hh - vh * vh) / J;  // std::pow(vh, 2) there
        constexpr Real umin = 100. * SMALL, Jmin = 100. * SMALL;
        Real scale = 0.;
        if (xi > xi_max) scale = smax(scale, xi_max / xi);
        if (P[0] < umin) scale = smax(scale, (ug0 - umin) / (ug0 - P[0]));
        if (P_rad[0] < Jmin) scale = smax(scale, (ur0 - Jmin) / (ur0 - P_rad[0]));
        if (!(scale > SMALL && scale >= 1.)) {  // the reference prints and gives up
          bad_guess = true;
          break;
        }
        scale *= 0.5;
        for (int m = 0; m < 4; m++)
          for (int n = 0; n < 4; n++) P[m] += (1. - scale) * jinv[m][n] * resid[n];
        status = srm.eval(P, U_mhd, U_rad, P_rad, dS);
        if (status == SUCCESS) bad_guess = false;
      }
    }
    if (bad_guess) break;
    for (int n = 0; n < 4; n++) {
      resid[n] = U_mhd[n] - srm.U_mhd_0[n] + dt * dS[n];
      if (std::isnan(resid[n])) {
        bad_guess = true;
        break;
      }
    }
    if (bad_guess) break;
    err = SMALL;
    Real max_div = SMALL;
    for (int n = 0; n < 4; n++)
      max_div = smax(max_div, std::fabs(U_mhd[n]) + std::fabs(srm.U_mhd_0[n]) + std::fabs(dt * dS[n]));
    for (int n = 0; n < 4; n++) {
      const Real sub = std::fabs(resid[n]) / max_div;
      if (sub > err) err = sub;
    }
    niter++;
    if (niter == rp.maxiter) break;
  } while (err > rp.tol);
  if (niter == rp.maxiter || err > rp.tol || std::isnan(U_rad[0]) || std::isnan(U_rad[1]) ||
      std::isnan(U_rad[2]) || std::isnan(U_rad[3]) || bad_guess)
    return false;
  dE = (U_rad[0] - R.U(PHX_RE, id)) / sdetgam;
  for (int a = 0; a < 3; a++) cov_dF(a) = (U_rad[a + 1] - R.U(PHX_RF + a, id)) / sdetgam;
  return true;
}

// MomentFluidSourceImpl, oned or fourd solver, one species
// (moments_source.cpp:203-965); fp: the fluid inversion's settings
// (update_fluid).  Returns 1 when the source update was applied.
int fluid_source(const RPar &rp, const phx_params &fp, const RBlk &R, int k, int j, int i, Real dt) {
  const long long id = R.B.idx(k, j, i);
  const RGeo G(R, CENT, k, j, i);
  const Real alpha = G.p.alpha, sdetgam = G.p.detgam;
  const Real alpha_max = rp.tau_max / (alpha * dt);
  const Real rho = R.fp(PHX_PRHO, id), ug = R.fp(PHX_PENG, id), Tf = R.fp(PHX_PTMP, id);
  Real W;
  const V3 con_v = con_v_at(R, id, G, &W);
  Real dE = 0.0;
  V3 cov_dF{{0.0, 0.0, 0.0}};
  bool success = false;
  bool oned = !rp.fourd;
  if (rp.fourd) {
    // fourd, falling back to the oned solver when it fails and
    // src_use_oned_backup is set (the reference's goto, :781-785); without
    // the fallback a failed zone keeps dE = cov_dF = 0 (left uninitialised
    // there) for the fluid update
    success = fourd_zone(rp, fp, R, G, id, dt, dE, cov_dF);
    oned = !success && rp.oned_backup;
  }
  if (oned) {
    const Real J0 = R.Q(PHX_RJ, id);
    const Real dtau = alpha * dt / W;
    RF root(rp.maxiter);
    TResidual res{rp, rho, ug, J0, dtau, alpha_max};
    bool ok;
    Real T1 = root.regula_falsi(res, 1.e-2 * Tf, 1.e2 * Tf, rp.tol * Tf, Tf, ok);
    Real fac = 10.;
    int tries = 0;
    while (!ok && tries < 4) {
      T1 = root.regula_falsi(res, 1.e-1 / fac * Tf, 1.e1 * fac * Tf, rp.tol * Tf, Tf, ok);
      tries++;
      fac *= 10.;
    }
    const Closure c(con_v, rp.m1, true, G.g());
    Real Estar = R.U(PHX_RE, id) / sdetgam;
    V3 Fstar{{R.U(PHX_RF, id) / sdetgam, R.U(PHX_RF + 1, id) / sdetgam, R.U(PHX_RF + 2, id) / sdetgam}};
    Real J = R.Q(PHX_RJ, id);
    V3 cov_H{{J * R.Q(PHX_RH, id), J * R.Q(PHX_RH + 1, id), J * R.Q(PHX_RH + 2, id)}};
    T2 Pi;
    c.TilPiFromPrim(J, cov_H, Pi);
    const Real JBB = rp.JBB(T1);
    Real kappaJ = smin(rp.kappaJ(rho, T1), alpha_max);
    Real kappaH = smin(rp.kappaS(rho, T1), alpha_max);
    kappaH += kappaJ;
    Real tauJ = alpha * dt * kappaJ;
    Real tauH = alpha * dt * kappaH;
    if (ok) {
      c.LinearSourceUpdate(Estar, Fstar, Pi, JBB, tauJ, tauH, dE, cov_dF);
      Estar += dE;
      for (int a = 0; a < 3; a++) Fstar(a) += cov_dF(a);
      success = c.Con2Prim(Estar, Fstar, Pi, J, cov_H) == SUCCESS;
    }
    if (!success && rp.oned_fixup == PHX_RAD_ONED_FIXUP_IGNORE_DJ) {
      Estar = R.U(PHX_RE, id) / sdetgam;
      for (int a = 0; a < 3; a++) Fstar(a) = R.U(PHX_RF + a, id) / sdetgam;
      const Real JBB2 = rp.JBB(Tf);
      const Real kJ = rp.kappaJ(rho, T1);
      const Real kH = rp.kappaS(rho, T1) + kJ;
      tauJ = alpha * dt * kJ;
      tauH = alpha * dt * kH;
      c.LinearSourceUpdate(Estar, Fstar, Pi, JBB2, tauJ, tauH, dE, cov_dF);
      Estar = R.U(PHX_RE, id) / sdetgam + dE;
      for (int a = 0; a < 3; a++) Fstar(a) = R.U(PHX_RF + a, id) / sdetgam + cov_dF(a);
      success = c.Con2Prim(Estar, Fstar, Pi, J, cov_H) == SUCCESS;
    } else if (!success && rp.oned_fixup == PHX_RAD_ONED_FIXUP_IGNORE_ALL) {
      dE = 0.;
      for (int a = 0; a < 3; a++) cov_dF(a) = 0.;
      success = true;
    }
  }
  if (success) {
    R.U(PHX_RE, id) += sdetgam * dE;
    for (int a = 0; a < 3; a++) R.U(PHX_RF + a, id) += sdetgam * cov_dF(a);
  }
  if (rp.update_fluid) {
    update_fluid_zone(rp, fp, R, G, k, j, i, id, dE, cov_dF);
    return success ? 1 : 0;
  }
  T2 Pi;
  Real E = R.U(PHX_RE, id) / sdetgam;
  V3 covF;
  Real J;
  V3 covH;
  {
    const Closure c(con_v, rp.m1, false, G.g());
    for (int a = 0; a < 3; a++) covF(a) = R.U(PHX_RF + a, id) / sdetgam;
    Real xi = 0.0, phi = PI;
    c.TilPiFromCon(E, covF, xi, phi, Pi);
    if (c.Con2Prim(E, covF, Pi, J, covH) == SUCCESS) {
      R.Q(PHX_RJ, id) = J;
      for (int a = 0; a < 3; a++) R.Q(PHX_RH + a, id) = covH(a) / J;
      return success ? 1 : 0;
    }
  }
  // failed inversion: the reference's zero-radiation state
  Real Wc;
  const V3 cv2 = con_v_at(R, id, G, &Wc);
  const Closure c(cv2, rp.m1, false, G.g());
  R.Q(PHX_RJ, id) = SMALL;
  J = R.Q(PHX_RJ, id);
  for (int a = 0; a < 3; a++) {
    R.Q(PHX_RH + a, id) = 0.;
    covH(a) = R.Q(PHX_RH + a, id) * J;
  }
  c.Prim2Con(J, covH, Pi, E, covF);
  R.U(PHX_RE, id) = E * sdetgam;
  for (int a = 0; a < 3; a++) R.U(PHX_RF + a, id) = covF(a) * sdetgam;
  return success ? 1 : 0;
}

// RadConservedToPrimitiveFixupImpl (fixup_radc2p.cpp:45-225) at an interior
// zone whose closure inversion failed: the c2pfail-weighted neighbour average
// of J and H_i / J (a failed neighbour contributes nothing), or J = 10 SMALL,
// H = 0; the xi ceiling on H / J; E, F_i from prim2con.
void rad_c2p_fixup_zone(const RPar &rp, const RBlk &R, int k, int j, int i) {
  const Blk &B = R.B;
  const long long id = B.idx(k, j, i);
  if (R.Q(PHX_RFAIL, id) != 0.0) return;
  const RGeo G(R, CENT, k, j, i);
  const V3 con_v = con_v_at(R, id, G);
  const long long di = 1, dj = B.n1t, dk = (long long)B.n1t * B.n2t;
  auto F = [&](long long o) { return R.Q(PHX_RFAIL, o); };
  auto nb = [&](int iv, long long o) { return F(o) != 0.0 ? F(o) * R.Q(iv, o) : 0.0; };
  auto fixv = [&](int iv, Real norm) {
    Real sum = nb(iv, id - di) + nb(iv, id + di);
    if (B.ndim > 1) {
      sum += nb(iv, id - dj) + nb(iv, id + dj);
      if (B.ndim == 3) sum += nb(iv, id - dk) + nb(iv, id + dk);
    }
    return norm * sum;
  };
  Real num_valid = F(id - di) + F(id + di);
  if (B.ndim > 1) num_valid += F(id - dj) + F(id + dj);
  if (B.ndim == 3) num_valid += F(id - dk) + F(id + dk);
  Real J;
  V3 Hr;
  if (num_valid > 0.5 && !rp.fixup_floors) {
    const Real norm = 1.0 / num_valid;
    J = fixv(PHX_RJ, norm);
    for (int a = 0; a < 3; a++) Hr(a) = fixv(PHX_RH + a, norm);
  } else {
    J = 10. * SMALL;
    for (int a = 0; a < 3; a++) Hr(a) = 0.;
  }
  const Real hh = G.mink ? ccov(Hr, Hr) : G.g3.contract_cov(Hr, Hr);
  const Real vh = cconcov(con_v, Hr);
  const Real xi = std::sqrt(hh - vh * vh);
  if (xi > rp.xi_ceiling)
    for (int a = 0; a < 3; a++) Hr(a) *= rp.xi_ceiling / xi;
  R.Q(PHX_RJ, id) = J;
  for (int a = 0; a < 3; a++) R.Q(PHX_RH + a, id) = Hr(a);
  const Closure c(con_v, rp.m1, true, G.g());
  V3 H{{Hr(0) * J, Hr(1) * J, Hr(2) * J}};
  T2 Pi;
  c.TilPiFromPrim(J, H, Pi);
  Real E;
  V3 Fc;
  c.Prim2Con(J, H, Pi, E, Fc);
  const Real sdetgam = G.p.detgam;
  R.U(PHX_RE, id) = sdetgam * E;
  for (int a = 0; a < 3; a++) R.U(PHX_RF + a, id) = sdetgam * Fc(a);
}

// ApplyFloorsImpl's radiation part (fixup.cpp:542-678, enable_rad_floors,
// one species) after the fluid part of the zone; flag: the fluid part acted.
void rad_floors_zone(const RPar &rp, const RBlk &R, int k, int j, int i, bool flag) {
  const long long id = R.B.idx(k, j, i);
  const RGeo G(R, CENT, k, j, i);
  const Real sdetgam = G.p.detgam;
  const V3 con_v = con_v_at(R, id, G);
  const Closure c(con_v, rp.m1, true, G.g());
  Real E, J;
  V3 F, H;
  T2 Pi;
  auto invert = [&]() {
    Real xi = 0.0, phi = std::acos(-1.0) * 1.000001;
    c.TilPiFromCon(E, F, xi, phi, Pi);
    c.Con2Prim(E, F, Pi, J, H);
    R.Q(PHX_RJ, id) = J;
    for (int a = 0; a < 3; a++) R.Q(PHX_RH + a, id) = H(a) / J;
  };
  if (flag) {
    E = R.U(PHX_RE, id) / sdetgam;
    for (int a = 0; a < 3; a++) F(a) = R.U(PHX_RF + a, id) / sdetgam;
    invert();
  }
  const Real dJ = rp.JFloor(R.B.Xc(1, i)) - R.Q(PHX_RJ, id);
  if (dJ > 0.) {
    const V3 zero{{0.0, 0.0, 0.0}};
    T2 Pz;
    for (int a = 0; a < 3; a++)
      for (int q = 0; q < 3; q++) Pz(a, q) = 0.0;
    const Closure c_iso(zero, rp.m1, true, G.g());
    c_iso.Prim2Con(dJ, zero, Pz, E, F);
    E += R.U(PHX_RE, id) / sdetgam;
    for (int a = 0; a < 3; a++) F(a) += R.U(PHX_RF + a, id) / sdetgam;
    R.U(PHX_RE, id) = E * sdetgam;
    for (int a = 0; a < 3; a++) R.U(PHX_RF + a, id) = F(a) * sdetgam;
    invert();
  }
  const V3 Hr{{R.Q(PHX_RH, id), R.Q(PHX_RH + 1, id), R.Q(PHX_RH + 2, id)}};
  const Real hh = G.mink ? ccov(Hr, Hr) : G.g3.contract_cov(Hr, Hr);
  const Real vh = cconcov(con_v, Hr);
  const Real xi = std::sqrt(hh - vh * vh);
  if (xi > rp.xi_ceiling) {
    J = R.Q(PHX_RJ, id);
    for (int a = 0; a < 3; a++) {
      H(a) = (rp.xi_ceiling / xi) * Hr(a) * J;
      R.Q(PHX_RH + a, id) = H(a) / J;
    }
    c.TilPiFromPrim(J, H, Pi);
    c.Prim2Con(J, H, Pi, E, F);
    R.U(PHX_RE, id) = E * sdetgam;
    for (int a = 0; a < 3; a++) R.U(PHX_RF + a, id) = F(a) * sdetgam;
  }
}

// radiation.cpp:585-648 (one species)
Real zone_dt(const RPar &rp, const RBlk &R, int k, int j, int i) {
  const long long id = R.B.idx(k, j, i);
  const RGeo G(R, CENT, k, j, i);
  const Real alpha = G.p.alpha;
  Real ldt = std::numeric_limits<Real>::max();
  const Real kappaH = R.Q(PHX_RKAPPAH, id);
  for (int d = 0; d < R.B.ndim; d++) {
    const Real sigp = alpha * std::sqrt(G.con(d, d)) - G.p.beta[d];
    const Real sigm = -alpha * std::sqrt(G.con(d, d)) - G.p.beta[d];
    const Real asym_sigl = alpha * R.fp(PHX_PVEL + d, id) - G.p.beta[d];
    const Real rad_speed = smax(std::fabs(sigm), std::fabs(sigp));
    const Real asym_speed = std::fabs(asym_sigl);
    const Real w = R.B.dx(d + 1);
    const Real dx = w * std::sqrt(G.cov(d, d));
    const Real a = tanh_r(ratio(1.0, std::fabs(kappaH * dx)));
    const Real csig = a * rad_speed + (1. - a) * asym_speed;
    ldt = smin(ldt, 1.0 / (csig / w));
  }
  return ldt;
}

}  // namespace rad
}  // namespace orc

extern "C" {
using namespace orc::rad;

void orc_rad_prim_to_con(const phx_rad_params *rp, const phx_params *p, const phx_block *fb, const phx_rad_block *rb,
                         phx_range ib, phx_range jb, phx_range kb) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = kb.s; k <= kb.e; k++)
    for (int j = jb.s; j <= jb.e; j++)
      for (int i = ib.s; i <= ib.e; i++) prim_to_con(P, R, k, j, i);
}

void orc_rad_con_to_prim(const phx_rad_params *rp, const phx_params *p, const phx_block *fb, const phx_rad_block *rb,
                         phx_range ib, phx_range jb, phx_range kb) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
  for (int k = kb.s; k <= kb.e; k++)
    for (int j = jb.s; j <= jb.e; j++)
      for (int i = ib.s; i <= ib.e; i++) con_to_prim(P, R, k, j, i);
}

void orc_rad_calculate_opacities(const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                                 const phx_rad_block *rb) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
  for (long long id = 0; id < R.B.N; id++) opacities(P, R, id);
}

// Every face the interior update reads: X1 faces i in [is, ie + 1] of
// interior rows, and likewise for X2, X3.
void orc_rad_calculate_fluxes(const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                              const phx_rad_block *rb) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
  const orc::Blk &B = R.B;
  for (int d = 0; d < B.ndim; d++) {
    const int ie = B.ie() + (d == 0), je = B.je() + (d == 1), ke = B.ke() + (d == 2);
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = B.ks(); k <= ke; k++)
      for (int j = B.js(); j <= je; j++)
        for (int i = B.is(); i <= ie; i++) face_flux(P, R, d, k, j, i);
  }
}

void orc_rad_update(const phx_rad_params *rp, const phx_block *fb, const phx_rad_block *rb, const double *base,
                    double *out, double beta, double dt) {
  const bool m1 = rp->method == PHX_RAD_M1;
  const RBlk R(fb, rb);
  // the geometric source reads the stage input: every zone's before the
  // in-place averaging below touches any
  std::vector<Real> gsrc;
  if (fb->geom && fb->geom->kind != PHX_GEOM_MINKOWSKI) {
    gsrc.assign(4 * (size_t)R.rvs, 0.0);
    const orc::Blk &Bk = R.B;
    for (int k = Bk.ks(); k <= Bk.ke(); k++)
      for (int j = Bk.js(); j <= Bk.je(); j++)
        for (int i = Bk.is(); i <= Bk.ie(); i++) {
          Real src[4];
          geometric_source(m1, R, k, j, i, src);
          for (int m = 0; m < 4; m++) gsrc[m * R.rvs + Bk.idx(k, j, i)] = src[m];
        }
  }
  const orc::Blk &B = R.B;
  const Real dx1 = fb->dx1, dx2 = fb->dx2, dx3 = fb->dx3;
  const Real A1 = dx2 * dx3, A2 = dx1 * dx3, A3 = dx1 * dx2, V = dx1 * dx2 * dx3;
  const Real bdt = beta * dt;
  const long long s1 = 1, s2 = B.n1t, s3 = (long long)B.n1t * B.n2t;
#pragma omp parallel for collapse(2) schedule(static)
  for (int m = 0; m < PHX_RNCONS; m++)
    for (int k = B.ks(); k <= B.ke(); k++)
      for (int j = B.js(); j <= B.je(); j++)
        for (int i = B.is(); i <= B.ie(); i++) {
          const long long id = B.idx(k, j, i);
          Real du = (A1 * R.F(0, m, id + s1) - A1 * R.F(0, m, id));
          if (B.ndim >= 2) du += A2 * R.F(1, m, id + s2) - A2 * R.F(1, m, id);
          if (B.ndim == 3) du += A3 * R.F(2, m, id + s3) - A3 * R.F(2, m, id);
          const Real r = -du / V + (gsrc.empty() ? 0.0 : gsrc[m * R.rvs + id]);  // + the geometric source
          rb->dudt[m * R.rvs + id] = r;
          Real u0 = R.U(m, id);
          u0 = beta * u0 + (1 - beta) * base[m * R.rvs + id];
          R.U(m, id) = u0;
          out[m * R.rvs + id] = u0 + bdt * r;
        }
}

long long orc_rad_fluid_source(const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                               const phx_rad_block *rb, double dt) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
  const orc::Blk &B = R.B;
  phx_params fp = *p;  // the inversion MomentFluidSourceImpl sets up
  fp.c2p_fail_on_floors = 1;
  fp.c2p_fail_on_ceilings = 1;
  long long applied = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) reduction(+ : applied)
  for (int k = B.ks(); k <= B.ke(); k++)
    for (int j = B.js(); j <= B.je(); j++)
      for (int i = B.is(); i <= B.ie(); i++) applied += fluid_source(P, fp, R, k, j, i, dt);
  return applied;
}

// CalculateGeometricSource into out[4][N] over the interior (FMKS blocks;
// zero on Minkowski), for tests of the source alone.
void orc_rad_geometric_source(const phx_rad_params *rp, const phx_block *fb, const phx_rad_block *rb, double *out) {
  const RBlk R(fb, rb);
  const orc::Blk &B = R.B;
  const bool curved = fb->geom && fb->geom->kind != PHX_GEOM_MINKOWSKI;
  for (int k = B.ks(); k <= B.ke(); k++)
    for (int j = B.js(); j <= B.je(); j++)
      for (int i = B.is(); i <= B.ie(); i++) {
        Real src[4] = {0.0, 0.0, 0.0, 0.0};
        if (curved) geometric_source(rp->method == PHX_RAD_M1, R, k, j, i, src);
        for (int m = 0; m < 4; m++) out[m * R.rvs + B.idx(k, j, i)] = src[m];
      }
}

void orc_rad_c2p_fixup(const phx_rad_params *rp, const phx_params *p, const phx_block *fb, const phx_rad_block *rb) {
  if (!p->enable_c2p_fixup) return;
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
  const orc::Blk &B = R.B;
  for (int k = B.ks(); k <= B.ke(); k++)
    for (int j = B.js(); j <= B.je(); j++)
      for (int i = B.is(); i <= B.ie(); i++) rad_c2p_fixup_zone(P, R, k, j, i);
}

// ApplyFloors with radiation active: the fluid part, then (enable_rad_floors)
// the radiation part, zone by zone over the range.
void orc_rad_apply_floors(const phx_rad_params *rp, const phx_params *p, const phx_block *fb, const phx_rad_block *rb,
                          phx_range ib, phx_range jb, phx_range kb) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
  std::vector<double> flag((size_t)R.B.N, 0.0);
  orc::apply_floors(*p, fb, ib, jb, kb, flag.data());
  if (!rp->enable_rad_floors || !p->enable_floors) return;
  for (int k = kb.s; k <= kb.e; k++)
    for (int j = jb.s; j <= jb.e; j++)
      for (int i = ib.s; i <= ib.e; i++) rad_floors_zone(P, R, k, j, i, flag[R.B.idx(k, j, i)] != 0.0);
}

void orc_rad_fill_ghosts_periodic(const phx_block *fb, const phx_rad_block *rb) {
  const RBlk R(fb, rb);
  phx_block tmp = *fb;
  tmp.var_stride = R.rvs;
  orc_fill_ghosts_periodic(&tmp, rb->cons, PHX_RNCONS);
  orc_fill_ghosts_periodic(&tmp, rb->prim, PHX_RFAIL + 1);
}

double orc_rad_estimate_timestep(const phx_rad_params *rp, const phx_params *p, const phx_block *fb,
                                 const phx_rad_block *rb) {
  const RPar P(*rp, *p);
  const RBlk R(fb, rb);
  const orc::Blk &B = R.B;
  Real min_dt = std::numeric_limits<Real>::max();
  for (int k = B.ks(); k <= B.ke(); k++)
    for (int j = B.js(); j <= B.je(); j++)
      for (int i = B.is(); i <= B.ie(); i++) min_dt = smin(min_dt, zone_dt(P, R, k, j, i));
  return rp->cfl * min_dt;
}

double orc_rad_tanh(double x) { return tanh_r(x); }

// phx_math.h's functions over an array (fn as PHX_MATH_*), for their tests.
void orc_math_eval(int fn, long long n, const double *x, const double *y, double *out) {
  for (long long q = 0; q < n; q++) {
    switch (fn) {
    case PHX_MATH_EXP: out[q] = phx_math::exp(x[q]); break;
    case PHX_MATH_LOG: out[q] = phx_math::log(x[q]); break;
    case PHX_MATH_SIN: out[q] = phx_math::sin(x[q]); break;
    case PHX_MATH_COS: out[q] = phx_math::cos(x[q]); break;
    default: out[q] = phx_math::pow(x[q], y[q]); break;
    }
  }
}

// ClosureM1::GetM1GuessesFromEddington (closure_m1.hpp:146-168) for n zones:
// the Eddington inversion's xi = |H| / J (capped at 0.99) and phi = 1.000001 pi,
// from E, F_i [3][n] and the fluid's coordinate velocity v^i [3][n].
void orc_rad_m1_guess(const double *E, const double *F, const double *v, long long n, double *xi_out,
                      double *phi_out) {
  for (long long z = 0; z < n; z++) {
    const V3 cv{{v[z], v[n + z], v[2 * n + z]}};
    const Closure c(cv, true, true);
    const V3 cF{{F[z], F[n + z], F[2 * n + z]}};
    T2 Pi;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Pi(i, j) = 0.0;
    Real JEdd;
    V3 HEdd;
    c.Con2Prim(E[z], cF, Pi, JEdd, HEdd);
    const Real vH = cconcov(cv, HEdd);
    const Real Hm = std::sqrt(ccov(HEdd, HEdd) - vH * vH);
    xi_out[z] = smin(ratio(Hm, JEdd), 0.99);
    phi_out[z] = 1.000001 * PI;
  }
}

}  // extern "C"
