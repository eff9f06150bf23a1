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
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "../include/phx_fluid.h"

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
      rflr = r0 * std::exp(ralpha * x1);
      sflr = s0 * std::exp(salpha * x1);
      break;
    case PHX_FLOOR_EXPX1_RHO_U: {
      Real scratch = r0 * std::exp(ralpha * x1);
      sflr = s0 * std::exp(salpha * x1) / std::max(rflr, scratch);
      rflr = scratch;
    } break;
    case PHX_FLOOR_X1_RHO_SIE:
      rflr = r0 * std::min(1.0, std::pow(x1, ralpha));
      sflr = s0 * std::min(1.0, std::pow(x1, salpha));
      break;
    default: {  // PHX_FLOOR_R_RHO_SIE
      Real r = std::sqrt(x1 * x1 + x2 * x2 + x3 * x3);
      rflr = r0 * std::min(1.0, std::pow(r, ralpha));
      sflr = s0 * std::min(1.0, std::pow(r, salpha));
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
    norm = 0.5 * M_PI * 1. / (1. + 1. / (alpha + 1.) * 1. / std::pow(xt, alpha));
  }
  // ---- McKinneyGammieRyan (mckinney_gammie_ryan.hpp:64-198)
  Real r_(Real X1) const {
    const Real hexp_dr = X1 - hexp_br;
    return std::exp(X1 + (hexp_dr > 0.) * hexp_csq * std::pow(hexp_dr, hexp_nsq));
  }
  Real thG_(Real X2) const { return M_PI * X2 + ((1. - h) / 2.) * std::sin(2. * M_PI * X2); }
  void thJ_(Real X2, Real &y, Real &thJ) const {
    y = 2. * X2 - 1.;
    thJ = norm * y * (1. + std::pow(y / xt, alpha) / (alpha + 1.)) + 0.5 * M_PI;
  }
  void th_(Real X1, Real X2, Real &y, Real &th) const {
    Real thG = thG_(X2);
    if (derefine_poles) {
      Real thJ;
      thJ_(X2, y, thJ);
      const Real fac = x0 - X1;
      th = thG + std::exp(smooth * fac) * (thJ - thG);
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
        std::exp(X1 + (hexp_dr > 0.) * hexp_csq * std::pow(hexp_dr, hexp_nsq)) *
        (1. + (hexp_dr > 0.) * hexp_csq * hexp_nsq * std::pow(hexp_dr, hexp_nsq - 1.));
    const Real dthGdX2 = M_PI + M_PI * (1 - h) * std::cos(2 * M_PI * X2);
    Real dthdX1, dthdX2;
    if (derefine_poles) {
      thJ_(X2, y, thJ);
      const Real thG = thG_(X2);
      const Real dydX2 = 2.;
      const Real dthJdy = norm * (1 + std::pow(y / xt, alpha));
      const Real dthJdX2 = dthJdy * dydX2;
      const Real fac = x0 - X1;
      dthdX1 = -smooth * (thJ - thG) * std::exp(smooth * fac);
      dthdX2 = dthGdX2 + std::exp(smooth * fac) * (dthJdX2 - dthGdX2);
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
    cth = std::cos(th);
    sth = std::sin(th);
    sth2 = sth * sth;
    rho2 = rho2_(r, cth);
  }
  Real ks_lapse(Real X1, Real X2) const {
    const Real r = std::abs(X1);
    const Real cth = std::cos(X2);
    const Real rho2 = rho2_(r, cth);
    return std::sqrt(ratio(rho2, 2 * r + rho2));
  }
  void ks_shift(Real X1, Real X2, Real beta[3]) const {
    Real r = std::abs(X1);
    Real cth = std::cos(X2);
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
    Real EPSFD = std::pow(std::numeric_limits<Real>::epsilon(), 1.0 / 3.0);
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
    Real EPSFD = std::pow(std::numeric_limits<Real>::epsilon(), 1.0 / 3.0);
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
C2PResult con2prim_core(const GeomPt &g, const EOS &eos, const Bounds &bounds, const phx_params &par,
                        Real x1, Real x2, Real x3, const ZoneRef &z, Real guess, Real sig[3],
                        const Real *learned = nullptr) {
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
  RootFind root(par.c2p_max_iter);
  bool bracketed = true;
  const Real mu = learned ? root.regula_falsi_learned(resid, learned[0], learned[1], learned[2], par.c2p_tol,
                                                      guess, bracketed, res.learned_accepted)
                          : root.regula_falsi(resid, 0.0, 1.0, par.c2p_tol, guess, bracketed);
  res.bracketed = bracketed;
  res.iterations = root.iteration_count;
  res.evals = root.evals;
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
  if (!bracketed) return res;
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
long long apply_floors(const phx_params &par, const phx_block *blk, phx_range ib, phx_range jb, phx_range kb) {
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
