// phx_m1.cu -- radiation moment transport (M1 and Eddington closures) on the
// device: one neutrino species, Minkowski metric, a static fluid background
// or (update_fluid) a fluid that exchanges energy and momentum with the
// radiation in the source step.
//
// Follows, in the reference's floating-point operation order (paths relative
// to the phoebus tree): radiation/closure.hpp:49-352 (ClosureEdd),
// closure_m1.hpp:31-372 (ClosureM1), local_three_geometry.hpp:140-185,
// linear_algebra.hpp:58-96, moments.cpp:61-995, moments_source.cpp:152-958
// (oned solver; update_fluid with the fluid's con2prim), radiation.cpp:585-648,
// root_find.hpp:111-160.  With the identity spatial metric each contraction
// keeps the order of its non-zero terms (for finite values the zero terms of
// the full 3x3 sums change no rounding).  std::pow(x, 2) and std::pow(x, 3)
// are products, and tanh is written out (Cody-Waite reduction + Taylor
// series) so that a CPU build without FMA contraction gives the same bits.
//
// One thread per zone (con2prim, source, prim2con, update) or per face
// (fluxes).  The fluxes of a face need only the row d of the pressure
// tensors P^i_j of its direction; the other rows are not formed.
#include <cfloat>

#include "phx_m1.cuh"

namespace phx {
namespace rad {

// Production-build arithmetic (the exact build keeps the reference's IEEE
// divisions): x / 3 as a product with 1/3, divisions by W as products with
// 1/W, shared reciprocals for repeated denominators.
#ifdef PHX_EXACT
#define D3(x) ((x) / 3)
#define DW(x) ((x) / W)
#else
#define D3(x) ((x) * (1.0 / 3.0))
#define DW(x) ((x) * iW)
#endif

// std::min / std::max (NaN handling of the reference)
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double sgn(double v) { return (double)((0.0 <= v) - (v < 0.0)); }

// tanh: e^y by Cody-Waite reduction y = n ln2 + r (32-bit head of ln2, so
// n * head is exact) and the Taylor series of e^r to degree 13; e^y - 1 by its
// Taylor series to degree 14 for |y| < 1/4; tanh x = -m / (2 + m) with
// m = e^{-2|x|} - 1.
constexpr double LN2_HI = 0.693147180369123816490;
constexpr double LN2_LO = 1.9082149292705877000e-10;
constexpr double INV_LN2 = 1.4426950408889634074;
__device__ __forceinline__ double exp_taylor(double r) {
  double p = 1.0 / 6227020800.0;
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
__device__ __forceinline__ double expm1_small(double y) {
  double p = 1.0 / 87178291200.0;
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
__device__ __forceinline__ double exp_neg(double y) {
  const double n = floor(y * INV_LN2 + 0.5);
  const double r = (y - n * LN2_HI) - n * LN2_LO;
  return ldexp(exp_taylor(r), (int)n);
}
__device__ __forceinline__ double tanh_r(double x) {
  const double ax = fabs(x);
  double t;
  if (ax > 22.0) {
    t = 1.0;
  } else {
    const double y = -2.0 * ax;
    const double m = (y > -0.25) ? expm1_small(y) : exp_neg(y) - 1.0;
    t = -m / (2.0 + m);
  }
  return copysign(t, x);
}

struct V3 {
  double d[3];
};
struct T2 {
  double d[3][3];
};

__device__ __forceinline__ double ccov(const V3 &a, const V3 &b) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) s += a.d[i] * b.d[i];
  return s;
}
__device__ __forceinline__ double gdelta(int i, int j) { return i == j ? 1.0 : 0.0; }
__device__ __forceinline__ double dop(double a, double b, double c, double d) {  // DifferenceOfProducts
  const double cd = c * d;
  const double err = fma(-c, d, cd);
  const double dp = fma(a, b, -cd);
  return dp + err;
}
__device__ __forceinline__ double lorentz3(const double vp[3]) {
  double vsq = 0.;
#pragma unroll
  for (int i = 0; i < 3; i++) vsq += vp[i] * vp[i];
  return sqrt(1. + vsq);
}

enum { SUCCESS = 0, FAILURE = 1, MODIFIED = 2 };
constexpr double PI = 3.141592653589793;
constexpr double SIN_PI = 1.2246467991473532e-16;

// LocalThreeGeometry (local_three_geometry.hpp:123-185) off Minkowski:
// gamma_ij of the location, gamma^ij from matrixInverse3x3 (the closure's
// own inverse, not the table's), the lapse.  Contractions in the
// reference's loop order.
struct G3 {
  double cov[3][3], con[3][3], alpha;
  __device__ __forceinline__ void lower(const V3 &a, V3 &o) const {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 3; j++) s += a.d[j] * cov[i][j];
      o.d[i] = s;
    }
  }
  __device__ __forceinline__ void raise(const V3 &a, V3 &o) const {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 3; j++) s += a.d[j] * con[i][j];
      o.d[i] = s;
    }
  }
  __device__ __forceinline__ double contract_cov(const V3 &a, const V3 &b) const {  // contractCov3Vectors
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) s += con[i][j] * a.d[i] * b.d[j];
    return s;
  }
};
// linear_algebra.hpp:67-89: adjugate over determinant (first-column expansion)
__device__ __forceinline__ G3 make_g3(const Pt &p) {
  G3 g;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) g.cov[a][b] = p.gcov[a + 1][b + 1];
  const double(&A)[3][3] = g.cov;
  double(&I)[3][3] = g.con;
  I[0][0] = dop(A[1][1], A[2][2], A[1][2], A[2][1]);
  I[1][0] = -dop(A[1][0], A[2][2], A[1][2], A[2][0]);
  I[2][0] = dop(A[1][0], A[2][1], A[1][1], A[2][0]);
  I[0][1] = -dop(A[0][1], A[2][2], A[0][2], A[2][1]);
  I[1][1] = dop(A[0][0], A[2][2], A[0][2], A[2][0]);
  I[2][1] = -dop(A[0][0], A[2][1], A[0][1], A[2][0]);
  I[0][2] = dop(A[0][1], A[1][2], A[0][2], A[1][1]);
  I[1][2] = -dop(A[0][0], A[1][2], A[0][2], A[1][0]);
  I[2][2] = dop(A[0][0], A[1][1], A[0][1], A[1][0]);
  const double det = fma(A[0][0], I[0][0], dop(A[2][0], I[2][0], A[1][0], -I[1][0]));
  const double invDet = 1.0 / det;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) I[a][b] *= invDet;
  g.alpha = p.alpha;
  return g;
}
// GetLorentzFactor with gamma_ij (relativity_utils.hpp:38-43)
__device__ __forceinline__ double lorentz_g(const double vp[3], const G3 &g) {
  double vsq = 0.;
#pragma unroll
  for (int ii = 0; ii < 3; ii++)
#pragma unroll
    for (int jj = 0; jj < 3; jj++) vsq += g.cov[ii][jj] * vp[ii] * vp[jj];
  return sqrt(1. + vsq);
}

#ifdef PHX_EXACT
constexpr bool kExactBuild = true;
#else
constexpr bool kExactBuild = false;
#endif

// ClosureEdd / ClosureM1 (M1).  MINK: the identity spatial metric, each
// contraction over its non-zero terms; otherwise geo (the LocalThreeGeometry
// of the zone or face) with the full 3x3 sums.
template <bool M1, bool MINK = true>
struct Closure {
  V3 con_v, cov_v;
  double W, W2, iW;
  bool robust;
  const G3 *geo;
  __device__ __forceinline__ Closure(const V3 &cv, bool rob, const G3 *g = nullptr) : robust(rob), geo(g) {
    con_v = cv;
    if constexpr (MINK) {
#pragma unroll
      for (int i = 0; i < 3; i++) cov_v.d[i] = 0.0 + cv.d[i];
    } else {
      geo->lower(cv, cov_v);
    }
    double v2 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) v2 += con_v.d[i] * cov_v.d[i];
    v2 = smin(v2, 0.9999);
    W = rsqrt_p(1 - v2);
    W2 = W * W;
    iW = rcp_p(W);
  }
  __device__ __forceinline__ void raise(const V3 &a, V3 &o) const {
    if constexpr (MINK) {
#pragma unroll
      for (int i = 0; i < 3; i++) o.d[i] = 0.0 + a.d[i];
    } else {
      geo->raise(a, o);
    }
  }
  // contractCov3Vectors
  __device__ __forceinline__ double ccv(const V3 &a, const V3 &b) const {
    if constexpr (MINK)
      return ccov(a, b);
    else
      return geo->contract_cov(a, b);
  }
  __device__ __forceinline__ double gcon(int i, int j) const {
    if constexpr (MINK)
      return gdelta(i, j);
    else
      return geo->con[i][j];
  }
  __device__ __forceinline__ void contractions(const T2 &Pi, V3 &cov_vPi, double &vvPi) const {
    vvPi = 0.0;
    V3 con_vPi;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      double c = 0.0;
#pragma unroll
      for (int j = 0; j < 3; j++) c += cov_v.d[j] * Pi.d[i][j];
      vvPi += cov_v.d[i] * c;
      con_vPi.d[i] = c;
      if constexpr (MINK) cov_vPi.d[i] = 0.0 + c;
    }
    if constexpr (!MINK) geo->lower(con_vPi, cov_vPi);
  }
  __device__ __forceinline__ void linear_source_update(double Estar, const V3 &Fs, const T2 &Pi, double JBB,
                                                       double tauJ, double tauH, double &dE, V3 &dF) const {
    double vvPi;
    V3 cvPi;
    contractions(Pi, cvPi, vvPi);
    double A00 = D3(4 * W2 - 1) + W2 * vvPi + W * tauJ;
    double A01 = 2 * W + tauH;
    double A10 = A00 - 1 - DW(tauJ);
    double A11 = A01 - DW(1.0);
    const double vFs = ccov(con_v, Fs);
    const double b0 = Estar + W * tauJ * JBB;
    const double b1 = vFs + DW(W2 - 1) * tauJ * JBB;
    const double invDet = rcp_p(dop(A00, A11, A01, A10));
    const double J = invDet * dop(A11, b0, A01, b1);
    const double zeta = invDet * dop(A00, b1, A10, b0);
    dE = D3(4 * W2 - 1 + 3 * W2 * vvPi) * J + 2 * W * zeta - Estar;
#ifndef PHX_EXACT
    const double iWt = rcp_p(W + tauH);
#endif
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double num = cov_v.d[i] * tauH * (D3(4 * W2) * J + W * zeta) + tauH * cvPi.d[i] * J +
                         tauJ * W2 * cov_v.d[i] * (JBB - J) + W * Fs.d[i];
#ifdef PHX_EXACT
      dF.d[i] = num / (W + tauH) - Fs.d[i];
#else
      dF.d[i] = num * iWt - Fs.d[i];
#endif
    }
  }
  __device__ __forceinline__ void prim2con(double J, const V3 &H, const T2 &Pi, double &E, V3 &F) const {
    double vvPi;
    V3 cvPi;
    contractions(Pi, cvPi, vvPi);
    const double vH = ccov(con_v, H);
    E = D3(4 * W2 - 1 + 3 * W2 * vvPi) * J + 2 * W * vH;
#pragma unroll
    for (int i = 0; i < 3; i++) F.d[i] = D3(4 * W2) * cov_v.d[i] * J + W * cov_v.d[i] * vH + W * H.d[i] + J * cvPi.d[i];
  }
  // row d of ClosureEdd::getConCovPFromPrim, before the lapse scaling
  __device__ __forceinline__ void concov_p_row(double J, const V3 &H, const T2 &Pi, int d, double P[3]) const {
    if constexpr (MINK) {
      const double conH_d = 0.0 + H.d[d];
#pragma unroll
      for (int j = 0; j < 3; j++)
        P[j] = 4.0 / 3.0 * W2 * con_v.d[d] * cov_v.d[j] * J + W * (con_v.d[d] * H.d[j] + cov_v.d[j] * conH_d) +
               J * (0.0 + Pi.d[d][j]);
    } else {
      V3 conH;
      geo->raise(H, conH);
#pragma unroll
      for (int j = 0; j < 3; j++) {
        double cc = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) cc += Pi.d[d][k] * geo->cov[k][j];
        P[j] = 4.0 / 3.0 * W2 * con_v.d[d] * cov_v.d[j] * J + W * (con_v.d[d] * H.d[j] + cov_v.d[j] * conH.d[d]) +
               J * cc;
      }
    }
    P[d] += D3(J);
  }
  // ClosureEdd::getConPFromPrim
  __device__ __forceinline__ void con_p(double J, const V3 &H, const T2 &Pi, T2 &P) const {
    V3 conH;
    raise(H, conH);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        P.d[i][j] = 4.0 / 3.0 * W2 * con_v.d[i] * con_v.d[j] * J + W * (con_v.d[i] * conH.d[j] + con_v.d[j] * conH.d[i]) +
                    J * Pi.d[i][j] + J / 3.0 * gcon(i, j);
  }
  __device__ __forceinline__ int con2prim(double E, const V3 &F, const T2 &Pi, double &J, V3 &H) const {
    double vvPi;
    V3 cvPi;
    contractions(Pi, cvPi, vvPi);
    const double vF = ccov(con_v, F);
    const double lam = D3(2.0 * W2 + 1.0) + (2.0 * W2 - 3.0) * W2 * vvPi;
#ifdef PHX_EXACT
    const double a = ratio(W2, lam) * ((4 * W2 / 3 - vvPi) * E - ((4 * W2 + 1) / 3 - W2 * vvPi) * vF);
    J = ratio((2 * W2 - 1) * E - 2 * W2 * vF, lam);
#else
    const double ilam = rcp_p(lam + (lam >= 0 ? kSMALL : -kSMALL));
    const double a = W2 * ilam * ((D3(4 * W2) - vvPi) * E - (D3(4 * W2 + 1) - W2 * vvPi) * vF);
    J = ((2 * W2 - 1) * E - 2 * W2 * vF) * ilam;
#endif
#pragma unroll
    for (int i = 0; i < 3; i++) H.d[i] = DW(F.d[i] - J * cvPi.d[i] - cov_v.d[i] * a);
    const double vh = ccov(con_v, H);
    const double xi = div_p(sqrt(ccv(H, H) - vh * vh), J);
    if (isnan(xi) || isnan(J)) return FAILURE;
    if (J < 0. || xi >= 1.0) {
      if (robust) {
        if (J < 0.) J = smin(J, 10. * kSMALL);
        if (xi >= 1.0) {
          const double sc = div_p(0.999, xi);
#pragma unroll
          for (int i = 0; i < 3; i++) H.d[i] *= sc;
        }
        return MODIFIED;
      }
      return FAILURE;
    }
    return SUCCESS;
  }
  __device__ __forceinline__ static double closure_fn(double xi) {
    return D3(1.0 - 2 * (xi * xi) + 4 * (xi * xi * xi));
  }
  __device__ __forceinline__ void tilpi_fill(const double f[3], double athin, T2 &Pi) const {
#ifdef PHX_EXACT
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        Pi.d[i][j] = f[i] * f[j] - (W2 * con_v.d[i] * con_v.d[j] + gcon(i, j)) / 3;
        Pi.d[i][j] *= athin;
      }
#else
    // Minkowski: symmetric, the upper triangle mirrored (gamma^ij from
    // matrixInverse3x3 need not be exactly symmetric: all nine otherwise)
    if constexpr (MINK) {
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
          const double v = (f[i] * f[j] - D3(W2 * con_v.d[i] * con_v.d[j] + gdelta(i, j))) * athin;
          Pi.d[i][j] = v;
          Pi.d[j][i] = v;
        }
    } else {
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) Pi.d[i][j] = (f[i] * f[j] - D3(W2 * con_v.d[i] * con_v.d[j] + geo->con[i][j])) * athin;
    }
#endif
  }
  // GetConTilPiFromPrim
  __device__ __forceinline__ void tilpi_from_prim(double J, const V3 &H, T2 &Pi) const {
    if constexpr (!M1) {
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) Pi.d[i][j] = 0.0;
    } else {
      V3 conH;
      raise(H, conH);
      double Hm = 0.0, vH = 0.0;
#pragma unroll
      for (int i = 0; i < 3; i++) Hm += H.d[i] * conH.d[i];
#pragma unroll
      for (int i = 0; i < 3; i++) vH += H.d[i] * con_v.d[i];
      Hm = sqrt(Hm - vH * vH);
      double f[3];
#ifdef PHX_EXACT
#pragma unroll
      for (int i = 0; i < 3; i++) f[i] = ratio(conH.d[i], Hm);
#else
      const double iHm = rcp_p(Hm + (Hm >= 0 ? kSMALL : -kSMALL));
#pragma unroll
      for (int i = 0; i < 3; i++) f[i] = (MINK ? H.d[i] : conH.d[i]) * iHm;
#endif
      const double xi = smax(smin(1.0, ratio_p(Hm, J)), 0.0);
      tilpi_fill(f, 0.5 * (3 * closure_fn(xi) - 1), Pi);
    }
  }
  __device__ __forceinline__ void angles_pressure(double xi, double phi, const V3 &g, const V3 &dd, T2 &Pi,
                                                  double f[3]) const {
    double s, c;
    if (phi == PI) {
      s = SIN_PI;
      c = -1.0;
    } else {
      s = sin(phi);
      c = cos(phi);
    }
#pragma unroll
    for (int i = 0; i < 3; i++) f[i] = -c * g.d[i] + s * dd.d[i];
    tilpi_fill(f, 0.5 * (3 * closure_fn(xi) - 1), Pi);
  }
  __device__ __forceinline__ void basis(const V3 &F, V3 &g, V3 &dd) const {
    V3 conF;
    raise(F, conF);
    double Fmag = 0.0, vl = 0.0, vv = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) Fmag += F.d[i] * conF.d[i];
    Fmag = sqrt(Fmag);
#pragma unroll
    for (int i = 0; i < 3; i++) vl += F.d[i] * con_v.d[i];
#ifndef PHX_EXACT
    const double iF = rcp_p(Fmag + kSMALL);
#endif
    vl = ratio_p(vl, Fmag);
#pragma unroll
    for (int i = 0; i < 3; i++) vv += cov_v.d[i] * con_v.d[i];
    const double lam = ratio_p(1.0, W * (1 - vl));
    const double aa = sqrt(vv * (1 + 10 * DBL_EPSILON) - vl * vl);
#ifndef PHX_EXACT
    const double iaa = rcp_p(aa + kSMALL);
#endif
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double cF = conF.d[i];
#ifdef PHX_EXACT
      g.d[i] = ratio(cF * lam, Fmag) - W * con_v.d[i];
      dd.d[i] = ratio(ratio(cF, Fmag) * (1 - lam / W) + con_v.d[i], aa);
#else
      g.d[i] = cF * lam * iF - W * con_v.d[i];
      dd.d[i] = (cF * iF * (1 - DW(lam)) + con_v.d[i]) * iaa;
#endif
    }
  }
  __device__ __forceinline__ double residual(double E, const V3 &F, double xi, double phi, const V3 &g,
                                             const V3 &dd) const {
    T2 Pi;
    double f[3];
    angles_pressure(xi, phi, g, dd, Pi, f);
    double J;
    V3 H;
    con2prim(E, F, Pi, J, H);
    double Hm = 0.0, vH = 0.0;
    if constexpr (MINK) {
#pragma unroll
      for (int i = 0; i < 3; i++) Hm += H.d[i] * H.d[i];
    } else {
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) Hm += H.d[i] * H.d[j] * geo->con[i][j];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) vH += con_v.d[i] * H.d[i];
    Hm = sqrt(Hm - vH * vH);
    return xi - ratio(Hm, J);
  }
  // SolveClosure with phi held at pi (the reference's update rule keeps it
  // there); the phi-perturbed residuals only feed the discarded 2x2 solve.
  // Exact build and curved metrics: the reference's central-difference
  // Newton, tensor arithmetic per residual.  Production build on Minkowski:
  // with phi fixed the rest-frame flux direction f is fixed, so
  // pi^ij(xi) = athin(xi) pi0^ij with athin = xi^2 (2 xi - 1), and every
  // quantity con2prim forms is a rational function of athin: the residual
  // and its exact derivative are scalar work (the difference quotient is
  // kept for the robust-rewrite branch and degenerate states).  Pi_out
  // (that path, phi = pi) receives athin(xi) pi0 for the caller's pressure
  // tensor.
  __device__ __forceinline__ void solve_closure(double E, V3 F, double &xi_io, double &phi_out,
                                                T2 *Pi_out = nullptr, bool *pi_done = nullptr) const {
    constexpr bool FD = kExactBuild || !MINK;
    const int max_iter = 30;
    const double tol = 1.e6 * DBL_EPSILON;
    const double eps = sqrt(10 * DBL_EPSILON);
    const double delta = 20 * DBL_EPSILON;
#pragma unroll
    for (int i = 0; i < 3; i++) F.d[i] = ratio(F.d[i], E) + 1.e3 * sgn(F.d[i]) * DBL_MIN;
    E = 1.0;
    V3 g, dd;
    basis(F, g, dd);
    int iter = 0;
    double fXi = 1.e3, fPhi = 1.e3;
    double xi = xi_io, phi = PI;
    if constexpr (FD) {
      do {
        const double xi_up = smin(xi * (1.0 + eps) + delta, 1.0);
        const double xi_lo = smax(xi * (1.0 - eps) - delta, 0.0);
        const double f_up = residual(E, F, xi_up, phi, g, dd);
        const double f_lo = residual(E, F, xi_lo, phi, g, dd);
        fXi = residual(E, F, xi, phi, g, dd);
        const double J00 = (f_up - f_lo) / (xi_up - xi_lo);
        const double dx0 = fXi / J00, dx1 = 0.0;
        fPhi = 0.0;
        double cdx = smin(dx0, xi - delta * xi);
        cdx = smax(cdx, xi - (1 - delta * (1 - xi)));
        double alpha = ratio(cdx, dx0);
        alpha = smin(alpha, 0.5 * 3.14159 / fabs(dx1));
        xi -= alpha * dx0;
        phi -= alpha * dx1;
        ++iter;
      } while (iter < max_iter && (fabs(fXi) > tol || fabs(fPhi) > tol));
    } else {
      double f[3];
#pragma unroll
      for (int i = 0; i < 3; i++) f[i] = g.d[i] + SIN_PI * dd.d[i];
      T2 Pi0;
      tilpi_fill(f, 1.0, Pi0);
      V3 C0;
      double V0;
      contractions(Pi0, C0, V0);
      const double vF = ccov(con_v, F);
      const double L0 = D3(2.0 * W2 + 1.0), c1 = (2.0 * W2 - 3.0) * W2;
      const double NJ = (2 * W2 - 1) * E - 2 * W2 * vF;
      const double K0 = D3(4 * W2) * E - D3(4 * W2 + 1) * vF, Kv = -E + W2 * vF;
      // residual at x; *df its derivative, NaN where the difference quotient is needed
      auto res = [&](double x, double *df) {
        const double at = x * x * (2 * x - 1);
        const double V = at * V0;
        const double lam = L0 + c1 * V;
        const double ilam = rcp_p(lam + (lam >= 0 ? kSMALL : -kSMALL));
        const double K = K0 + V * Kv;
        const double A = W2 * ilam * K;
        const double J = NJ * ilam;
        const double Ja = J * at;
        V3 H;
#pragma unroll
        for (int i = 0; i < 3; i++) H.d[i] = (F.d[i] - Ja * C0.d[i] - cov_v.d[i] * A) * iW;
        const double vh = ccov(con_v, H);
        const double s0 = sqrt(ccov(H, H) - vh * vh);
        const double iJ = rcp_p(J + (J >= 0 ? kSMALL : -kSMALL));
        const double xc = s0 * iJ;
        double sH = s0;
        const bool modified = robust && !isnan(xc) && !isnan(J) && (J < 0. || xc >= 1.0);
        if (modified && xc >= 1.0) sH = s0 * (0.999 * rcp_p(xc));
        if (df) {
          if (modified || !(s0 > 0.0)) {
            *df = __longlong_as_double(0x7ff8000000000000ll);
          } else {
            const double dat = x * (6 * x - 2);
            const double dV = dat * V0;
            const double dilam = -(c1 * dV) * ilam * ilam;
            const double dJ = NJ * dilam;
            const double dA = W2 * (dilam * K + ilam * (Kv * dV));
            const double dJa = dJ * at + J * dat;
            double hdh = 0.0, vdh = 0.0;
#pragma unroll
            for (int i = 0; i < 3; i++) {
              const double dH = (-dJa * C0.d[i] - cov_v.d[i] * dA) * iW;
              hdh += H.d[i] * dH;
              vdh += con_v.d[i] * dH;
            }
            const double ds0 = (hdh - vh * vdh) * rcp_p(s0);
            *df = 1.0 - (ds0 - s0 * dJ * iJ) * iJ;
          }
        }
        return x - sH * iJ;
      };
      do {
        const double xi_up = smin(xi * (1.0 + eps) + delta, 1.0);
        const double xi_lo = smax(xi * (1.0 - eps) - delta, 0.0);
        double J00;
        fXi = res(xi, &J00);
        if (!isfinite(J00)) J00 = (res(xi_up, nullptr) - res(xi_lo, nullptr)) / (xi_up - xi_lo);
        const double dx0 = fXi / J00, dx1 = 0.0;
        fPhi = 0.0;
        double cdx = smin(dx0, xi - delta * xi);
        cdx = smax(cdx, xi - (1 - delta * (1 - xi)));
        double alpha = ratio(cdx, dx0);
        alpha = smin(alpha, 0.5 * 3.14159 / fabs(dx1));
        xi -= alpha * dx0;
        phi -= alpha * dx1;
        ++iter;
      } while (iter < max_iter && (fabs(fXi) > tol || fabs(fPhi) > tol));
      if (Pi_out && phi == PI) {
        const double at = 0.5 * (3 * closure_fn(xi) - 1);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) Pi_out->d[i][j] = Pi0.d[i][j] * at;
        *pi_done = true;
      }
    }
    xi_io = xi;
    phi_out = phi;
  }
  // GetConTilPiFromCon
  __device__ __forceinline__ void tilpi_from_con(double E, const V3 &F, double &xi, double &phi, T2 &Pi) const {
    if constexpr (!M1) {
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) Pi.d[i][j] = 0.0;
      xi = 0.0;
      phi = PI;
    } else {
      bool done = false;
      solve_closure(E, F, xi, phi, &Pi, &done);
      if (!done) {
        V3 g, dd;
        basis(F, g, dd);
        double f[3];
        angles_pressure(xi, phi, g, dd, Pi, f);
      }
    }
  }
};

// RadiationFloors::GetRadiationFloors (fixup.hpp:166-177) at X1 = x1:
// ConstantJ, or ExpX1J J0 exp(J_alpha x1) with the project's exp (the one the
// oracle uses, so both agree bit for bit)
__device__ __forceinline__ double j_floor_at(const RPar &p, double x1) {
  return p.floor_expx1 ? p.J_floor * phx_math::exp(p.J_alpha * x1) : p.J_floor;
}

// ---------------------------------------------------------------- views
// The geometry a moment task reads at one location (loc 0 centre and X3
// faces, 1 X1 face, 2 X2 face): the table values and, off Minkowski, the
// LocalThreeGeometry built from them.  Minkowski: lapse 1, shift 0, identity.
template <bool MINK>
struct RGeo {
  Pt p;
  G3 g;
  __device__ __forceinline__ RGeo(const BView &b, int loc, int j, int i) {
    if constexpr (!MINK) {
      load_pt(b, loc, j, i, p);
      g = make_g3(p);
    }
  }
  __device__ __forceinline__ const G3 *geo() const { return MINK ? nullptr : &g; }
  __device__ __forceinline__ double alpha() const { return MINK ? 1.0 : p.alpha; }
  __device__ __forceinline__ double beta(int d) const { return MINK ? 0.0 : p.beta[d]; }
  __device__ __forceinline__ double sdetgam() const { return MINK ? 1.0 : p.detgam; }
  __device__ __forceinline__ double cov(int a, int c) const { return MINK ? gdelta(a, c) : p.gcov[a + 1][c + 1]; }
  __device__ __forceinline__ double con(int a, int c) const { return MINK ? gdelta(a, c) : p.gamcon[a][c]; }
};

// The fluid three-velocity (W v^i) / W, W of gamma_ij.
template <bool MINK = true>
__device__ __forceinline__ V3 fluid_v(const BView &b, long long id, const G3 *g = nullptr, double *Wout = nullptr) {
  const double vp[3] = {b.prim[PHX_PVEL * b.vs + id], b.prim[(PHX_PVEL + 1) * b.vs + id],
                        b.prim[(PHX_PVEL + 2) * b.vs + id]};
  double W;
  if constexpr (MINK)
    W = lorentz3(vp);
  else
    W = lorentz_g(vp, *g);
  if (Wout) *Wout = W;
  V3 v;
  v.d[0] = vp[0] / W;
  v.d[1] = vp[1] / W;
  v.d[2] = vp[2] / W;
  return v;
}
__device__ __forceinline__ void zone_of(const Range3 &r, long long t, int &k, int &j, int &i) {
  const int ni = r.ie - r.is + 1, nj = r.je - r.js + 1;
  i = r.is + (int)(t % ni);
  j = r.js + (int)((t / ni) % nj);
  k = r.ks + (int)(t / ((long long)ni * nj));
}
__host__ __device__ inline long long range_count(const Range3 &r) {
  return (long long)(r.ie - r.is + 1) * (r.je - r.js + 1) * (r.ke - r.ks + 1);
}

// ---------------------------------------------------- MomentPrim2Con
template <bool M1, bool MINK>
__global__ void __launch_bounds__(128) k_p2c(RPar p, BView b, RView r, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long id = b.idx(k, j, i), vs = r.vs;
  const RGeo<MINK> G(b, 0, j, i);
  const Closure<M1, MINK> c(fluid_v<MINK>(b, id, G.geo()), true, G.geo());
  const double J = r.prim[PHX_RJ * vs + id];
  V3 H;
#pragma unroll
  for (int a = 0; a < 3; a++) H.d[a] = r.prim[(PHX_RH + a) * vs + id] * J;
  T2 Pi;
  c.tilpi_from_prim(J, H, Pi);
  double E;
  V3 F;
  c.prim2con(J, H, Pi, E, F);
  const double sdetgam = G.sdetgam();
  r.cons[PHX_RE * vs + id] = sdetgam * E;
#pragma unroll
  for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = sdetgam * F.d[a];
}

// ---------------------------------------------------- MomentCon2Prim
template <bool M1, bool MINK>
__global__ void __launch_bounds__(128) k_c2p(RPar p, BView b, RView r, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long id = b.idx(k, j, i), vs = r.vs;
  const RGeo<MINK> G(b, 0, j, i);
  const double isdetgam = 1.0 / G.sdetgam();
  const Closure<M1, MINK> c(fluid_v<MINK>(b, id, G.geo()), p.robust != 0, G.geo());
  double E = r.cons[PHX_RE * vs + id] * isdetgam;
  V3 F;
#pragma unroll
  for (int a = 0; a < 3; a++) F.d[a] = r.cons[(PHX_RF + a) * vs + id] * isdetgam;
  double xi = 0.0, phi = PI;
  if constexpr (M1) {
    xi = r.prim[PHX_RXI * vs + id];
    phi = 1.0001 * r.prim[PHX_RPHI * vs + id];
  }
  T2 Pi;
  c.tilpi_from_con(E, F, xi, phi, Pi);
  if constexpr (M1) {
    r.prim[PHX_RXI * vs + id] = xi;
    r.prim[PHX_RPHI * vs + id] = phi;
  }
  double J;
  V3 H;
  int st = c.con2prim(E, F, Pi, J, H);
  if (st == MODIFIED) {
    c.prim2con(J, H, Pi, E, F);
    r.cons[PHX_RE * vs + id] = E / isdetgam;
#pragma unroll
    for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = F.d[a] / isdetgam;
    st = SUCCESS;
  }
  r.prim[PHX_RJ * vs + id] = J;
#ifdef PHX_EXACT
#pragma unroll
  for (int a = 0; a < 3; a++) r.prim[(PHX_RH + a) * vs + id] = ratio(H.d[a], J);
#else
  const double iJ = rcp_p(J + (J >= 0 ? kSMALL : -kSMALL));
#pragma unroll
  for (int a = 0; a < 3; a++) r.prim[(PHX_RH + a) * vs + id] = H.d[a] * iJ;
#endif
  r.prim[PHX_RFAIL * vs + id] = st == SUCCESS ? 1.0 : 0.0;
}

// ------------------------------------------ MomentCalculateOpacities
__global__ void __launch_bounds__(256) k_opacities(RPar p, BView b, RView r, long long n) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n) return;
  const double rho = b.prim[PHX_PRHO * b.vs + id], T = b.prim[PHX_PTMP * b.vs + id];
  const double kJ = rho * p.kappa_a;
  const double kH = kJ + rho * p.kappa_s;
  r.prim[PHX_RJBB * r.vs + id] = p.jbb * (T * T) * (T * T);
  r.prim[PHX_RKAPPAJ * r.vs + id] = kJ;
  r.prim[PHX_RKAPPAH * r.vs + id] = kH;
}

// --------------------------------------------------------- fluxes
// One face state: E, F_i, and the flux of direction d (con_F^d and row d of
// P^i_j) for the closure's velocity, J and H_i.
// ClosureEdd::getFluxesFromPrim: con_F^d = alpha gamma^{dj} F_j and
// alpha P^d_j (on Minkowski the lapse scalings by 1 are exact and skipped).
template <bool M1, int d, bool MINK>
__device__ __forceinline__ void face_state(const Closure<M1, MINK> &c, double J, const V3 &H, double &E, V3 &F,
                                           double &Fd, double P[3]) {
  T2 Pi;
  c.tilpi_from_prim(J, H, Pi);
  c.concov_p_row(J, H, Pi, d, P);
  c.prim2con(J, H, Pi, E, F);
  if constexpr (MINK) {
    Fd = 0.0 + F.d[d];
  } else {
    V3 conF;
    c.geo->raise(F, conF);
#pragma unroll
    for (int a = 0; a < 3; a++) P[a] *= c.geo->alpha;
    Fd = conF.d[d] * c.geo->alpha;
  }
}

template <bool M1, int RECON, int d, bool MINK>
__global__ void __launch_bounds__(128) k_fluxes(RPar p, BView b, RView r, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long vs = r.vs, fvs = b.vs;
  const long long st = d == 0 ? 1 : (d == 1 ? (long long)b.n1t : (long long)b.n1t * b.n2t);
  const long long id = b.idx(k, j, i), idm = id - st;
  // reconstruction: J, H/J (rad prims 0..3) and u^i (fluid prims 1..3)
  double ql[7], qr[7];
#pragma unroll
  for (int n = 0; n < 7; n++) {
    const double *base = n < 4 ? r.prim + n * vs : b.prim + (PHX_PVEL + n - 4) * fvs;
    const double q0 = base[idm - 2 * st], q1 = base[idm - st], q2 = base[idm], q3 = base[id], q4 = base[id + st],
                 q5 = base[id + 2 * st];
    double a, c;
    recon<RECON>(q0, q1, q2, q3, q4, ql[n], a);
    recon<RECON>(q1, q2, q3, q4, q5, c, qr[n]);
  }
  // dJ at the face (moments.cpp:412-455)
  const int dj = b.ndim > 1 ? 1 : 0, dk = b.ndim > 2 ? 1 : 0;
  const double *Jp = r.prim + PHX_RJ * vs;
  auto Jat = [&](int kk, int jj, int ii) { return Jp[b.idx(kk, jj, ii)]; };
  const double idx = 1.0 / b.dx[0], idx4 = 0.25 * idx;
  const double idy = 1.0 / b.dx[1], idy4 = 0.25 * idy;
  const double idz = 1.0 / b.dx[2], idz4 = 0.25 * idz;
  V3 dJ;
  if constexpr (d == 0) {
    dJ.d[0] = (Jat(k, j, i) - Jat(k, j, i - 1)) * idx;
    dJ.d[1] = (Jat(k, j + dj, i) + Jat(k, j + dj, i - 1) - Jat(k, j - dj, i) - Jat(k, j - dj, i - 1)) * idy4;
    dJ.d[2] = (Jat(k + dk, j, i) + Jat(k + dk, j, i - 1) - Jat(k - dk, j, i) - Jat(k - dk, j, i - 1)) * idz4;
  } else if constexpr (d == 1) {
    dJ.d[0] = (Jat(k, j, i + 1) + Jat(k, j - dj, i + 1) - Jat(k, j, i - 1) - Jat(k, j - dj, i - 1)) * idx4;
    dJ.d[1] = (Jat(k, j, i) - Jat(k, j - dj, i)) * idy;
    dJ.d[2] = (Jat(k + dk, j, i) + Jat(k + dk, j - dj, i) - Jat(k - dk, j, i) - Jat(k - dk, j - dj, i)) * idz4;
  } else {
    dJ.d[0] = (Jat(k, j, i + 1) + Jat(k - dk, j, i + 1) - Jat(k, j, i - 1) - Jat(k - dk, j, i - 1)) * idx4;
    dJ.d[1] = (Jat(k, j + dj, i) + Jat(k - dk, j + dj, i) - Jat(k, j - dj, i) - Jat(k - dk, j - dj, i)) * idy4;
    dJ.d[2] = (Jat(k, j, i) - Jat(k - dk, j, i)) * idz;
  }
  const RGeo<MINK> G(b, d == 0 ? 1 : (d == 1 ? 2 : 0), j, i);  // X3 faces: the centre table
  const double dx = b.dx[d] * sqrt(G.cov(d, d));
  double vpl[3] = {ql[4], ql[5], ql[6]}, vpr[3] = {qr[4], qr[5], qr[6]};
  double Wl, Wr;
  if constexpr (MINK) {
    Wl = lorentz3(vpl);
    Wr = lorentz3(vpr);
  } else {
    Wl = lorentz_g(vpl, G.g);
    Wr = lorentz_g(vpr, G.g);
  }
  if (p.bounds) {
    if (Wl > p.W_ceiling) {
      const double rescale = sqrt(p.W_ceiling * p.W_ceiling - 1.) / (Wl * Wl - 1.);
#pragma unroll
      for (int a = 0; a < 3; a++) vpl[a] *= rescale;
      Wl = p.W_ceiling;
    }
    if (Wr > p.W_ceiling) {
      const double rescale = sqrt(p.W_ceiling * p.W_ceiling - 1.) / (Wr * Wr - 1.);
#pragma unroll
      for (int a = 0; a < 3; a++) vpr[a] *= rescale;
      Wr = p.W_ceiling;
    }
  }
  V3 vl, vr;
  const double iWl = rcp_p(Wl), iWr = rcp_p(Wr);
#pragma unroll
  for (int a = 0; a < 3; a++) {
#ifdef PHX_EXACT
    vl.d[a] = vpl[a] / Wl;
    vr.d[a] = vpr[a] / Wr;
#else
    vl.d[a] = vpl[a] * iWl;
    vr.d[a] = vpr[a] * iWr;
#endif
  }
  const double alpha = G.alpha(), beta_d = G.beta(d);
  const double sigp = alpha * sqrt(G.con(d, d)) - beta_d;
  const double sigm = -alpha * sqrt(G.con(d, d)) - beta_d;
  const double asym_sigl = alpha * vl.d[d] - beta_d;
  const double asym_sigr = alpha * vr.d[d] - beta_d;
  double Jl = ql[0], Jr = qr[0];
  if (p.bounds) {
    const double Jf = j_floor_at(p, d == 0 ? b.Xf(0, i) : b.Xc(0, i));  // at the face (moments.cpp:562-575)
    Jl = smax(Jl, Jf);
    Jr = smax(Jr, Jf);
  }
  V3 Hl, Hr;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    Hl.d[a] = Jl * ql[1 + a];
    Hr.d[a] = Jr * qr[1 + a];
  }
#ifdef PHX_EXACT
  if (p.bounds) {
#else
  // with the ceiling at DBL_MAX (radiation ceilings off) no finite xi
  // exceeds it, and an infinite xi needs J = 0, where H = J q is already 0
  if (p.bounds && p.xi_ceiling < kDBLMAX) {
#endif
    const double vhl = ccov(vl, Hl), vhr = ccov(vr, Hr);
    const double hhl = MINK ? ccov(Hl, Hl) : G.g.contract_cov(Hl, Hl);
    const double hhr = MINK ? ccov(Hr, Hr) : G.g.contract_cov(Hr, Hr);
    const double xil = div_p(sqrt(hhl - vhl * vhl), Jl);
    const double xir = div_p(sqrt(hhr - vhr * vhr), Jr);
    if (xil > p.xi_ceiling) {
#pragma unroll
      for (int a = 0; a < 3; a++) Hl.d[a] *= p.xi_ceiling / xil;
    }
    if (xir > p.xi_ceiling) {
#pragma unroll
      for (int a = 0; a < 3; a++) Hr.d[a] *= p.xi_ceiling / xir;
    }
  }
  const double *kH = r.prim + PHX_RKAPPAH * vs;
  const double kappaH = sqrt(kH[id] * kH[idm]);
  const double aw = tanh_r(ratio(1.0, fabs(kappaH * dx)));
  const double kappaH_min = 1.e-20;
  V3 Has;
#ifdef PHX_EXACT
#pragma unroll
  for (int a = 0; a < 3; a++) Has.d[a] = ratio(-dJ.d[a], 3 * kappaH + 3 * kappaH_min);
#else
  const double ik = rcp_p(3 * kappaH + 3 * kappaH_min + kSMALL);
#pragma unroll
  for (int a = 0; a < 3; a++) Has.d[a] = -dJ.d[a] * ik;
#endif
  const Closure<M1, MINK> cl(vl, true, G.geo()), cr(vr, true, G.geo());
  double El, Er, Fdl, Fdr, Fdl_a, Fdr_a, Pl[3], Pr[3], Pl_a[3], Pr_a[3], Ed;
  V3 Fl, Fr, Fd_scr;
  face_state<M1, d, MINK>(cl, Jl, Has, Ed, Fd_scr, Fdl_a, Pl_a);
  face_state<M1, d, MINK>(cr, Jr, Has, Ed, Fd_scr, Fdr_a, Pr_a);
  face_state<M1, d, MINK>(cl, Jl, Hl, El, Fl, Fdl, Pl);
  face_state<M1, d, MINK>(cr, Jr, Hr, Er, Fr, Fdr, Pr);
  Fdl = aw * Fdl + (1 - aw) * Fdl_a;
  Fdr = aw * Fdr + (1 - aw) * Fdr_a;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    Pl[a] = aw * Pl[a] + (1 - aw) * Pl_a[a];
    Pr[a] = aw * Pr[a] + (1 - aw) * Pr_a[a];
  }
  const double rad_sigspeed = smax(fabs(sigm), fabs(sigp));
  const double asym_sigspeed = smax(fabs(asym_sigl), fabs(asym_sigr));
  const double sigspeed = aw * rad_sigspeed + (1. - aw) * asym_sigspeed;
  Fdl -= beta_d * El;
  Fdr -= beta_d * Er;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    Pl[a] -= beta_d * Fl.d[a];
    Pr[a] -= beta_d * Fr.d[a];
  }
  const double sdetgam = G.sdetgam();
  double *fl = r.flux + (long long)d * PHX_RNCONS * vs;
  const bool zero = !MINK && sdetgam < kSMALL;
  fl[PHX_RE * vs + id] = zero ? 0.0 : 0.5 * sdetgam * (Fdl + Fdr + sigspeed * (El - Er));
#pragma unroll
  for (int a = 0; a < 3; a++)
    fl[(PHX_RF + a) * vs + id] = zero ? 0.0 : 0.5 * sdetgam * (Pl[a] + Pr[a] + sigspeed * (Fl.d[a] - Fr.d[a]));
}

// CalculateGeometricSourceImpl (moments.cpp:764-885) of one zone off
// Minkowski, from the stage input E, F_i and the stored J, H_i: the
// radiation stress tensor T^{mu nu} (E n n + F n + n F + P), the connection
// coefficients 0.5 (dg_{b a, c} + dg_{c a, b} - dg_{b c, a}) of the derivative
// table, row 0 of g^{mu nu} (cached_system.hpp:281-299) and d ln(alpha).
// src: the densitised sources of E and F_1..3.
template <bool M1>
__device__ void geometric_source(const BView &b, const RView &r, int k, int j, int i, double src[4]) {
  const long long id = b.idx(k, j, i), vs = r.vs;
  const RGeo<false> G(b, 0, j, i);
  const Closure<M1, false> c(fluid_v<false>(b, id, &G.g), true, &G.g);
  const double alp = G.p.alpha, sdetgam = G.p.detgam;
  double alpha2 = alp;
  alpha2 *= alpha2;
  const double g0[4] = {-ratio_p(1, alpha2), ratio_p(G.p.beta[0], alpha2), ratio_p(G.p.beta[1], alpha2),
                        ratio_p(G.p.beta[2], alpha2)};
  const long long pitch = (long long)b.n2t * b.n1t, off = (long long)j * b.n1t + i;
  double dg[4][4][4];
#pragma unroll
  for (int mu = 0; mu < 4; mu++)
#pragma unroll
    for (int nu = 0; nu < 4; nu++) {
      dg[mu][nu][0] = 0.0;
#pragma unroll
      for (int s = 1; s < 4; s++) dg[mu][nu][s] = __ldg(b.gderiv + (PHX_GD_DG + 3 * flat2(mu, nu) + s - 1) * pitch + off);
    }
  auto gam = [&](int a, int bb, int cc) { return 0.5 * (dg[bb][a][cc] + dg[cc][a][bb] - dg[bb][cc][a]); };
  double dlnalp[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int s = 1; s < 4; s++) dlnalp[s] = __ldg(b.gderiv + (PHX_GD_DALPHA + s - 1) * pitch + off);
  const double con_n[4] = {1. / alp, -G.p.beta[0] / alp, -G.p.beta[1] / alp, -G.p.beta[2] / alp};
  const double E = r.cons[PHX_RE * vs + id] / sdetgam;
  const double J = r.prim[PHX_RJ * vs + id];
  V3 covF, covH, conF;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    covF.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam;
    covH.d[a] = J * r.prim[(PHX_RH + a) * vs + id];
  }
  T2 Pi, P;
  c.tilpi_from_prim(J, covH, Pi);
  c.con_p(J, covH, Pi, P);
  G.g.raise(covF, conF);
  double T[4][4];
#pragma unroll
  for (int mu = 0; mu < 4; mu++)
#pragma unroll
    for (int nu = 0; nu < 4; nu++) T[mu][nu] = 0.0 + con_n[mu] * con_n[nu] * E;
#pragma unroll
  for (int mu = 0; mu < 4; mu++)
#pragma unroll
    for (int ii = 0; ii < 3; ii++) {
      T[mu][ii + 1] += con_n[mu] * conF.d[ii];
      T[ii + 1][mu] += con_n[mu] * conF.d[ii];
    }
#pragma unroll
  for (int ii = 0; ii < 3; ii++)
#pragma unroll
    for (int jj = 0; jj < 3; jj++) T[ii + 1][jj + 1] += P.d[ii][jj];
  double TGam = 0.0;
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int n = 0; n < 4; n++) {
      double gam0 = 0.;
#pragma unroll
      for (int q = 0; q < 4; q++) gam0 += g0[q] * gam(q, m, n);
      TGam += T[m][n] * gam0;
    }
  double Ta = 0.0;
#pragma unroll
  for (int m = 0; m < 4; m++) Ta += T[m][0] * dlnalp[m];
  src[0] = sdetgam * alp * alp * (Ta - TGam);
#pragma unroll
  for (int l = 0; l < 3; l++) {
    double sm = 0.0;
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
      for (int n = 0; n < 4; n++) sm += T[m][n] * (dg[n][l + 1][m] - gam(l + 1, n, m));
    src[1 + l] = alp * sdetgam * sm;
  }
}

// ------------------------------------------ divergence + RK update
template <bool M1, bool MINK>
__global__ void __launch_bounds__(256) k_update(BView b, RView r, const double *base, double *out, double beta,
                                                double dt, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long id = b.idx(k, j, i), vs = r.vs;
  // SumData: the geometric source (zero on Minkowski), from the stage input
  double src[4] = {0.0, 0.0, 0.0, 0.0};
  if constexpr (!MINK) geometric_source<M1>(b, r, k, j, i, src);
  const double dx1 = b.dx[0], dx2 = b.dx[1], dx3 = b.dx[2];
  const double A1 = dx2 * dx3, A2 = dx1 * dx3, A3 = dx1 * dx2, V = dx1 * dx2 * dx3;
  const double bdt = beta * dt;
  const long long s2 = b.n1t, s3 = (long long)b.n1t * b.n2t;
#pragma unroll
  for (int m = 0; m < PHX_RNCONS; m++) {
    const double *F0 = r.flux + (long long)m * vs;
    const double *F1 = r.flux + (long long)(PHX_RNCONS + m) * vs;
    const double *F2 = r.flux + (long long)(2 * PHX_RNCONS + m) * vs;
    double du = (A1 * F0[id + 1] - A1 * F0[id]);
    if (b.ndim >= 2) du += A2 * F1[id + s2] - A2 * F1[id];
    if (b.ndim == 3) du += A3 * F2[id + s3] - A3 * F2[id];
    const double rr = -du / V + src[m];
    r.dudt[m * vs + id] = rr;
    double u0 = r.cons[m * vs + id];
    u0 = beta * u0 + (1 - beta) * base[m * vs + id];
    r.cons[m * vs + id] = u0;
    out[m * vs + id] = u0 + bdt * rr;
  }
}

// ------------------------------------------ MomentFluidSource (oned)
struct TRes {
  const RPar *p;
  double rho, ug0, J0, dtau, amax;
#ifndef PHX_EXACT
  // gray opacity: kappa does not depend on T, so both denominators are fixed
  // per zone (production build: two reciprocals instead of a division per
  // evaluation)
  double dk, i1, i2;
  __device__ __forceinline__ void prepare() {
    dk = dtau * smin(rho * p->kappa_a, amax);
    i1 = rcp_p(1. + dk);
    i2 = rcp_p(ug0 + J0);
  }
  __device__ __forceinline__ double operator()(double T) const {
    const double JBB = p->jbb * (T * T) * (T * T);
    const double dJ = (J0 + dk * JBB) * i1 - J0;
    const double ug1 = rho * (p->Cv * T);
    return ((ug1 - ug0) + dJ) * i2;
  }
#else
  __device__ __forceinline__ void prepare() {}
  __device__ __forceinline__ double operator()(double T) const {
    double kappa = rho * p->kappa_a;
    kappa = smin(kappa, amax);
    const double JBB = p->jbb * (T * T) * (T * T);
    const double dJ = (J0 + dtau * kappa * JBB) / (1. + dtau * kappa) - J0;
    const double ug1 = rho * (p->Cv * T);
    return ((ug1 - ug0) + dJ) / (ug0 + J0);
  }
#endif
};
// RootFind::regula_falsi with a status; the iteration count persists across
// calls (the reference reuses one RootFind for its re-bracketing tries).
__device__ __forceinline__ double regula_falsi(const TRes &f, double a, double b, double tol, double guess,
                                               int &count, int max_iter, bool &ok) {
  double ya, yb;
  if (a <= guess && b >= guess) {
    ya = f(guess);
    yb = f(b);
    if (ya * yb > 0.0) {
      yb = ya;
      b = guess;
      ya = f(a);
    } else {
      a = guess;
    }
  } else {
    ya = f(a);
    yb = f(b);
  }
  if (ya * yb > 0.0) {
    ok = false;
    return guess;
  }
  const double sign = (ya < 0 ? 1.0 : -1.0);
  ya *= sign;
  yb *= sign;
  int b1 = 0, b2 = 0;
  while (b - a > 2.0 * tol && count < max_iter) {
    const double c = (a * yb - b * ya) / (yb - ya);
    if (c == a) {
      b = a;
      count++;
      continue;
    } else if (c == b) {
      a = b;
      count++;
      continue;
    }
    const double yc = sign * f(c);
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
    count++;
  }
  ok = count != max_iter;
  return 0.5 * (a + b);
}

// con2prim_robust's solve (con2prim_robust.hpp:299-453) of one zone of the
// fluid block (g: its centre geometry; unused on Minkowski) with
// MomentFluidSourceImpl's settings (fp fails on floors and ceilings), from
// the stored mu.  The lane iterates on its own.  Writes the primitives, the
// cell speeds and, when bounds were used, the conserved variables.  True on
// success; an unbracketed root is a failure.
template <bool MINK>
__device__ bool fluid_invert(const Par &fp, const BView &b, const Pt &g, int k, int j, int i, long long id) {
  const long long vs = b.vs;
  double U[PHX_NCONS];
#pragma unroll
  for (int m = 0; m < PHX_NCONS; m++) U[m] = b.cons[m * vs + id];
  Residual res;
  double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0;
  if (!c2p_setup<MINK>(fp, g, U, b.Xc(0, i), b.Xc(1, j), b.Xc(2, k), res, rcon, rcov, bu, Bprim, bdotr))
    return false;
  const double guess = b.prim[PHX_PMU * vs + id];
  RFState st;
  rf_start<false>(fp, res, true, 0.0, 1.0, guess, nullptr, st);
  rf_iterate<false>(fp, res, true, st, fp.c2p_max_iter);
  C2POut out{0, 0, false, true, false, false};
  const double mu = rf_result(st, guess, out);
  double prim[PHX_NPRIM], sig[3];
  bool used_bounds;
  c2p_finish<MINK>(fp, g, res, mu, rcon, bu, Bprim, bdotr, prim, U, sig, used_bounds);
  for (int v = 0; v < PHX_NPRIM; v++) {
    if (v >= PHX_PB && v < PHX_PB + 3 && !fp.mhd) continue;
    b.prim[v * vs + id] = prim[v];
  }
  if (used_bounds) {
    b.cons[PHX_CRHO * vs + id] = U[PHX_CRHO];
    b.cons[PHX_CENG * vs + id] = U[PHX_CENG];
    for (int m = 0; m < 3; m++) b.cons[(PHX_CMOM + m) * vs + id] = U[PHX_CMOM + m];
  }
  for (int d = 0; d < b.ndim; d++) b.cell_sig[d * vs + id] = sig[d];
  const int num_nans = isnan(U[PHX_CRHO]) + isnan(U[PHX_CMOM]) + isnan(U[PHX_CENG]);
  bool ok = out.bracketed && num_nans == 0;
  if (fp.fail_on_floors && (res.used_density_floor || res.used_energy_floor)) ok = false;
  if (fp.fail_on_ceilings && res.used_gamma_max) ok = false;
  return ok;
}

// update_fluid (moments_source.cpp:807-965): the fluid gives up the energy
// and momentum the radiation took (dE, dF: the source solve's last values,
// applied to the fluid whether or not the radiation kept them), is inverted,
// and the closure inversion runs with the new fluid velocity.  When either
// inversion fails, the fluid becomes a near-vacuum at rest (rho = u =
// 10 SMALL, P, T and -- as the reference stores it -- the bulk modulus in
// the gamma1 slot, then prim2con of D, S, tau) and the radiation the
// J = SMALL, H = 0 state of that fluid's closure, with the tilde-pressure
// tensor of the inversion that failed (zero when the fluid inversion failed).
template <bool M1, bool MINK>
__device__ void source_update_fluid(const Par &fp, const BView &b, const RView &r, const RGeo<MINK> &G, int k, int j,
                                    int i, long long id, double dE, const V3 &dF) {
  const long long vs = r.vs, fvs = b.vs;
  const double sdetgam = G.sdetgam();
  b.cons[PHX_CENG * fvs + id] -= sdetgam * dE;
#pragma unroll
  for (int a = 0; a < 3; a++) b.cons[(PHX_CMOM + a) * fvs + id] -= sdetgam * dF.d[a];
  T2 Pi;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int c = 0; c < 3; c++) Pi.d[a][c] = 0.0;
  double E = r.cons[PHX_RE * vs + id] / sdetgam;
  V3 F, H;
  double J;
#pragma unroll
  for (int a = 0; a < 3; a++) F.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam;
  if (fluid_invert<MINK>(fp, b, G.p, k, j, i, id)) {
    const Closure<M1, MINK> c(fluid_v<MINK>(b, id, G.geo()), false, G.geo());
    double xi = 0.0, phi = PI;
    c.tilpi_from_con(E, F, xi, phi, Pi);
    if (c.con2prim(E, F, Pi, J, H) == SUCCESS) {
      r.prim[PHX_RJ * vs + id] = J;
#pragma unroll
      for (int a = 0; a < 3; a++) r.prim[(PHX_RH + a) * vs + id] = div_p(H.d[a], J);
      return;
    }
  }
  double *P = b.prim + id;
  P[PHX_PRHO * fvs] = 10. * kSMALL;
  P[PHX_PENG * fvs] = 10. * kSMALL;
#pragma unroll
  for (int a = 0; a < 3; a++) P[(PHX_PVEL + a) * fvs] = 0.;
  P[PHX_PPRS * fvs] = eos_P_rho_sie(fp, P[PHX_PRHO * fvs], ratio(P[PHX_PENG * fvs], P[PHX_PRHO * fvs]));
  P[PHX_PTMP * fvs] = eos_T_rho_sie(fp, P[PHX_PRHO * fvs], ratio(P[PHX_PENG * fvs], P[PHX_PRHO * fvs]));
  P[PHX_PGM1 * fvs] = eos_bmod_rho_T(fp, P[PHX_PRHO * fvs], P[PHX_PTMP * fvs]);
  const double vp[3] = {P[PHX_PVEL * fvs], P[(PHX_PVEL + 1) * fvs], P[(PHX_PVEL + 2) * fvs]};
  double bp[3] = {0.0, 0.0, 0.0};
  if (fp.mhd)
#pragma unroll
    for (int a = 0; a < 3; a++) bp[a] = P[(PHX_PB + a) * fvs];
  double D, tau, S[3], bc[3], sig[3];
  p2c<MINK>(P[PHX_PRHO * fvs], vp, bp, P[PHX_PENG * fvs], P[PHX_PPRS * fvs], P[PHX_PGM1 * fvs], G.p, sdetgam, D, S,
            bc, tau, sig);
  b.cons[PHX_CRHO * fvs + id] = D;
#pragma unroll
  for (int a = 0; a < 3; a++) b.cons[(PHX_CMOM + a) * fvs + id] = S[a];
  b.cons[PHX_CENG * fvs + id] = tau;
  const Closure<M1, MINK> c(fluid_v<MINK>(b, id, G.geo()), false, G.geo());
  r.prim[PHX_RJ * vs + id] = kSMALL;
  J = r.prim[PHX_RJ * vs + id];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    r.prim[(PHX_RH + a) * vs + id] = 0.;
    H.d[a] = r.prim[(PHX_RH + a) * vs + id] * J;
  }
  c.prim2con(J, H, Pi, E, F);
  r.cons[PHX_RE * vs + id] = E * sdetgam;
#pragma unroll
  for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = F.d[a] * sdetgam;
}

// ------------------------------------------------------ fourd solver
// moments_source.cpp:39-150 (SourceResidual4) and :489-786 for one zone:
// Newton's method over the fluid's P = (u, W v^i) for
// U_mhd(P) - U_mhd_0 + dt S(P, P_rad) = 0, where the radiation takes up what
// the fluid loses (U_rad = U_rad_0 - (U_mhd - U_mhd_0)) and P_rad = (J, H_i)
// is its closure inversion with the guess's velocity.  As in the reference:
// the fluid enters prim2con with B = 0 (the B primitives are declared a
// second time in an inner block there and never reach the solver); kappaH is
// the absorption coefficient taken twice, both capped at 1e5; the closure
// solve starts from xi = 0.5 (SolveClosure's default; the reference passes
// an uninitialised local).
template <bool M1, bool MINK>
struct SrcRes4 {
  const RPar &p;
  const Par &fp;
  const RGeo<MINK> &G;
  double rho, sdetgam, alpha;
  double U0[4], R0[4];  // U_mhd_0, U_rad_0
  __device__ __forceinline__ void mhd_cons(const double P[4], double U[4]) const {
    const double Pg = eos_P_rho_sie(fp, rho, div_p(P[0], rho));
    const double gam1 = div_p(eos_bmod_rho_sie(fp, rho, div_p(P[0], rho)), Pg);
    const double bp[3] = {0.0, 0.0, 0.0};
    double D, bc[3];
    p2c<MINK>(rho, &P[1], bp, P[0], Pg, gam1, G.p, sdetgam, D, &U[1], bc, U[0], nullptr);
  }
  __device__ __forceinline__ double W_of(const double P[4]) const {
    double W = 0.;
#pragma unroll
    for (int ii = 0; ii < 3; ii++)
#pragma unroll
      for (int jj = 0; jj < 3; jj++) W += G.cov(ii, jj) * P[ii + 1] * P[jj + 1];
    return sqrt(1. + W);
  }
  // U_mhd, U_rad, P_rad and the source at P; the closure inversion's status
  __device__ __forceinline__ int eval(const double P[4], double U[4], double Ur[4], double Pr[4], double S[4]) const {
    mhd_cons(P, U);
#pragma unroll
    for (int n = 0; n < 4; n++) Ur[n] = R0[n] - (U[n] - U0[n]);
    const double E = div_p(Ur[0], sdetgam);
    V3 F;
#pragma unroll
    for (int a = 0; a < 3; a++) F.d[a] = div_p(Ur[a + 1], sdetgam);
    const double W = W_of(P);
    V3 cv;
#pragma unroll
    for (int a = 0; a < 3; a++) cv.d[a] = div_p(P[a + 1], W);
    const Closure<M1, MINK> c(cv, true, G.geo());
    double xi = 0.5, phi = PI;
    T2 Pi;
    c.tilpi_from_con(E, F, xi, phi, Pi);
    V3 H;
    const int st = c.con2prim(E, F, Pi, Pr[0], H);
#pragma unroll
    for (int a = 0; a < 3; a++) Pr[a + 1] = H.d[a];
    // CalculateSource
    const double Tg = eos_T_rho_sie(fp, rho, div_p(P[0], rho));
    const double JBB = p.jbb * (Tg * Tg) * (Tg * Tg);
    double kappaJ = rho * p.kappa_a;
    double kappaH = kappaJ + rho * p.kappa_a;
    kappaH = smin(kappaH, 1.e5);
    kappaJ = smin(kappaJ, 1.e5);
    double cov_v[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int ii = 0; ii < 3; ii++)
#pragma unroll
      for (int jj = 0; jj < 3; jj++) cov_v[ii] += div_p(G.cov(ii, jj) * P[jj + 1], W);
    double vdH = 0.;
#pragma unroll
    for (int ii = 0; ii < 3; ii++) vdH += div_p(P[ii + 1], W) * Pr[ii + 1];
    S[0] = alpha * sdetgam * (kappaJ * W * (JBB - Pr[0]) - kappaH * vdH);
#pragma unroll
    for (int ii = 0; ii < 3; ii++)
      S[ii + 1] = alpha * sdetgam * (kappaJ * W * cov_v[ii] * (JBB - Pr[0]) - kappaH * Pr[1 + ii]);
    return st;
  }
};

// LinearAlgebra::matrixInverse4x4 (linear_algebra.hpp:90-147): the adjugate
// from 3x3 minors over the determinant expanded along the first row.
__device__ __forceinline__ double minor3(const double m[16], int r0, int r1, int r2, int c0, int c1, int c2) {
  return m[4 * r0 + c0] * (m[4 * r1 + c1] * m[4 * r2 + c2] - m[4 * r2 + c1] * m[4 * r1 + c2]) -
         m[4 * r0 + c1] * (m[4 * r1 + c0] * m[4 * r2 + c2] - m[4 * r2 + c0] * m[4 * r1 + c2]) +
         m[4 * r0 + c2] * (m[4 * r1 + c0] * m[4 * r2 + c1] - m[4 * r2 + c0] * m[4 * r1 + c1]);
}
__device__ __forceinline__ void inverse4x4(const double a[4][4], double inv[4][4]) {
  const double *m = &a[0][0];
  double *o = &inv[0][0];
  const int R[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
#pragma unroll
  for (int col = 0; col < 4; col++)
#pragma unroll
    for (int row = 0; row < 4; row++) {
      const double mn = minor3(m, R[col][0], R[col][1], R[col][2], R[row][0], R[row][1], R[row][2]);
      o[4 * row + col] = ((row + col) % 2 == 0) ? mn : -mn;
    }
  const double det = m[0] * minor3(m, 1, 2, 3, 1, 2, 3) - m[1] * minor3(m, 1, 2, 3, 0, 2, 3) +
                     m[2] * minor3(m, 1, 2, 3, 0, 1, 3) - m[3] * minor3(m, 1, 2, 3, 0, 1, 2);
#pragma unroll
  for (int i = 0; i < 16; i++) o[i] = o[i] / det;
}

// The Newton iterations (see the oracle's fourd_zone for the steps).  True
// on success, with dE, dF the radiation's change per sqrt(gamma).
template <bool M1, bool MINK>
__device__ bool fourd_zone(const RPar &p, const Par &fp, const BView &b, const RView &r, const RGeo<MINK> &G,
                           long long id, double dt, double &dE, V3 &dF) {
  const long long vs = r.vs, fvs = b.vs;
  const double rho = b.prim[PHX_PRHO * fvs + id];
  double P[4] = {b.prim[PHX_PENG * fvs + id], b.prim[PHX_PVEL * fvs + id], b.prim[(PHX_PVEL + 1) * fvs + id],
                 b.prim[(PHX_PVEL + 2) * fvs + id]};
  SrcRes4<M1, MINK> srm{p, fp, G, rho, G.sdetgam(), G.alpha(), {}, {}};
  srm.mhd_cons(P, srm.U0);
#pragma unroll
  for (int n = 0; n < 4; n++) srm.R0[n] = r.cons[(PHX_RE + n) * vs + id];
  const double eps = p.fd_eps, xi_max = p.xi_ceiling;
  double U[4], Ur[4], Pr[4], dS[4], res[4];
  int status = srm.eval(P, U, Ur, Pr, dS);
#pragma unroll
  for (int n = 0; n < 4; n++) res[n] = U[n] - srm.U0[n] + dt * dS[n];
  double err = 1.e100;
  int niter = 0;
  bool bad = false;
  do {
    double jac[4][4];
    double mag_min = DBL_MAX;
#pragma unroll
    for (int m = 0; m < 4; m++)
      if (fabs(P[m]) > 0.) mag_min = smin(mag_min, fabs(P[m]));
    bool bad_m = false, bad_p = false;
    for (int m = 0; m < 4; m++) {
      double Pm[4] = {P[0], P[1], P[2], P[3]}, Pp[4] = {P[0], P[1], P[2], P[3]};
      const double step = smax(eps * mag_min, eps * fabs(P[m]));
      Pm[m] -= step;
      Pp[m] += step;
      double Um[4], Urm[4], Prm[4], dSm[4], Up[4], Urp[4], Prp[4], dSp[4];
      if (srm.eval(Pm, Um, Urm, Prm, dSm) == FAILURE) bad_m = true;
      if (srm.eval(Pp, Up, Urp, Prp, dSp) == FAILURE) bad_p = true;
#pragma unroll
      for (int n = 0; n < 4; n++) {
        const double fpl = Up[n] - srm.U0[n] + dt * dSp[n];
        const double fmi = Um[n] - srm.U0[n] + dt * dSm[n];
        jac[n][m] = div_p(fpl - fmi, Pp[m] - Pm[m]);
      }
    }
    if (bad_m && bad_p) {
      bad = true;
      break;
    } else if (bad_m || bad_p) {  // one-sided from the guess, on the good side
      const double side = bad_m ? 1.0 : -1.0;
      for (int m = 0; m < 4; m++) {
        double Ps[4] = {P[0], P[1], P[2], P[3]};
        Ps[m] += side * smax(eps * mag_min, eps * fabs(Ps[m]));
        double Us[4], Urs[4], Prs[4], dSs[4];
        srm.eval(Ps, Us, Urs, Prs, dSs);
#pragma unroll
        for (int n = 0; n < 4; n++) {
          const double fs = Us[n] - srm.U0[n] + dt * dSs[n];
          const double fg = U[n] - srm.U0[n] + dt * dS[n];
          jac[n][m] = bad_m ? div_p(fs - fg, Ps[m] - P[m]) : div_p(fg - fs, P[m] - Ps[m]);
        }
      }
    }
    double jinv[4][4];
    inverse4x4(jac, jinv);
    if (!bad) {
      const double ug0 = P[0], ur0 = Pr[0];
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) P[m] -= jinv[m][n] * res[n];
      status = srm.eval(P, U, Ur, Pr, dS);
      if (status == FAILURE) bad = true;
      if (bad) {
        V3 H;
#pragma unroll
        for (int a = 0; a < 3; a++) H.d[a] = div_p(Pr[a + 1], Pr[0]);
        double hh = 0.0;
        if constexpr (MINK) {
#pragma unroll
          for (int a = 0; a < 3; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) hh += gdelta(a, c) * H.d[a] * H.d[c];
        } else {
          hh = G.g.contract_cov(H, H);
        }
        double vh = 0.0;
#pragma unroll
        for (int a = 0; a < 3; a++) vh += P[a + 1] * H.d[a];
        const double xi = div_p(sqrt(hh - vh * vh), Pr[0]);
        constexpr double umin = 100. * kSMALL, Jmin = 100. * kSMALL;
        double scale = 0.;
        if (xi > xi_max) scale = smax(scale, div_p(xi_max, xi));
        if (P[0] < umin) scale = smax(scale, div_p(ug0 - umin, ug0 - P[0]));
        if (Pr[0] < Jmin) scale = smax(scale, div_p(ur0 - Jmin, ur0 - Pr[0]));
        if (!(scale > kSMALL && scale >= 1.)) {  // the reference prints and gives up
          bad = true;
          break;
        }
        scale *= 0.5;
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
          for (int n = 0; n < 4; n++) P[m] += (1. - scale) * jinv[m][n] * res[n];
        status = srm.eval(P, U, Ur, Pr, dS);
        if (status == SUCCESS) bad = false;
      }
    }
    if (bad) break;
#pragma unroll
    for (int n = 0; n < 4; n++) res[n] = U[n] - srm.U0[n] + dt * dS[n];
    if (isnan(res[0]) || isnan(res[1]) || isnan(res[2]) || isnan(res[3])) {
      bad = true;
      break;
    }
    err = kSMALL;
    double max_div = kSMALL;
#pragma unroll
    for (int n = 0; n < 4; n++) max_div = smax(max_div, fabs(U[n]) + fabs(srm.U0[n]) + fabs(dt * dS[n]));
#pragma unroll
    for (int n = 0; n < 4; n++) {
      const double sub = div_p(fabs(res[n]), max_div);
      if (sub > err) err = sub;
    }
    niter++;
    if (niter == p.maxiter) break;
  } while (err > p.tol);
  if (niter == p.maxiter || err > p.tol || isnan(Ur[0]) || isnan(Ur[1]) || isnan(Ur[2]) || isnan(Ur[3]) || bad)
    return false;
  dE = div_p(Ur[0] - r.cons[PHX_RE * vs + id], srm.sdetgam);
#pragma unroll
  for (int a = 0; a < 3; a++) dF.d[a] = div_p(Ur[a + 1] - r.cons[(PHX_RF + a) * vs + id], srm.sdetgam);
  return true;
}

template <bool M1, bool UPD, bool MINK, bool FOURD>
__global__ void __launch_bounds__(128) k_source(RPar p, Par fp, BView b, RView r, double dt, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long id = b.idx(k, j, i), vs = r.vs, fvs = b.vs;
  const RGeo<MINK> G(b, 0, j, i);
  const double alpha = G.alpha(), sdetgam = G.sdetgam();
  const double amax = p.tau_max / (alpha * dt);
  const double rho = b.prim[PHX_PRHO * fvs + id], ug = b.prim[PHX_PENG * fvs + id],
               Tf = b.prim[PHX_PTMP * fvs + id];
  double W;
  const V3 cv = fluid_v<MINK>(b, id, G.geo(), &W);
  double dE = 0.0;
  V3 dF;
  dF.d[0] = dF.d[1] = dF.d[2] = 0.0;
  bool success = false;
  T2 Pi;
  bool oned = !FOURD;
  if constexpr (FOURD) {
    // fourd, falling back to oned when it fails and src_use_oned_backup is
    // set (the reference's goto); without the fallback a failed zone keeps
    // dE = dF = 0 for the fluid update (uninitialised in the reference)
    success = fourd_zone<M1, MINK>(p, fp, b, r, G, id, dt, dE, dF);
    oned = !success && p.oned_backup;
  }
  if (oned) {
    const double J0 = r.prim[PHX_RJ * vs + id];
    const double dtau = alpha * dt / W;
    TRes res{&p, rho, ug, J0, dtau, amax};
    res.prepare();
    int count = 0;
    bool ok;
    double T1 = regula_falsi(res, 1.e-2 * Tf, 1.e2 * Tf, p.tol * Tf, Tf, count, p.maxiter, ok);
    double fac = 10.;
    for (int tries = 0; !ok && tries < 4; tries++) {
      T1 = regula_falsi(res, 1.e-1 / fac * Tf, 1.e1 * fac * Tf, p.tol * Tf, Tf, count, p.maxiter, ok);
      fac *= 10.;
    }
    const Closure<M1, MINK> c(cv, true, G.geo());
    double Es = r.cons[PHX_RE * vs + id] / sdetgam;
    V3 Fs;
#pragma unroll
    for (int a = 0; a < 3; a++) Fs.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam;
    double J = r.prim[PHX_RJ * vs + id];
    V3 H;
#pragma unroll
    for (int a = 0; a < 3; a++) H.d[a] = J * r.prim[(PHX_RH + a) * vs + id];
    c.tilpi_from_prim(J, H, Pi);
    const double JBB = p.jbb * (T1 * T1) * (T1 * T1);
    const double kappaJ = smin(rho * p.kappa_a, amax);
    double kappaH = smin(rho * p.kappa_s, amax);
    kappaH += kappaJ;
    double tauJ = alpha * dt * kappaJ;
    double tauH = alpha * dt * kappaH;
    if (ok) {
      c.linear_source_update(Es, Fs, Pi, JBB, tauJ, tauH, dE, dF);
      Es += dE;
#pragma unroll
      for (int a = 0; a < 3; a++) Fs.d[a] += dF.d[a];
      success = c.con2prim(Es, Fs, Pi, J, H) == SUCCESS;
    }
    if (!success && p.oned_fixup == PHX_RAD_ONED_FIXUP_IGNORE_DJ) {
      Es = r.cons[PHX_RE * vs + id] / sdetgam;
#pragma unroll
      for (int a = 0; a < 3; a++) Fs.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam;
      const double JBB2 = p.jbb * (Tf * Tf) * (Tf * Tf);
      const double kJ = rho * p.kappa_a;
      const double kH2 = rho * p.kappa_s + kJ;
      tauJ = alpha * dt * kJ;
      tauH = alpha * dt * kH2;
      c.linear_source_update(Es, Fs, Pi, JBB2, tauJ, tauH, dE, dF);
      Es = r.cons[PHX_RE * vs + id] / sdetgam + dE;
#pragma unroll
      for (int a = 0; a < 3; a++) Fs.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam + dF.d[a];
      success = c.con2prim(Es, Fs, Pi, J, H) == SUCCESS;
    } else if (!success && p.oned_fixup == PHX_RAD_ONED_FIXUP_IGNORE_ALL) {
      dE = 0.;
      dF.d[0] = dF.d[1] = dF.d[2] = 0.;
      success = true;
    }
  }
  if (success) {
    r.cons[PHX_RE * vs + id] += sdetgam * dE;
#pragma unroll
    for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] += sdetgam * dF.d[a];
  }
  if constexpr (UPD) {
    source_update_fluid<M1, MINK>(fp, b, r, G, k, j, i, id, dE, dF);
    return;
  }
  double E = r.cons[PHX_RE * vs + id] / sdetgam;
  V3 F, H;
  double J;
  const Closure<M1, MINK> cf(cv, false, G.geo());
#pragma unroll
  for (int a = 0; a < 3; a++) F.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam;
  double xi = 0.0, phi = PI;
  cf.tilpi_from_con(E, F, xi, phi, Pi);
  if (cf.con2prim(E, F, Pi, J, H) == SUCCESS) {
    r.prim[PHX_RJ * vs + id] = J;
#pragma unroll
    for (int a = 0; a < 3; a++) r.prim[(PHX_RH + a) * vs + id] = div_p(H.d[a], J);
    return;
  }
  // failed inversion: the reference's zero-radiation state
  r.prim[PHX_RJ * vs + id] = kSMALL;
  J = r.prim[PHX_RJ * vs + id];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    r.prim[(PHX_RH + a) * vs + id] = 0.;
    H.d[a] = r.prim[(PHX_RH + a) * vs + id] * J;
  }
  cf.prim2con(J, H, Pi, E, F);
  r.cons[PHX_RE * vs + id] = E * sdetgam;
#pragma unroll
  for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = F.d[a] * sdetgam;
}

// ------------------------------------- RadConservedToPrimitiveFixup
// fixup_radc2p.cpp:45-225 over the interior: a zone whose closure inversion
// failed (c2pfail = 0) takes the average of J and H_i / J over its face
// neighbours weighted by their c2pfail flags (strategy interpolate, at least
// one valid neighbour), else J = 10 SMALL, H = 0; H / J is then held to the
// xi ceiling and E, F_i follow from prim2con with the zone's fluid velocity.
// A failed neighbour contributes nothing; the reference multiplies it by its
// zero flag in place while other zones are rewritten, which is the same
// whenever the failed zones hold finite values.
template <bool M1, bool MINK>
__global__ void __launch_bounds__(128) k_rad_c2p_fixup(RPar p, BView b, RView r, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long id = b.idx(k, j, i), vs = r.vs;
  const double *F = r.prim + PHX_RFAIL * vs;
  if (F[id] != 0.0) return;
  const long long di = 1, dj = b.n1t, dk = (long long)b.n1t * b.n2t;
  const RGeo<MINK> G(b, 0, j, i);
  const V3 cv = fluid_v<MINK>(b, id, G.geo());
  auto nb = [&](int iv, long long o) { return F[o] != 0.0 ? F[o] * r.prim[iv * vs + o] : 0.0; };
  auto fixv = [&](int iv, double inv_mask_sum) {
    double s = nb(iv, id - di) + nb(iv, id + di);
    if (b.ndim > 1) {
      s += nb(iv, id - dj) + nb(iv, id + dj);
      if (b.ndim == 3) s += nb(iv, id - dk) + nb(iv, id + dk);
    }
    return inv_mask_sum * s;
  };
  double num_valid = F[id - di] + F[id + di];
  if (b.ndim > 1) num_valid += F[id - dj] + F[id + dj];
  if (b.ndim == 3) num_valid += F[id - dk] + F[id + dk];
  double J;
  V3 Hr;
  if (num_valid > 0.5 && !p.rad_fixup_floors) {
    const double norm = 1.0 / num_valid;
    J = fixv(PHX_RJ, norm);
#pragma unroll
    for (int a = 0; a < 3; a++) Hr.d[a] = fixv(PHX_RH + a, norm);
  } else {
    J = 10. * kSMALL;
    Hr.d[0] = Hr.d[1] = Hr.d[2] = 0.;
  }
  {
    const double hh = MINK ? ccov(Hr, Hr) : G.g.contract_cov(Hr, Hr);
    const double vh = ccov(cv, Hr);
    const double xi = sqrt(hh - vh * vh);
    if (xi > p.xi_ceiling) {
#pragma unroll
      for (int a = 0; a < 3; a++) Hr.d[a] *= p.xi_ceiling / xi;
    }
  }
  r.prim[PHX_RJ * vs + id] = J;
#pragma unroll
  for (int a = 0; a < 3; a++) r.prim[(PHX_RH + a) * vs + id] = Hr.d[a];
  const Closure<M1, MINK> c(cv, true, G.geo());
  V3 H;
#pragma unroll
  for (int a = 0; a < 3; a++) H.d[a] = Hr.d[a] * J;
  T2 Pi;
  c.tilpi_from_prim(J, H, Pi);
  double E;
  V3 Fc;
  c.prim2con(J, H, Pi, E, Fc);
  const double sdetgam = G.sdetgam();
  r.cons[PHX_RE * vs + id] = sdetgam * E;
#pragma unroll
  for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = sdetgam * Fc.d[a];
}

// ------------------------------------- ApplyFloors, radiation part
// fixup.cpp:542-678 (enable_rad_floors, one species), after the fluid part
// of the same zone: with the fluid's velocity as the floors left it, the
// closure inversion is redone where the fluid floors or ceilings acted
// (flag != 0), from xi = 0; a J below the floor gains an isotropic
// normal-observer radiation field of the missing J (added to E, F_i, then
// inverted again); H / J above the xi ceiling is scaled down and E, F_i
// recomputed.
template <bool M1, bool MINK>
__global__ void __launch_bounds__(128) k_rad_floors(RPar p, BView b, RView r, const double *flag, Range3 rg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= range_count(rg)) return;
  int k, j, i;
  zone_of(rg, t, k, j, i);
  const long long id = b.idx(k, j, i), vs = r.vs;
  const RGeo<MINK> G(b, 0, j, i);
  const double sdetgam = G.sdetgam();
  const V3 cv = fluid_v<MINK>(b, id, G.geo());
  const Closure<M1, MINK> c(cv, true, G.geo());
  double E, J;
  V3 F, H;
  T2 Pi;
  auto invert = [&]() {  // GetConTilPiFromCon from xi = 0, then Con2Prim; J, H / J stored
    double xi = 0.0, phi = PI * 1.000001;
    c.tilpi_from_con(E, F, xi, phi, Pi);
    c.con2prim(E, F, Pi, J, H);
    r.prim[PHX_RJ * vs + id] = J;
#pragma unroll
    for (int a = 0; a < 3; a++) r.prim[(PHX_RH + a) * vs + id] = H.d[a] / J;
  };
  if (flag[id] != 0.0) {
    E = r.cons[PHX_RE * vs + id] / sdetgam;
#pragma unroll
    for (int a = 0; a < 3; a++) F.d[a] = r.cons[(PHX_RF + a) * vs + id] / sdetgam;
    invert();
  }
  const double dJ = j_floor_at(p, b.Xc(0, i)) - r.prim[PHX_RJ * vs + id];
  if (dJ > 0.) {
    V3 zero, Hz;
    zero.d[0] = zero.d[1] = zero.d[2] = 0.0;
    Hz = zero;
    T2 Pz;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int q = 0; q < 3; q++) Pz.d[a][q] = 0.0;
    const Closure<M1, MINK> c_iso(zero, true, G.geo());
    c_iso.prim2con(dJ, Hz, Pz, E, F);
    E += r.cons[PHX_RE * vs + id] / sdetgam;
#pragma unroll
    for (int a = 0; a < 3; a++) F.d[a] += r.cons[(PHX_RF + a) * vs + id] / sdetgam;
    r.cons[PHX_RE * vs + id] = E * sdetgam;
#pragma unroll
    for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = F.d[a] * sdetgam;
    invert();
  }
  V3 Hr;
#pragma unroll
  for (int a = 0; a < 3; a++) Hr.d[a] = r.prim[(PHX_RH + a) * vs + id];
  const double hh = MINK ? ccov(Hr, Hr) : G.g.contract_cov(Hr, Hr);
  const double vh = ccov(cv, Hr);
  const double xi = sqrt(hh - vh * vh);
  if (xi > p.xi_ceiling) {
    J = r.prim[PHX_RJ * vs + id];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      H.d[a] = (p.xi_ceiling / xi) * Hr.d[a] * J;
      r.prim[(PHX_RH + a) * vs + id] = H.d[a] / J;
    }
    c.tilpi_from_prim(J, H, Pi);
    c.prim2con(J, H, Pi, E, F);
    r.cons[PHX_RE * vs + id] = E * sdetgam;
#pragma unroll
    for (int a = 0; a < 3; a++) r.cons[(PHX_RF + a) * vs + id] = F.d[a] * sdetgam;
  }
}

// ------------------------------------------------------- timestep
__global__ void k_dt_init(unsigned long long *scratch) { *scratch = 0x7fefffffffffffffull; }
template <bool MINK>
__global__ void __launch_bounds__(256) k_dt(RPar p, BView b, RView r, Range3 rg, unsigned long long *scratch) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = DBL_MAX;
  if (t < range_count(rg)) {
    int k, j, i;
    zone_of(rg, t, k, j, i);
    const long long id = b.idx(k, j, i);
    const RGeo<MINK> G(b, 0, j, i);
    const double alpha = G.alpha();
    const double kappaH = r.prim[PHX_RKAPPAH * r.vs + id];
    for (int d = 0; d < b.ndim; d++) {
      const double sigp = alpha * sqrt(G.con(d, d)) - G.beta(d);
      const double sigm = -alpha * sqrt(G.con(d, d)) - G.beta(d);
      const double asym_sigl = alpha * b.prim[(PHX_PVEL + d) * b.vs + id] - G.beta(d);
      const double rad_speed = smax(fabs(sigm), fabs(sigp));
      const double asym_speed = fabs(asym_sigl);
      const double w = b.dx[d];
      const double dx = w * sqrt(G.cov(d, d));
      const double a = tanh_r(ratio(1.0, fabs(kappaH * dx)));
      const double csig = a * rad_speed + (1. - a) * asym_speed;
      v = smin(v, 1.0 / (csig / w));
    }
  }
  // non-negative doubles order like their bit patterns; NaN zones are
  // skipped like the reference's min (a NaN never compares less)
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = fmin(v, sm[w]);
    if (v >= 0.0) atomicMin(scratch, (unsigned long long)__double_as_longlong(v));
  }
}
__global__ void k_dt_final(const unsigned long long *scratch, double cfl, double *out) {
  *out = cfl * __longlong_as_double((long long)*scratch);
}

// ------------------------------------------------------- launchers
namespace {
inline unsigned blocks_for(long long n, int T) { return (unsigned)((n + T - 1) / T); }
Range3 interior3(const BView &b) {
  return {b.ng, b.ng + b.nx1 - 1, b.ndim >= 2 ? b.ng : 0, b.ndim >= 2 ? b.ng + b.nx2 - 1 : 0,
          b.ndim >= 3 ? b.ng : 0, b.ndim >= 3 ? b.ng + b.nx3 - 1 : 0};
}
}  // namespace

// Every launcher picks the closure (M1 or Eddington) and the metric
// (Minkowski, or the block's FMKS tables) at run time.
void launch_p2c(const RPar &p, const BView &b, const RView &r, Range3 rg, cudaStream_t s) {
  const long long n = range_count(rg);
  if (n <= 0) return;
  const unsigned g = blocks_for(n, 128);
  if (b.fmks) {
    if (p.m1)
      k_p2c<true, false><<<g, 128, 0, s>>>(p, b, r, rg);
    else
      k_p2c<false, false><<<g, 128, 0, s>>>(p, b, r, rg);
  } else {
    if (p.m1)
      k_p2c<true, true><<<g, 128, 0, s>>>(p, b, r, rg);
    else
      k_p2c<false, true><<<g, 128, 0, s>>>(p, b, r, rg);
  }
}

void launch_c2p(const RPar &p, const BView &b, const RView &r, Range3 rg, cudaStream_t s) {
  const long long n = range_count(rg);
  if (n <= 0) return;
  const unsigned g = blocks_for(n, 128);
  if (b.fmks) {
    if (p.m1)
      k_c2p<true, false><<<g, 128, 0, s>>>(p, b, r, rg);
    else
      k_c2p<false, false><<<g, 128, 0, s>>>(p, b, r, rg);
  } else {
    if (p.m1)
      k_c2p<true, true><<<g, 128, 0, s>>>(p, b, r, rg);
    else
      k_c2p<false, true><<<g, 128, 0, s>>>(p, b, r, rg);
  }
}

void launch_opacities(const RPar &p, const BView &b, const RView &r, cudaStream_t s) {
  const long long n = (long long)b.n1t * b.n2t * b.n3t;
  k_opacities<<<blocks_for(n, 256), 256, 0, s>>>(p, b, r, n);
}

template <bool M1, int RECON, bool MINK>
static void fluxes_r(const BView &b, const RPar &p, const RView &r, int d, Range3 rg, unsigned g, cudaStream_t s) {
  if (d == 0)
    k_fluxes<M1, RECON, 0, MINK><<<g, 128, 0, s>>>(p, b, r, rg);
  else if (d == 1)
    k_fluxes<M1, RECON, 1, MINK><<<g, 128, 0, s>>>(p, b, r, rg);
  else
    k_fluxes<M1, RECON, 2, MINK><<<g, 128, 0, s>>>(p, b, r, rg);
}

template <bool M1, bool MINK>
static void fluxes_t(const RPar &p, const BView &b, const RView &r, int d, Range3 rg, cudaStream_t s) {
  const unsigned g = blocks_for(range_count(rg), 128);
  switch (p.recon) {
  case PHX_RECON_WENO5Z: fluxes_r<M1, PHX_RECON_WENO5Z, MINK>(b, p, r, d, rg, g, s); break;
  case PHX_RECON_MP5: fluxes_r<M1, PHX_RECON_MP5, MINK>(b, p, r, d, rg, g, s); break;
  case PHX_RECON_LINEAR: fluxes_r<M1, PHX_RECON_LINEAR, MINK>(b, p, r, d, rg, g, s); break;
  default: fluxes_r<M1, PHX_RECON_CONSTANT, MINK>(b, p, r, d, rg, g, s); break;
  }
}

void launch_fluxes(const RPar &p, const BView &b, const RView &r, cudaStream_t s) {
  for (int d = 0; d < b.ndim; d++) {
    Range3 rg = interior3(b);
    if (d == 0) rg.ie += 1;
    if (d == 1) rg.je += 1;
    if (d == 2) rg.ke += 1;
    if (b.fmks) {
      if (p.m1)
        fluxes_t<true, false>(p, b, r, d, rg, s);
      else
        fluxes_t<false, false>(p, b, r, d, rg, s);
    } else {
      if (p.m1)
        fluxes_t<true, true>(p, b, r, d, rg, s);
      else
        fluxes_t<false, true>(p, b, r, d, rg, s);
    }
  }
}

void launch_update(const RPar &p, const BView &b, const RView &r, const double *base, double *out, double beta,
                   double dt, cudaStream_t s) {
  const Range3 rg = interior3(b);
  const unsigned g = blocks_for(range_count(rg), 256);
  if (!b.fmks)
    k_update<true, true><<<g, 256, 0, s>>>(b, r, base, out, beta, dt, rg);
  else if (p.m1)
    k_update<true, false><<<g, 256, 0, s>>>(b, r, base, out, beta, dt, rg);
  else
    k_update<false, false><<<g, 256, 0, s>>>(b, r, base, out, beta, dt, rg);
}

// the fourd solver is its own instantiation, so the oned kernels keep the
// registers they need
template <bool MINK, bool FOURD>
static void source_s(const RPar &p, const Par &fp, const BView &b, const RView &r, double dt, Range3 rg,
                     unsigned g, cudaStream_t s) {
  if (p.m1) {
    if (p.update_fluid)
      k_source<true, true, MINK, FOURD><<<g, 128, 0, s>>>(p, fp, b, r, dt, rg);
    else
      k_source<true, false, MINK, FOURD><<<g, 128, 0, s>>>(p, fp, b, r, dt, rg);
  } else {
    if (p.update_fluid)
      k_source<false, true, MINK, FOURD><<<g, 128, 0, s>>>(p, fp, b, r, dt, rg);
    else
      k_source<false, false, MINK, FOURD><<<g, 128, 0, s>>>(p, fp, b, r, dt, rg);
  }
}
template <bool MINK>
static void source_t(const RPar &p, const Par &fp, const BView &b, const RView &r, double dt, Range3 rg, unsigned g,
                     cudaStream_t s) {
  if (p.fourd)
    source_s<MINK, true>(p, fp, b, r, dt, rg, g, s);
  else
    source_s<MINK, false>(p, fp, b, r, dt, rg, g, s);
}

void launch_source(const RPar &p, const Par &fp, const BView &b, const RView &r, double dt, cudaStream_t s) {
  const Range3 rg = interior3(b);
  const unsigned g = blocks_for(range_count(rg), 128);
  if (b.fmks)
    source_t<false>(p, fp, b, r, dt, rg, g, s);
  else
    source_t<true>(p, fp, b, r, dt, rg, g, s);
}

// ------------------------------------------ boundary exchange of a tiled mesh
// The radiation half of PhoebusDriver's exchange (phoebus_driver.cpp:646-668)
// for one ghost: every radiation field with Metadata::FillGhost (E, F_i and
// J, H_i/J, xi, phi, c2pfail; radiation.cpp:448-474, 506-508).  Inside the
// domain the owner's values are copied.  Beyond a physical face the boundary
// functions act on every FillGhost field (phoebus_boundaries.cpp:42-254): the
// mapped cell's value, with bc_vars = conserved scaled at each face by
// robust::ratio(DetGamma(cell), DetGamma(source)) -- the radiation primitives
// too, since they carry FillGhost under either bc_vars -- and F_d, H_d
// negated across a reflect face along d (Metadata::Vector); the polar faces
// negate only the fluid's v^2 and B^2 (PolarInnerX2 / PolarOuterX2).
// ConvertBoundaryConditions (:303-445) then, in the outer-X1 slab of an FMKS
// mesh with the inflow check, removes radiation flux entering the domain
// (H^1 < 0: H^1 = 0, |H| capped at 0.99, H_i lowered again), and with
// bc_vars = primitive rebuilds E, F_i from J, H_i and the fluid velocity of
// the ghost (MomentPrim2Con over the physical slabs).
template <bool M1, bool MINK>
__global__ void __launch_bounds__(128) k_mesh_ghost(RPar p, const BView *views, const RView *rviews, MeshDev m,
                                                    int blk, int inflow) {
  const BView &b = views[blk];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)b.n1t * b.n2t * b.n3t) return;
  const GhostMap q = map_ghost(views, m, blk, t);
  if (!q.ghost) return;
  const RView &r = rviews[blk], &sr = rviews[q.src];
  constexpr int NP = PHX_RFAIL + 1;  // the FillGhost primitives
  double U[PHX_RNCONS], P[NP];
#pragma unroll
  for (int v = 0; v < PHX_RNCONS; v++) U[v] = sr.cons[v * sr.vs + q.sid];
#pragma unroll
  for (int v = 0; v < NP; v++) P[v] = sr.prim[v * sr.vs + q.sid];
  if (q.physical) {
    const bool conserved = m.bc_vars == PHX_BC_VARS_CONSERVED;
    for (int d = 0; d < b.ndim; d++) {
      if (!q.phys[d]) continue;
      const double sg = q.reflect[d] ? -1.0 : 1.0;
      double gr = 1.0;  // DetGamma = 1 in Minkowski: ratio(1, 1) = 1
      if (!MINK && conserved) gr = ghost_gratio(b, q, d);
#pragma unroll
      for (int v = 0; v < PHX_RNCONS; v++) {
        const double s = v == PHX_RF + d ? sg : 1.0;
        U[v] = conserved ? s * gr * U[v] : s * U[v];
      }
#pragma unroll
      for (int v = 0; v < NP; v++) {
        const double s = v == PHX_RH + d ? sg : 1.0;
        P[v] = conserved ? s * gr * P[v] : s * P[v];
      }
    }
    const RGeo<MINK> G(b, 0, q.loc[1], q.loc[0]);
    if constexpr (!MINK) {
      if (inflow && q.outer_x1) {  // no flux of radiation into the domain (:383-411)
        double Hcon[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++) Hcon[a] += G.con(a, c) * P[PHX_RH + c];
        if (Hcon[0] < 0.) {
          Hcon[0] = 0.;
          double xi = 0.;
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) xi += G.cov(a, c) * Hcon[a] * Hcon[c];
          xi = sqrt(xi);
          if (xi > 0.99)
            for (int a = 0; a < 3; a++) Hcon[a] *= 0.99 / xi;
          for (int a = 0; a < 3; a++) {
            P[PHX_RH + a] = 0.;
            for (int c = 0; c < 3; c++) P[PHX_RH + a] += G.cov(a, c) * Hcon[c];
          }
        }
      }
    }
    if (!conserved) {  // MomentPrim2Con (moments.cpp:198-275) at the ghost
      const Closure<M1, MINK> c(fluid_v<MINK>(b, q.id, G.geo()), true, G.geo());
      const double J = P[PHX_RJ];
      V3 H;
#pragma unroll
      for (int a = 0; a < 3; a++) H.d[a] = P[PHX_RH + a] * J;
      T2 Pi;
      c.tilpi_from_prim(J, H, Pi);
      double E;
      V3 F;
      c.prim2con(J, H, Pi, E, F);
      const double sdetgam = G.sdetgam();
      U[PHX_RE] = sdetgam * E;
#pragma unroll
      for (int a = 0; a < 3; a++) U[PHX_RF + a] = sdetgam * F.d[a];
    }
  }
#pragma unroll
  for (int v = 0; v < PHX_RNCONS; v++) r.cons[v * r.vs + q.id] = U[v];
#pragma unroll
  for (int v = 0; v < NP; v++) r.prim[v * r.vs + q.id] = P[v];
}

void launch_mesh_ghosts(const RPar &p, bool mink, const BView &b, const BView *views, const RView *rviews,
                        const MeshDev &m, int blk, int inflow, cudaStream_t s) {
  const unsigned g = blocks_for((long long)b.n1t * b.n2t * b.n3t, 128);
  if (p.m1) {
    if (mink)
      k_mesh_ghost<true, true><<<g, 128, 0, s>>>(p, views, rviews, m, blk, 0);
    else
      k_mesh_ghost<true, false><<<g, 128, 0, s>>>(p, views, rviews, m, blk, inflow);
  } else {
    if (mink)
      k_mesh_ghost<false, true><<<g, 128, 0, s>>>(p, views, rviews, m, blk, 0);
    else
      k_mesh_ghost<false, false><<<g, 128, 0, s>>>(p, views, rviews, m, blk, inflow);
  }
}

// FixFluxes' radiation part (fixup.cpp:728-1078) on one physical face of a
// block: the direction-d fluxes of the moments in mask (bit m: conserved
// moment m) set to 0 at local face index f, over the interior of the other
// axes.
__global__ void __launch_bounds__(256) k_fix_face(BView b, RView r, int d, int f, unsigned mask) {
  const int ng = b.ng;
  const int e1 = b.nx1, e2 = b.ndim >= 2 ? b.nx2 : 1, e3 = b.ndim >= 3 ? b.nx3 : 1;
  const int na = d == 0 ? e2 : e1, nb = d == 2 ? e2 : e3;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int a = (int)(t % na), c = (int)(t / na);
  const int o2 = b.ndim >= 2 ? ng : 0, o3 = b.ndim >= 3 ? ng : 0;
  const int i = d == 0 ? f : ng + a;
  const int j = d == 1 ? f : (d == 0 ? o2 + a : o2 + c);
  const int k = d == 2 ? f : o3 + c;
  const long long id = b.idx(k, j, i);
#pragma unroll
  for (int m = 0; m < PHX_RNCONS; m++)
    if ((mask >> m) & 1u) r.flux[((long long)d * PHX_RNCONS + m) * r.vs + id] = 0.0;
}

void launch_fix_face(const BView &b, const RView &r, int d, int f, unsigned mask, cudaStream_t s) {
  const long long e1 = b.nx1, e2 = b.ndim >= 2 ? b.nx2 : 1, e3 = b.ndim >= 3 ? b.nx3 : 1;
  const long long n = d == 0 ? e2 * e3 : (d == 1 ? e1 * e3 : e1 * e2);
  k_fix_face<<<blocks_for(n, 256), 256, 0, s>>>(b, r, d, f, mask);
}

void launch_ghosts(const BView &b, const RView &r, cudaStream_t s) {
  BView v = b;
  v.vs = r.vs;
  launch_ghost_periodic(v, r.cons, PHX_RNCONS, s);
  launch_ghost_periodic(v, r.prim, PHX_RFAIL + 1, s);
}

void launch_rad_c2p_fixup(const RPar &p, const BView &b, const RView &r, cudaStream_t s) {
  const Range3 rg = interior3(b);
  const unsigned g = blocks_for(range_count(rg), 128);
  if (b.fmks) {
    if (p.m1)
      k_rad_c2p_fixup<true, false><<<g, 128, 0, s>>>(p, b, r, rg);
    else
      k_rad_c2p_fixup<false, false><<<g, 128, 0, s>>>(p, b, r, rg);
  } else {
    if (p.m1)
      k_rad_c2p_fixup<true, true><<<g, 128, 0, s>>>(p, b, r, rg);
    else
      k_rad_c2p_fixup<false, true><<<g, 128, 0, s>>>(p, b, r, rg);
  }
}

void launch_rad_floors(const RPar &p, const BView &b, const RView &r, const double *flag, Range3 rg,
                       cudaStream_t s) {
  const long long n = range_count(rg);
  if (n <= 0) return;
  const unsigned g = blocks_for(n, 128);
  if (b.fmks) {
    if (p.m1)
      k_rad_floors<true, false><<<g, 128, 0, s>>>(p, b, r, flag, rg);
    else
      k_rad_floors<false, false><<<g, 128, 0, s>>>(p, b, r, flag, rg);
  } else {
    if (p.m1)
      k_rad_floors<true, true><<<g, 128, 0, s>>>(p, b, r, flag, rg);
    else
      k_rad_floors<false, true><<<g, 128, 0, s>>>(p, b, r, flag, rg);
  }
}

void launch_dt(const RPar &p, const BView &b, const RView &r, unsigned long long *scratch, double *dt_out,
               cudaStream_t s) {
  const Range3 rg = interior3(b);
  k_dt_init<<<1, 1, 0, s>>>(scratch);
  if (b.fmks)
    k_dt<false><<<blocks_for(range_count(rg), 256), 256, 0, s>>>(p, b, r, rg, scratch);
  else
    k_dt<true><<<blocks_for(range_count(rg), 256), 256, 0, s>>>(p, b, r, rg, scratch);
  k_dt_final<<<1, 1, 0, s>>>(scratch, p.cfl, dt_out);
}

}  // namespace rad
}  // namespace phx
