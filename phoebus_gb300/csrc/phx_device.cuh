// phx_device.cuh -- per-zone FP64 physics of the phoebus fluid hot path, on
// the device.
//
// Every function follows the operation order of the phoebus source it cites
// (paths relative to the phoebus tree), so that the exact build (nvcc
// -fmad=false) reproduces a CPU build without FMA contraction bit for bit.
// Minkowski is folded at compile time: with gcov = diag(-1,1,1,1), lapse 1,
// shift 0, each metric contraction of the reference reduces to the same
// sequence of roundings on its nonzero terms (x * 1 = x, s + (+-0) = s), so the
// folded form is bit-identical for finite states and saves most of the FP64
// work of the general contraction.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/phx_fluid.h"
#include "phx_math.h"

namespace phx {

// ------------------------------------------------------------ robust.hpp
constexpr double kSMALL = 10 * 2.2250738585072014e-308;  // 10 * DBL_MIN
constexpr double kEPS = 10 * 2.220446049250313e-16;      // 10 * DBL_EPSILON
constexpr double kDBLMAX = 1.7976931348623157e308;

// std::max / std::min as the reference calls them: the first argument comes
// back when the comparison is false, so a NaN there propagates (fmax / fmin
// would drop it).  The exact build keeps that for bit-for-bit parity on
// every input, NaN states included; the production build uses the one-
// instruction fmax / fmin (the two differ only where an argument is NaN).
__device__ __forceinline__ double rmax(double a, double b) {
#ifdef PHX_EXACT
  return (a < b) ? b : a;
#else
  return fmax(a, b);
#endif
}
__device__ __forceinline__ double rmin(double a, double b) {
#ifdef PHX_EXACT
  return (b < a) ? b : a;
#else
  return fmin(a, b);
#endif
}
__device__ __forceinline__ double make_positive(double v) { return rmax(v, kEPS); }
__device__ __forceinline__ double make_bounded(double v, double vmin, double vmax) {
  return rmin(rmax(v, vmin + kEPS), vmax * (1.0 - kEPS));
}
__device__ __forceinline__ double ratio(double a, double b) {
  const double sgn = b >= 0 ? 1.0 : -1.0;
  return a / (b + sgn * kSMALL);
}

// 1/x from the hardware reciprocal seed r and one third-order step
// r (1 + e + e^2), e = 1 - x r: the relative error goes from e to e^3 (the
// seed's e is below 2^-19.9 over the normal range, so e^3 is below 2^-59),
// three FP64 instructions where two Newton steps take four.  Within an ulp of
// the correctly rounded 1/x (2^28 random normal x: 0.03% one ulp off, none
// more); callers guarantee a normal, finite argument.
__device__ __forceinline__ double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
// biased exponent of a double, on the integer pipe
__device__ __forceinline__ int dexp(double x) { return (__double2hiint(x) >> 20) & 0x7ff; }

// 1/x for the production build (IEEE division in the exact build); falls back
// to the division when x is outside the normal range the Newton form handles.
__device__ __forceinline__ double rcp_p(double x) {
#ifdef PHX_EXACT
  return 1.0 / x;
#else
  const int e = dexp(x);
  return (e >= 16 && e <= 2030) ? rcp_nr(x) : 1.0 / x;
#endif
}
// a / b: IEEE division in the exact build, a * rcp_p(b) in the production build
__device__ __forceinline__ double div_p(double a, double b) {
#ifdef PHX_EXACT
  return a / b;
#else
  return a * rcp_p(b);
#endif
}
// 1/sqrt(x) from the hardware seed y and one third-order step: with
// h = 1 - x y^2, (1 - h)^(-1/2) = 1 + h/2 + 3h^2/8 + O(h^3), so
// y (1 + h (1/2 + 3h/8)) cuts the relative error from h/2 (the seed's, below
// 2^-20) to about 5h^3/16 (normal, finite x > 0); five FP64 instructions where
// two Newton steps take eight.  Within two ulps of 1.0 / sqrt(x) over 2^28
// random normal x.  The production build's replacement for 1 / sqrt(x); the
// exact build divides.
__device__ __forceinline__ double rsqrt_nr(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double h = fma(-(x * y), y, 1.0);
  return fma(y * h, fma(0.375, h, 0.5), y);
}
__device__ __forceinline__ double rsqrt_p(double x) {
#ifdef PHX_EXACT
  return 1.0 / sqrt(x);
#else
  const int e = dexp(x);
  return (e >= 16 && e <= 2030) ? rsqrt_nr(x) : 1.0 / sqrt(x);
#endif
}
// robust::ratio with the production-build reciprocal
__device__ __forceinline__ double ratio_p(double a, double b) {
#ifdef PHX_EXACT
  return ratio(a, b);
#else
  const double sgn = b >= 0 ? 1.0 : -1.0;
  return a * rcp_p(b + sgn * kSMALL);
#endif
}

// ---------------------------------------------------------- parameters
// Device copy of the fluid / fixup / eos params (phx_params), with the
// fixup package's defaults already resolved (fixup.cpp:120-180).
// Reconstructed variables the flux kernels read from memory.  The exact
// build reconstructs all PHX_NRECON, as the reference does
// (fluid.cpp:272-286).  Under the ideal gas gamma1 = bulk modulus / P is the
// constant Gamma (every zone's stored value is Gamma to a few ulps), so the
// production build reconstructs the first PHX_NRECON - 1 and gives both face
// states gamma1 = Gamma (recon_gamma1): one variable fewer staged, held in
// registers and reconstructed per cell and direction.
#ifdef PHX_EXACT
constexpr int kReconLoad = PHX_NRECON;
#else
constexpr int kReconLoad = PHX_NRECON - 1;
static_assert(PHX_PGM1 == PHX_NRECON - 1, "gamma1 is the last reconstructed variable");
#endif

struct Par {
  double gm1, Cv;
  double rho_min_eos, sie_min_eos;
  double c2p_tol;
  int c2p_max_iter;
  double fsf;  // c2p_floor_scale_fac
  int fail_on_floors, fail_on_ceilings;
  int mhd;
  int floor_type;
  double r0, s0, ralpha, salpha;
  double g0, smax0;
  double bsqorho0, bsqou0;
  int recon, riemann;
  double cfl;
  int c2p_fixup, strategy_floors, enable_floors, enable_mhd_floors;
  double vsq_max;  // 1 - 1 / g0^2 (the gamma ceiling as a v^2 bound)
  double iCv;      // 1 / Cv, formed on the host (production-build temperature)
  int fix_flux;      // fixup/enable_flux_fixup
  int inflow_check;  // fixup/enable_ox1_fmks_inflow_check
};

// Face states of gamma1 where the production build does not reconstruct it.
__device__ __forceinline__ void recon_gamma1(const Par &p, double *ql, double *qr) {
  if constexpr (kReconLoad < PHX_NRECON) {
    ql[PHX_PGM1] = p.gm1 + 1.0;
    qr[PHX_PGM1] = p.gm1 + 1.0;
  }
}

// ------------------------------------------------ singularity-eos IdealGas
__device__ __forceinline__ double eos_P_rho_sie(const Par &p, double rho, double sie) {
  return fmax(0.0, p.gm1 * rho * sie);
}
__device__ __forceinline__ double eos_T_rho_sie(const Par &p, double rho, double sie) {
#ifdef PHX_EXACT
  return fmax(0.0, div_p(sie, p.Cv));
#else
  return fmax(0.0, sie * p.iCv);  // production build: the host's 1/Cv
#endif
}
__device__ __forceinline__ double eos_P_rho_T(const Par &p, double rho, double T) {
  return fmax(0.0, p.gm1 * rho * p.Cv * T);
}
__device__ __forceinline__ double eos_bmod_rho_T(const Par &p, double rho, double T) {
  return fmax(0.0, (p.gm1 + 1) * p.gm1 * rho * p.Cv * T);
}
__device__ __forceinline__ double eos_bmod_rho_sie(const Par &p, double rho, double sie) {
  return fmax(0.0, p.gm1 * (p.gm1 + 1) * rho * sie);
}

// ------------------------------------------------------- fixup.hpp Bounds
// Bounds::GetFloors in two parts.  floor_point holds what depends on the
// position only (for ExpX1RhoSie two exponentials); floors_from finishes
// the floors from it and the density passed in (only ExpX1RhoU's sie floor
// depends on that density).  A zone's con2prim evaluates its floors at every
// residual and both states of a face at the face's position, so they compute
// floor_point once and reuse it: the same values as get_floors, bit for bit.
struct FloorPt {
  double r, s;
};
__device__ __forceinline__ FloorPt floor_point(const Par &p, double x1, double x2, double x3) {
  FloorPt f;
  switch (p.floor_type) {
  case PHX_FLOOR_CONSTANT_RHO_SIE:
    f.r = p.r0;
    f.s = p.s0;
    break;
  case PHX_FLOOR_EXPX1_RHO_SIE:
  case PHX_FLOOR_EXPX1_RHO_U:  // s: the sie floor's numerator
    f.r = p.r0 * phx_math::exp(p.ralpha * x1);
    f.s = p.s0 * phx_math::exp(p.salpha * x1);
    break;
  case PHX_FLOOR_X1_RHO_SIE:
    f.r = p.r0 * fmin(1.0, phx_math::pow(x1, p.ralpha));
    f.s = p.s0 * fmin(1.0, phx_math::pow(x1, p.salpha));
    break;
  default: {
    double r = sqrt(x1 * x1 + x2 * x2 + x3 * x3);
    f.r = p.r0 * fmin(1.0, phx_math::pow(r, p.ralpha));
    f.s = p.s0 * fmin(1.0, phx_math::pow(r, p.salpha));
  } break;
  }
  return f;
}
// True when the floors depend on X1 alone (all types but RRhoSie).
__device__ __forceinline__ bool floors_x1_only(const Par &p) { return p.floor_type != PHX_FLOOR_R_RHO_SIE; }
__device__ __forceinline__ void floors_from(const Par &p, const FloorPt &f, double &rflr, double &sflr) {
  if (p.floor_type == PHX_FLOOR_EXPX1_RHO_U) {
    sflr = f.s / rmax(rflr, f.r);
  } else {
    sflr = f.s;
  }
  rflr = f.r;
  rflr = rmax(rflr, p.rho_min_eos);
  sflr = rmax(sflr, p.sie_min_eos);
}
__device__ __forceinline__ void get_floors(const Par &p, double x1, double x2, double x3,
                                           double &rflr, double &sflr) {
  floors_from(p, floor_point(p, x1, x2, x3), rflr, sflr);
}

// ------------------------------------------------------------ block view
struct BView {
  int n1t, n2t, n3t, ndim, ng, nx1, nx2, nx3;
  long long vs;
  double x0[3], dx[3];
  double *prim, *cons, *flux, *face_sig, *cell_sig, *fail, *src, *emf, *dudt;
  const double *gcent, *gface1, *gface2, *gderiv;
  int fmks;
  __device__ __forceinline__ long long idx(int k, int j, int i) const {
    return ((long long)k * n2t + j) * n1t + i;
  }
  __device__ __forceinline__ double Xc(int d, int ix) const { return x0[d] + (ix + 0.5) * dx[d]; }
  __device__ __forceinline__ double Xf(int d, int ix) const { return x0[d] + ix * dx[d]; }
  __device__ __forceinline__ int is() const { return ng; }
  __device__ __forceinline__ int ie() const { return ng + nx1 - 1; }
  __device__ __forceinline__ int js() const { return ndim >= 2 ? ng : 0; }
  __device__ __forceinline__ int je() const { return ndim >= 2 ? ng + nx2 - 1 : 0; }
  __device__ __forceinline__ int ks() const { return ndim >= 3 ? ng : 0; }
  __device__ __forceinline__ int ke() const { return ndim >= 3 ? ng + nx3 - 1 : 0; }
};

// ------------------------------------------------------------- geometry
// Point geometry (values at a cell centre or a face).
struct Pt {
  double alpha, beta[3], gcov[4][4], gamcon[3][3], detgam;
};

__device__ __forceinline__ int flat2(int m, int n) {
  // Flatten2 (geometry_utils.hpp:180-185): symmetric 4x4 packing
  const int lo = m < n ? m : n, hi = m < n ? n : m;
  return hi * (hi + 1) / 2 + lo;
}

// loc: 0 = centre (and X3 face), 1 = X1 face, 2 = X2 face
__device__ __forceinline__ void load_pt(const BView &b, int loc, int j, int i, Pt &p) {
  const double *t;
  long long pitch, off;
  if (loc == 1) {
    t = b.gface1;
    pitch = (long long)b.n2t * (b.n1t + 1);
    off = (long long)j * (b.n1t + 1) + i;
  } else if (loc == 2) {
    t = b.gface2;
    pitch = (long long)(b.n2t + 1) * b.n1t;
    off = (long long)j * b.n1t + i;
  } else {
    t = b.gcent;
    pitch = (long long)b.n2t * b.n1t;
    off = (long long)j * b.n1t + i;
  }
  p.alpha = __ldg(t + PHX_G_ALPHA * pitch + off);
#pragma unroll
  for (int d = 0; d < 3; d++) p.beta[d] = __ldg(t + (PHX_G_BETA + d) * pitch + off);
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int n = 0; n < 4; n++) p.gcov[m][n] = __ldg(t + (PHX_G_GCOV + flat2(m, n)) * pitch + off);
#pragma unroll
  for (int m = 0; m < 3; m++)
#pragma unroll
    for (int n = 0; n < 3; n++) p.gamcon[m][n] = __ldg(t + (PHX_G_GAMCON + flat2(m, n)) * pitch + off);
  p.detgam = __ldg(t + PHX_G_DETGAM * pitch + off);
}

// Point geometry of zone q from a [PHX_GEOM_NLOC][pitch] table.
__device__ __forceinline__ void load_pt_flat(const double *t, long long pitch, long long q, Pt &p) {
  p.alpha = __ldg(t + PHX_G_ALPHA * pitch + q);
#pragma unroll
  for (int d = 0; d < 3; d++) p.beta[d] = __ldg(t + (PHX_G_BETA + d) * pitch + q);
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int n = 0; n < 4; n++) p.gcov[m][n] = __ldg(t + (PHX_G_GCOV + flat2(m, n)) * pitch + q);
#pragma unroll
  for (int m = 0; m < 3; m++)
#pragma unroll
    for (int n = 0; n < 3; n++) p.gamcon[m][n] = __ldg(t + (PHX_G_GAMCON + flat2(m, n)) * pitch + q);
  p.detgam = __ldg(t + PHX_G_DETGAM * pitch + q);
}

// a_m = gamma_mn a^n (the spatial metric lowers a vector).
__device__ __forceinline__ void lower_sp(const Pt &g, const double a[3], double out[3]) {
#pragma unroll
  for (int m = 0; m < 3; m++) out[m] = g.gcov[m + 1][1] * a[0] + g.gcov[m + 1][2] * a[1] + g.gcov[m + 1][3] * a[2];
}
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// sum_{m,n} gcov[m+1][n+1] a[m] b[n]: the reference's nine-term loop in the
// exact build; a . (gamma b) in the production build (12 FP64 instructions
// instead of 18).
template <bool MINK>
__device__ __forceinline__ double dot_sp(const Pt &g, const double a[3], const double b[3]) {
  if constexpr (MINK) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  } else {
#ifdef PHX_EXACT
    double s = 0.0;
#pragma unroll
    for (int m = 0; m < 3; m++)
#pragma unroll
      for (int n = 0; n < 3; n++) s += g.gcov[m + 1][n + 1] * a[m] * b[n];
    return s;
#else
    double bl[3];
    lower_sp(g, b, bl);
    return dot3(a, bl);
#endif
  }
}

// ------------------------------------------------- relativity_utils.hpp
template <bool MINK>
__device__ __forceinline__ double lorentz(const Pt &g, const double v[3]) {
  return sqrt(1. + dot_sp<MINK>(g, v, v));
}

// The outer-X1 inflow check of one ghost zone (ConvertBoundaryConditions,
// phoebus_boundaries.cpp:366-397): where u^1 = v^1 - W beta^1 / alpha < 0,
// the three-velocity v / W keeps its X2 and X3 components, takes
// beta^1 / alpha along X1, and is turned back into W v.  v: W v^i in place.
__device__ __forceinline__ void ox1_inflow_fix(const Pt &gm, double v[3]) {
  double W = lorentz<false>(gm, v);
  const double ucon1 = v[0] - W * gm.beta[0] / gm.alpha;
  if (ucon1 < 0) {
    double vcon[3] = {v[0] / W, v[1] / W, v[2] / W};
    vcon[0] = gm.beta[0] / gm.alpha;
    const double vsq = dot_sp<false>(gm, vcon, vcon);
    W = 1. / sqrt(1. - vsq);
    for (int d = 0; d < 3; d++) v[d] = W * vcon[d];
  }
}

// ---------------------------------------------------------- prim2con.hpp
// signal_speeds (prim2con.hpp:24-46); ndim entries written.
template <bool MINK>
__device__ __forceinline__ void signal_speeds(double rho, double u, double p, double bsq,
                                              const double v[3], double vsq, double gam1,
                                              const Pt &g, double *sig) {
  const double rho_rel = rho + u + p;
#ifdef PHX_EXACT
  const double vasq = div_p(bsq, rho_rel + bsq);
  double cssq = div_p(gam1 * p, rho_rel);
#else
  // production build: one reciprocal of the product of the two denominators
  // where it is normal
  double vasq, cssq;
  const double dAB = (rho_rel + bsq) * rho_rel;
  const int eAB = dexp(dAB);
  if (eAB >= 16 && eAB <= 2030) {
    const double rAB = rcp_nr(dAB);
    vasq = bsq * (rho_rel * rAB);
    cssq = gam1 * p * ((rho_rel + bsq) * rAB);
  } else {
    vasq = div_p(bsq, rho_rel + bsq);
    cssq = div_p(gam1 * p, rho_rel);
  }
#endif
  cssq += vasq - cssq * vasq;
  const double alpha = MINK ? 1.0 : g.alpha;
  const double vcoff = div_p(alpha, 1.0 - vsq * cssq);
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const double gmm = MINK ? 1.0 : g.gamcon[m][m];
#ifdef PHX_EXACT
    const double vpm = sqrt(cssq * (1.0 - vsq) * (gmm * (1.0 - vsq * cssq) - v[m] * v[m] * (1.0 - cssq)));
#else
    // production build: sqrt(x) as x rsqrt(x) for normal x > 0 (zero, negative
    // and extreme arguments take the IEEE square root)
    const double vpm_sq = cssq * (1.0 - vsq) * (gmm * (1.0 - vsq * cssq) - v[m] * v[m] * (1.0 - cssq));
    const int ev = dexp(vpm_sq);
    const double vpm = (vpm_sq > 0.0 && ev >= 16 && ev <= 2030) ? vpm_sq * rsqrt_nr(vpm_sq) : sqrt(vpm_sq);
#endif
    double vp = vcoff * (v[m] * (1.0 - cssq) + vpm);
    double vm = vcoff * (v[m] * (1.0 - cssq) - vpm);
    if constexpr (!MINK) {
      vp -= g.beta[m];
      vm -= g.beta[m];
    }
    sig[m] = rmax(fabs(vp), fabs(vm));
  }
}

// p2c (prim2con.hpp:48-102)
template <bool MINK>
__device__ __forceinline__ void p2c(double rho, const double vp[3], const double b[3], double u,
                                    double p, double gam1, const Pt &g, double gdet, double &D,
                                    double S[3], double bcons[3], double &tau, double *sig) {
  const double W = lorentz<MINK>(g, vp);
  const double iW = rcp_p(W);
  double v[3] = {vp[0] * iW, vp[1] * iW, vp[2] * iW};
  double vsq, Bsq, Bdotv;
  if constexpr (MINK) {
    // the reference accumulates the three sums interleaved; each is independent
    vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    Bsq = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    Bdotv = b[0] * v[0] + b[1] * v[1] + b[2] * v[2];
  } else {
    vsq = 0.0;
    Bsq = 0.0;
    Bdotv = 0.0;
#pragma unroll
    for (int ii = 0; ii < 3; ii++)
#pragma unroll
      for (int jj = 0; jj < 3; jj++) {
        vsq += g.gcov[ii + 1][jj + 1] * v[ii] * v[jj];
        Bsq += g.gcov[ii + 1][jj + 1] * b[ii] * b[jj];
        Bdotv += g.gcov[ii + 1][jj + 1] * b[ii] * v[jj];
      }
  }
  const double b0 = W * Bdotv;
  const double alpha = MINK ? 1.0 : g.alpha;
  double bcon[4];
  bcon[0] = W * Bdotv / alpha;
#pragma unroll
  for (int m = 0; m < 3; m++) {
    if constexpr (MINK)
      bcon[m + 1] = b[m] * iW + Bdotv * W * v[m];
    else
      bcon[m + 1] = b[m] * iW + Bdotv * W * (v[m] - g.beta[m] / alpha);
  }
  const double bsq = Bsq * iW * iW + Bdotv * Bdotv;
  double bcov[3];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    if constexpr (MINK) {
      bcov[m] = bcon[m + 1];
    } else {
      bcov[m] = 0.0;
#pragma unroll
      for (int n = 0; n < 4; n++) bcov[m] += g.gcov[m + 1][n] * bcon[n];
    }
  }
  D = gdet * rho * W;
  const double rho_rel = (rho + u + p + bsq) * W * W;
#pragma unroll
  for (int m = 0; m < 3; m++) {
    double vcov;
    if constexpr (MINK) {
      vcov = v[m];
    } else {
      vcov = 0.0;
#pragma unroll
      for (int n = 0; n < 3; n++) vcov += g.gcov[m + 1][n + 1] * v[n];
    }
    S[m] = gdet * (rho_rel * vcov - b0 * bcov[m]);
    bcons[m] = gdet * b[m];
  }
  tau = gdet * (rho_rel - (p + 0.5 * bsq) - b0 * b0) - D;
  if (sig != nullptr) signal_speeds<MINK>(rho, u, p, bsq, v, vsq, gam1, g, sig);
}

// -------------------------------------------------- reconstruction.hpp
__device__ __forceinline__ double mc(double dm, double dp, double alpha) {
#ifdef PHX_EXACT
  const double dc = (dm * dp > 0.0) * 0.5 * (dm + dp);
#else
  // a select instead of the product with the converted comparison: two fewer
  // FP64 instructions; only the sign of a zero slope can differ
  const double dc = dm * dp > 0.0 ? 0.5 * (dm + dp) : 0.0;
#endif
#ifdef PHX_EXACT
  // std::min (reconstruction.hpp:106): a NaN slope propagates, as fmin would not
  const double m1 = (fabs(dp) < fabs(dm)) ? fabs(dp) : fabs(dm);
  const double m2 = alpha * m1;
  return copysign((m2 < fabs(dc)) ? m2 : fabs(dc), dc);
#else
  return copysign(fmin(fabs(dc), alpha * fmin(fabs(dm), fabs(dp))), dc);
#endif
}
__device__ __forceinline__ void recon_plm(double qm, double q0, double qp, double &ql, double &qr) {
  double dq = qp - q0;
  dq = mc(q0 - qm, dq, 1.5);
  ql = q0 + 0.5 * dq;
  qr = q0 - 0.5 * dq;
}
__device__ __forceinline__ void recon_weno5z(double q0, double q1, double q2, double q3, double q4,
                                             double &ql, double &qr) {
  constexpr double a00 = 1.0 / 3.0, a01 = -7.0 / 6.0, a02 = 11.0 / 6.0;
  constexpr double a10 = -1.0 / 6.0, a11 = 5.0 / 6.0, a12 = 1.0 / 3.0;
  constexpr double a20 = 1.0 / 3.0, a21 = 5.0 / 6.0, a22 = -1.0 / 6.0;
  constexpr double g0 = 0.1, g1 = 0.6, g2 = 0.3;
  constexpr double eps = 1e-100;
  constexpr double t13 = 13.0 / 3.0;
  double a = q0 - 2 * q1 + q2;
  double b = q0 - 4.0 * q1 + 3.0 * q2;
  double beta0 = t13 * a * a + b * b + eps;
  a = q1 - 2.0 * q2 + q3;
  b = q3 - q1;
  double beta1 = t13 * a * a + b * b + eps;
  a = q2 - 2.0 * q3 + q4;
  b = q4 - 4.0 * q3 + 3.0 * q2;
  double beta2 = t13 * a * a + b * b + eps;
  const double tau5 = fabs(beta2 - beta0);
  beta0 = (beta0 + tau5) / beta0;
  beta1 = (beta1 + tau5) / beta1;
  beta2 = (beta2 + tau5) / beta2;
  double w0 = g0 * beta0 + eps;
  double w1 = g1 * beta1 + eps;
  double w2 = g2 * beta2 + eps;
  double wsum = 1.0 / (w0 + w1 + w2);
  ql = w0 * (a00 * q0 + a01 * q1 + a02 * q2);
  ql += w1 * (a10 * q1 + a11 * q2 + a12 * q3);
  ql += w2 * (a20 * q2 + a21 * q3 + a22 * q4);
  ql *= wsum;
  const double alpha_l = 3.0 * wsum * w0 * w1 * w2 / (g2 * w0 * w1 + g1 * w0 * w2 + g0 * w1 * w2) + eps;
  w0 = g0 * beta2 + eps;
  w1 = g1 * beta1 + eps;
  w2 = g2 * beta0 + eps;
  wsum = 1.0 / (w0 + w1 + w2);
  qr = w0 * (a00 * q4 + a01 * q3 + a02 * q2);
  qr += w1 * (a10 * q3 + a11 * q2 + a12 * q1);
  qr += w2 * (a20 * q2 + a21 * q1 + a22 * q0);
  qr *= wsum;
  const double alpha_r = 3.0 * wsum * w0 * w1 * w2 / (g2 * w0 * w1 + g1 * w0 * w2 + g0 * w1 * w2) + eps;
  double dq = q3 - q2;
  dq = mc(q2 - q1, dq, 2.0);
  const double alpha_lin = 2.0 * alpha_l * alpha_r / (alpha_l + alpha_r);
  ql = alpha_lin * ql + (1.0 - alpha_lin) * (q2 + 0.5 * dq);
  qr = alpha_lin * qr + (1.0 - alpha_lin) * (q2 - 0.5 * dq);
}
// ---- production-build WENO5-Z: same mathematics, fewer FP64 instructions.
// WENO5-Z as reconstruction.hpp:127-183, rearranged.
//  - The nonlinear weights are gamma_k bp_k, bp_k = 1 + tau5 / beta_k,
//    normalised by their sums S_l, S_r; the three 1/beta_k come from one
//    reciprocal of beta0 beta1 beta2.  (The reference's + eps on a weight is
//    below half an ulp of gamma_k bp_k >= 0.1 and drops out.)
//  - The blend factor: with normalised weights w_k = gamma_k bp_k / S,
//    alpha = 3 w0 w1 w2 / (g2 w0 w1 + g1 w0 w2 + g0 w1 w2) = 3 / (S R) with
//    R = sum_k 1/bp_k, the same for both faces, so the harmonic mean
//    alpha_lin = 2 alpha_l alpha_r / (alpha_l + alpha_r) = 6 / (R (S_l + S_r)).
//    1/bp_k = beta_k / (beta_k + tau5): with M the larger of beta0, beta2 and
//    m the smaller, beta_m + tau5 = beta_M, so 1/bp_m = beta_m / beta_M from
//    the reciprocal above, and 1/bp_M, 1/bp_1 share one reciprocal of
//    (2 beta_M - beta_m)(beta1 + tau5).  (The reference's + eps on alpha_l,
//    alpha_r moves alpha_lin only where alpha_lin < 1e-90.)  alpha_lin and
//    the weights' normalisations 1 / S_l, 1 / S_r come from one reciprocal of
//    R (S_l + S_r) S_l S_r.
//  - The MC slope of the blend, mc(q2 - q1, q3 - q2, 2), doubled, on the
//    integer pipe: the sign test, the minima of magnitudes and the power-of-two
//    scale act on the bit patterns; the sum dm + dp is the slope b1 = q3 - q1
//    the smoothness indicator already forms.
// Three reciprocals (three FP64 instructions each) and about 90 FP64
// instructions for both face states.  Every intermediate stays in the normal
// range for |q| < 1e50; outside it (checked on the exponents) the reference
// sequence is used.
__device__ __forceinline__ void recon_weno5z_fast(double q0, double q1, double q2, double q3, double q4,
                                                  double &ql, double &qr) {
  constexpr double g0 = 0.1, g1 = 0.6, g2 = 0.3;
  constexpr double eps = 1e-100;
  constexpr double t13 = 13.0 / 3.0;
  // second differences a_k and one-sided slopes b_k of the three stencils;
  // beta_k = 13/3 a_k^2 + b_k^2 + eps with eps folded into the b^2 product.
  // These keep the reference's operation order: in near-flat regions the
  // weights follow the rounding of a_k and b_k (differences of nearly equal
  // indicators), and forming them from first differences instead moved
  // signal speeds of a 256^3 shear layer 1.7e-12 away from the reference's.
  const double a0 = q0 - 2 * q1 + q2, b0 = q0 - 4.0 * q1 + 3.0 * q2;
  const double a1 = q1 - 2.0 * q2 + q3, b1 = q3 - q1;
  const double a2 = q2 - 2.0 * q3 + q4, b2 = q4 - 4.0 * q3 + 3.0 * q2;
  const double beta0 = fma(t13 * a0, a0, fma(b0, b0, eps));
  const double beta1 = fma(t13 * a1, a1, fma(b1, b1, eps));
  const double beta2 = fma(t13 * a2, a2, fma(b2, b2, eps));
  const double d20 = beta2 - beta0;
  const double tau5 = fabs(d20);
  const double b01 = beta0 * beta1;
  const double prod = b01 * beta2;
  const int ep = dexp(prod);
  if (ep < 16 || ep > 2030) {  // outside [~1e-303, ~1e303]: reference sequence
    recon_weno5z(q0, q1, q2, q3, q4, ql, qr);
    return;
  }
  const double rp = rcp_nr(prod);
  const double t = beta2 * rp;
  const double ib0 = beta1 * t, ib2 = b01 * rp;  // 1/beta0, 1/beta2
  const double bp0 = fma(tau5, ib0, 1.0);
  const double bp1 = fma(tau5, beta0 * t, 1.0);
  const double bp2 = fma(tau5, ib2, 1.0);
  const bool big2 = __double2hiint(d20) >= 0;  // beta2 >= beta0
  const double bM = big2 ? beta2 : beta0, bm = big2 ? beta0 : beta2;
  const double X1 = fma(2.0, bM, -bm), Y1 = beta1 + tau5;
  const double X = X1 * Y1;
  const double wl0 = g0 * bp0, wl1 = g1 * bp1, wl2 = g2 * bp2;
  const double wr0 = g0 * bp2, wr2 = g2 * bp0;
  const double Sl = wl0 + wl1 + wl2, Sr = wr0 + wl1 + wr2;
  const double SS = Sl * Sr, S2 = Sl + Sr;
  const int ex = dexp(X), eSS = dexp(SS), eS2 = dexp(S2);
  // R in [1/2, 3] and S_l, S_r >= 1: R S2 SS lies in [1, 2^1021) below the sum bound
  if (ex < 16 || ex > 2030 || eSS > 2030 || eS2 > 2027 || eSS + eS2 > 3060) {
    recon_weno5z(q0, q1, q2, q3, q4, ql, qr);
    return;
  }
  const double rx = rcp_nr(X);
  const double R = fma(bm, big2 ? ib2 : ib0, fma(bM, Y1 * rx, beta1 * (X1 * rx)));
  // one reciprocal Z = 1 / (R S2 S_l S_r) gives alpha_lin / 4 = 1.5 S_l S_r Z and
  // the candidates' normalisation with the blend factor folded in:
  // alpha_lin / (12 S_l) = S_r Z / 2, alpha_lin / (12 S_r) = S_l Z / 2
  const double Z = rcp_nr(R * S2 * SS);
  const double aq = (1.5 * SS) * Z;  // alpha_lin / 4
  const double hZ = 0.5 * Z;
  const double zl = hZ * Sr, zr = hZ * Sl;
  // 2 mc(q2 - q1, q3 - q2, 2) = copysign(min(|dm + dp|, 4 min(|dm|, |dp|)),
  // dm + dp) where dm dp > 0, else 0 (finite dm, dp: |q| < 1e50 here)
  const long long MAG = 0x7fffffffffffffffLL;
  const long long idm = __double_as_longlong(q2 - q1), idp = __double_as_longlong(q3 - q2);
  const long long isum = __double_as_longlong(b1);
  const long long adm = idm & MAG, adp = idp & MAG, asum = isum & MAG;
  const bool same = ((idm ^ idp) >= 0) && adm != 0 && adp != 0;
  const long long a4 = (adm < adp ? adm : adp) + (2LL << 52);
  const double dq2 = same ? __longlong_as_double((asum < a4 ? asum : a4) | (isum & ~MAG)) : 0.0;
  // candidate values as q2 plus a twelfth of a_k +- 3 b_k: for ql (upper
  // face) (a0 + 3 b0), (a1 + 3 b1), (a2 - 3 b2); for qr (lower face, the
  // mirrored stencils) (a2 + 3 b2), (a1 - 3 b1), (a0 - 3 b0); the weights sum
  // to one, so sum_k w_k c_k = q2 + sum_k w_k (c_k - q2).  Then the blend
  // alpha q + (1 - alpha) p with p = q2 +- dq2 / 4 as p -+ (alpha / 4) dq2 +
  // alpha (q - q2), alpha (q - q2) = (sum_k w_k (a_k +- 3 b_k)) alpha / (12 S).
  const double sl = wl0 * fma(3.0, b0, a0) + wl1 * fma(3.0, b1, a1) + wl2 * fma(-3.0, b2, a2);
  const double sr = wr0 * fma(3.0, b2, a2) + wl1 * fma(-3.0, b1, a1) + wr2 * fma(-3.0, b0, a0);
  ql = fma(sl, zl, fma(-aq, dq2, fma(0.25, dq2, q2)));
  qr = fma(sr, zr, fma(aq, dq2, fma(-0.25, dq2, q2)));
}

__device__ __forceinline__ double minmod(double a, double b) {
  return a * b > 0.0 ? (fabs(a) < fabs(b) ? a : b) : 0.0;
}
// MP5 value at the face j+1/2 from f_{j-2} .. f_{j+2}: the monotonicity-
// preserving fifth-order scheme of Suresh & Huynh (1997, J. Comput. Phys.
// 136, 83-99; alpha = 4, eps = 1e-12).  The fifth-order interface value is
// kept when it lies between f_j and the monotonicity bound f_MP; otherwise
// it is clipped to [f_min, f_max], built from the minmod4-limited
// curvatures at j+1/2 and j-1/2 and the upper-limit (UL), average (AV),
// median (MD) and large-curvature (LC) values.  The operations are in the
// order of the reference (reconstruction.hpp:186-244), which bitwise parity
// needs; minmod4(a, b, c, d) is minmod(minmod(a, b), minmod(c, d)).
__device__ __forceinline__ double mp5_face(double fm2, double fm1, double f0, double fp1, double fp2) {
  constexpr double alpha = 4.0, eps = 1.e-12;
  double f = 2.0 * fm2 - 13.0 * fm1 + 47.0 * f0 + 27.0 * fp1 - 3.0 * fp2;
#ifdef PHX_EXACT
  f /= 60.0;
#else
  f *= 1.0 / 60.0;  // a product instead of the IEEE division (an ulp apart)
#endif
  const double f_mp = f0 + minmod(fp1 - f0, alpha * (f0 - fm1));
  if ((f - f0) * (f - f_mp) <= eps) return f;
  const double curv_m = fm2 + f0 - 2.0 * fm1;  // second differences at j-1, j, j+1
  const double curv_0 = fm1 + fp1 - 2.0 * f0;
  const double curv_p = f0 + fp2 - 2.0 * fp1;
  const double m4_plus = minmod(minmod(4.0 * curv_0 - curv_p, 4.0 * curv_p - curv_0), minmod(curv_0, curv_p));
  const double m4_minus = minmod(minmod(4.0 * curv_m - curv_0, 4.0 * curv_0 - curv_m), minmod(curv_0, curv_m));
  const double f_ul = f0 + alpha * (f0 - fm1);
  const double f_av = 0.5 * (f0 + fp1);
  const double f_md = f_av - 0.5 * m4_plus;
  const double f_lc = 0.5 * (3.0 * f0 - fm1) + 4.0 / 3.0 * m4_minus;
  const double f_min = fmax(fmin(fmin(f0, fp1), f_md), fmin(fmin(f0, f_ul), f_lc));
  const double f_max = fmin(fmax(fmax(f0, fp1), f_md), fmax(fmax(f0, f_ul), f_lc));
  return f + minmod(f_min - f, f_max - f);  // the median of f, f_min, f_max
}

// 5-point (or 3-point) reconstruction of one variable.  ql = value at the
// upper face of the cell, qr = value at its lower face.
template <int RECON>
__device__ __forceinline__ void recon(double qm2, double qm1, double q0, double qp1, double qp2,
                                      double &ql, double &qr) {
  if constexpr (RECON == PHX_RECON_WENO5Z) {
#ifdef PHX_EXACT
    recon_weno5z(qm2, qm1, q0, qp1, qp2, ql, qr);
#else
    recon_weno5z_fast(qm2, qm1, q0, qp1, qp2, ql, qr);
#endif
  } else if constexpr (RECON == PHX_RECON_MP5) {
    ql = mp5_face(qm2, qm1, q0, qp1, qp2);
    qr = mp5_face(qp2, qp1, q0, qm1, qm2);
  } else if constexpr (RECON == PHX_RECON_LINEAR) {
    recon_plm(qm1, q0, qp1, ql, qr);
  } else {
    ql = q0;
    qr = q0;
  }
}

// ------------------------------------------------------- riemann.hpp
struct Face {
  Pt g;          // face geometry (unused for Minkowski)
  double gdet;   // DetG: 1 for Minkowski, alpha * detgam from the cache
  double gammadet;
  double gdd;
  FloorPt fl;    // floor_point at the face, shared by its two states
};

// prim_to_flux (riemann.hpp:88-209) for face direction DIR (0-based).
template <bool MINK, int DIR>
__device__ __forceinline__ void prim_to_flux(const Par &par, const Face &f, const double q[PHX_NRECON],
                                             double &vm, double &vp, double U[PHX_NCONS],
                                             double F[PHX_NCONS], double sie_max, double gam_max) {
  const Pt &g = f.g;
  double rho_floor = q[PHX_PRHO];
  double sie_floor;
  floors_from(par, f.fl, rho_floor, sie_floor);
  const double rho = rmax(q[PHX_PRHO], rho_floor);
  double vpcon[3] = {q[PHX_PVEL], q[PHX_PVEL + 1], q[PHX_PVEL + 2]};
#ifdef PHX_EXACT
  double W = lorentz<MINK>(g, vpcon);
#else
  const double Wsq0 = 1. + dot_sp<MINK>(g, vpcon, vpcon);
  const double iW0 = rsqrt_p(Wsq0);
  double W = Wsq0 * iW0;
#endif
#ifndef PHX_EXACT
  bool capped = false;  // a velocity cap changed v: W is formed again below
#endif
  if (W > gam_max) {
    const double rescale = sqrt((gam_max * gam_max - 1.) / (W * W - 1.));
#pragma unroll
    for (int ii = 0; ii < 3; ii++) vpcon[ii] *= rescale;
#ifndef PHX_EXACT
    capped = true;
#endif
  }
  const double qe = q[PHX_PENG];
#ifdef PHX_EXACT
  double vcon[3] = {vpcon[0] / W, vpcon[1] / W, vpcon[2] / W};
  const double sie_q = q[PHX_PENG] / rho;
  const bool above_floor = sie_q > sie_floor, above_max = sie_q > sie_max;
#else
  double vcon[3] = {vpcon[0] * iW0, vpcon[1] * iW0, vpcon[2] * iW0};
  // u / rho > s as u > rho s for rho > 0 (no reciprocal; the products are the
  // bounded energies anyway); the quotient only where rho <= 0
  bool above_floor, above_max;
  if (rho > 0.0) {
    above_floor = qe > rho * sie_floor;
    above_max = qe > rho * sie_max;
  } else {
    const double sie_q = qe * rcp_p(rho);
    above_floor = sie_q > sie_floor;
    above_max = sie_q > sie_max;
  }
#endif
  double Bcon[3] = {0.0, 0.0, 0.0};
  const double u = (above_floor ? (above_max ? rho * sie_max : qe) : rho * sie_floor);
  const double P = rmax(q[PHX_PPRS], 0.0);
  const double gamma1 = q[PHX_PGM1];
  if (par.mhd) {
    Bcon[0] = q[PHX_PB];
    Bcon[1] = q[PHX_PB + 1];
    Bcon[2] = q[PHX_PB + 2];
  }
  double vsq, Bdotv, BdotB;
  if constexpr (MINK) {
    vsq = vcon[0] * vcon[0] + vcon[1] * vcon[1] + vcon[2] * vcon[2];
    Bdotv = Bcon[0] * vcon[0] + Bcon[1] * vcon[1] + Bcon[2] * vcon[2];
    BdotB = Bcon[0] * Bcon[0] + Bcon[1] * Bcon[1] + Bcon[2] * Bcon[2];
  } else {
    vsq = 0.0;
    Bdotv = 0.0;
    BdotB = 0.0;
#ifdef PHX_EXACT
#pragma unroll
    for (int m = 0; m < 3; m++)
#pragma unroll
      for (int n = 0; n < 3; n++) {
        vsq += g.gcov[m + 1][n + 1] * vcon[m] * vcon[n];
        Bdotv += g.gcov[m + 1][n + 1] * Bcon[m] * vcon[n];
        BdotB += g.gcov[m + 1][n + 1] * Bcon[m] * Bcon[n];
      }
#endif
  }
#ifndef PHX_EXACT
  // production build: the lowered v and B serve the three contractions here
  // and the covariant momentum / field terms below
  double vlo[3], Blo[3];
  if constexpr (!MINK) {
    lower_sp(g, vcon, vlo);
    lower_sp(g, Bcon, Blo);
    vsq = dot3(vcon, vlo);
    Bdotv = dot3(Bcon, vlo);
    BdotB = dot3(Bcon, Blo);
  }
#endif
#ifdef PHX_EXACT
  const double vsq_max = 1.0 - 1.0 / (gam_max * gam_max);
#else
  const double vsq_max = par.vsq_max;  // 1 - 1 / gam_max^2, formed on the host
#endif
  if (vsq > vsq_max) {
    double scale = vsq_max / vsq;
    vsq *= scale;
    scale = sqrt(scale);
    Bdotv *= scale;
#pragma unroll
    for (int m = 0; m < 3; m++) vcon[m] *= scale;
#ifndef PHX_EXACT
    if constexpr (!MINK)
#pragma unroll
      for (int m = 0; m < 3; m++) vlo[m] *= scale;
    capped = true;
#endif
  }
#ifdef PHX_EXACT
  W = 1.0 / sqrt(1 - vsq);
#else
  // production build: W = 1/s with s = sqrt(1 - v^2); divisions by W and W^2
  // become products with s and s^2.  Without a cap v^2 = 1 - 1/W0^2, so W
  // stays W0 and s is the 1/W0 formed above (no second rsqrt)
  double sW = iW0;
  if (capped) {
    W = rsqrt_p(1 - vsq);
    sW = (1 - vsq) * W;
  }
#endif
  const double vel = vcon[DIR];
  const double alpha = MINK ? 1.0 : g.alpha;
#ifdef PHX_EXACT
#define PHX_BOA(m) (g.beta[m] / alpha)
#else
  const double ialpha = MINK ? 1.0 : rcp_p(alpha);
#define PHX_BOA(m) (g.beta[m] * ialpha)
#endif
  double vtil;
  if constexpr (MINK)
    vtil = vel;
  else
    vtil = vel - PHX_BOA(DIR);
  U[PHX_CRHO] = rho * W;
  F[PHX_CRHO] = U[PHX_CRHO] * vtil;
  const double b0 = W * Bdotv;
#ifdef PHX_EXACT
  const double bsq = (BdotB + b0 * b0) / (W * W);
  const double rhohWsq = (rho + u + P) * W * W;
  const double bsqWsq = bsq * W * W;
#else
  // production build: bsq W^2 = B.B + b0^2 (sW = 1/W), W^2 formed once
  const double Wsq = W * W;
  const double bsqWsq = fma(b0, b0, BdotB);
  const double bsq = bsqWsq * (sW * sW);
  const double rhohWsq = (rho + u + P) * Wsq;
#endif
  const double ptot = P + 0.5 * bsq;
#pragma unroll
  for (int m = 0; m < 3; m++) {
    double bcovm, vcovm;
#ifdef PHX_EXACT
#define PHX_DIV_W(x) ((x) / W)
#else
#define PHX_DIV_W(x) ((x) * sW)
#endif
    if constexpr (MINK) {
      // gcov[m+1][0] = 0: first term is +-0; then only n = m+1 survives
      bcovm = PHX_DIV_W(Bcon[m]) + b0 * vcon[m];
      vcovm = vcon[m];
    } else {
#ifdef PHX_EXACT
      bcovm = g.gcov[m + 1][0] * b0 / alpha;
      vcovm = 0.0;
#pragma unroll
      for (int n = 1; n < 4; n++) {
        bcovm += g.gcov[m + 1][n] * (PHX_DIV_W(Bcon[n - 1]) + b0 * (vcon[n - 1] - PHX_BOA(n - 1)));
        vcovm += g.gcov[m + 1][n] * vcon[n - 1];
      }
#else
      // g_{m0} = gamma_mn beta^n: the shift terms cancel, b_m = B_m / W + b0 v_m
      bcovm = Blo[m] * sW + b0 * vlo[m];
      vcovm = vlo[m];
#endif
    }
    U[PHX_CMOM + m] = (rhohWsq + bsqWsq) * vcovm - b0 * bcovm;
    F[PHX_CMOM + m] = U[PHX_CMOM + m] * vtil + ptot * (double)(DIR == m) - PHX_DIV_W(bcovm * Bcon[DIR]);
#undef PHX_DIV_W
  }
#ifdef PHX_EXACT
  U[PHX_CENG] = rhohWsq + bsqWsq - ptot - b0 * b0 - U[PHX_CRHO];
#else
  U[PHX_CENG] = rhohWsq + BdotB - ptot - U[PHX_CRHO];  // bsq W^2 - b0^2 = B.B
#endif
  F[PHX_CENG] = U[PHX_CENG] * vtil + ptot * vel - Bdotv * Bcon[DIR];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    U[PHX_CB + m] = Bcon[m];
    if constexpr (MINK) {
#ifdef PHX_EXACT
      F[PHX_CB + m] = U[PHX_CB + m] * vtil - Bcon[DIR] * vcon[m];
#else
      // production build: B^d v^d - B^d v^d is 0 as the reference computes it
      // (equal products); contracted into an FMA it would be the product's
      // rounding error instead
      F[PHX_CB + m] = m == DIR ? 0.0 : U[PHX_CB + m] * vtil - Bcon[DIR] * vcon[m];
#endif
    } else {
      F[PHX_CB + m] = U[PHX_CB + m] * vtil - Bcon[DIR] * (vcon[m] - PHX_BOA(m));
    }
  }
#undef PHX_BOA
#ifdef PHX_EXACT
  const double vasq = bsqWsq / make_positive(rhohWsq + bsqWsq);
  const double cssq = make_bounded(gamma1 * P * W * W / make_positive(rhohWsq), 0.0, 1.0);
#else
  // one reciprocal of the product of the two denominators when it is normal
  const double dA = make_positive(rhohWsq + bsqWsq), dB = make_positive(rhohWsq);
  const double dAB = dA * dB;
  const int eAB = dexp(dAB);
  double vasq, cs_raw;
  if (eAB >= 16 && eAB <= 2030) {
    const double rAB = rcp_nr(dAB);
    vasq = bsqWsq * (dB * rAB);
    cs_raw = gamma1 * P * Wsq * (dA * rAB);
  } else {
    vasq = bsqWsq * rcp_p(dA);
    cs_raw = gamma1 * P * Wsq * rcp_p(dB);
  }
  const double cssq = make_bounded(cs_raw, 0.0, 1.0);
#endif
  const double cmsq = make_bounded(cssq + vasq * (1.0 - cssq), 0.0, 1.0);
  const double vcoff = div_p(alpha, 1.0 - vsq * cmsq);
  const double v0 = vel * (1.0 - cmsq);
  const double gdd = MINK ? 1.0 : f.gdd;
#ifdef PHX_EXACT
  const double vpm = sqrt(make_positive(cmsq * (1.0 - vsq) * (gdd * (1.0 - vsq * cmsq) - vel * v0)));
#else
  const double vpm_sq = make_positive(cmsq * (1.0 - vsq) * (gdd * (1.0 - vsq * cmsq) - vel * v0));
  const double vpm = vpm_sq * rsqrt_p(vpm_sq);  // vpm_sq >= 10 DBL_EPSILON > 0
#endif
  vp = vcoff * (v0 + vpm);
  vm = vcoff * (v0 - vpm);
  if constexpr (!MINK) {
    vp -= g.beta[DIR];
    vm -= g.beta[DIR];
  }
}

}  // namespace phx
