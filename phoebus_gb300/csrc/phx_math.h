// phx_math.h -- exp, log, sin, cos and pow written out from their series.
//
// The FMKS geometry (mckinney_gammie_ryan.hpp, spherical_kerr_schild.hpp)
// and the floors (fixup.hpp) call exp, sin, cos and pow.  CUDA's and the C
// library's versions of these differ by ulps, and the finite-difference
// metric derivatives (geometry_utils.hpp:153-178, step eps^(1/3)) amplify an
// ulp of the metric about 1.6e5 times.  Here the functions are written with
// IEEE operations only -- +, -, *, /, fma, rint and exact scaling by powers
// of two, each correctly rounded -- so that the CUDA kernels and the CPU
// oracle (which includes this header) compute them bit for bit alike:
//
//   exp  Cody-Waite reduction x = n ln2 + r (ln2 split in a 42-bit head and
//        a tail, so n ln2_hi is exact), |r| <= ln2 / 2, Taylor series of e^r
//        to degree 14 (truncation below 1e-19 relative) by Horner's rule with
//        fused multiply-adds, then the exact scaling by 2^n.
//   sin, cos  reduction by pi/2 in three parts (33 + 33 + 53 bits: exact
//        products for |n| < 2^20), |r| <= pi/4, Taylor series of sin r to
//        degree 19 and of cos r to degree 20 (truncation below 1e-19),
//        quadrant from n mod 4.  Accurate for |x| < 1e6 (the geometry's
//        angles are below 10).
//   log  x = 2^e m with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with
//        s = (m - 1) / (m + 1), |s| < 0.172, the atanh series to s^23.
//   pow  an integer exponent of magnitude <= 64 by binary powering in
//        double-double arithmetic (exact sign for a negative base), otherwise
//        exp(y log x) for x > 0.
//
// Measured against the C library (tests/test_cpu_math.py): exp within 1
// ulp, sin, cos and log within 2; pow within 1 ulp for integer exponents and
// within 2 |y log x| + 2 ulp otherwise.  The constants are the mathematical values
// (1/k!, 1/(2k+1), ln 2, pi/2) rounded to double, written in hexadecimal.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define PHX_MATH_FN __host__ __device__ __forceinline__
#else
#include <cmath>
#define PHX_MATH_FN inline
#endif

namespace phx_math {

constexpr double LN2_HI = 0x1.62e42fefa3800p-1;  // ln 2 to 42 bits: n LN2_HI is exact for |n| < 2^11
constexpr double LN2_LO = 0x1.ef35793c76730p-45;  // ln 2 - LN2_HI
constexpr double INV_LN2 = 0x1.71547652b82fep+0;
constexpr double PIO2_1 = 0x1.921fb54400000p+0;  // pi/2 to 33 bits
constexpr double PIO2_2 = 0x1.0b4611a600000p-34;  // the next 33 bits
constexpr double PIO2_3 = 0x1.3198a2e037073p-69;  // the rest
constexpr double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
constexpr double SQRT2 = 0x1.6a09e667f3bcdp+0;
// 1/k!, k = 0..14 (Taylor series of e^r)
#define PHX_MATH_EXP_C \
  {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1, 0x1.5555555555555p-3, \
   0x1.5555555555555p-5, 0x1.1111111111111p-7, 0x1.6c16c16c16c17p-10, \
   0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, \
   0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26, 0x1.1eed8eff8d898p-29, \
   0x1.6124613a86d09p-33, 0x1.93974a8c07c9dp-37}
// (-1)^k / (2k+1)!, k = 0..9 (sin r = r sum_k c_k r^2k)
#define PHX_MATH_SIN_C \
  {0x1.0000000000000p+0, -0x1.5555555555555p-3, 0x1.1111111111111p-7, \
   -0x1.a01a01a01a01ap-13, 0x1.71de3a556c734p-19, -0x1.ae64567f544e4p-26, \
   0x1.6124613a86d09p-33, -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49, \
   -0x1.2f49b46814157p-57}
// (-1)^k / (2k)!, k = 0..10 (cos r = sum_k c_k r^2k)
#define PHX_MATH_COS_C \
  {0x1.0000000000000p+0, -0x1.0000000000000p-1, 0x1.5555555555555p-5, \
   -0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16, -0x1.27e4fb7789f5cp-22, \
   0x1.1eed8eff8d898p-29, -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45, \
   -0x1.6827863b97d97p-53, 0x1.e542ba4020225p-62}
// 1 / (2k+1), k = 0..11 (log m = 2 s sum_k c_k s^2k, the atanh series)
#define PHX_MATH_LOG_C \
  {0x1.0000000000000p+0, 0x1.5555555555555p-2, 0x1.999999999999ap-3, 0x1.2492492492492p-3, \
   0x1.c71c71c71c71cp-4, 0x1.745d1745d1746p-4, 0x1.3b13b13b13b14p-4, 0x1.1111111111111p-4, \
   0x1.e1e1e1e1e1e1ep-5, 0x1.af286bca1af28p-5, 0x1.8618618618618p-5, 0x1.642c8590b2164p-5}

// ---- single correctly rounded operations that no compiler may contract
PHX_MATH_FN double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
PHX_MATH_FN double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
PHX_MATH_FN double fma_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
PHX_MATH_FN double div_(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
PHX_MATH_FN double rint_(double x) {  // round to nearest, ties to even
#ifdef __CUDA_ARCH__
  return rint(x);
#else
  return std::nearbyint(x);
#endif
}
PHX_MATH_FN double from_bits(uint64_t u) {
  double d;
  memcpy(&d, &u, sizeof(d));
  return d;
}
PHX_MATH_FN uint64_t to_bits(double d) {
  uint64_t u;
  memcpy(&u, &d, sizeof(u));
  return u;
}
PHX_MATH_FN double inf() { return from_bits(0x7ff0000000000000ull); }
PHX_MATH_FN double qnan() { return from_bits(0x7ff8000000000000ull); }
// 2^k for -1022 <= k <= 1023 (a normal power of two)
PHX_MATH_FN double pow2i(int k) { return from_bits((uint64_t)(k + 1023) << 52); }

// ---- exp
PHX_MATH_FN double exp(double x) {
  if (!(x == x)) return x;
  if (x > 709.782712893384) return inf();  // e^x above the largest double
  if (x < -745.2) return 0.0;              // below half the smallest subnormal
  const double n = rint_(mul(x, INV_LN2));
  double r = fma_(-n, LN2_HI, x);
  r = fma_(-n, LN2_LO, r);
  const double C[15] = PHX_MATH_EXP_C;
  double p = C[14];
#pragma unroll
  for (int k = 13; k >= 0; k--) p = fma_(p, r, C[k]);
  // scale by 2^n in two exact steps (n in [-1075, 1024]); only a subnormal
  // result rounds, once, in the second
  const int ni = (int)n, k1 = ni / 2, k2 = ni - k1;
  return mul(mul(p, pow2i(k1)), pow2i(k2));
}

// ---- sin and cos of the reduced argument |r| <= pi/4 (+ rounding)
PHX_MATH_FN double sin_r(double r) {
  const double s = mul(r, r);
  const double C[10] = PHX_MATH_SIN_C;
  double p = C[9];
#pragma unroll
  for (int k = 8; k >= 1; k--) p = fma_(p, s, C[k]);
  return fma_(mul(r, s), p, r);  // r + r^3 (c_1 + c_2 r^2 + ...)
}
PHX_MATH_FN double cos_r(double r) {
  const double s = mul(r, r);
  const double C[11] = PHX_MATH_COS_C;
  double p = C[10];
#pragma unroll
  for (int k = 9; k >= 1; k--) p = fma_(p, s, C[k]);
  return fma_(s, p, 1.0);
}
// x = n pi/2 + r; returns r and the quadrant n mod 4
PHX_MATH_FN double reduce_pio2(double x, int &quadrant) {
  const double n = rint_(mul(x, TWO_OVER_PI));
  double r = fma_(-n, PIO2_1, x);
  r = fma_(-n, PIO2_2, r);
  r = fma_(-n, PIO2_3, r);
  const long long ni = (long long)n;
  quadrant = (int)(ni & 3);
  return r;
}
PHX_MATH_FN double sin(double x) {
  if (!(x - x == 0.0)) return qnan();  // NaN or infinite
  int q;
  const double r = reduce_pio2(x, q);
  switch (q) {
  case 0: return sin_r(r);
  case 1: return cos_r(r);
  case 2: return -sin_r(r);
  default: return -cos_r(r);
  }
}
PHX_MATH_FN double cos(double x) {
  if (!(x - x == 0.0)) return qnan();
  int q;
  const double r = reduce_pio2(x, q);
  switch (q) {
  case 0: return cos_r(r);
  case 1: return -sin_r(r);
  case 2: return -cos_r(r);
  default: return sin_r(r);
  }
}

// ---- log
PHX_MATH_FN double log(double x) {
  if (!(x == x)) return x;
  if (x < 0.0) return qnan();
  if (x == 0.0) return -inf();
  if (x == inf()) return x;
  int e = 0;
  if (x < 0x1p-1022) {  // subnormal: scale into the normal range (exact)
    x = mul(x, 0x1p54);
    e = -54;
  }
  const uint64_t u = to_bits(x);
  e += (int)((u >> 52) & 0x7ff) - 1023;
  double m = from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);  // [1, 2)
  if (m > SQRT2) {
    m = mul(m, 0.5);
    e += 1;
  }
  const double f = add(m, -1.0);  // exact (Sterbenz)
  const double s = div_(f, add(2.0, f));
  const double z = mul(s, s);
  const double C[12] = PHX_MATH_LOG_C;
  double p = C[11];
#pragma unroll
  for (int k = 10; k >= 1; k--) p = fma_(p, z, C[k]);
  const double s2 = add(s, s);
  const double lm = fma_(mul(s2, z), p, s2);  // 2 s (1 + z/3 + z^2/5 + ...)
  const double de = (double)e;
  return fma_(de, LN2_HI, fma_(de, LN2_LO, lm));
}

// ---- pow
// (ah + al) *= (bh + bl) in double-double: the head product exactly as
// p + e (e = fma(ah, bh, -p)), plus the cross terms, renormalised.
PHX_MATH_FN void dd_mul(double &ah, double &al, double bh, double bl) {
  const double p = mul(ah, bh);
  const double e = fma_(ah, bh, -p);
  const double t = fma_(ah, bl, fma_(al, bh, e));
  const double h = add(p, t);
  al = add(t, -add(h, -p));  // exact when |p| >= |t| (fast two-sum)
  ah = h;
}
PHX_MATH_FN double pow(double x, double y) {
  if (y == 0.0) return 1.0;
  if (!(x == x) || !(y == y)) return qnan();
  const double yi = rint_(y);
  if (yi == y && y <= 64.0 && y >= -64.0) {  // integer exponent: binary powering
    // in double-double arithmetic (the products' rounding errors carried by
    // fma), so the result is rounded about once
    int k = (int)(y < 0 ? -y : y);
    double bh = x, bl = 0.0, rh = 1.0, rl = 0.0;
    while (k) {
      if (k & 1) dd_mul(rh, rl, bh, bl);
      k >>= 1;
      if (k) dd_mul(bh, bl, bh, bl);
    }
    if (y < 0) {  // 1 / (rh + rl) = q (1 + (1 - q rh) - q rl) to first order
      const double q = div_(1.0, rh);
      const double res = fma_(-q, rh, 1.0);
      return fma_(q, fma_(-q, rl, res), q);
    }
    return add(rh, rl);
  }
  if (x < 0.0) return qnan();
  if (x == 0.0) return y > 0 ? 0.0 : inf();
  return exp(mul(y, log(x)));
}

}  // namespace phx_math
