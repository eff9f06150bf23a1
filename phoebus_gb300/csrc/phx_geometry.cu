// phx_geometry.cu -- FMKS metric tables on the device.
//
// FMKS = Modified<SphericalKerrSchild, McKinneyGammieRyan> (fmks.hpp:44).
// The tables are the reference's cached geometry with axisymmetry
// (cached_system.hpp:560-640, the analytic-derivative branch): per (j, i) of
// a block, at cell centres and X1/X2 faces, alpha, beta, gcov, gamcon and
// sqrt(gamma); at cell centres the finite-difference derivatives of ln alpha
// and g_{mu nu} (geometry_utils.hpp:89-178).  The metric does not depend on
// X3, so X3 faces share the centre table.
//
// exp, sin, cos and pow are phx_math.h's (the oracle evaluates the same
// operations), and this file is compiled without contraction in both library
// builds, so the tables equal the oracle's bit for bit.
#include "phx_fmks.cuh"

namespace phx {

__global__ void k_geom_loc(FmksDev f, double x01, double dx1, double x02, double dx2, int nj, int ni,
                           int locd, double *t) {
  const long long n = (long long)nj * ni;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % ni), j = (int)(q / ni);
  const double X1 = locd == 1 ? x01 + i * dx1 : x01 + (i + 0.5) * dx1;
  const double X2 = locd == 2 ? x02 + j * dx2 : x02 + (j + 0.5) * dx2;
  f.point(X1, X2, t + q, n);
}

__global__ void k_geom_deriv(FmksDev f, double x01, double dx1, double x02, double dx2, int nj, int ni,
                             double *t) {
  const long long n = (long long)nj * ni;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % ni), j = (int)(q / ni);
  const double X1 = x01 + (i + 0.5) * dx1;
  const double X2 = x02 + (j + 0.5) * dx2;
  const double EPSFD = f.epsfd;
  // GradLnAlpha (geometry_utils.hpp:89-119); the X3 derivative is 0 exactly
  // (identical lapse at X3 +- dx) and is stored as the reference computes it.
  for (int d = 1; d < 4; d++) {
    double da;
    if (d == 3) {
      da = 0.0;  // alphap - alpham = 0 exactly and the divisor is positive: +0
    } else {
      const double Xd = d == 1 ? X1 : X2;
      const double dx = fmax(fabs(Xd), 1.0) * EPSFD;
      const double am = d == 1 ? f.Lapse(X1 - dx, X2) : f.Lapse(X1, X2 - dx);
      const double ap = d == 1 ? f.Lapse(X1 + dx, X2) : f.Lapse(X1, X2 + dx);
      da = ratio(ap - am, dx * (am + ap));
    }
    t[(PHX_GD_DALPHA + d - 1) * n + q] = da;
  }
  // SetMetricGradientByFD (geometry_utils.hpp:149-178)
  for (int d = 1; d < 4; d++) {
    double gl[4][4], gr[4][4];
    double dx;
    if (d == 3) {  // gr - gl = 0 exactly, divided by a positive step: +0
      for (int mu = 0; mu < 4; mu++)
        for (int nu = mu; nu < 4; nu++) t[(PHX_GD_DG + 3 * flat2(mu, nu) + 2) * n + q] = 0.0;
      continue;
    }
    const double Xd = d == 1 ? X1 : X2;
    dx = fmax(fabs(Xd), 1.0) * EPSFD;
    if (d == 1) {
      f.SpacetimeMetric(X1 + dx, X2, gr);
      f.SpacetimeMetric(X1 - dx, X2, gl);
    } else {
      f.SpacetimeMetric(X1, X2 + dx, gr);
      f.SpacetimeMetric(X1, X2 - dx, gl);
    }
    for (int mu = 0; mu < 4; mu++)
      for (int nu = mu; nu < 4; nu++)
        t[(PHX_GD_DG + 3 * flat2(mu, nu) + d - 1) * n + q] = ratio(gr[mu][nu] - gl[mu][nu], 2 * dx);
  }
}

__global__ void k_geom_points(FmksDev f, long long n, const double *x1, const double *x2, double *t) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  f.point(x1[q], x2[q], t + q, n);
}


void launch_geom_points(const phx_geometry &g, long long n, const double *x1, const double *x2, double *geom,
                        cudaStream_t s) {
  if (n <= 0) return;
  const FmksDev f = make_fmks(g);
  const int T = 128;
  k_geom_points<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(f, n, x1, x2, geom);
}

// The library's exp / log / sin / cos / pow over an array, and the
// reciprocal and inverse square root of the kernels' arithmetic (their
// validation).
__global__ void k_math_eval(int fn, long long n, const double *x, const double *y, double *out) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double a = x[q];
  double r;
  switch (fn) {
  case PHX_MATH_EXP: r = phx_math::exp(a); break;
  case PHX_MATH_LOG: r = phx_math::log(a); break;
  case PHX_MATH_SIN: r = phx_math::sin(a); break;
  case PHX_MATH_COS: r = phx_math::cos(a); break;
  case PHX_MATH_RCP: r = rcp_p(a); break;
  case PHX_MATH_RSQRT: r = rsqrt_p(a); break;
  default: r = phx_math::pow(a, y[q]); break;
  }
  out[q] = r;
}

void launch_math_eval(int fn, long long n, const double *x, const double *y, double *out, cudaStream_t s) {
  if (n <= 0) return;
  k_math_eval<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(fn, n, x, y, out);
}

void launch_geom_fmks(const phx_geometry &g, const BView &b, cudaStream_t s) {
  const FmksDev f = make_fmks(g);
  const int T = 128;
  auto grid = [&](long long n) { return (unsigned)((n + T - 1) / T); };
  const int n1t = b.n1t, n2t = b.n2t;
  k_geom_loc<<<grid((long long)n2t * n1t), T, 0, s>>>(f, b.x0[0], b.dx[0], b.x0[1], b.dx[1], n2t, n1t, 0, g.cent);
  k_geom_loc<<<grid((long long)n2t * (n1t + 1)), T, 0, s>>>(f, b.x0[0], b.dx[0], b.x0[1], b.dx[1], n2t, n1t + 1, 1, g.face1);
  k_geom_loc<<<grid((long long)(n2t + 1) * n1t), T, 0, s>>>(f, b.x0[0], b.dx[0], b.x0[1], b.dx[1], n2t + 1, n1t, 2, g.face2);
  k_geom_deriv<<<grid((long long)n2t * n1t), T, 0, s>>>(f, b.x0[0], b.dx[0], b.x0[1], b.dx[1], n2t, n1t, g.deriv);
}

}  // namespace phx
