// phx_torus.cu -- the magnetised Fishbone-Moncrief torus problem generator.
//
// The initial state of phoebus's torus problem for the ideal gas: the
// per-block ProblemGenerator (pgen/torus.cpp:130-474) and the mesh-wide
// field normalisation of PostInitializationModifier (torus.cpp:525-740,
// ComputeBetas :844-924), with the Fishbone-Moncrief helpers lfish_calc,
// log_enthalpy, GetStateFromEnthalpy and ucon_norm (torus.cpp:743-843) and the
// Boyer-Lindquist metric and BL -> FMKS velocity transform
// (boyer_lindquist.hpp, mckinney_gammie_ryan.hpp:111-151).  The reference
// evaluates the axisymmetric solution at every (k, j, i); here one 2D pass
// per block evaluates it per (j, i) and a 3D pass adds the k-dependent parts
// (the pressure noise and the floors), which gives the same values.  The
// noise draw is a counter-based SplitMix64 uniform (the reference's Kokkos
// pool is seeded by the clock).  Compiled without contraction in both
// library builds, with phx_math.h's exp / log / sin / cos / pow: the state
// equals the oracle's restatement bit for bit.
#include <cstring>

#include "phx_fmks.cuh"

namespace phx {

struct TorusDev {
  FmksDev f;
  double a, rin, l, kappa, gam, Cv, rho_rmax, u_jitter;
  unsigned long long seed;
};

// ---- torus.cpp:743-843 (ideal gas)
__host__ __device__ inline double lfish_calc(double r, double a) {
  using phx_math::pow;
  return (((pow(a, 2) - 2. * a * sqrt(r) + pow(r, 2)) *
           ((-2. * a * r * (pow(a, 2) - 2. * a * sqrt(r) + pow(r, 2))) / sqrt(2. * a * sqrt(r) + (-3. + r) * r) +
            ((a + (-2. + r) * sqrt(r)) * (pow(r, 3) + pow(a, 2) * (2. + r))) /
                sqrt(1 + (2. * a) / pow(r, 1.5) - 3. / r))) /
          (pow(r, 3) * sqrt(2. * a * sqrt(r) + (-3. + r) * r) * (pow(a, 2) + (-2. + r) * r)));
}

__host__ __device__ inline double log_enthalpy(double r, double th, double a, double rin, double l, double &uphi) {
  const double sth = phx_math::sin(th);
  const double cth = phx_math::cos(th);
  const double DD = r * r - 2. * r + a * a;
  const double AA = (r * r + a * a) * (r * r + a * a) - DD * a * a * sth * sth;
  const double SS = r * r + a * a * cth * cth;
  const double thin = M_PI / 2.;
  const double sthin = phx_math::sin(thin);
  const double cthin = phx_math::cos(thin);
  const double DDin = rin * rin - 2. * rin + a * a;
  const double AAin = (rin * rin + a * a) * (rin * rin + a * a) - DDin * a * a * sthin * sthin;
  const double SSin = rin * rin + a * a * cthin * cthin;
  uphi = 0.0;
  const double lnh =
      0.5 * phx_math::log((1. + sqrt(1. + 4. * (l * l * SS * SS) * DD / (AA * AA * sth * sth))) / (SS * DD / AA)) -
      0.5 * sqrt(1. + 4. * (l * l * SS * SS) * DD / (AA * AA * sth * sth)) - 2. * a * r * l / AA -
      (0.5 * phx_math::log((1. + sqrt(1. + 4. * (l * l * SSin * SSin) * DDin / (AAin * AAin * sthin * sthin))) /
                           (SSin * DDin / AAin)) -
       0.5 * sqrt(1. + 4. * (l * l * SSin * SSin) * DDin / (AAin * AAin * sthin * sthin)) -
       2. * a * rin * l / AAin);
  if (lnh > 0.0) {
    const double expm2chi = SS * SS * DD / (AA * AA * sth * sth);
    const double up1 = sqrt((-1. + sqrt(1. + 4. * l * l * expm2chi)) / 2.);
    uphi = 2. * a * r * sqrt(1. + up1 * up1) / sqrt(AA * SS * DD) + sqrt(SS / AA) * up1 / sth;
  }
  return lnh;
}

__host__ __device__ inline void state_from_enthalpy(double hm1, double kappa, double gam, double rho_rmax,
                                                    double &rho_out, double &u_out) {
  rho_out = phx_math::pow(hm1 * (gam - 1.) / (kappa * gam), 1. / (gam - 1.));
  u_out = kappa * phx_math::pow(rho_out, gam) / (gam - 1.) / rho_rmax;
  rho_out /= rho_rmax;
}

__host__ __device__ inline double ucon_norm(const double ucon[4], const double gcov[4][4]) {
  const double AA = gcov[0][0];
  const double BB = 2. * (gcov[0][1] * ucon[1] + gcov[0][2] * ucon[2] + gcov[0][3] * ucon[3]);
  const double CC = 1. + gcov[1][1] * ucon[1] * ucon[1] + gcov[2][2] * ucon[2] * ucon[2] +
                    gcov[3][3] * ucon[3] * ucon[3] +
                    2. * (gcov[1][2] * ucon[1] * ucon[2] + gcov[1][3] * ucon[1] * ucon[3] +
                          gcov[2][3] * ucon[2] * ucon[3]);
  const double discr = BB * BB - 4. * AA * CC;
  return (-BB - sqrt(discr)) / (2. * AA);
}

__device__ inline double rratio(double a, double b) {  // robust::ratio
  const double sgn = b >= 0 ? 1.0 : -1.0;
  return a / (b + sgn * kSMALL);
}

// Boyer-Lindquist g_{mu nu} (boyer_lindquist.hpp:77-95, ComputeDeltaMu_ :262-280)
__device__ inline void bl_gcov(double a, double X1, double X2, double g[4][4]) {
  const double a2 = a * a;
  const double r = fabs(X1), th = X2;
  const double sth = phx_math::sin(th), cth = phx_math::cos(th);
  const double r2 = r * r, r3 = r2 * r;
  const double DD = 1. - rratio(2., r) + rratio(a2, r2);
  const double mu = 1. + rratio(a2 * cth * cth, r2);
  const double sth2 = sth * sth;
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) g[m][n] = 0.0;
  g[0][0] = -(1.0 - rratio(2.0, r * mu));
  g[0][3] = g[3][0] = -rratio(2.0 * a * sth2, r * mu);
  g[1][1] = mu / DD;
  g[2][2] = r2 * mu;
  g[3][3] = r2 * sth2 * (1.0 + rratio(a2, r2) + rratio(2.0 * a2 * sth2, r3 * mu));
}

// McKinneyGammieRyan::bl_to_fmks (mckinney_gammie_ryan.hpp:119-151)
__device__ inline void bl_to_fmks(const FmksDev &f, double x1, double x2, double a, const double ucon_bl[4],
                                  double ucon_fmks[4]) {
  double trans[4][4];
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) trans[m][n] = 0.0;
  const double r = f.r_(x1);
  const double idenom = 1.0 / (r * r - 2.0 * r + a * a);
  trans[0][0] = 1.0;
  trans[0][1] = 2.0 * r * idenom;
  trans[1][1] = 1.0;
  trans[2][2] = 1.0;
  trans[3][1] = a * idenom;
  trans[3][3] = 1.0;
  double ucon_ks[4] = {0.0, 0.0, 0.0, 0.0};
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) ucon_ks[mu] += trans[mu][nu] * ucon_bl[nu];
  double C[3], Jcov[3][3], Jcon[3][3];
  f.transform(x1, x2, C, Jcov, Jcon);
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) trans[m][n] = 0.0;
  trans[0][0] = 1.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) trans[i + 1][j + 1] = Jcon[i][j];
  for (int mu = 0; mu < 4; mu++) ucon_fmks[mu] = 0.0;
  for (int mu = 0; mu < 4; mu++)
    for (int nu = 0; nu < 4; nu++) ucon_fmks[mu] += trans[mu][nu] * ucon_ks[nu];
}

// Plane scratch of a block: per (j, i) the solution before the noise and the
// floors, and the field before the normalisation.
enum { TP_RHO = 0, TP_U, TP_WV1, TP_WV2, TP_WV3, TP_B1, TP_B2, TP_NVAR };

// torus.cpp:279-338 for one (j, i) (nsub = 1, x3-independent parts)
__global__ void k_torus_plane(TorusDev t, BView b, double *S) {
  const long long n = (long long)b.n1t * b.n2t;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % b.n1t), j = (int)(q / b.n1t);
  const double dx_sub = b.dx[0] / 1;
  const double dy_sub = b.dx[1] / 1;
  double rho_acc = 0.0, u_acc = 0.0, v_acc[3] = {0.0, 0.0, 0.0};
  const double x1 = b.Xf(0, i) + (0 + 0.5) * dx_sub;
  const double x2 = b.Xf(1, j) + (0 + 0.5) * dy_sub;
  const double r = t.f.r_(x1);
  double y, th;
  t.f.th_(x1, x2, y, th);
  double lnh = -1.0, uphi = 0.0;
  if (r > t.rin) lnh = log_enthalpy(r, th, t.a, t.rin, t.l, uphi);
  if (lnh > 0.0) {
    const double hm1 = phx_math::exp(lnh) - 1.;
    double rho, u;
    state_from_enthalpy(hm1, t.kappa, t.gam, t.rho_rmax, rho, u);
    double ucon_bl[4] = {0.0, 0.0, 0.0, uphi};
    double gcov[4][4];
    bl_gcov(t.a, r, th, gcov);
    ucon_bl[0] = ucon_norm(ucon_bl, gcov);
    double ucon[4];
    bl_to_fmks(t.f, x1, x2, t.a, ucon_bl, ucon);
    const double lapse = t.f.Lapse(x1, x2);
    double beta[3];
    t.f.Shift(x1, x2, beta);
    t.f.SpacetimeMetric(x1, x2, gcov);
    ucon[0] = ucon_norm(ucon, gcov);
    const double W = lapse * ucon[0];
    const double vcon[3] = {ucon[1] / W + beta[0] / lapse, ucon[2] / W + beta[1] / lapse,
                            ucon[3] / W + beta[2] / lapse};
    rho_acc += rho / (1 * 1);
    u_acc += u / (1 * 1);
    for (int d = 0; d < 3; d++) v_acc[d] += W * vcon[d] / (1 * 1);
  }
  S[TP_RHO * n + q] = rho_acc;
  S[TP_U * n + q] = u_acc;
  for (int d = 0; d < 3; d++) S[(TP_WV1 + d) * n + q] = v_acc[d];
}

// the floored density of cell (j, i) at k = kb.s (torus.cpp:340-349), which the
// vector potential reads
__device__ inline double torus_rho_floored(const Par &p, const BView &b, const double *S, long long n, int j, int i) {
  const double rho = S[TP_RHO * n + (long long)j * b.n1t + i];
  double rhoflr = 0, epsflr;
  get_floors(p, b.Xc(0, i), b.Xc(1, j), b.Xc(2, 0), rhoflr, epsflr);
  return rho < rhoflr ? rhoflr : rho;
}

// A_phi at the corners and the poloidal field (torus.cpp:452-488): A(j, i)
// for j in [jb.s+1, jb.e], i in [ib.s+1, ib.e] (0 elsewhere), the field for
// j <= jb.e-1, i <= ib.e-1 (the last row and column keep 0)
__global__ void k_torus_field(Par p, BView b, double *S) {
  const long long n = (long long)b.n1t * b.n2t;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % b.n1t), j = (int)(q / b.n1t);
  double B1 = 0.0, B2 = 0.0;
  if (j <= b.n2t - 2 && i <= b.n1t - 2) {
    auto A = [&](int jj, int ii) -> double {
      if (jj < 1 || ii < 1) return 0.0;
      const double rho_av = 0.25 * (torus_rho_floored(p, b, S, n, jj, ii) + torus_rho_floored(p, b, S, n, jj, ii - 1) +
                                    torus_rho_floored(p, b, S, n, jj - 1, ii) +
                                    torus_rho_floored(p, b, S, n, jj - 1, ii - 1));
      const double qq = rho_av - 0.2;
      return qq > 0 ? qq : 0.0;
    };
    const double a00 = A(j, i), a10 = A(j + 1, i), a01 = A(j, i + 1), a11 = A(j + 1, i + 1);
    const double gamdet = b.gcent[PHX_G_DETGAM * n + q];
    B1 = -(a00 - a10 + a01 - a11) / (2.0 * b.dx[1] * gamdet);
    B2 = (a00 + a10 - a01 - a11) / (2.0 * b.dx[0] * gamdet);
  }
  S[TP_B1 * n + q] = B1;
  S[TP_B2 * n + q] = B2;
}

__device__ inline double torus_uniform(unsigned long long seed, unsigned long long idx) {
  // SplitMix64 of the counter (seed, stream 0, idx) -> [0, 1), 53 bits
  unsigned long long z = seed * 0x100000001B3ull;
  z += (idx + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// torus.cpp:279-367 per (k, j, i): the solution from the plane, the noise on
// u, the floors, T, P, gamma1; the field from the plane
__global__ void k_torus_fill(TorusDev t, Par p, BView b, const double *S, unsigned long long noise0) {
  const long long N = (long long)b.n1t * b.n2t * b.n3t;
  const long long n = (long long)b.n1t * b.n2t;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N) return;
  const int i = (int)(q % b.n1t), j = (int)((q / b.n1t) % b.n2t), k = (int)(q / n);
  const long long c = (long long)j * b.n1t + i;
  double *P = b.prim + q;
  const long long vs = b.vs;
  double rho = S[TP_RHO * n + c];
  double eng = S[TP_U * n + c];
  eng *= (1. + t.u_jitter * (torus_uniform(t.seed, noise0 + (unsigned long long)q) - 0.5));
  double rhoflr = 0, epsflr;
  get_floors(p, b.Xc(0, i), b.Xc(1, j), b.Xc(2, k), rhoflr, epsflr);
  rho = rho < rhoflr ? rhoflr : rho;
  eng = eng / rho < epsflr ? rho * epsflr : eng;
  // singularity-eos IdealGas (eos_phoebus.cpp:73-95)
  const double T = fmax(0.0, (eng / rho) / t.Cv);
  const double Pr = fmax(0.0, p.gm1 * rho * t.Cv * T);
  const double bmod = fmax(0.0, (p.gm1 + 1) * p.gm1 * rho * t.Cv * T);
  P[PHX_PRHO * vs] = rho;
  P[PHX_PENG * vs] = eng;
  for (int d = 0; d < 3; d++) P[(PHX_PVEL + d) * vs] = S[(TP_WV1 + d) * n + c];
  P[PHX_PTMP * vs] = T;
  P[PHX_PPRS * vs] = Pr;
  P[PHX_PGM1 * vs] = bmod / Pr;
  P[PHX_PB * vs] = S[TP_B1 * n + c];
  P[(PHX_PB + 1) * vs] = S[TP_B2 * n + c];
  P[(PHX_PB + 2) * vs] = 0.0;
  P[PHX_PMU * vs] = 0.0;
}

__device__ inline void atomic_max_nonneg(unsigned long long *w, double v) {
  if (v >= 0.0) atomicMax(w, (unsigned long long)__double_as_longlong(v));  // order of non-negative doubles
}

// ComputeBetas (torus.cpp:844-924): max P and max b^2 over the interior
__global__ void k_torus_maxima(BView b, unsigned long long *red) {
  const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1, nk = b.ndim >= 3 ? b.nx3 : 1;
  const long long n = (long long)ni * nj * nk;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double pr = 0.0, bsq = 0.0;
  if (t < n) {
    const int i = b.ng + (int)(t % ni);
    const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
    const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
    const long long id = b.idx(k, j, i);
    const long long nn = (long long)b.n1t * b.n2t, c = (long long)j * b.n1t + i;
    double gcov[3][3];
    for (int m = 0; m < 3; m++)
      for (int l = 0; l < 3; l++) gcov[m][l] = b.gcent[(PHX_G_GCOV + flat2(m + 1, l + 1)) * nn + c];
    const double vp[3] = {b.prim[PHX_PVEL * b.vs + id], b.prim[(PHX_PVEL + 1) * b.vs + id],
                          b.prim[(PHX_PVEL + 2) * b.vs + id]};
    const double Bp[3] = {b.prim[PHX_PB * b.vs + id], b.prim[(PHX_PB + 1) * b.vs + id],
                          b.prim[(PHX_PB + 2) * b.vs + id]};
    // GetLorentzFactor, GetMagneticFieldSquared (relativity_utils.hpp:38-43, 131-164)
    double vsq = 0.;
    for (int m = 0; m < 3; m++)
      for (int l = 0; l < 3; l++) vsq += gcov[m][l] * vp[m] * vp[l];
    const double W = sqrt(1. + vsq);
    double Bsq = 0, Bdotv = 0;
    for (int m = 0; m < 3; m++)
      for (int l = 0; l < 3; l++) {
        Bdotv += gcov[m][l] * rratio(vp[m], W) * Bp[l];
        Bsq += gcov[m][l] * Bp[m] * Bp[l];
      }
    bsq = rratio(Bsq, W * W) + Bdotv * Bdotv;
    pr = b.prim[PHX_PPRS * b.vs + id];
  }
  for (int o = 16; o > 0; o >>= 1) {
    pr = fmax(pr, __shfl_xor_sync(0xffffffffu, pr, o));
    bsq = fmax(bsq, __shfl_xor_sync(0xffffffffu, bsq, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_nonneg(&red[0], pr);
    atomic_max_nonneg(&red[1], bsq);
  }
}

// torus.cpp:728-738: the interior field times the normalisation factor
__global__ void k_torus_scale_field(BView b, double fac) {
  const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1, nk = b.ndim >= 3 ? b.nx3 : 1;
  const long long n = (long long)ni * nj * nk;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = b.ng + (int)(t % ni);
  const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
  const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
  const long long id = b.idx(k, j, i);
  for (int d = 0; d < 3; d++) b.prim[(PHX_PB + d) * b.vs + id] *= fac;
}

// ---- host side
cudaError_t torus_init(const Par &p, const phx_geometry &g, const phx_torus_params &tp, const BView *views, int n,
                       double *scratch, unsigned long long *red, DevStats *stats, unsigned int *err, double *fac_out,
                       cudaStream_t s) {
  TorusDev t;
  t.f = make_fmks(g);
  t.a = g.a;
  t.rin = tp.rin;
  t.l = lfish_calc(tp.rmax, g.a);
  t.kappa = tp.kappa;
  t.gam = p.gm1 + 1.0;
  t.Cv = p.Cv;
  t.u_jitter = tp.u_jitter;
  t.seed = tp.seed;
  // torus.cpp:270-276: the enthalpy at the pressure maximum sets the density scale
  double uphi_rmax;
  const double hm1_rmax = phx_math::exp(log_enthalpy(tp.rmax, 0.5 * M_PI, g.a, tp.rin, t.l, uphi_rmax)) - 1.0;
  double u_rmax;
  state_from_enthalpy(hm1_rmax, tp.kappa, t.gam, 1.0, t.rho_rmax, u_rmax);
  const int T = 128;
  // ProblemGenerator, block by block (noise counters continue across blocks)
  unsigned long long noise0 = 0;
  for (int q = 0; q < n; q++) {
    const BView &b = views[q];
    const long long n2 = (long long)b.n1t * b.n2t, N = n2 * b.n3t;
    k_torus_plane<<<(unsigned)((n2 + T - 1) / T), T, 0, s>>>(t, b, scratch);
    k_torus_field<<<(unsigned)((n2 + T - 1) / T), T, 0, s>>>(p, b, scratch);
    k_torus_fill<<<(unsigned)((N + T - 1) / T), T, 0, s>>>(t, p, b, scratch, noise0);
    const Range3 all{0, b.n1t - 1, 0, b.n2t - 1, 0, b.n3t - 1};
    launch_p2c(p, b, all, s);                     // fluid::PrimitiveToConserved
    launch_floors(p, b, all, stats, err, s);      // fixup::ApplyFloors
    noise0 += (unsigned long long)N;
  }
  // PostInitializationModifier: HARM-style normalisation max P / max (b^2 / 2)
  cudaError_t e = cudaMemsetAsync(red, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  for (int q = 0; q < n; q++) {
    const BView &b = views[q];
    const long long ni = (long long)b.nx1 * (b.ndim >= 2 ? b.nx2 : 1) * (b.ndim >= 3 ? b.nx3 : 1);
    k_torus_maxima<<<(unsigned)((ni + T - 1) / T), T, 0, s>>>(b, red);
  }
  unsigned long long hred[2];
  if ((e = cudaMemcpyAsync(hred, red, sizeof(hred), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  double pmax, bsqmax;
  memcpy(&pmax, &hred[0], sizeof(double));
  memcpy(&bsqmax, &hred[1], sizeof(double));
  const double half_bsq = 0.5 * bsqmax;
  const double beta_pmax = pmax / (half_bsq + (half_bsq >= 0 ? 1.0 : -1.0) * kSMALL);  // robust::ratio
  const double fac = tp.magnetized ? sqrt(beta_pmax / tp.target_beta) : 0;
  for (int q = 0; q < n; q++) {
    const BView &b = views[q];
    const long long ni = (long long)b.nx1 * (b.ndim >= 2 ? b.nx2 : 1) * (b.ndim >= 3 ? b.nx3 : 1);
    k_torus_scale_field<<<(unsigned)((ni + T - 1) / T), T, 0, s>>>(b, fac);
    launch_p2c(p, b, Range3{0, b.n1t - 1, 0, b.n2t - 1, 0, b.n3t - 1}, s);
  }
  if (fac_out) *fac_out = fac;
  return cudaGetLastError();
}

}  // namespace phx
