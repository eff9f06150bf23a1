// phx_stage.cu -- stage glue around the flux and con2prim kernels:
//   FluxCT (fluid.cpp:775-841), geometric sources (fluid.cpp:566-657 with
//   tmunu.hpp:62-131), FluxDivergence + SumData + Average/UpdateIndependentData
//   (phoebus_driver.cpp:547-577), periodic ghost exchange, and
//   EstimateTimestepBlock (fluid.cpp:899-944) as an on-device min-reduction.
#include "phx_kernels.cuh"

namespace phx {

__device__ __forceinline__ double &FX(const BView &b, int d, int m, long long id) {
  return b.flux[((long long)d * PHX_NCONS + m) * b.vs + id];
}

// ---------------------------------------------------------------- FluxCT
// Bodies take the face index t over the (nx1+1)(nx2+1)(nx3+1) interior
// corners (3D) or (nx1+1)(nx2+1) (2D), starting at (ng, ng, ng).
__device__ __forceinline__ void emf3d_at(const BView &b, long long t) {
  const int ni = b.nx1 + 1, nj = b.nx2 + 1;
  const int i = b.ng + (int)(t % ni);
  const int j = b.ng + (int)((t / ni) % nj);
  const int k = b.ng + (int)(t / ((long long)ni * nj));
  const long long id = b.idx(k, j, i);
  const long long dk = (long long)b.n1t * b.n2t, dj = b.n1t;
  const int B1 = PHX_CB, B2 = PHX_CB + 1, B3 = PHX_CB + 2;
  b.emf[id] = 0.25 * (FX(b, 1, B3, id) + FX(b, 1, B3, id - dk) - FX(b, 2, B2, id) - FX(b, 2, B2, id - dj));
  b.emf[b.vs + id] = -0.25 * (FX(b, 0, B3, id) + FX(b, 0, B3, id - dk) - FX(b, 2, B1, id) - FX(b, 2, B1, id - 1));
  b.emf[2 * b.vs + id] = 0.25 * (FX(b, 0, B2, id) + FX(b, 0, B2, id - dj) - FX(b, 1, B1, id) - FX(b, 1, B1, id - 1));
}
__device__ __forceinline__ void ctflux3d_at(const BView &b, long long t) {
  const int ni = b.nx1 + 1, nj = b.nx2 + 1;
  const int i = b.ng + (int)(t % ni);
  const int j = b.ng + (int)((t / ni) % nj);
  const int k = b.ng + (int)(t / ((long long)ni * nj));
  const long long id = b.idx(k, j, i);
  const long long dk = (long long)b.n1t * b.n2t, dj = b.n1t;
  const double *e0 = b.emf, *e1 = b.emf + b.vs, *e2 = b.emf + 2 * b.vs;
  const int B1 = PHX_CB, B2 = PHX_CB + 1, B3 = PHX_CB + 2;
  FX(b, 0, B1, id) = 0.0;
  FX(b, 0, B2, id) = 0.5 * (e2[id] + e2[id + dj]);
  FX(b, 0, B3, id) = -0.5 * (e1[id] + e1[id + dk]);
  FX(b, 1, B1, id) = -0.5 * (e2[id] + e2[id + 1]);
  FX(b, 1, B2, id) = 0.0;
  FX(b, 1, B3, id) = 0.5 * (e0[id] + e0[id + dk]);
  FX(b, 2, B1, id) = 0.5 * (e1[id] + e1[id + 1]);
  FX(b, 2, B2, id) = -0.5 * (e0[id] + e0[id + dj]);
  FX(b, 2, B3, id) = 0.0;
}
__device__ __forceinline__ void emf2d_at(const BView &b, long long t) {
  const int ni = b.nx1 + 1;
  const int i = b.ng + (int)(t % ni);
  const int j = b.ng + (int)(t / ni);
  const long long id = b.idx(0, j, i), dj = b.n1t;
  const int B1 = PHX_CB, B2 = PHX_CB + 1;
  b.emf[id] = 0.25 * (FX(b, 0, B2, id) + FX(b, 0, B2, id - dj) - FX(b, 1, B1, id) - FX(b, 1, B1, id - 1));
}
__device__ __forceinline__ void ctflux2d_at(const BView &b, long long t) {
  const int ni = b.nx1 + 1;
  const int i = b.ng + (int)(t % ni);
  const int j = b.ng + (int)(t / ni);
  const long long id = b.idx(0, j, i), dj = b.n1t;
  const int B1 = PHX_CB, B2 = PHX_CB + 1;
  FX(b, 0, B1, id) = 0.0;
  FX(b, 0, B2, id) = 0.5 * (b.emf[id] + b.emf[id + dj]);
  FX(b, 1, B1, id) = -0.5 * (b.emf[id] + b.emf[id + 1]);
  FX(b, 1, B2, id) = 0.0;
}

__global__ void k_emf3d(BView b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) emf3d_at(b, t);
}
__global__ void k_ctflux3d(BView b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) ctflux3d_at(b, t);
}
__global__ void k_emf2d(BView b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) emf2d_at(b, t);
}
__global__ void k_ctflux2d(BView b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) ctflux2d_at(b, t);
}

long long fluxct_count(const BView &b) {
  if (b.ndim == 3) return (long long)(b.nx1 + 1) * (b.nx2 + 1) * (b.nx3 + 1);
  if (b.ndim == 2) return (long long)(b.nx1 + 1) * (b.nx2 + 1);
  return 0;
}

void launch_fluxct(const BView &b, cudaStream_t s) {
  const int T = 256;
  const long long n = fluxct_count(b);
  if (n == 0) return;
  const unsigned g = (unsigned)((n + T - 1) / T);
  if (b.ndim == 3) {
    k_emf3d<<<g, T, 0, s>>>(b, n);
    k_ctflux3d<<<g, T, 0, s>>>(b, n);
  } else {
    k_emf2d<<<g, T, 0, s>>>(b, n);
    k_ctflux2d<<<g, T, 0, s>>>(b, n);
  }
}

// -------------------------------------- FluxDivergence + RK2 stage update
// dudt = -(A1 dF1 + A2 dF2 + A3 dF3) / V (+ src for S_i, tau);
// u0 = beta u0 + (1 - beta) base; out = u0 + (beta dt) dudt.
// t runs over the interior zones.
__device__ __forceinline__ void update_at(const BView &b, const double *base, double *out, double beta, double bdt,
                                          int ncons, long long t) {
  const double dx1 = b.dx[0], dx2 = b.dx[1], dx3 = b.dx[2];
  const double A1 = dx2 * dx3, A2 = dx1 * dx3, A3 = dx1 * dx2, V = dx1 * dx2 * dx3;
  const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1;
  const int i = b.ng + (int)(t % ni);
  const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
  const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
  const long long id = b.idx(k, j, i);
  const long long dk = (long long)b.n1t * b.n2t, dj = b.n1t;
#ifndef PHX_EXACT
  const double iV = rcp_p(V);  // one reciprocal for the ncons divisions by the volume
#endif
  for (int m = 0; m < ncons; m++) {
    double du = (A1 * FX(b, 0, m, id + 1) - A1 * FX(b, 0, m, id));
    if (b.ndim >= 2) du += A2 * FX(b, 1, m, id + dj) - A2 * FX(b, 1, m, id);
    if (b.ndim == 3) du += A3 * FX(b, 2, m, id + dk) - A3 * FX(b, 2, m, id);
#ifdef PHX_EXACT
    double r = -du / V;
#else
    double r = -du * iV;
#endif
    if (m >= 1 && m <= 4 && b.src != nullptr) r = r + b.src[(m - 1) * b.vs + id];
    const long long vid = m * b.vs + id;
    if (b.dudt != nullptr) b.dudt[vid] = r;
    if (out != nullptr) {
      double u0 = b.cons[vid];
      u0 = beta * u0 + (1 - beta) * base[vid];
      b.cons[vid] = u0;
      out[vid] = u0 + bdt * r;
    }
  }
}

__global__ void __launch_bounds__(256) k_update(BView b, const double *base, double *out, double beta,
                                                double bdt, int ncons, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) update_at(b, base, out, beta, bdt, ncons, t);
}

long long interior_count(const BView &b) {
  return (long long)b.nx1 * (b.ndim >= 2 ? b.nx2 : 1) * (b.ndim >= 3 ? b.nx3 : 1);
}

void launch_update(const Par &p, const BView &b, const double *base, double *out, double beta,
                   double dt, cudaStream_t s) {
  const long long n = interior_count(b);
  const int T = 256;
  k_update<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(b, base, out, beta, beta * dt, p.mhd ? PHX_NCONS : 5, n);
}

// ------------------------------------------------ periodic ghost exchange
__device__ __forceinline__ int wrap(int x, int ng, int n) {
  if (x < ng) return x + n;
  if (x >= ng + n) return x - n;
  return x;
}
__device__ __forceinline__ void ghost_at(const BView &b, double *field, int nvar, long long t) {
  const int i = (int)(t % b.n1t);
  const int j = (int)((t / b.n1t) % b.n2t);
  const int k = (int)(t / ((long long)b.n1t * b.n2t));
  const int si = wrap(i, b.ng, b.nx1);
  const int sj = b.ndim >= 2 ? wrap(j, b.ng, b.nx2) : j;
  const int sk = b.ndim >= 3 ? wrap(k, b.ng, b.nx3) : k;
  if (si == i && sj == j && sk == k) return;
  const long long d = b.idx(k, j, i), src = b.idx(sk, sj, si);
  for (int v = 0; v < nvar; v++) field[v * b.vs + d] = field[v * b.vs + src];
}
__global__ void __launch_bounds__(256) k_ghost(BView b, double *field, int nvar, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) ghost_at(b, field, nvar, t);
}

void launch_ghost_periodic(const BView &b, double *field, int nvar, cudaStream_t s) {
  const long long n = (long long)b.n1t * b.n2t * b.n3t;
  const int T = 256;
  k_ghost<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(b, field, nvar, n);
}

// ------------------------------------------------------------ timestep
__global__ void k_dt_init(unsigned long long *scratch) { *scratch = 0x7ff0000000000000ull; }
__global__ void __launch_bounds__(256) k_dt(BView b, int use_face, unsigned long long *scratch, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 1.7976931348623157e308;
  if (t < n) {
    const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1;
    const int i = b.ng + (int)(t % ni);
    const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
    const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
    const long long id = b.idx(k, j, i);
    double ldt = 0.0;
    for (int d = 0; d < b.ndim; d++) {
      double ms = b.cell_sig[d * b.vs + id];
      if (use_face) {
        const long long off = d == 0 ? 1 : (d == 1 ? (long long)b.n1t : (long long)b.n1t * b.n2t);
        ms = fmax(ms, fmax(b.face_sig[d * b.vs + id], b.face_sig[d * b.vs + id + off]));
      }
      ldt += ms / b.dx[d];
    }
    v = 1.0 / (ldt + 1.e-50);
  }
  // positive doubles order like their bit patterns
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = fmin(v, sm[w]);
    if (!(v >= 0.0)) v = 1.7976931348623157e308;  // all-NaN block: skipped, like the serial min
    atomicMin(scratch, (unsigned long long)__double_as_longlong(v));
  }
}
__global__ void k_dt_final(const unsigned long long *scratch, double cfl, double *out) {
  *out = cfl * __longlong_as_double((long long)*scratch);
}

void launch_dt(const Par &p, const BView &b, int use_face, unsigned long long *scratch, double *dt_out,
               cudaStream_t s) {
  const long long n = (long long)b.nx1 * (b.ndim >= 2 ? b.nx2 : 1) * (b.ndim >= 3 ? b.nx3 : 1);
  const int T = 256;
  k_dt_init<<<1, 1, 0, s>>>(scratch);
  k_dt<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(b, use_face, scratch, n);
  k_dt_final<<<1, 1, 0, s>>>(scratch, p.cfl, dt_out);
}

// ------------------------------------------------------------- sources
template <bool MINK>
__device__ __forceinline__ void sources_at(const Par &p, const BView &b, long long t) {
  const int ni = b.nx1, nj = b.ndim >= 2 ? b.nx2 : 1;
  const int i = b.ng + (int)(t % ni);
  const int j = (b.ndim >= 2 ? b.ng : 0) + (int)((t / ni) % nj);
  const int k = (b.ndim >= 3 ? b.ng : 0) + (int)(t / ((long long)ni * nj));
  const long long id = b.idx(k, j, i);
  const long long vs = b.vs;
  const double *P = b.prim + id;
  const double rho = P[PHX_PRHO * vs], uu = P[PHX_PENG * vs], Pr = P[PHX_PPRS * vs];
  const double vp[3] = {P[PHX_PVEL * vs], P[(PHX_PVEL + 1) * vs], P[(PHX_PVEL + 2) * vs]};
  double bf[3] = {0.0, 0.0, 0.0};
  if (p.mhd) {
    bf[0] = P[PHX_PB * vs];
    bf[1] = P[(PHX_PB + 1) * vs];
    bf[2] = P[(PHX_PB + 2) * vs];
  }
  if constexpr (MINK) {
    // All metric derivatives vanish: every source is exactly +0 for a finite
    // stress-energy tensor, NaN otherwise (as in the reference's arithmetic).
    const double chk = rho + uu + Pr + vp[0] + vp[1] + vp[2] + bf[0] + bf[1] + bf[2];
    const double z = isfinite(chk) ? 0.0 : __longlong_as_double(0x7ff8000000000000ll);
    for (int l = 0; l < 4; l++) b.src[l * vs + id] = z;
  } else {
    Pt g;
    load_pt(b, 0, j, i, g);
#ifdef PHX_EXACT
    double vsqw = 0.;
    for (int ii = 0; ii < 3; ii++)
      for (int jj = 0; jj < 3; jj++) vsqw += g.gcov[ii + 1][jj + 1] * vp[ii] * vp[jj];
    const double W = sqrt(1. + vsqw);
    double Bdotv = 0.0, Bsq = 0.0;
    for (int ii = 0; ii < 3; ii++)
      for (int jj = 0; jj < 3; jj++) {
        Bdotv += bf[ii] * (vp[jj] / W) * g.gcov[ii + 1][jj + 1];
        Bsq += bf[ii] * bf[jj] * g.gcov[ii + 1][jj + 1];
      }
#else
    double vlo[3], blo[3];  // the lowered vectors serve the three contractions
    lower_sp(g, vp, vlo);
    lower_sp(g, bf, blo);
    const double W = sqrt(1. + dot3(vp, vlo));
    const double Bdotv = div_p(dot3(bf, vlo), W);
    const double Bsq = dot3(bf, blo);
#endif
    const double iW = ratio_p(1., W);
    const double alpha = g.alpha;
    double u[4], bb[4];
    u[0] = ratio_p(W, fabs(alpha));
    bb[0] = u[0] * Bdotv;
    for (int l = 1; l < 4; ++l) {
      u[l] = vp[l - 1] - u[0] * g.beta[l - 1];
      bb[l] = iW * (bf[l - 1] + alpha * bb[0] * u[l]);
    }
    const double bsq = Bsq * iW * iW + Bdotv * Bdotv;
    double gi[4][4];
    {
      double alpha2 = g.alpha;
      alpha2 *= alpha2;
      gi[0][0] = -ratio_p(1, alpha2);
      for (int mu = 0; mu < 3; mu++) gi[mu + 1][0] = gi[0][mu + 1] = ratio_p(g.beta[mu], alpha2);
      for (int mu = 0; mu < 3; mu++)
        for (int nu = 0; nu < 3; nu++) {
          gi[mu + 1][nu + 1] = g.gamcon[mu][nu];
          gi[mu + 1][nu + 1] -= gi[0][mu + 1] * gi[0][nu + 1] * alpha2;
        }
    }
    const double A = rho + uu + Pr + bsq;
    const double Bt = Pr + 0.5 * bsq;
    double T[4][4];
    for (int mu = 0; mu < 4; mu++)
      for (int nu = 0; nu < 4; nu++) T[mu][nu] = A * u[mu] * u[nu] + Bt * gi[mu][nu] - bb[mu] * bb[nu];
    const double gdet = g.alpha * g.detgam;
    const long long pitch = (long long)b.n2t * b.n1t, off = (long long)j * b.n1t + i;
    double dg[4][4][4];
    for (int mu = 0; mu < 4; mu++)
      for (int nu = 0; nu < 4; nu++) {
        dg[mu][nu][0] = 0.0;
        for (int s = 1; s < 4; s++) dg[mu][nu][s] = __ldg(b.gderiv + (PHX_GD_DG + 3 * flat2(mu, nu) + s - 1) * pitch + off);
      }
    // Gamma[a][b][c] = 0.5 (dg[b][a][c] + dg[c][a][b] - dg[b][c][a]) is formed on the fly
    auto gam = [&](int a, int bb_, int c) { return 0.5 * (dg[bb_][a][c] + dg[c][a][bb_] - dg[bb_][c][a]); };
    for (int l = 0; l < 3; l++) {
      double src_mom = 0.0;
      for (int m = 0; m < 4; m++)
        for (int nn = 0; nn < 4; nn++) src_mom += T[m][nn] * (dg[nn][l + 1][m] - gam(l + 1, nn, m));
      b.src[l * vs + id] = gdet * src_mom;
    }
    double TGam = 0.0;
    const double inv_alpha2 = ratio_p(1, alpha * alpha);
    const double gcon0[4] = {-inv_alpha2, inv_alpha2 * g.beta[0], inv_alpha2 * g.beta[1], inv_alpha2 * g.beta[2]};
    for (int m = 0; m < 4; m++)
      for (int nn = 0; nn < 4; nn++) {
        double gam0 = 0;
        for (int r = 0; r < 4; r++) gam0 += gcon0[r] * gam(r, m, nn);
        TGam += T[m][nn] * gam0;
      }
    double Ta = 0.0;
    double da[4] = {0.0, 0.0, 0.0, 0.0};
    for (int d = 1; d < 4; d++) da[d] = __ldg(b.gderiv + (PHX_GD_DALPHA + d - 1) * pitch + off);
    for (int m = 0; m < 4; m++) Ta += T[m][0] * da[m];
    b.src[3 * vs + id] = gdet * alpha * (Ta - TGam);
  }
}

template <bool MINK>
__global__ void __launch_bounds__(128) k_sources(Par p, BView b, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) sources_at<MINK>(p, b, t);
}

void launch_sources(const Par &p, const BView &b, cudaStream_t s) {
  const long long n = interior_count(b);
  const int T = 128;
  if (b.fmks)
    k_sources<false><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(p, b, n);
  else
    k_sources<true><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(p, b, n);
}

// ------------------------------------------------------------- batched
// Persistent CTAs walk a work list of (block, [first, last)) items; each
// thread handles index first + threadIdx.x of its item's block.
template <bool MINK>
__global__ void __launch_bounds__(128) kb_sources(Par p, const BView *views, const WorkItem *items, int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) sources_at<MINK>(p, views[w.block], t);
  }
}
template <int NDIM, bool EMF>
__global__ void __launch_bounds__(256) kb_fluxct(const BView *views, const WorkItem *items, int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) {
      const BView &b = views[w.block];
      if constexpr (NDIM == 3) {
        if constexpr (EMF) emf3d_at(b, t); else ctflux3d_at(b, t);
      } else {
        if constexpr (EMF) emf2d_at(b, t); else ctflux2d_at(b, t);
      }
    }
  }
}
// beta_dt (device): beta and dt of the stage, read at run time so that a
// captured graph serves every step.
__global__ void __launch_bounds__(256) kb_update(const BView *views, const double *const *base, double *const *out,
                                                 const double *beta_dt, int ncons, const WorkItem *items,
                                                 int nitems) {
  const double beta = beta_dt[0], bdt = beta_dt[0] * beta_dt[1];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) update_at(views[w.block], base[w.block], out[w.block], beta, bdt, ncons, t);
  }
}
__global__ void __launch_bounds__(256) kb_ghost(const BView *views, int nvar, const WorkItem *items, int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) {
      const BView &b = views[w.block];
      ghost_at(b, b.cons, nvar, t);
    }
  }
}

// Ghost zone t of block blk on a tiled mesh (phx_mesh).  Each active axis
// maps the ghost's global cell: periodic axes wrap, gr_outflow clamps to the
// boundary cell (OutflowInnerX1 & co., phoebus_boundaries.cpp:115-150,
// 215-254, GenericBC Outflow), reflect and polar mirror it about the face
// (GenericBC Reflect :42-113, PolarInnerX2 :153-184, PolarOuterX2 :186-213).
// Parthenon applies the faces one after the other (X1, X2, X3; each over the
// whole extent of the other axes), so a ghost in several boundary slabs ends
// up with the source cell of all axes' maps; its value passes through the
// faces in that order.
//   Inside the domain (block faces, periodic wraps): the owner's exchanged
//   variables are copied (conserved; with bc_vars = primitive also the
//   primitives).
//   bc_vars = conserved, physical slab: the source's conserved variables,
//   scaled at each face by sgn * robust::ratio(DetGamma(cell), DetGamma(its
//   mapped cell)) where the cell is the one that face's loop sets (axes before
//   it at the ghost's own index, axes after it already mapped); sgn negates
//   the vector components along a reflect axis.  With the outer-X1 inflow
//   check on an FMKS mesh, launch_ox1_inflow (phx_c2p.cu) then takes the
//   outer-X1 slab through con2prim, the check and prim2con.
//   bc_vars = primitive, physical slab: primitives from the source with the
//   rule's signs (the velocity and B components along a reflect axis, v^2 and
//   B^2 across a polar face), the outer-X1 inflow check
//   (ConvertBoundaryConditions, phoebus_boundaries.cpp:366-397), then
//   prim2con with the ghost's own metric (PrimitiveToConservedRegion,
//   fluid.cpp:368-449: cons and cell speeds).
template <bool MINK>
__device__ __forceinline__ void mesh_ghost_at(const Par &p, const BView *views, const MeshDev &m, int blk,
                                              long long t) {
  const BView &b = views[blk];
  const GhostMap q = map_ghost(views, m, blk, t);
  if (!q.ghost) return;
  const int nd = b.ndim;
  const bool physical = q.physical, outer_x1 = q.outer_x1;
  double sgn_v[3];  // sign of the axis-d vector components from a mirror
  for (int d = 0; d < 3; d++) sgn_v[d] = q.mirror[d] ? -1.0 : 1.0;
  const BView &sb = views[q.src];
  const long long sid = q.sid, id = q.id;
  const int *loc = q.loc;
  const int ncons = p.mhd ? PHX_NCONS : PHX_CB;
  const bool prim_vars = m.bc_vars == PHX_BC_VARS_PRIMITIVE;
  if (!physical) {
    if (prim_vars)
      for (int v = 0; v < PHX_NPRIM; v++) {
        if (v >= PHX_PB && v < PHX_PB + 3 && !p.mhd) continue;
        b.prim[v * b.vs + id] = sb.prim[v * sb.vs + sid];
      }
    for (int v = 0; v < ncons; v++) b.cons[v * b.vs + id] = sb.cons[v * sb.vs + sid];
    return;
  }
  if (!prim_vars) {
    double U[PHX_NCONS];
    for (int v = 0; v < ncons; v++) U[v] = sb.cons[v * sb.vs + sid];
    for (int d = 0; d < nd; d++) {
      if (!q.phys[d]) continue;
      double gr = 1.0;  // DetGamma = 1 in Minkowski: ratio(1, 1) = 1
      if constexpr (!MINK) gr = ghost_gratio(b, q, d);
      for (int v = 0; v < ncons; v++) {
        const double sg = (v == PHX_CMOM + d || v == PHX_CB + d) ? sgn_v[d] : 1.0;
        U[v] = sg * gr * U[v];
      }
    }
    for (int v = 0; v < ncons; v++) b.cons[v * b.vs + id] = U[v];
    return;
  }
  double P[PHX_NPRIM];
  for (int v = 0; v < PHX_NPRIM; v++) P[v] = sb.prim[v * sb.vs + sid];
  for (int d = 0; d < 3; d++) {
    P[PHX_PVEL + d] = sgn_v[d] * P[PHX_PVEL + d];
    P[PHX_PB + d] = sgn_v[d] * P[PHX_PB + d];
  }
  Pt gm{};
  if constexpr (!MINK) {
    load_pt(b, 0, loc[1], loc[0], gm);
    if (outer_x1 && p.inflow_check) {  // enforce u^1 >= 0
      double v[3] = {P[PHX_PVEL], P[PHX_PVEL + 1], P[PHX_PVEL + 2]};
      ox1_inflow_fix(gm, v);
      for (int d = 0; d < 3; d++) P[PHX_PVEL + d] = v[d];
    }
  }
  const double vel[3] = {P[PHX_PVEL], P[PHX_PVEL + 1], P[PHX_PVEL + 2]};
  double bp[3] = {0.0, 0.0, 0.0};
  if (p.mhd)
    for (int d = 0; d < 3; d++) bp[d] = P[PHX_PB + d];
  double D, tau, S[3], bc[3], sig[3];
  p2c<MINK>(P[PHX_PRHO], vel, bp, P[PHX_PENG], P[PHX_PPRS], P[PHX_PGM1], gm, MINK ? 1.0 : gm.detgam, D, S, bc, tau,
            sig);
  for (int v = 0; v < PHX_NPRIM; v++) {
    if (v >= PHX_PB && v < PHX_PB + 3 && !p.mhd) continue;
    b.prim[v * b.vs + id] = P[v];
  }
  b.cons[PHX_CRHO * b.vs + id] = D;
  b.cons[PHX_CENG * b.vs + id] = tau;
  for (int d = 0; d < 3; d++) b.cons[(PHX_CMOM + d) * b.vs + id] = S[d];
  if (p.mhd)
    for (int d = 0; d < 3; d++) b.cons[(PHX_CB + d) * b.vs + id] = bc[d];
  for (int d = 0; d < b.ndim; d++) b.cell_sig[d * b.vs + id] = sig[d];
}

template <bool MINK>
__global__ void __launch_bounds__(128) kb_mesh_exchange(Par p, const BView *views, MeshDev m, const WorkItem *items,
                                                        int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) mesh_ghost_at<MINK>(p, views, m, w.block, t);
  }
}

void launch_mesh_exchange(const Par &p, bool mink, const BView *views, const MeshDev &m, const WorkItem *items,
                          int nitems, int grid, cudaStream_t s) {
  if (nitems <= 0) return;
  if (mink)
    kb_mesh_exchange<true><<<persistent_grid(kb_mesh_exchange<true>, 128, 0, nitems, grid), 128, 0, s>>>(
        p, views, m, items, nitems);
  else
    kb_mesh_exchange<false><<<persistent_grid(kb_mesh_exchange<false>, 128, 0, nitems, grid), 128, 0, s>>>(
        p, views, m, items, nitems);
}

// FixFluxes (fixup.cpp:728-1078) at face t of block blk's physical-boundary
// faces (fix_face_counts order).  The density-flux clamps keep the
// reference's std::min / std::max operand order (a NaN flux stays NaN).
__device__ __forceinline__ void fixflux_at(const Par &p, const BView &b, const int origin[3], const int n[3],
                                           const int bc_lo[3], const int bc_hi[3], long long t) {
  const int nx[3] = {b.nx1, b.nx2, b.nx3};
  long long cnt[6];
  fix_face_counts(b.ndim, nx, origin, n, bc_lo, bc_hi, cnt);
  int f = 0;
  while (f < 6 && t >= cnt[f]) t -= cnt[f++];
  if (f == 6) return;
  const int dir = f >> 1;
  const bool hi = f & 1;
  const int bc = hi ? bc_hi[dir] : bc_lo[dir];
  int i, j, k;
  if (dir == 0) {
    const int ny = b.ndim >= 2 ? b.nx2 : 1;
    i = hi ? b.ie() + 1 : b.is();
    j = b.js() + (int)(t % ny);
    k = b.ks() + (int)(t / ny);
  } else if (dir == 1) {
    i = b.is() + (int)(t % b.nx1);
    j = hi ? b.je() + 1 : b.js();
    k = b.ks() + (int)(t / b.nx1);
  } else {
    i = b.is() + (int)(t % b.nx1);
    j = b.js() + (int)(t / b.nx1);
    k = hi ? b.ke() + 1 : b.ks();
  }
  const long long id = b.idx(k, j, i);
  auto F = [&](int d, int v) -> double * { return b.flux + ((long long)d * PHX_NCONS + v) * b.vs; };
  double *fr = F(dir, PHX_CRHO);
  if (bc == PHX_BC_OUTFLOW) {  // gr_outflow: no mass inflow
    const double x = fr[id];
    fr[id] = hi ? ((x < 0.0) ? 0.0 : x) : ((0.0 < x) ? 0.0 : x);
  } else if (bc == PHX_BC_REFLECT) {
    fr[id] = 0.0;
    F(dir, PHX_CENG)[id] = 0.0;
    if (dir == 1) {
      F(dir, PHX_CMOM + 0)[id] = 0.0;
      F(dir, PHX_CMOM + 2)[id] = 0.0;
    }
  } else if (bc == PHX_BC_POLAR && dir == 1) {
    fr[id] = 0.0;
    F(1, PHX_CENG)[id] = 0.0;
    for (int d = 0; d < 3; d++) F(1, PHX_CMOM + d)[id] = 0.0;
    if (p.mhd) {
      for (int d = 0; d < 3; d++) F(1, PHX_CB + d)[id] = 0.0;
      // the B^2 fluxes of the ghost row mirror those of the interior row
      const long long in = hi ? b.idx(k, j - 1, i) : id, out = hi ? id : b.idx(k, j - 1, i);
      F(0, PHX_CB + 1)[out] = -F(0, PHX_CB + 1)[in];
      if (b.ndim == 3) F(2, PHX_CB + 1)[out] = -F(2, PHX_CB + 1)[in];
    }
  }
}

__global__ void __launch_bounds__(128) kb_fix_fluxes(Par p, const BView *views, MeshDev m, const WorkItem *items,
                                                     int nitems) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) fixflux_at(p, views[w.block], m.origin + 3 * w.block, m.n, m.bc_lo, m.bc_hi, t);
  }
}

void launch_fix_fluxes(const Par &p, const BView *views, const MeshDev &m, const WorkItem *items, int nitems,
                       int grid, cudaStream_t s) {
  if (nitems <= 0) return;
  kb_fix_fluxes<<<persistent_grid(kb_fix_fluxes, 128, 0, nitems, grid), 128, 0, s>>>(p, views, m, items, nitems);
}

// One block whose faces' boundary kinds are given (PHX_BC_PERIODIC for a
// face with a neighbour): the block is its own mesh.
struct FaceBC {
  int lo[3], hi[3];
};
__global__ void __launch_bounds__(128) k_fix_fluxes(Par p, BView b, FaceBC bc, long long count) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int origin[3] = {0, 0, 0}, n[3] = {b.nx1, b.nx2, b.nx3};
  if (t < count) fixflux_at(p, b, origin, n, bc.lo, bc.hi, t);
}

void launch_fix_fluxes_block(const Par &p, const BView &b, const int bc_lo[3], const int bc_hi[3], cudaStream_t s) {
  FaceBC bc;
  const int origin[3] = {0, 0, 0}, nx[3] = {b.nx1, b.nx2, b.nx3};
  for (int d = 0; d < 3; d++) {
    bc.lo[d] = bc_lo[d];
    bc.hi[d] = bc_hi[d];
  }
  long long cnt[6], tot = 0;
  fix_face_counts(b.ndim, nx, origin, nx, bc.lo, bc.hi, cnt);
  for (long long c : cnt) tot += c;
  if (tot == 0) return;
  k_fix_fluxes<<<(unsigned)((tot + 127) / 128), 128, 0, s>>>(p, b, bc, tot);
}

void launch_sources_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems, int grid,
                            cudaStream_t s) {
  if (nitems <= 0) return;
  if (mink)
    kb_sources<true><<<persistent_grid(kb_sources<true>, 128, 0, nitems, grid), 128, 0, s>>>(p, views, items, nitems);
  else
    kb_sources<false><<<persistent_grid(kb_sources<false>, 128, 0, nitems, grid), 128, 0, s>>>(p, views, items,
                                                                                              nitems);
}
void launch_fluxct_batched(int ndim, const BView *views, const WorkItem *items, int nitems, int grid, cudaStream_t s) {
  if (nitems <= 0) return;
  const int g = persistent_grid(kb_fluxct<3, true>, 256, 0, nitems, grid);
  if (ndim == 3) {
    kb_fluxct<3, true><<<g, 256, 0, s>>>(views, items, nitems);
    kb_fluxct<3, false><<<g, 256, 0, s>>>(views, items, nitems);
  } else if (ndim == 2) {
    kb_fluxct<2, true><<<g, 256, 0, s>>>(views, items, nitems);
    kb_fluxct<2, false><<<g, 256, 0, s>>>(views, items, nitems);
  }
}
void launch_update_batched(const Par &p, const BView *views, const double *const *base, double *const *out,
                           const double *beta_dt, const WorkItem *items, int nitems, int grid, cudaStream_t s) {
  if (nitems <= 0) return;
  kb_update<<<persistent_grid(kb_update, 256, 0, nitems, grid), 256, 0, s>>>(views, base, out, beta_dt,
                                                                           p.mhd ? PHX_NCONS : 5, items, nitems);
}
void launch_ghost_batched(const BView *views, int nvar, const WorkItem *items, int nitems, int grid, cudaStream_t s) {
  if (nitems <= 0) return;
  kb_ghost<<<persistent_grid(kb_ghost, 256, 0, nitems, grid), 256, 0, s>>>(views, nvar, items, nitems);
}

// ------------------------------------------------------- FP64 peak probe
// Independent FMA chains (8 per thread) so the pipe, not latency, limits.
__global__ void __launch_bounds__(256) k_fp64_probe(double *out, int iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
  double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
  const double m = 0.999999999, c = 1e-12;
  for (int it = 0; it < iters; it++) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 12345.678) out[0] = r;  // keep the chains alive
}
void launch_fp64_probe(double *out, int iters, cudaStream_t s, int *nthreads_out) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 8;
  k_fp64_probe<<<blocks, 256, 0, s>>>(out, iters);
  *nthreads_out = blocks * 256;
}

}  // namespace phx
