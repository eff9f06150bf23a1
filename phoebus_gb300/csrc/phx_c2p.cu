// phx_c2p.cu -- prim2con and robust con2prim kernels
// (fluid.cpp:368-449 PrimitiveToConservedRegion, fluid.cpp:477-517
// ConservedToPrimitiveRobust).  One zone per thread over the index box; the
// con2prim loop exits on a warp vote.
#include "phx_kernels.cuh"

namespace phx {

__device__ __forceinline__ void box_index(const Range3 &r, long long t, int &k, int &j, int &i) {
  const int ni = r.ie - r.is + 1, nj = r.je - r.js + 1;
  i = r.is + (int)(t % ni);
  const long long q = t / ni;
  j = r.js + (int)(q % nj);
  k = r.ks + (int)(q / nj);
}

template <bool MINK>
__global__ void __launch_bounds__(128) k_p2c(Par p, BView b, Range3 r, long long ntot) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntot) return;
  int k, j, i;
  box_index(r, t, k, j, i);
  const long long id = b.idx(k, j, i);
  Pt g{};
  if constexpr (!MINK) load_pt(b, 0, j, i, g);
  const double *P = b.prim + id;
  const long long vs = b.vs;
  const double vel[3] = {P[PHX_PVEL * vs], P[(PHX_PVEL + 1) * vs], P[(PHX_PVEL + 2) * vs]};
  double bp[3] = {0.0, 0.0, 0.0};
  if (p.mhd) {
    bp[0] = P[PHX_PB * vs];
    bp[1] = P[(PHX_PB + 1) * vs];
    bp[2] = P[(PHX_PB + 2) * vs];
  }
  double D, tau, S[3], bc[3], sig[3];
  const double gdet = MINK ? 1.0 : g.detgam;
  p2c<MINK>(P[PHX_PRHO * vs], vel, bp, P[PHX_PENG * vs], P[PHX_PPRS * vs], P[PHX_PGM1 * vs], g,
            gdet, D, S, bc, tau, sig);
  double *U = b.cons + id;
  U[PHX_CRHO * vs] = D;
  U[PHX_CENG * vs] = tau;
  U[PHX_CMOM * vs] = S[0];
  U[(PHX_CMOM + 1) * vs] = S[1];
  U[(PHX_CMOM + 2) * vs] = S[2];
  if (p.mhd) {
    U[PHX_CB * vs] = bc[0];
    U[(PHX_CB + 1) * vs] = bc[1];
    U[(PHX_CB + 2) * vs] = bc[2];
  }
  for (int d = 0; d < b.ndim; d++) b.cell_sig[d * vs + id] = sig[d];
}

void launch_p2c(const Par &p, const BView &b, Range3 r, cudaStream_t s) {
  const long long n = (long long)(r.ie - r.is + 1) * (r.je - r.js + 1) * (r.ke - r.ks + 1);
  if (n <= 0) return;
  const int T = 128;
  const unsigned grid = (unsigned)((n + T - 1) / T);
  if (b.fmks)
    k_p2c<false><<<grid, T, 0, s>>>(p, b, r, n);
  else
    k_p2c<true><<<grid, T, 0, s>>>(p, b, r, n);
}

// ----------------------------------------------------------- con2prim
constexpr int C2P_THREADS = 128;

template <bool MINK>
__global__ void __launch_bounds__(C2P_THREADS) k_c2p(Par p, BView b, Range3 r, long long ntot,
                                                      DevStats *stats, unsigned int *err) {
  __shared__ unsigned int s_hist[PHX_C2P_HIST];
  __shared__ unsigned long long s_cnt[5];
  if (stats) {
    for (int h = threadIdx.x; h < PHX_C2P_HIST; h += blockDim.x) s_hist[h] = 0;
    if (threadIdx.x < 5) s_cnt[threadIdx.x] = 0;
    __syncthreads();
  }
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = t < ntot;
  int k = 0, j = 0, i = 0;
  if (valid) box_index(r, t, k, j, i);
  const long long id = b.idx(k, j, i);
  const long long vs = b.vs;
  Pt g{};
  if constexpr (!MINK) {
    if (valid) load_pt(b, 0, j, i, g);
  }
  double U[PHX_NCONS];
  bool setup_ok = false;
  Residual res;
  double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0, guess = 0.0;
  if (valid) {
#pragma unroll
    for (int m = 0; m < PHX_NCONS; m++) U[m] = b.cons[m * vs + id];
    const double x1 = b.Xc(0, i), x2 = b.Xc(1, j), x3 = b.Xc(2, k);
    setup_ok = c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
    guess = b.prim[PHX_PMU * vs + id];
  }
  C2POut out{0, 0, false, true, false};
  const double mu = regula_falsi_warp(p, res, valid && setup_ok, 0.0, 1.0, guess, out);
  if (valid) {
    bool success = false;
    if (setup_ok) {
      double prim[PHX_NPRIM], sig[3];
      bool used_bounds;
      c2p_finish<MINK>(p, g, res, mu, rcon, bu, Bprim, bdotr, prim, U, sig, used_bounds);
      double *P = b.prim + id;
#pragma unroll
      for (int v = 0; v < PHX_NPRIM; v++) {
        if (v >= PHX_PB && v < PHX_PB + 3 && !p.mhd) continue;
        P[v * vs] = prim[v];
      }
      if (used_bounds) {
        b.cons[PHX_CRHO * vs + id] = U[PHX_CRHO];
        b.cons[PHX_CENG * vs + id] = U[PHX_CENG];
#pragma unroll
        for (int m = 0; m < 3; m++) b.cons[(PHX_CMOM + m) * vs + id] = U[PHX_CMOM + m];
      }
      for (int d = 0; d < b.ndim; d++) b.cell_sig[d * vs + id] = sig[d];
      const int num_nans = isnan(U[PHX_CRHO]) + isnan(U[PHX_CMOM]) + isnan(U[PHX_CENG]);
      success = out.bracketed && num_nans == 0;
      if (p.fail_on_floors && (res.used_density_floor || res.used_energy_floor)) success = false;
      if (p.fail_on_ceilings && res.used_gamma_max) success = false;
      if (!out.bracketed) atomicOr(err, ERR_UNBRACKETED);
    }
    b.fail[id] = success ? 1.0 : 0.0;
    if (stats) {
      const int h = out.iterations < PHX_C2P_HIST ? out.iterations : PHX_C2P_HIST - 1;
      atomicAdd(&s_hist[h], 1u);
      atomicAdd(&s_cnt[0], (unsigned long long)out.iterations);
      atomicAdd(&s_cnt[1], (unsigned long long)out.evals);
      if (!success) atomicAdd(&s_cnt[2], 1ull);
      if (setup_ok && !out.bracketed) atomicAdd(&s_cnt[3], 1ull);
      atomicAdd(&s_cnt[4], 1ull);
    }
  }
  if (stats) {
    __syncthreads();
    for (int h = threadIdx.x; h < PHX_C2P_HIST; h += blockDim.x)
      if (s_hist[h]) atomicAdd(&stats->hist[h], (unsigned long long)s_hist[h]);
    if (threadIdx.x == 0) {
      atomicAdd(&stats->iterations, s_cnt[0]);
      atomicAdd(&stats->residual_evals, s_cnt[1]);
      atomicAdd(&stats->failures, s_cnt[2]);
      atomicAdd(&stats->unbracketed, s_cnt[3]);
      atomicAdd(&stats->zones, s_cnt[4]);
    }
  }
}

void launch_c2p(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                const float *mlp_w, cudaStream_t s) {
  (void)mlp_w;
  const long long n = (long long)(r.ie - r.is + 1) * (r.je - r.js + 1) * (r.ke - r.ks + 1);
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + C2P_THREADS - 1) / C2P_THREADS);
  if (b.fmks)
    k_c2p<false><<<grid, C2P_THREADS, 0, s>>>(p, b, r, n, stats, err);
  else
    k_c2p<true><<<grid, C2P_THREADS, 0, s>>>(p, b, r, n, stats, err);
}

}  // namespace phx
