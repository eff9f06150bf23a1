// phx_c2p.cu -- prim2con and robust con2prim kernels
// (fluid.cpp:368-449 PrimitiveToConservedRegion, fluid.cpp:477-517
// ConservedToPrimitiveRobust).  One zone per thread over the index box; the
// con2prim loop exits on a warp vote.
#include "phx_mlp.cuh"

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

template <bool MINK>
__global__ void __launch_bounds__(128) k_p2c_zones(Par p, long long n, const double *prim, const double *geom,
                                                   double *cons, double *cell_sig) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  Pt g{};
  if constexpr (!MINK) load_pt_flat(geom, n, q, g);
  const double *P = prim + q;
  const double vel[3] = {P[PHX_PVEL * n], P[(PHX_PVEL + 1) * n], P[(PHX_PVEL + 2) * n]};
  double bp[3] = {0.0, 0.0, 0.0};
  if (p.mhd) {
    bp[0] = P[PHX_PB * n];
    bp[1] = P[(PHX_PB + 1) * n];
    bp[2] = P[(PHX_PB + 2) * n];
  }
  double D, tau, S[3], bc[3], sig[3];
  const double gdet = MINK ? 1.0 : g.detgam;
  p2c<MINK>(P[PHX_PRHO * n], vel, bp, P[PHX_PENG * n], P[PHX_PPRS * n], P[PHX_PGM1 * n], g, gdet, D, S, bc,
            tau, sig);
  double *U = cons + q;
  U[PHX_CRHO * n] = D;
  U[PHX_CENG * n] = tau;
#pragma unroll
  for (int m = 0; m < 3; m++) U[(PHX_CMOM + m) * n] = S[m];
  if (p.mhd)
#pragma unroll
    for (int m = 0; m < 3; m++) U[(PHX_CB + m) * n] = bc[m];
  if (cell_sig)
#pragma unroll
    for (int d = 0; d < 3; d++) cell_sig[d * n + q] = sig[d];
}

void launch_p2c_zones(const Par &p, long long n, const double *prim, const double *geom, double *cons,
                      double *cell_sig, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (geom)
    k_p2c_zones<false><<<grid, 128, 0, s>>>(p, n, prim, geom, cons, cell_sig);
  else
    k_p2c_zones<true><<<grid, 128, 0, s>>>(p, n, prim, geom, cons, cell_sig);
}

// ----------------------------------------------------------- con2prim
// One generic kernel over "zone accessors": a block index box (the
// reference's ConservedToPrimitiveRegion) or a list of independent zones with
// per-zone geometry.  LEARNED fuses the learned start: per warp, the setup
// invariants of its 32 zones go through the tensor-core network, and the
// resulting bracket starts the unchanged FP64 root find.
constexpr int C2P_THREADS = 128;
constexpr int C2P_WARPS = C2P_THREADS / 32;

// Zones of a block index box.
struct BoxZones {
  BView b;
  Range3 r;
  __device__ __forceinline__ long long id(long long t, int &k, int &j, int &i) const {
    box_index(r, t, k, j, i);
    return b.idx(k, j, i);
  }
  template <bool MINK>
  __device__ __forceinline__ void load(long long t, long long &id, Pt &g, double U[PHX_NCONS], double &x1, double &x2,
                                       double &x3, double &guess) const {
    int k, j, i;
    id = this->id(t, k, j, i);
    if constexpr (!MINK) load_pt(b, 0, j, i, g);
#pragma unroll
    for (int m = 0; m < PHX_NCONS; m++) U[m] = b.cons[m * b.vs + id];
    x1 = b.Xc(0, i);
    x2 = b.Xc(1, j);
    x3 = b.Xc(2, k);
    guess = b.prim[PHX_PMU * b.vs + id];
  }
  __device__ __forceinline__ void store(long long id, const Par &p, const double prim[PHX_NPRIM],
                                        const double U[PHX_NCONS], bool used_bounds, const double sig[3]) const {
    double *P = b.prim + id;
    const long long vs = b.vs;
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
  }
  __device__ __forceinline__ void store_fail(long long id, double f) const { b.fail[id] = f; }
};

// Independent zones, arrays [var][n]; geometry [PHX_GEOM_NLOC][n].
struct ListZones {
  long long n;
  double *cons, *prim, *fail, *cell_sig;
  const double *geom, *coords;
  template <bool MINK>
  __device__ __forceinline__ void load(long long t, long long &id, Pt &g, double U[PHX_NCONS], double &x1, double &x2,
                                       double &x3, double &guess) const {
    id = t;
    if constexpr (!MINK) load_pt_flat(geom, n, t, g);
#pragma unroll
    for (int m = 0; m < PHX_NCONS; m++) U[m] = cons[m * n + t];
    x1 = coords ? coords[t] : 0.0;
    x2 = coords ? coords[n + t] : 0.0;
    x3 = coords ? coords[2 * n + t] : 0.0;
    guess = prim[PHX_PMU * n + t];
  }
  __device__ __forceinline__ void store(long long id, const Par &p, const double pr[PHX_NPRIM],
                                        const double U[PHX_NCONS], bool used_bounds, const double sig[3]) const {
#pragma unroll
    for (int v = 0; v < PHX_NPRIM; v++) {
      if (v >= PHX_PB && v < PHX_PB + 3 && !p.mhd) continue;
      prim[v * n + id] = pr[v];
    }
    if (used_bounds) {
      cons[PHX_CRHO * n + id] = U[PHX_CRHO];
      cons[PHX_CENG * n + id] = U[PHX_CENG];
#pragma unroll
      for (int m = 0; m < 3; m++) cons[(PHX_CMOM + m) * n + id] = U[PHX_CMOM + m];
    }
    if (cell_sig)
#pragma unroll
      for (int d = 0; d < 3; d++) cell_sig[d * n + id] = sig[d];
  }
  __device__ __forceinline__ void store_fail(long long id, double f) const { fail[id] = f; }
};

// Shared memory of the learned variant: packed weights + per-warp scratch.
struct C2PLearnedSmem {
  MlpPacked w;
  uint32_t xs[C2P_WARPS][128];
  float os[C2P_WARPS][64];
};

// CTAs walk chunks of C2P_THREADS zones (grid-stride); with LEARNED the
// weights are staged once per CTA.
template <class Z, bool MINK, bool LEARNED>
__global__ void __launch_bounds__(C2P_THREADS) k_c2p(Par p, Z zones, long long ntot, const MlpPacked *mlp,
                                                      DevStats *stats, unsigned int *err) {
  extern __shared__ __align__(16) unsigned char c2p_dyn[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ unsigned int s_hist[PHX_C2P_HIST];
  __shared__ unsigned long long s_cnt[6];
  if (stats) {
    for (int h = threadIdx.x; h < PHX_C2P_HIST; h += blockDim.x) s_hist[h] = 0;
    if (threadIdx.x < 6) s_cnt[threadIdx.x] = 0;
  }
  C2PLearnedSmem *L = reinterpret_cast<C2PLearnedSmem *>(c2p_dyn);
  if constexpr (LEARNED) {
    if (!mlp_stage_weights(&L->w, mlp, &bar, err)) return;
  } else {
    __syncthreads();
  }
  const int warp = threadIdx.x >> 5;
  for (long long base = (long long)blockIdx.x * C2P_THREADS; base < ntot;
       base += (long long)gridDim.x * C2P_THREADS) {
    const long long t = base + threadIdx.x;
    const bool valid = t < ntot;
    long long id = 0;
    Pt g{};
    double U[PHX_NCONS];
    bool setup_ok = false;
    Residual res;
    double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0, guess = 0.0;
    if (valid) {
      double x1, x2, x3;
      zones.template load<MINK>(t, id, g, U, x1, x2, x3, guess);
      setup_ok = c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
    }
    C2POut out{0, 0, false, true, false, false};
    double mu;
    if constexpr (LEARNED) {
      float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (valid && setup_ok) c2p_features(res, f);
      float o0, o1;
      mlp_warp_forward(L->w, f, L->xs[warp], L->os[warp], o0, o1);
      double lb[3];
      mlp_bracket(o0, o1, lb);
      mu = regula_falsi_warp<true>(p, res, valid && setup_ok, 0.0, 1.0, guess, out, lb);
    } else {
      mu = regula_falsi_warp<false>(p, res, valid && setup_ok, 0.0, 1.0, guess, out);
    }
    if (valid) {
      bool success = false;
      if (setup_ok) {
        double prim[PHX_NPRIM], sig[3];
        bool used_bounds;
        c2p_finish<MINK>(p, g, res, mu, rcon, bu, Bprim, bdotr, prim, U, sig, used_bounds);
        zones.store(id, p, prim, U, used_bounds, sig);
        const int num_nans = isnan(U[PHX_CRHO]) + isnan(U[PHX_CMOM]) + isnan(U[PHX_CENG]);
        success = out.bracketed && num_nans == 0;
        if (p.fail_on_floors && (res.used_density_floor || res.used_energy_floor)) success = false;
        if (p.fail_on_ceilings && res.used_gamma_max) success = false;
        if (!out.bracketed) atomicOr(err, ERR_UNBRACKETED);
      }
      zones.store_fail(id, success ? 1.0 : 0.0);
      if (stats) {
        const int h = out.iterations < PHX_C2P_HIST ? out.iterations : PHX_C2P_HIST - 1;
        atomicAdd(&s_hist[h], 1u);
        atomicAdd(&s_cnt[0], (unsigned long long)out.iterations);
        atomicAdd(&s_cnt[1], (unsigned long long)out.evals);
        if (!success) atomicAdd(&s_cnt[2], 1ull);
        if (setup_ok && !out.bracketed) atomicAdd(&s_cnt[3], 1ull);
        atomicAdd(&s_cnt[4], 1ull);
        if (out.learned) atomicAdd(&s_cnt[5], 1ull);
      }
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
      atomicAdd(&stats->learned_accepted, s_cnt[5]);
    }
  }
}

// Plain launches cover the zones with one chunk per CTA; learned launches
// cap the grid at a few CTAs per SM so that each CTA stages the weights once
// for many chunks.
template <class Z, bool MINK>
static void launch_c2p_any(const Par &p, const Z &z, long long n, const MlpPacked *mlp, DevStats *stats,
                           unsigned int *err, cudaStream_t s) {
  if (n <= 0) return;
  long long grid = (n + C2P_THREADS - 1) / C2P_THREADS;
  if (mlp) {
    static int nsm = 0;
    if (!nsm) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      cudaFuncSetAttribute(k_c2p<Z, MINK, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(C2PLearnedSmem));
    }
    const long long cap = (long long)nsm * 8;
    if (grid > cap) grid = cap;
    k_c2p<Z, MINK, true><<<(unsigned)grid, C2P_THREADS, sizeof(C2PLearnedSmem), s>>>(p, z, n, mlp, stats, err);
  } else {
    k_c2p<Z, MINK, false><<<(unsigned)grid, C2P_THREADS, 0, s>>>(p, z, n, nullptr, stats, err);
  }
}

void launch_c2p(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                const MlpPacked *mlp, cudaStream_t s) {
  const long long n = (long long)(r.ie - r.is + 1) * (r.je - r.js + 1) * (r.ke - r.ks + 1);
  const BoxZones z{b, r};
  if (b.fmks)
    launch_c2p_any<BoxZones, false>(p, z, n, mlp, stats, err, s);
  else
    launch_c2p_any<BoxZones, true>(p, z, n, mlp, stats, err, s);
}

void launch_c2p_zones(const Par &p, long long n, double *cons, double *prim, const double *geom, double *fail,
                      double *cell_sig, const double *coords, DevStats *stats, unsigned int *err,
                      const MlpPacked *mlp, cudaStream_t s) {
  const ListZones z{n, cons, prim, fail, cell_sig, geom, coords};
  if (geom)
    launch_c2p_any<ListZones, false>(p, z, n, mlp, stats, err, s);
  else
    launch_c2p_any<ListZones, true>(p, z, n, mlp, stats, err, s);
}

}  // namespace phx
