// phx_c2p.cu -- prim2con and robust con2prim kernels
// (fluid.cpp:368-449 PrimitiveToConservedRegion, fluid.cpp:477-517
// ConservedToPrimitiveRobust).  One zone per thread over the index box; the
// con2prim loop exits on a warp vote.
#include <cstdlib>

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
// per-zone geometry.  The learned start runs as two kernels per chunk of
// zones: k_mlp_bracket (setup invariants -> tensor-core network -> bracket
// (m, lo, hi), 24 bytes per zone in a context scratch) and k_c2p<LEARNED>,
// whose unchanged FP64 root find starts from that bracket.  Keeping the
// network out of the root-find kernel keeps that kernel's instruction
// footprint small (fused, the two codes thrashed the instruction cache).
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
  // the stored mu of zone t alone (the learned start's cold-zone test)
  __device__ __forceinline__ double guess_of(long long t) const {
    int k, j, i;
    return b.prim[PHX_PMU * b.vs + id(t, k, j, i)];
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
    guess = prim ? prim[PHX_PMU * n + t] : 0.0;
  }
  __device__ __forceinline__ double guess_of(long long t) const { return prim ? prim[PHX_PMU * n + t] : 0.0; }
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

// The learned start of zones t0 .. t0 + count - 1 into brk[3][count]
// (NaN where the setup rejects the zone).  CTAs stage the packed weights
// once and walk chunks of 128 zones, one tensor-core tile per chunk.
struct BracketSmem {
  MlpPacked w;
  MlpTile tile;
};
static_assert(C2P_THREADS == 128, "one network tile row per thread");
// more than 1/9 of an SM's shared memory: at most 8 CTAs resident, whose TMEM
// columns (8 x 64) fit the SM's 512, so tcgen05.alloc never waits on another CTA
static_assert(sizeof(BracketSmem) * 9 > 228 * 1024, "TMEM columns of the resident CTAs");

template <class Z, bool MINK>
__global__ void __launch_bounds__(C2P_THREADS) k_mlp_bracket(Par p, Z zones, long long t0, long long count,
                                                             const MlpPacked *mlp, double *brk, unsigned int *err) {
  extern __shared__ __align__(128) unsigned char brk_dyn[];
  __shared__ __align__(8) uint64_t bar;
  BracketSmem *S = reinterpret_cast<BracketSmem *>(brk_dyn);
  if (!mlp_stage_weights(&S->w, mlp, &bar, err)) return;
  mlp_tc_init(&S->tile);
  unsigned phase = 0;
  for (long long base = (long long)blockIdx.x * C2P_THREADS; base < count;
       base += (long long)gridDim.x * C2P_THREADS) {
    const long long q = base + threadIdx.x;
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool ok = false;
    // warm zones (a stored mu > 0) keep the reference's start: their stored
    // mu is the only value read, and the root find reads no bracket for them
    const bool cold = q < count && !(zones.guess_of(t0 + q) > 0.0);
    if (cold) {
      long long id;
      Pt g{};
      double U[PHX_NCONS], x1, x2, x3, guess;
      zones.template load<MINK>(t0 + q, id, g, U, x1, x2, x3, guess);
      ok = c2p_features_fp32<MINK>(p, g, U, x1, x2, x3, f) && mlp_in_box(S->w, f);
    }
    if (!__syncthreads_or(cold)) continue;  // whole chunk warm: no network
    float o0, o1;
    if (!mlp_cta_forward(S->w, &S->tile, f, phase, err, o0, o1)) break;
    if (cold) {
      double lb[3];
      mlp_bracket(o0, o1, lb);
      const double nan = __longlong_as_double(0x7ff8000000000000ll);
      for (int c = 0; c < 3; c++) brk[c * count + q] = ok ? lb[c] : nan;
    }
  }
  mlp_tc_finish(&S->tile);
}

// Per-zone statistics into the block's shared counters.
__device__ __forceinline__ void c2p_tally(unsigned int *s_hist, unsigned long long *s_cnt, const C2POut &out,
                                          bool setup_ok, bool success) {
  const int h = out.iterations < PHX_C2P_HIST ? out.iterations : PHX_C2P_HIST - 1;
  atomicAdd(&s_hist[h], 1u);
  atomicAdd(&s_cnt[0], (unsigned long long)out.iterations);
  atomicAdd(&s_cnt[1], (unsigned long long)out.evals);
  if (!success) atomicAdd(&s_cnt[2], 1ull);
  if (setup_ok && !out.bracketed) atomicAdd(&s_cnt[3], 1ull);
  atomicAdd(&s_cnt[4], 1ull);
  if (out.learned) atomicAdd(&s_cnt[5], 1ull);
}

__device__ __forceinline__ void c2p_flush_stats(DevStats *stats, const unsigned int *s_hist,
                                                const unsigned long long *s_cnt) {
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

// Finish one zone after its root find: unwrap mu, store, fail flag, stats.
template <class Z, bool MINK>
__device__ __forceinline__ void c2p_complete(const Par &p, const Z &zones, long long id, const Pt &g, Residual &res,
                                             double mu, const double rcon[3], const double bu[3],
                                             const double Bprim[3], double bdotr, double U[PHX_NCONS],
                                             bool setup_ok, const C2POut &out, DevStats *stats, unsigned int *s_hist,
                                             unsigned long long *s_cnt, unsigned int *err) {
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
  if (stats) c2p_tally(s_hist, s_cnt, out, setup_ok, success);
}

// Zones whose root find is still running after the first kernel's iteration
// cap: chunk offset and the saved RFState (it, evals, b1, b2 in 16/16/14/14
// bits, then the sign and learned bits).
struct RetryBuf {
  int *count;
  int *idx;
  double *a, *b, *ya, *yb;
  unsigned long long *packed;
};

__device__ __forceinline__ unsigned long long rf_pack(const RFState &s) {
  return (unsigned long long)(s.it & 0xffff) | ((unsigned long long)(s.evals & 0xffff) << 16) |
         ((unsigned long long)(s.b1 & 0x3fff) << 32) | ((unsigned long long)(s.b2 & 0x3fff) << 46) |
         ((unsigned long long)(s.sign < 0.0) << 60) | ((unsigned long long)s.learned << 61);
}
__device__ __forceinline__ void rf_unpack(unsigned long long w, RFState &s) {
  s.it = (int)(w & 0xffff);
  s.evals = (int)((w >> 16) & 0xffff);
  s.b1 = (int)((w >> 32) & 0x3fff);
  s.b2 = (int)((w >> 46) & 0x3fff);
  s.sign = ((w >> 60) & 1) ? -1.0 : 1.0;
  s.learned = (w >> 61) & 1;
  s.bracketed = true;
}

// con2prim of zones t0 .. t0 + count - 1, one zone per thread.  LEARNED:
// the start bracket of zone t is brk[c * count + t - t0].  A lane that has
// not converged after cap iterations saves its state to rb (warp-aggregated
// append) and leaves the zone to k_c2p_retry, so that one slow zone does not
// hold 31 finished lanes of its warp.
template <class Z, bool MINK, bool LEARNED>
__global__ void __launch_bounds__(C2P_THREADS) k_c2p(Par p, Z zones, long long t0, long long count,
                                                      const double *brk, int cap, RetryBuf rb, DevStats *stats,
                                                      unsigned int *err) {
  __shared__ unsigned int s_hist[PHX_C2P_HIST];
  __shared__ unsigned long long s_cnt[6];
  if (stats) {
    for (int h = threadIdx.x; h < PHX_C2P_HIST; h += blockDim.x) s_hist[h] = 0;
    if (threadIdx.x < 6) s_cnt[threadIdx.x] = 0;
    __syncthreads();
  }
  const long long q = (long long)blockIdx.x * C2P_THREADS + threadIdx.x;
  const bool valid = q < count;
  long long id = 0;
  Pt g{};
  double U[PHX_NCONS];
  bool setup_ok = false;
  Residual res;
  double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0, guess = 0.0;
  if (valid) {
    double x1, x2, x3;
    zones.template load<MINK>(t0 + q, id, g, U, x1, x2, x3, guess);
    setup_ok = c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
  }
  const bool run = valid && setup_ok;
  RFState st;
  if constexpr (LEARNED) {
    double lb[3] = {0.0, 0.0, 0.0};
    if (valid && !(guess > 0.0)) {  // brackets exist for cold zones only
      lb[0] = brk[q];
      lb[1] = brk[count + q];
      lb[2] = brk[2 * count + q];
    }
    rf_start<true>(p, res, run, 0.0, 1.0, guess, lb, st);
  } else {
    rf_start<false>(p, res, run, 0.0, 1.0, guess, nullptr, st);
  }
  rf_iterate(p, res, run, st, cap);
  const bool defer = run && rf_running(p, st);
  const unsigned m = __ballot_sync(0xffffffffu, defer);
  if (m) {
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(rb.count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (defer) {
      const int pos = base + __popc(m & ((1u << lane) - 1u));
      rb.idx[pos] = (int)q;
      rb.a[pos] = st.a;
      rb.b[pos] = st.b;
      rb.ya[pos] = st.ya;
      rb.yb[pos] = st.yb;
      rb.packed[pos] = rf_pack(st);
    }
  }
  if (valid && !defer) {
    C2POut out{0, 0, false, true, false, false};
    const double mu = rf_result(st, guess, out);
    c2p_complete<Z, MINK>(p, zones, id, g, res, mu, rcon, bu, Bprim, bdotr, U, setup_ok, out, stats, s_hist, s_cnt,
                          err);
  }
  if (stats) c2p_flush_stats(stats, s_hist, s_cnt);
}

// The deferred zones of a chunk: reload, set up again (the same
// deterministic setup), restore the root-find state and iterate to the end.
template <class Z, bool MINK>
__global__ void __launch_bounds__(C2P_THREADS) k_c2p_retry(Par p, Z zones, long long t0, RetryBuf rb, DevStats *stats,
                                                            unsigned int *err) {
  __shared__ unsigned int s_hist[PHX_C2P_HIST];
  __shared__ unsigned long long s_cnt[6];
  if (stats) {
    for (int h = threadIdx.x; h < PHX_C2P_HIST; h += blockDim.x) s_hist[h] = 0;
    if (threadIdx.x < 6) s_cnt[threadIdx.x] = 0;
    __syncthreads();
  }
  const int n = *rb.count;
  for (long long base = (long long)blockIdx.x * C2P_THREADS; base < n; base += (long long)gridDim.x * C2P_THREADS) {
    const long long k = base + threadIdx.x;
    const bool valid = k < n;
    long long id = 0;
    Pt g{};
    double U[PHX_NCONS];
    bool setup_ok = false;
    Residual res;
    double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0, guess = 0.0;
    RFState st{};
    if (valid) {
      double x1, x2, x3;
      zones.template load<MINK>(t0 + rb.idx[k], id, g, U, x1, x2, x3, guess);
      setup_ok = c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
      st.a = rb.a[k];
      st.b = rb.b[k];
      st.ya = rb.ya[k];
      st.yb = rb.yb[k];
      rf_unpack(rb.packed[k], st);
    }
    rf_iterate(p, res, valid && setup_ok, st, p.c2p_max_iter);
    if (valid) {
      C2POut out{0, 0, false, true, false, false};
      const double mu = rf_result(st, guess, out);
      c2p_complete<Z, MINK>(p, zones, id, g, res, mu, rcon, bu, Bprim, bdotr, U, setup_ok, out, stats, s_hist,
                            s_cnt, err);
    }
  }
  if (stats) c2p_flush_stats(stats, s_hist, s_cnt);
}

static int num_sms() {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm > 0 ? nsm : 1;
}

template <class Z, bool MINK>
static void launch_bracket_any(const Par &p, const Z &z, long long t0, long long count, const MlpPacked *mlp,
                               double *brk, unsigned int *err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_mlp_bracket<Z, MINK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(BracketSmem));
    attr = true;
  }
  long long grid = (count + C2P_THREADS - 1) / C2P_THREADS;
  const long long cap = (long long)num_sms() * 8;
  if (grid > cap) grid = cap;
  k_mlp_bracket<Z, MINK><<<(unsigned)grid, C2P_THREADS, sizeof(BracketSmem), s>>>(p, z, t0, count, mlp, brk, err);
}

// Zones per chunk of C2P_CHUNK; per chunk: [bracket launch], root-find
// launch with an iteration cap, retry launch over the deferred zones.  The
// caps default to a little above the mean iteration count of each start on
// Kerr-Schild zones at tolerance 1e-10; PHX_C2P_CAP_PLAIN /
// PHX_C2P_CAP_LEARNED in the environment override them (read once).
static int cap_from_env(const char *name, int dflt) {
  const char *v = getenv(name);
  const int c = v ? atoi(v) : 0;
  return c > 0 ? c : dflt;
}

template <class Z, bool MINK>
static void launch_c2p_any(const Par &p, const Z &z, long long n, const MlpPacked *mlp, const C2PScratch &scr,
                           DevStats *stats, unsigned int *err, cudaStream_t s) {
  if (n <= 0) return;
  static const int cap_plain = cap_from_env("PHX_C2P_CAP_PLAIN", 12);
  static const int cap_learned = cap_from_env("PHX_C2P_CAP_LEARNED", 6);
  const int cap = mlp ? cap_learned : cap_plain;
  RetryBuf rb{scr.count, scr.idx, scr.a, scr.b, scr.ya, scr.yb, scr.packed};
  const unsigned retry_grid = (unsigned)num_sms() * 4;
  for (long long t0 = 0; t0 < n; t0 += C2P_CHUNK) {
    const long long m = n - t0 < C2P_CHUNK ? n - t0 : C2P_CHUNK;
    const long long grid = (m + C2P_THREADS - 1) / C2P_THREADS;
    cudaMemsetAsync(scr.count, 0, sizeof(int), s);
    if (mlp) {
      launch_bracket_any<Z, MINK>(p, z, t0, m, mlp, scr.brk, err, s);
      k_c2p<Z, MINK, true><<<(unsigned)grid, C2P_THREADS, 0, s>>>(p, z, t0, m, scr.brk, cap, rb, stats, err);
    } else {
      k_c2p<Z, MINK, false><<<(unsigned)grid, C2P_THREADS, 0, s>>>(p, z, t0, m, nullptr, cap, rb, stats, err);
    }
    k_c2p_retry<Z, MINK><<<retry_grid, C2P_THREADS, 0, s>>>(p, z, t0, rb, stats, err);
  }
}

void launch_c2p(const Par &p, const BView &b, Range3 r, DevStats *stats, unsigned int *err,
                const MlpPacked *mlp, const C2PScratch &scr, cudaStream_t s) {
  const long long n = (long long)(r.ie - r.is + 1) * (r.je - r.js + 1) * (r.ke - r.ks + 1);
  const BoxZones z{b, r};
  if (b.fmks)
    launch_c2p_any<BoxZones, false>(p, z, n, mlp, scr, stats, err, s);
  else
    launch_c2p_any<BoxZones, true>(p, z, n, mlp, scr, stats, err, s);
}

void launch_c2p_zones(const Par &p, long long n, double *cons, double *prim, const double *geom, double *fail,
                      double *cell_sig, const double *coords, DevStats *stats, unsigned int *err,
                      const MlpPacked *mlp, const C2PScratch &scr, cudaStream_t s) {
  const ListZones z{n, cons, prim, fail, cell_sig, geom, coords};
  if (geom)
    launch_c2p_any<ListZones, false>(p, z, n, mlp, scr, stats, err, s);
  else
    launch_c2p_any<ListZones, true>(p, z, n, mlp, scr, stats, err, s);
}

void launch_mlp_bracket(const Par &p, long long n, const double *cons, const double *geom, const double *coords,
                        const MlpPacked *mlp, double *bracket, unsigned int *err, cudaStream_t s) {
  if (n <= 0) return;
  const ListZones z{n, const_cast<double *>(cons), nullptr, nullptr, nullptr, geom, coords};
  if (geom)
    launch_bracket_any<ListZones, false>(p, z, 0, n, mlp, bracket, err, s);
  else
    launch_bracket_any<ListZones, true>(p, z, 0, n, mlp, bracket, err, s);
}

// ------------------------------------------------------------- batched
// con2prim over the entire zones of many blocks: persistent CTAs walk
// (block, [first, last)) items; the root find runs to completion in place
// (no iteration cap: the retry list is per chunk of one zone list).
// Learned start of the batched con2prim: item it's zone first + tid gets
// its bracket at brk[c * (nitems * C2P_THREADS) + it * C2P_THREADS + tid]
// (c = 0, 1, 2); plane 3 holds its pass (1.0 cold: no stored mu > 0, the
// learned start; 0.0 warm: the plain start from the stored mu), written by
// the warm pass, which runs first and counts the cold zones in the word after
// plane 3.  This kernel and the cold pass return at once when that count is
// zero (a running simulation has no cold zones), and each zone is inverted
// exactly once even when a warm zone's new mu is not positive.  A 128-zone
// tile none of whose cold zones has features inside the network's input box
// skips the network.
template <bool MINK>
__global__ void __launch_bounds__(C2P_THREADS) kb_mlp_bracket(Par p, const BView *views, const WorkItem *items,
                                                              int nitems, const MlpPacked *mlp, double *brk,
                                                              unsigned int *err) {
  extern __shared__ __align__(128) unsigned char kbb_dyn[];
  __shared__ __align__(8) uint64_t bar;
  BracketSmem *S = reinterpret_cast<BracketSmem *>(kbb_dyn);
  const long long stride = (long long)nitems * C2P_THREADS;
  if (*reinterpret_cast<const unsigned long long *>(brk + 4 * stride) == 0) return;  // no cold zone
  if (!mlp_stage_weights(&S->w, mlp, &bar, err)) return;
  mlp_tc_init(&S->tile);
  unsigned phase = 0;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const BView &bv = views[w.block];
    const BoxZones zones{bv, Range3{0, bv.n1t - 1, 0, bv.n2t - 1, 0, bv.n3t - 1}};
    const long long q = w.first + threadIdx.x;
    const long long o = (long long)it * C2P_THREADS + threadIdx.x;
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool ok = false;
    const bool cold = q < w.last && brk[3 * stride + o] == 1.0;
    if (cold) {
      long long id;
      Pt g{};
      double U[PHX_NCONS], x1, x2, x3, guess;
      zones.template load<MINK>(q, id, g, U, x1, x2, x3, guess);
      ok = c2p_features_fp32<MINK>(p, g, U, x1, x2, x3, f) && mlp_in_box(S->w, f);
    }
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    if (!__syncthreads_or(ok)) {  // no usable start in this tile: no network
      if (cold)
        for (int c = 0; c < 3; c++) brk[c * stride + o] = nan;
      continue;
    }
    float o0, o1;
    if (!mlp_cta_forward(S->w, &S->tile, f, phase, err, o0, o1)) break;
    if (cold) {
      double lb[3];
      mlp_bracket(o0, o1, lb);
      for (int c = 0; c < 3; c++) brk[c * stride + o] = ok ? lb[c] : nan;
    }
  }
  mlp_tc_finish(&S->tile);
}

// only: 0 every zone; 1 the warm zones alone (this pass classifies every
// zone into plane 3 of brk and counts the cold ones); 2 the cold zones alone,
// as the warm pass classified them.  With the learned start the plan runs the
// plain kernel over the warm zones and the learned one over the cold zones,
// so warm zones (all of them once a run is under way) go through exactly the
// plain kernel's code.
template <bool MINK, bool LEARNED>
__global__ void __launch_bounds__(C2P_THREADS) kb_c2p(Par p, const BView *views, const WorkItem *items, int nitems,
                                                       double *brk, DevStats *stats, unsigned int *err, int only) {
  if (only == 2 && *reinterpret_cast<const unsigned long long *>(brk + 4 * (long long)nitems * C2P_THREADS) == 0)
    return;  // no cold zone
  __shared__ unsigned int s_hist[PHX_C2P_HIST];
  __shared__ unsigned long long s_cnt[6];
  if (stats) {
    for (int h = threadIdx.x; h < PHX_C2P_HIST; h += blockDim.x) s_hist[h] = 0;
    if (threadIdx.x < 6) s_cnt[threadIdx.x] = 0;
    __syncthreads();
  }
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const BView &bv = views[w.block];
    const BoxZones zones{bv, Range3{0, bv.n1t - 1, 0, bv.n2t - 1, 0, bv.n3t - 1}};
    const long long q = w.first + threadIdx.x;
    bool valid = q < w.last;
    if (only) {
      const long long stride = (long long)nitems * C2P_THREADS, o = (long long)it * C2P_THREADS + threadIdx.x;
      if (only == 1) {
        const bool cold = valid && !(zones.guess_of(q) > 0.0);
        if (valid) brk[3 * stride + o] = cold ? 1.0 : 0.0;
        const unsigned m = __ballot_sync(0xffffffffu, cold);
        if (m && (threadIdx.x & 31) == 0)
          atomicAdd(reinterpret_cast<unsigned long long *>(brk + 4 * stride), (unsigned long long)__popc(m));
        valid = valid && !cold;
      } else {
        valid = valid && brk[3 * stride + o] == 1.0;
      }
    }
    if (!__any_sync(0xffffffffu, valid)) continue;  // nothing for this warp in this pass
    long long id = 0;
    Pt g{};
    double U[PHX_NCONS];
    bool setup_ok = false;
    Residual res;
    double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0, guess = 0.0;
    if (valid) {
      double x1, x2, x3;
      zones.template load<MINK>(q, id, g, U, x1, x2, x3, guess);
      setup_ok = c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
    }
    RFState st;
    if constexpr (LEARNED) {
      const long long stride = (long long)nitems * C2P_THREADS, o = (long long)it * C2P_THREADS + threadIdx.x;
      double lb[3] = {0.0, 0.0, 0.0};
      if (valid && !(guess > 0.0)) {  // brackets exist for cold zones only
        lb[0] = brk[o];
        lb[1] = brk[stride + o];
        lb[2] = brk[2 * stride + o];
      }
      rf_start<true>(p, res, valid && setup_ok, 0.0, 1.0, guess, lb, st);
    } else {
      rf_start<false>(p, res, valid && setup_ok, 0.0, 1.0, guess, nullptr, st);
    }
    rf_iterate(p, res, valid && setup_ok, st, p.c2p_max_iter);
    if (valid) {
      C2POut out{0, 0, false, true, false, false};
      const double mu = rf_result(st, guess, out);
      c2p_complete<BoxZones, MINK>(p, zones, id, g, res, mu, rcon, bu, Bprim, bdotr, U, setup_ok, out, stats, s_hist,
                                   s_cnt, err);
    }
  }
  if (stats) c2p_flush_stats(stats, s_hist, s_cnt);
}

template <bool MINK>
static void c2p_batched_t(const Par &p, const BView *views, const WorkItem *items, int nitems, int grid,
                          const MlpPacked *mlp, double *brk, DevStats *stats, unsigned int *err, cudaStream_t s) {
  if (mlp) {
    static_assert(sizeof(BracketSmem) <= 48 * 1024, "no opt-in attribute needed (launches may be captured)");
    // warm pass (classifies and counts), bracket kernel, cold pass
    cudaMemsetAsync(brk + 4 * (long long)nitems * C2P_THREADS, 0, sizeof(unsigned long long), s);
    kb_c2p<MINK, false><<<persistent_grid(kb_c2p<MINK, false>, C2P_THREADS, 0, nitems, grid), C2P_THREADS, 0, s>>>(
        p, views, items, nitems, brk, stats, err, 1);
    kb_mlp_bracket<MINK><<<persistent_grid(kb_mlp_bracket<MINK>, C2P_THREADS, sizeof(BracketSmem), nitems, 0),
                           C2P_THREADS, sizeof(BracketSmem), s>>>(p, views, items, nitems, mlp, brk, err);
    kb_c2p<MINK, true><<<persistent_grid(kb_c2p<MINK, true>, C2P_THREADS, 0, nitems, grid), C2P_THREADS, 0, s>>>(
        p, views, items, nitems, brk, stats, err, 2);
  } else {
    kb_c2p<MINK, false><<<persistent_grid(kb_c2p<MINK, false>, C2P_THREADS, 0, nitems, grid), C2P_THREADS, 0, s>>>(
        p, views, items, nitems, nullptr, stats, err, 0);
  }
}

// bc_vars = conserved with the outer-X1 inflow check on an FMKS mesh
// (ConvertBoundaryConditions, phoebus_boundaries.cpp:333-340, 366-397, 416):
// after the exchange, the outer-X1 ghost slab of each block on the physical
// outer X1 face goes through con2prim (ConservedToPrimitiveRegion: the plain
// start from the stored mu, floors, the fail flag), the inflow check on the
// primitives it left, and prim2con with the zone's own metric (conserved
// variables and cell speeds).  Item zone t of a block is the slab zone
// i = n1t - ng + t % ng, j = (t / ng) % n2t, k = t / (ng n2t).
__global__ void __launch_bounds__(C2P_THREADS) kb_ox1_inflow(Par p, const BView *views, const WorkItem *items,
                                                              int nitems, unsigned int *err) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const BView &bv = views[w.block];
    const BoxZones zones{bv, Range3{bv.n1t - bv.ng, bv.n1t - 1, 0, bv.n2t - 1, 0, bv.n3t - 1}};
    const long long q = w.first + threadIdx.x;
    const bool valid = q < w.last;
    if (!__any_sync(0xffffffffu, valid)) continue;
    long long id = 0;
    Pt g{};
    double U[PHX_NCONS];
    bool setup_ok = false;
    Residual res;
    double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0, guess = 0.0;
    if (valid) {
      double x1, x2, x3;
      zones.template load<false>(q, id, g, U, x1, x2, x3, guess);
      setup_ok = c2p_setup<false>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr);
    }
    RFState st;
    rf_start<false>(p, res, valid && setup_ok, 0.0, 1.0, guess, nullptr, st);
    rf_iterate(p, res, valid && setup_ok, st, p.c2p_max_iter);
    if (!valid) continue;
    C2POut out{0, 0, false, true, false, false};
    const double mu = rf_result(st, guess, out);
    c2p_complete<BoxZones, false>(p, zones, id, g, res, mu, rcon, bu, Bprim, bdotr, U, setup_ok, out, nullptr,
                                  nullptr, nullptr, err);
    double *P = bv.prim + id;
    const long long vs = bv.vs;
    double vel[3] = {P[PHX_PVEL * vs], P[(PHX_PVEL + 1) * vs], P[(PHX_PVEL + 2) * vs]};
    ox1_inflow_fix(g, vel);
    for (int d = 0; d < 3; d++) P[(PHX_PVEL + d) * vs] = vel[d];
    double bp[3] = {0.0, 0.0, 0.0};
    if (p.mhd)
      for (int d = 0; d < 3; d++) bp[d] = P[(PHX_PB + d) * vs];
    double D, tau, S[3], bc[3], sig[3];
    p2c<false>(P[PHX_PRHO * vs], vel, bp, P[PHX_PENG * vs], P[PHX_PPRS * vs], P[PHX_PGM1 * vs], g, g.detgam, D, S,
               bc, tau, sig);
    double *C = bv.cons + id;
    C[PHX_CRHO * vs] = D;
    C[PHX_CENG * vs] = tau;
    for (int d = 0; d < 3; d++) C[(PHX_CMOM + d) * vs] = S[d];
    if (p.mhd)
      for (int d = 0; d < 3; d++) C[(PHX_CB + d) * vs] = bc[d];
    for (int d = 0; d < bv.ndim; d++) bv.cell_sig[d * vs + id] = sig[d];
  }
}

void launch_ox1_inflow(const Par &p, const BView *views, const WorkItem *items, int nitems, int grid,
                       unsigned int *err, cudaStream_t s) {
  if (nitems <= 0) return;
  kb_ox1_inflow<<<persistent_grid(kb_ox1_inflow, C2P_THREADS, 0, nitems, grid), C2P_THREADS, 0, s>>>(
      p, views, items, nitems, err);
}

void launch_c2p_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems, int grid,
                        const MlpPacked *mlp, double *brk, DevStats *stats, unsigned int *err, cudaStream_t s) {
  if (nitems <= 0) return;
  if (mink)
    c2p_batched_t<true>(p, views, items, nitems, grid, mlp, brk, stats, err, s);
  else
    c2p_batched_t<false>(p, views, items, nitems, grid, mlp, brk, stats, err, s);
}

}  // namespace phx
