// phx_flux.cu -- fluid::CalculateFluxes (fluid.cpp:659-773) as fused
// reconstruction + Riemann kernels, one launch per direction.
//
// The reference reconstructs every variable into ql/qr arrays (K1) and then
// solves one Riemann problem per face (K2).  Here each face's two states are
// produced and consumed in registers:
//   X1: a CTA stages four (k, j) pencils' reconstructed primitive rows in
//       shared memory with one tiled TMA copy per pencil
//       (cp.async.bulk.tensor through a 5-D tensor map of the primitive
//       array: i split in S rows of n1t/S, j, k, variable), completing on an
//       mbarrier (1-D cp.async.bulk per row, or plain loads, where the block
//       shape does not admit the map); lanes reconstruct consecutive cells and
//       the left state of face i (the upper-face value of cell i-1) moves to
//       lane i with __shfl_up_sync.
//   X2, X3: a thread sweeps a segment of faces along the direction with the
//       5-point stencil window and the previous cell's upper-face state held
//       in registers; consecutive lanes are consecutive i (coalesced).
// Faces computed, per direction d: along d [s, e+1]; transverse active
// directions [s-1, e+1].  These are all the faces FluxDivergence, FluxCT and
// EstimateTimestep read.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "phx_kernels.cuh"
#include "phx_bulk.cuh"

namespace phx {

constexpr unsigned FULL = 0xffffffffu;

// Riemann solve + store for one face (riemann.hpp:256-301).
// col: the face's floor_point when the caller holds it (a sweep across X1
// faces' constant X1 when the floors depend on X1 alone), else null.
template <bool MINK, int DIR>
__device__ __forceinline__ void face_flux(const Par &p, const BView &b, int k, int j, int i,
                                          const double ql[PHX_NRECON], const double qr[PHX_NRECON],
                                          const FloorPt *col = nullptr) {
  Face f;
  if constexpr (!MINK) {
    load_pt(b, DIR == 0 ? 1 : (DIR == 1 ? 2 : 0), j, i, f.g);
    f.gdet = f.g.alpha * f.g.detgam;
    f.gammadet = f.g.detgam;
    f.gdd = f.g.gamcon[DIR][DIR];
  }
  if (col) {
    f.fl = *col;
  } else {
    f.fl = floor_point(p, DIR == 0 ? b.Xf(0, i) : b.Xc(0, i), DIR == 1 ? b.Xf(1, j) : b.Xc(1, j),
                       DIR == 2 ? b.Xf(2, k) : b.Xc(2, k));
  }
  const double gam_max = p.g0, sie_max = p.smax0;
  double Ul[PHX_NCONS], Fl[PHX_NCONS], Ur[PHX_NCONS], Fr[PHX_NCONS];
  double vml, vpl, vmr, vpr;
  prim_to_flux<MINK, DIR>(p, f, ql, vml, vpl, Ul, Fl, sie_max, gam_max);
  prim_to_flux<MINK, DIR>(p, f, qr, vmr, vpr, Ur, Fr, sie_max, gam_max);
  const double gdet = MINK ? 1.0 : f.gdet;
  const double gammadet = MINK ? 1.0 : f.gammadet;
  const long long id = b.idx(k, j, i);
  double *fx = b.flux + (long long)DIR * PHX_NCONS * b.vs + id;
  const int ncons = p.mhd ? PHX_NCONS : 5;
  double sig;
  if (p.riemann == PHX_RIEMANN_LLF) {
    const double cmax = rmax(rmax(-vml, vpl), rmax(-vmr, vpr));
#pragma unroll
    for (int m = 0; m < PHX_NCONS; m++)
      if (m < ncons) fx[m * b.vs] = 0.5 * ((Fl[m] + Fr[m]) * gdet - cmax * ((Ur[m] - Ul[m]) * gammadet));
    sig = cmax;
  } else {
    const double cl = rmin(rmin(vml, vmr), 0.0);
    const double cr = rmax(rmax(vpl, vpr), 0.0);
    const double crcl = cr * cl;
    const double inv_cr_cl = ratio_p(1.0, cr - cl);
#ifdef PHX_EXACT
#pragma unroll
    for (int m = 0; m < PHX_NCONS; m++)
      if (m < ncons)
        fx[m * b.vs] = ((cr * Fl[m] - cl * Fr[m]) * gdet + crcl * (Ur[m] - Ul[m]) * gammadet) * inv_cr_cl;
#else
    // the per-face factors formed once: F_l cr' - F_r cl' + (U_r - U_l) c'
    const double crg = cr * gdet * inv_cr_cl, clg = cl * gdet * inv_cr_cl, cc = crcl * gammadet * inv_cr_cl;
#pragma unroll
    for (int m = 0; m < PHX_NCONS; m++)
      if (m < ncons) fx[m * b.vs] = fma(crg, Fl[m], fma(-clg, Fr[m], cc * (Ur[m] - Ul[m])));
#endif
    sig = rmax(-cl, cr);
  }
  b.face_sig[(long long)DIR * b.vs + id] = sig;
}

// ------------------------------------------------------------------ X1
// Resident CTAs per SM the register allocation of the sweep kernels is
// bounded for (launch bounds); 1 leaves the compiler free (no spills).
#ifndef PHX_SWEEP_MINB
#define PHX_SWEEP_MINB 1
#endif

constexpr int X1_WARPS = 4;    // warps per CTA
constexpr int X1_PENCILS = 4;  // (k, j) pencils staged per CTA

// A CTA stages np pencils (kReconLoad primitive rows each) in shared memory
// with TMA copies completing on one mbarrier.  Its warps then walk the pencils'
// cells as one flattened list [pencil][cell is-1 .. ie+1] in chunks of 32
// cells that overlap by one: lane L reconstructs its cell, takes the
// upper-face state of the cell on its left from lane L-1 (__shfl_up_sync) and
// solves the Riemann problem of its lower face; lane 0 only supplies its
// state to lane 1 (its own face belongs to the previous chunk's lane 31).

// X1 face ranges of a block: pencils (k, j) over k in [ks-dk, ke+dk],
// j in [js-dj, je+dj]; pencil pen is (klo + pen / nj, jlo + pen % nj).
struct X1Range {
  int jlo, nj, klo, npencil;
};
__host__ __device__ __forceinline__ X1Range x1_range(const BView &b) {
  const int dk = b.ndim == 3 ? 1 : 0, dj = b.ndim > 1 ? 1 : 0;
  const int js = dj ? b.ng : 0, je = dj ? b.ng + b.nx2 - 1 : 0;
  const int ks = dk ? b.ng : 0, ke = dk ? b.ng + b.nx3 - 1 : 0;
  X1Range r;
  r.jlo = js - dj;
  r.nj = je - js + 1 + 2 * dj;
  r.klo = ks - dk;
  r.npencil = r.nj * (ke - ks + 1 + 2 * dk);
  return r;
}
__host__ __device__ __forceinline__ bool x1_tma_ok(const BView &b) {
  return (b.n1t % 2 == 0) && (b.vs % 2 == 0) && ((reinterpret_cast<uintptr_t>(b.prim) & 15) == 0);
}
// Staging modes of the X1 kernels.
enum X1Mode { X1_LOADS = 0, X1_BULK = 1, X1_TENSOR = 2 };

// Shared-memory doubles per staged pencil: its kReconLoad rows of n1t,
// rounded up to 128 bytes (the alignment of a tiled TMA destination).
__host__ __device__ __forceinline__ long long x1_pencil_stride(const BView &b) {
  return ((long long)kReconLoad * b.n1t + 15) / 16 * 16;
}

// One tiled TMA copy: box {n1t/S, S, 1, 1, kReconLoad} of the 5-D map at
// (0, 0, j, k, 0) -> a pencil's kReconLoad rows, contiguous in shared memory.
__device__ __forceinline__ void tensor_g2s_5d(void *dst, const CUtensorMap *map, int j, int k, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(j), "r"(k), "r"(0), "r"(smem_u32(bar))
      : "memory");
}

// Stage pencils p0 .. p0+np-1 into rows (pencil pp at rows + pp * pencil
// stride; mbarrier phase parity `phase` for the TMA modes).  Returns false,
// with ERR_TIMEOUT set, when the bounded wait gave up; every thread returns
// the same value.
__device__ __forceinline__ bool x1_stage(const BView &b, const X1Range &xr, int p0, int np, int mode,
                                         const CUtensorMap *map, double *rows, uint64_t *bar, unsigned phase,
                                         unsigned int *err) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n1t = b.n1t;
  const long long pst = x1_pencil_stride(b);
  if (mode == X1_TENSOR && (smem_u32(rows) & 127u) != 0) mode = X1_BULK;  // tiled TMA wants 128-byte rows
  if (mode == X1_TENSOR) {
    if (threadIdx.x == 0) {
      mbar_expect_tx(bar, (unsigned)(n1t * sizeof(double)) * kReconLoad * np);
      for (int pp = 0; pp < np; pp++) {
        const int pen = p0 + pp;
        tensor_g2s_5d(rows + pp * pst, map, xr.jlo + pen % xr.nj, xr.klo + pen / xr.nj, bar);
      }
    }
    return mbar_wait_block(bar, phase, MBAR_SPIN_LIMIT, err);
  }
  if (mode == X1_BULK) {
    const unsigned bytes = (unsigned)(n1t * sizeof(double));
    if (threadIdx.x == 0) mbar_expect_tx(bar, bytes * kReconLoad * np);
    __syncthreads();
    // one bulk copy per (pencil, variable) row; a CTA may stage more rows
    // than it has threads
    for (int r = threadIdx.x; r < np * kReconLoad; r += blockDim.x) {
      const int pp = r / kReconLoad, v = r % kReconLoad;
      const int pen = p0 + pp;
      const long long base = b.idx(xr.klo + pen / xr.nj, xr.jlo + pen % xr.nj, 0);
      bulk_g2s(rows + pp * pst + (long long)v * n1t, b.prim + v * b.vs + base, bytes, bar);
    }
    return mbar_wait_block(bar, phase, MBAR_SPIN_LIMIT, err);
  }
  for (int r = warp; r < np * kReconLoad; r += (int)(blockDim.x >> 5)) {
    const int pp = r / kReconLoad, v = r % kReconLoad;
    const int pen = p0 + pp;
    const long long base = b.idx(xr.klo + pen / xr.nj, xr.jlo + pen % xr.nj, 0);
    for (int i = lane; i < n1t; i += 32) rows[pp * pst + (long long)v * n1t + i] = b.prim[v * b.vs + base + i];
  }
  __syncthreads();
  return true;
}

template <int RECON, bool MINK>
__device__ __forceinline__ void x1_compute(const Par &p, const BView &b, const X1Range &xr, int p0, int np,
                                           const double *rows) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = (int)(blockDim.x >> 5);
  const int n1t = b.n1t;
  const int c0 = b.is() - 1;
  const int ncell = b.ie() + 1 - c0 + 1;  // cells is-1 .. ie+1 per pencil
  const int nslot = np * ncell;
  const int nchunk = (nslot - 1 + 30) / 31;
  for (int ch = warp; ch < nchunk; ch += nwarps) {
    const int slot = ch * 31 + lane;
    const bool have = slot < nslot;
    const int pp = have ? slot / ncell : 0;
    const int c = c0 + (have ? slot % ncell : 0);
    const double *prow = rows + pp * x1_pencil_stride(b);
    double ql[PHX_NRECON], qr[PHX_NRECON];
#pragma unroll
    for (int v = 0; v < kReconLoad; v++) {
      const double *r = prow + v * n1t;
      if (have) {
        if constexpr (RECON == PHX_RECON_WENO5Z || RECON == PHX_RECON_MP5)
          recon<RECON>(r[c - 2], r[c - 1], r[c], r[c + 1], r[c + 2], ql[v], qr[v]);
        else if constexpr (RECON == PHX_RECON_LINEAR)
          recon<RECON>(0.0, r[c - 1], r[c], r[c + 1], 0.0, ql[v], qr[v]);
        else
          recon<RECON>(0.0, 0.0, r[c], 0.0, 0.0, ql[v], qr[v]);
      } else {
        ql[v] = qr[v] = 0.0;
      }
    }
    double left[PHX_NRECON];
#pragma unroll
    for (int v = 0; v < kReconLoad; v++) left[v] = __shfl_up_sync(FULL, ql[v], 1);
    recon_gamma1(p, left, qr);
    // face of cell c: left state from cell c-1 (same pencil when c > is-1)
    if (have && lane > 0 && c > c0) {
      const int pen = p0 + pp;
      face_flux<MINK, 0>(p, b, xr.klo + pen / xr.nj, xr.jlo + pen % xr.nj, c, left, qr);
    }
  }
}

template <int RECON, bool MINK>
__global__ void __launch_bounds__(32 * X1_WARPS)
    k_flux_x1(Par p, BView b, int mode, const __grid_constant__ CUtensorMap map, unsigned int *err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  double *rows = reinterpret_cast<double *>(smem_raw);
  const X1Range xr = x1_range(b);
  const int p0 = blockIdx.x * X1_PENCILS;
  const int np = min(X1_PENCILS, xr.npencil - p0);
  if (mode != X1_LOADS && threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (!x1_stage(b, xr, p0, np, mode, &map, rows, &bar, 0u, err)) return;
  x1_compute<RECON, MINK>(p, b, xr, p0, np, rows);
}

// Batched X1: a persistent CTA walks the work list; item = (block, first
// pencil, pencil count).  The mbarrier is reused with alternating phase.
// maps[b] / modes[b]: block b's tensor map and staging mode.
template <int RECON, bool MINK>
__global__ void __launch_bounds__(32 * X1_WARPS) kb_flux_x1(Par p, const BView *views, const WorkItem *items,
                                                            int nitems, const CUtensorMap *maps, const int *modes,
                                                            unsigned int *err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  double *rows = reinterpret_cast<double *>(smem_raw);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned phase = 0;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const BView &b = views[w.block];
    const X1Range xr = x1_range(b);
    const int mode = modes[w.block];
    if (!x1_stage(b, xr, (int)w.first, (int)(w.last - w.first), mode, maps + w.block, rows, &bar, phase, err))
      return;
    if (mode != X1_LOADS) phase ^= 1u;
    x1_compute<RECON, MINK>(p, b, xr, (int)w.first, (int)(w.last - w.first), rows);
    __syncthreads();  // rows are rewritten by the next item
  }
}

// ------------------------------------------------------ X1 tensor maps
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;  // callers on several host threads look it up once
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

// The 5-D map of a block's reconstructed primitive planes: dimensions
// (n1t / S, S, n2t, n3t, kReconLoad) with byte strides (8, 8 n1t / S, 8 n1t,
// 8 n1t n2t, 8 vs), box (n1t / S, S, 1, 1, kReconLoad): one copy moves one
// (k, j) pencil's rows.  S is the smallest split with n1t / S <= 256 (the
// box limit) and n1t / S even (16-byte rows).  False (mode falls back) when
// no split fits, the strides are not multiples of 16 bytes, the base is not
// 16-byte aligned, or the encode is refused.
bool x1_encode_map(const BView &b, CUtensorMap *map) {
  if (!x1_tma_ok(b)) return false;
  int S = 0;
  for (int s = 1; s <= 8 && !S; s++)
    if (b.n1t % s == 0 && (b.n1t / s) % 2 == 0 && b.n1t / s <= 256) S = s;
  if (!S) return false;
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t h = (cuuint64_t)(b.n1t / S);
  const cuuint64_t dim[5] = {h, (cuuint64_t)S, (cuuint64_t)b.n2t, (cuuint64_t)b.n3t, (cuuint64_t)kReconLoad};
  const cuuint64_t stride[4] = {h * 8, (cuuint64_t)b.n1t * 8, (cuuint64_t)b.n1t * b.n2t * 8, (cuuint64_t)b.vs * 8};
  const cuuint32_t box[5] = {(cuuint32_t)h, (cuuint32_t)S, 1, 1, (cuuint32_t)kReconLoad};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, b.prim, dim, stride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// PHX_X1_STAGING=loads or =bulk in the environment forces a simpler mode
// (read at every call; the three modes give identical fluxes).
int x1_mode(const BView &b, CUtensorMap *map) {
  const char *force = getenv("PHX_X1_STAGING");
  if (force && strcmp(force, "loads") == 0) return X1_LOADS;
  if (!(force && strcmp(force, "bulk") == 0) && x1_encode_map(b, map)) return X1_TENSOR;
  return x1_tma_ok(b) ? X1_BULK : X1_LOADS;
}

// The failure path of the bounded waits above, driven on purpose: one CTA
// arms an mbarrier for 16 bytes and issues no copy, so the phase never
// completes and nothing is in flight; mbar_wait_block gives up after `limit`
// polls, sets ERR_TIMEOUT and the CTA returns.
__global__ void __launch_bounds__(128) k_wait_probe(long long limit, unsigned int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_expect_tx(&bar, 16u);
  mbar_wait_block(&bar, 0u, limit, err);
  __syncthreads();
  if (threadIdx.x == 0) mbar_inval(&bar);
}

void launch_wait_probe(long long limit, unsigned int *err, cudaStream_t s) {
  k_wait_probe<<<1, 128, 0, s>>>(limit, err);
}

// ------------------------------------------------------------- sweeps
// Thread = (transverse a, transverse c, segment).  DIR 1: a = i, c = k;
// DIR 2: a = i, c = j; DIR 0 (fallback for X1): a = j, c = k.
template <int RECON, bool MINK, int DIR>
__device__ __forceinline__ void sweep_at(const Par &p, const BView &b, int alo, int na, int clo, int nc, int f0,
                                         int nface, int seg, int nseg, long long t) {
  const int a = alo + (int)(t % na);
  const long long q = t / na;
  const int s = (int)(q % nseg);
  const int cc = clo + (int)(q / nseg);
  const int fbeg = f0 + s * seg;
  const int fend = min(f0 + nface - 1, fbeg + seg - 1);
  if (fbeg > fend) return;
  // position along the sweep direction -> (k, j, i)
  auto kji = [&](int x, int &k, int &j, int &i) {
    if constexpr (DIR == 0) {
      i = x;
      j = a;
      k = cc;
    } else if constexpr (DIR == 1) {
      i = a;
      j = x;
      k = cc;
    } else {
      i = a;
      j = cc;
      k = x;
    }
  };
  long long stride;
  if constexpr (DIR == 0)
    stride = 1;
  else if constexpr (DIR == 1)
    stride = b.n1t;
  else
    stride = (long long)b.n1t * b.n2t;
  int k0, j0, i0;
  kji(fbeg - 1, k0, j0, i0);
  const double *pc = b.prim + b.idx(k0, j0, i0);  // cell fbeg-1
  const long long vs = b.vs;
  double w[kReconLoad][5];
#pragma unroll
  for (int v = 0; v < kReconLoad; v++)
#pragma unroll
    for (int o = 0; o < 4; o++) w[v][o + 1] = pc[v * vs + (o - 2) * stride];  // cells x-2..x+1
  double prev_ql[PHX_NRECON];
  // X2 and X3 faces of this column share X1 (= the cell centre of column a)
  FloorPt col{};
  const bool use_col = DIR != 0 && floors_x1_only(p);
  if (use_col) col = floor_point(p, b.Xc(0, a), 0.0, 0.0);
  for (int x = fbeg - 1; x <= fend; x++) {
    const double *pn = pc + (long long)(x - (fbeg - 1)) * stride;
    double ql[PHX_NRECON], qr[PHX_NRECON];
#pragma unroll
    for (int v = 0; v < kReconLoad; v++) {
#pragma unroll
      for (int o = 0; o < 4; o++) w[v][o] = w[v][o + 1];
      w[v][4] = pn[v * vs + 2 * stride];
      recon<RECON>(w[v][0], w[v][1], w[v][2], w[v][3], w[v][4], ql[v], qr[v]);
    }
    if (x >= fbeg) {
      int k, j, i;
      kji(x, k, j, i);
      recon_gamma1(p, prev_ql, qr);
      face_flux<MINK, DIR>(p, b, k, j, i, prev_ql, qr, use_col ? &col : nullptr);
    }
#pragma unroll
    for (int v = 0; v < kReconLoad; v++) prev_ql[v] = ql[v];
  }
}

template <int RECON, bool MINK, int DIR>
__global__ void __launch_bounds__(128, PHX_SWEEP_MINB)
    k_flux_sweep(Par p, BView b, int alo, int na, int clo, int nc, int f0, int nface, int seg, int nseg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)na * nc * nseg) sweep_at<RECON, MINK, DIR>(p, b, alo, na, clo, nc, f0, nface, seg, nseg, t);
}

// Sweep geometry of a block for DIR 1 (X2 faces: j in [js, je+1], i in
// [is-1, ie+1], k in [ks-dk, ke+dk]) and DIR 2 (X3 faces: k in [ks, ke+1],
// i in [is-1, ie+1], j in [js-1, je+1]); threads per block na * nc * nseg.
struct SweepRange {
  int alo, na, clo, nc, f0, nface, seg, nseg;
};
__host__ __device__ __forceinline__ SweepRange sweep_range(const BView &b, int dir, int seg_target) {
  const int dk = b.ndim == 3 ? 1 : 0;
  const int is = b.ng, ie = b.ng + b.nx1 - 1;
  const int js = b.ng, je = b.ng + b.nx2 - 1;
  const int ks = dk ? b.ng : 0, ke = dk ? b.ng + b.nx3 - 1 : 0;
  SweepRange r;
  r.alo = is - 1;
  r.na = ie - is + 3;
  if (dir == 1) {
    r.clo = ks - dk;
    r.nc = ke - ks + 1 + 2 * dk;
    r.f0 = js;
    r.nface = je - js + 2;
  } else {
    r.clo = js - 1;
    r.nc = je - js + 3;
    r.f0 = ks;
    r.nface = ke - ks + 2;
  }
  r.nseg = (r.nface + seg_target - 1) / seg_target;
  r.seg = (r.nface + r.nseg - 1) / r.nseg;
  return r;
}

template <int RECON, bool MINK, int DIR>
__global__ void __launch_bounds__(128, PHX_SWEEP_MINB) kb_flux_sweep(Par p, const BView *views, const WorkItem *items, int nitems,
                                                     int seg_target) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const long long t = w.first + threadIdx.x;
    if (t < w.last) {
      const BView &b = views[w.block];
      const SweepRange r = sweep_range(b, DIR, seg_target);
      sweep_at<RECON, MINK, DIR>(p, b, r.alo, r.na, r.clo, r.nc, r.f0, r.nface, r.seg, r.nseg, t);
    }
  }
}

template <int RECON, bool MINK, int DIR>
static void launch_sweep(const Par &p, const BView &b, int alo, int na, int clo, int nc, int f0,
                         int nface, cudaStream_t s) {
  const int target = 32;
  const int nseg = (nface + target - 1) / target;
  const int seg = (nface + nseg - 1) / nseg;
  const long long total = (long long)na * nc * nseg;
  const int T = 128;
  k_flux_sweep<RECON, MINK, DIR><<<(unsigned)((total + T - 1) / T), T, 0, s>>>(p, b, alo, na, clo, nc,
                                                                            f0, nface, seg, nseg);
}

template <int RECON, bool MINK>
static void launch_fluxes_t(const Par &p, const BView &b, unsigned int *err, cudaStream_t s) {
  const int ndim = b.ndim;
  const int dk = ndim == 3 ? 1 : 0, dj = ndim > 1 ? 1 : 0;
  const int is = b.ng, ie = b.ng + b.nx1 - 1;
  const int js = dj ? b.ng : 0, je = dj ? b.ng + b.nx2 - 1 : 0;
  const int ks = dk ? b.ng : 0, ke = dk ? b.ng + b.nx3 - 1 : 0;
  // X1 faces: i in [is, ie+1]; j in [js-dj, je+dj]; k in [ks-dk, ke+dk]
  {
    const X1Range xr = x1_range(b);
    const int jlo = xr.jlo, nj = xr.nj, klo = xr.klo, nk = xr.npencil / xr.nj;
    const size_t smem = (size_t)X1_PENCILS * x1_pencil_stride(b) * sizeof(double);
    if (smem <= 200 * 1024) {
      auto kern = k_flux_x1<RECON, MINK>;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      CUtensorMap map;
      memset(&map, 0, sizeof(map));
      const int mode = x1_mode(b, &map);
      kern<<<(xr.npencil + X1_PENCILS - 1) / X1_PENCILS, 32 * X1_WARPS, smem, s>>>(p, b, mode, map, err);
    } else {
      launch_sweep<RECON, MINK, 0>(p, b, jlo, nj, klo, nk, is, ie - is + 2, s);
    }
  }
  if (ndim >= 2) {  // X2 faces: j in [js, je+1]; i in [is-1, ie+1]; k in [ks-dk, ke+dk]
    launch_sweep<RECON, MINK, 1>(p, b, is - 1, ie - is + 3, ks - dk, ke - ks + 1 + 2 * dk, js,
                                 je - js + 2, s);
  }
  if (ndim >= 3) {  // X3 faces: k in [ks, ke+1]; i in [is-1, ie+1]; j in [js-1, je+1]
    launch_sweep<RECON, MINK, 2>(p, b, is - 1, ie - is + 3, js - 1, je - js + 3, ks, ke - ks + 2, s);
  }
}

void launch_fluxes_err(const Par &p, const BView &b, unsigned int *err, cudaStream_t s) {
  const bool mink = !b.fmks;
  switch (p.recon) {
  case PHX_RECON_WENO5Z:
    mink ? launch_fluxes_t<PHX_RECON_WENO5Z, true>(p, b, err, s)
         : launch_fluxes_t<PHX_RECON_WENO5Z, false>(p, b, err, s);
    break;
  case PHX_RECON_MP5:
    mink ? launch_fluxes_t<PHX_RECON_MP5, true>(p, b, err, s) : launch_fluxes_t<PHX_RECON_MP5, false>(p, b, err, s);
    break;
  case PHX_RECON_LINEAR:
    mink ? launch_fluxes_t<PHX_RECON_LINEAR, true>(p, b, err, s)
         : launch_fluxes_t<PHX_RECON_LINEAR, false>(p, b, err, s);
    break;
  default:
    mink ? launch_fluxes_t<PHX_RECON_CONSTANT, true>(p, b, err, s)
         : launch_fluxes_t<PHX_RECON_CONSTANT, false>(p, b, err, s);
    break;
  }
}

// ------------------------------------------------------------- batched
int x1_npencil(const BView &b) { return x1_range(b).npencil; }
bool x1_tma_ok_host(const BView &b) { return x1_tma_ok(b); }
long long x1_pencil_stride_host(const BView &b) { return x1_pencil_stride(b); }
long long sweep_threads(const BView &b, int dir, int seg_target) {
  const SweepRange r = sweep_range(b, dir, seg_target);
  return (long long)r.na * r.nc * r.nseg;
}

template <int RECON, bool MINK>
static void x1_prepare_t(size_t smem) {
  static size_t set = 0;  // largest dynamic shared memory already allowed
  if (smem > set) {
    cudaFuncSetAttribute(kb_flux_x1<RECON, MINK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set = smem;
  }
}

template <int RECON, bool MINK>
static void x1_batched_t(const Par &p, const BView *views, const WorkItem *items, int nitems, int grid, size_t smem,
                         const CUtensorMap *maps, const int *modes, unsigned int *err, cudaStream_t s) {
  auto kern = kb_flux_x1<RECON, MINK>;
  x1_prepare_t<RECON, MINK>(smem);
  kern<<<persistent_grid(kern, 32 * X1_WARPS, smem, nitems, grid), 32 * X1_WARPS, smem, s>>>(
      p, views, items, nitems, maps, modes, err);
}

template <int RECON, bool MINK>
static void sweep_batched_t(const Par &p, int dir, const BView *views, const WorkItem *items, int nitems, int grid,
                            int seg_target, cudaStream_t s) {
  if (dir == 1)
    kb_flux_sweep<RECON, MINK, 1><<<persistent_grid(kb_flux_sweep<RECON, MINK, 1>, 128, 0, nitems, grid), 128, 0, s>>>(
        p, views, items, nitems, seg_target);
  else
    kb_flux_sweep<RECON, MINK, 2><<<persistent_grid(kb_flux_sweep<RECON, MINK, 2>, 128, 0, nitems, grid), 128, 0, s>>>(
        p, views, items, nitems, seg_target);
}

#define PHX_RECON_DISPATCH(FN, ...)                                                         \
  switch (p.recon) {                                                                        \
  case PHX_RECON_WENO5Z:                                                                    \
    mink ? FN<PHX_RECON_WENO5Z, true>(__VA_ARGS__) : FN<PHX_RECON_WENO5Z, false>(__VA_ARGS__); \
    break;                                                                                  \
  case PHX_RECON_MP5:                                                                       \
    mink ? FN<PHX_RECON_MP5, true>(__VA_ARGS__) : FN<PHX_RECON_MP5, false>(__VA_ARGS__);     \
    break;                                                                                  \
  case PHX_RECON_LINEAR:                                                                    \
    mink ? FN<PHX_RECON_LINEAR, true>(__VA_ARGS__) : FN<PHX_RECON_LINEAR, false>(__VA_ARGS__); \
    break;                                                                                  \
  default:                                                                                  \
    mink ? FN<PHX_RECON_CONSTANT, true>(__VA_ARGS__) : FN<PHX_RECON_CONSTANT, false>(__VA_ARGS__); \
    break;                                                                                  \
  }

void launch_flux_x1_batched(const Par &p, bool mink, const BView *views, const WorkItem *items, int nitems, int grid,
                            size_t smem, const CUtensorMap *maps, const int *modes, unsigned int *err,
                            cudaStream_t s) {
  if (nitems <= 0) return;
  PHX_RECON_DISPATCH(x1_batched_t, p, views, items, nitems, grid, smem, maps, modes, err, s)
}

void prepare_flux_x1_batched(const Par &p, bool mink, size_t smem) {
  PHX_RECON_DISPATCH(x1_prepare_t, smem)
}

void launch_flux_sweep_batched(const Par &p, bool mink, int dir, const BView *views, const WorkItem *items,
                               int nitems, int grid, int seg_target, cudaStream_t s) {
  if (nitems <= 0) return;
  PHX_RECON_DISPATCH(sweep_batched_t, p, dir, views, items, nitems, grid, seg_target, s)
}

}  // namespace phx
