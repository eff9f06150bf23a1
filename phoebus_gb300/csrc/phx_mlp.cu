// phx_mlp.cu -- the learned con2prim start: packing, feature extraction,
// tensor-core inference and FP32 training kernels (no reference
// counterpart; the network only chooses where the reference's unchanged
// FP64 regula falsi starts, root_find.hpp:110-167).
//
// Training (k_mlp_grad + k_mlp_adamw): one CTA of 256 threads works on tiles
// of 64 samples with all weights and activations in shared memory.  Forward
// and backward are register-tiled FP32 products (each thread a 4 x 4 block);
// the weight-gradient products walk the sample index in a lane-rotated order
// so that the shared-memory reads of a warp fall in distinct banks.  Weight
// gradients stay in registers over a CTA's tiles and are added to the global
// gradient once per CTA.  The forward pass multiplies BF16-rounded weights
// and inputs, as the tensor-core inference does (the gradient passes straight
// through the rounding).
#include "phx_mlp.cuh"

namespace phx {

// ------------------------------------------------------------------ packing
__device__ __forceinline__ float mlp_w(const float *theta, int off, int N, int K, int n, int k) {
  return (n < N && k < K) ? theta[off + n * K + k] : 0.0f;
}

__global__ void k_mlp_pack(const float *theta, MlpPacked *out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int E1 = 64 * 16, E2 = 64 * 64, E4 = 16 * 64;
  if (t < E1 + 2 * E2 + E4) {
    // element (n, k) of an N x K weight matrix, K-major core-matrix layout
    int e = t, off, N, K, KP;
    uint16_t *dst;
    if (e < E1) {
      off = MLP_OFF_W1, N = 64, K = PHX_MLP_IN, KP = 16, dst = out->w1;
    } else if ((e -= E1) < E2) {
      off = MLP_OFF_W2, N = 64, K = 64, KP = 64, dst = out->w2;
    } else if ((e -= E2) < E2) {
      off = MLP_OFF_W3, N = 64, K = 64, KP = 64, dst = out->w3;
    } else {
      e -= E2;
      off = MLP_OFF_W4, N = PHX_MLP_OUT, K = 64, KP = 64, dst = out->w4;
    }
    const int n = e / KP, k = e % KP;
    dst[kmaj_off(n, k, KP) / 2] = __bfloat16_as_ushort(__float2bfloat16_rn(mlp_w(theta, off, N, K, n, k)));
  } else if ((t -= E1 + 2 * E2 + E4) < 64 * 3 + 8) {
    if (t < 64)
      out->b1[t] = theta[MLP_OFF_B1 + t];
    else if (t < 128)
      out->b2[t - 64] = theta[MLP_OFF_B2 + t - 64];
    else if (t < 192)
      out->b3[t - 128] = theta[MLP_OFF_B3 + t - 128];
    else
      out->b4[t - 192] = (t - 192) < PHX_MLP_OUT ? theta[MLP_OFF_B4 + t - 192] : 0.0f;
  }
}

void launch_mlp_pack(const float *theta, MlpPacked *out, cudaStream_t s) {
  const int n = 64 * 16 + 2 * 64 * 64 + 16 * 64 + 64 * 3 + 8;
  k_mlp_pack<<<(n + 255) / 256, 256, 0, s>>>(theta, out);
}

// ------------------------------------------------------------- input box
// Floats ordered as ints: non-negative floats keep their bits, negative ones
// flip the magnitude bits, so int order equals float order (NaN excluded).
__device__ __forceinline__ int mlp_fkey(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float mlp_funkey(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

__global__ void k_mlp_box_reset(MlpPacked *out) {
  const int c = threadIdx.x;
  if (c < 8) {
    out->xlo[c] = -INFINITY;
    out->xhi[c] = INFINITY;
  }
}

__global__ void k_mlp_box_init(int *keys) {
  const int c = threadIdx.x;
  if (c < PHX_MLP_IN) {
    keys[c] = 0x7fffffff;                // running min
    keys[PHX_MLP_IN + c] = (int)0x80000000;  // running max
  }
}

__global__ void __launch_bounds__(256) k_mlp_box_reduce(const float *x, long long n, int *keys) {
  __shared__ int smin[PHX_MLP_IN], smax[PHX_MLP_IN];
  if (threadIdx.x < PHX_MLP_IN) {
    smin[threadIdx.x] = 0x7fffffff;
    smax[threadIdx.x] = (int)0x80000000;
  }
  __syncthreads();
  for (int c = 0; c < PHX_MLP_IN; c++) {
    int lo = 0x7fffffff, hi = (int)0x80000000;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
      const float f = x[c * n + q];
      if (isfinite(f)) {
        lo = min(lo, mlp_fkey(f));
        hi = max(hi, mlp_fkey(f));
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&smin[c], lo);
      atomicMax(&smax[c], hi);
    }
  }
  __syncthreads();
  if (threadIdx.x < PHX_MLP_IN) {
    atomicMin(&keys[threadIdx.x], smin[threadIdx.x]);
    atomicMax(&keys[PHX_MLP_IN + threadIdx.x], smax[threadIdx.x]);
  }
}

__global__ void k_mlp_box_finish(const int *keys, float margin, MlpPacked *out) {
  const int c = threadIdx.x;
  if (c < PHX_MLP_IN) {
    const int klo = keys[c], khi = keys[PHX_MLP_IN + c];
    if (klo > khi) {  // no finite sample: leave the input unbounded
      out->xlo[c] = -INFINITY;
      out->xhi[c] = INFINITY;
      return;
    }
    const float lo = mlp_funkey(klo), hi = mlp_funkey(khi), w = margin * (hi - lo);
    out->xlo[c] = lo - w;
    out->xhi[c] = hi + w;
  } else if (c < 8) {
    out->xlo[c] = -INFINITY;
    out->xhi[c] = INFINITY;
  }
}

void launch_mlp_box_reset(MlpPacked *out, cudaStream_t s) { k_mlp_box_reset<<<1, 32, 0, s>>>(out); }

void launch_mlp_box_from(const float *x, long long n, float margin, int *keys, MlpPacked *out, cudaStream_t s) {
  k_mlp_box_init<<<1, 32, 0, s>>>(keys);
  if (n > 0) {
    long long grid = (n + 255) / 256;
    if (grid > 152 * 4) grid = 152 * 4;
    k_mlp_box_reduce<<<(unsigned)grid, 256, 0, s>>>(x, n, keys);
  }
  k_mlp_box_finish<<<1, 32, 0, s>>>(keys, margin, out);
}

// ----------------------------------------------------------------- features
template <bool MINK>
__global__ void __launch_bounds__(128) k_mlp_features(Par p, long long n, const double *cons, const double *geom,
                                                      const double *coords, float *x) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  Pt g{};
  if constexpr (!MINK) load_pt_flat(geom, n, q, g);
  double U[PHX_NCONS];
  for (int m = 0; m < PHX_NCONS; m++) U[m] = cons[m * n + q];
  const double x1 = coords ? coords[q] : 0.0, x2 = coords ? coords[n + q] : 0.0,
               x3 = coords ? coords[2 * n + q] : 0.0;
  Residual res;
  double rcon[3], rcov[3], bu[3], Bprim[3] = {0.0, 0.0, 0.0}, bdotr = 0.0;
  float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (c2p_setup<MINK>(p, g, U, x1, x2, x3, res, rcon, rcov, bu, Bprim, bdotr)) c2p_features(res, f);
  for (int c = 0; c < PHX_MLP_IN; c++) x[c * n + q] = f[c];
}

void launch_mlp_features(const Par &p, long long n, const double *cons, const double *geom, const double *coords,
                         float *x, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (geom)
    k_mlp_features<false><<<grid, 128, 0, s>>>(p, n, cons, geom, coords, x);
  else
    k_mlp_features<true><<<grid, 128, 0, s>>>(p, n, cons, geom, coords, x);
}

// --------------------------------------------------- inference on features
struct MlpFwdSmem {
  MlpPacked w;
  MlpTile tile;
};
// more than 1/9 of an SM's shared memory: at most 8 CTAs resident, whose TMEM
// columns (8 x 64) fit the SM's 512, so tcgen05.alloc never waits on another CTA
static_assert(sizeof(MlpFwdSmem) * 9 > 228 * 1024, "TMEM columns of the resident CTAs");

__global__ void __launch_bounds__(128) k_mlp_forward(const MlpPacked *mlp, long long n, const float *x, float *out,
                                                     unsigned int *err) {
  extern __shared__ __align__(128) unsigned char fwd_dyn[];
  __shared__ __align__(8) uint64_t bar;
  MlpFwdSmem *S = reinterpret_cast<MlpFwdSmem *>(fwd_dyn);
  if (!mlp_stage_weights(&S->w, mlp, &bar, err)) return;
  mlp_tc_init(&S->tile);
  unsigned phase = 0;
  for (long long base = (long long)blockIdx.x * 128; base < n; base += (long long)gridDim.x * 128) {
    const long long q = base + threadIdx.x;
    float f[6];
    for (int c = 0; c < 6; c++) f[c] = q < n ? x[c * n + q] : 0.0f;
    float o0, o1;
    if (!mlp_cta_forward(S->w, &S->tile, f, phase, err, o0, o1)) break;
    if (q < n) {
      out[q] = o0;
      out[n + q] = o1;
    }
  }
  mlp_tc_finish(&S->tile);
}

void launch_mlp_forward(const MlpPacked *mlp, long long n, const float *x, float *out, unsigned int *err,
                        cudaStream_t s) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpFwdSmem));
    attr = true;
  }
  long long grid = (n + 127) / 128;
  if (grid > 152 * 8) grid = 152 * 8;
  k_mlp_forward<<<(unsigned)grid, 128, sizeof(MlpFwdSmem), s>>>(mlp, n, x, out, err);
}

// ------------------------------------------------------------------ training
constexpr int TR_T = 64;         // samples per tile
constexpr int TR_THREADS = 256;  // 16 x 16 threads, each a 4 x 4 block of a 64 x 64 product
constexpr float GELU_C = 0.7978845608028654f;
constexpr float GELU_A = 0.044715f;

// Every array starts on a 16-byte boundary (float4 accesses).
struct TrainSmem {
  alignas(16) float W1T[PHX_MLP_IN][64];             // [in][out] for the forward product
  alignas(16) float W2[64 * 64];                     // [out][in] for the backward product
  alignas(16) float W2T[64 * 64];                    // [in][out] for the forward product
  alignas(16) float W3[64 * 64];
  alignas(16) float W3T[64 * 64];
  alignas(16) float W4[PHX_MLP_OUT][64];
  alignas(16) float b1[64];
  alignas(16) float b2[64];
  alignas(16) float b3[64];
  alignas(16) float b4[4];
  alignas(16) float xT[8][TR_T];                     // BF16-rounded inputs [feature][sample]
  alignas(16) float z1[64 * TR_T];                   // pre-activations [neuron][sample]
  alignas(16) float z2[64 * TR_T];
  alignas(16) float z3[64 * TR_T];
  alignas(16) float a1[64 * TR_T];                   // GELU outputs
  alignas(16) float a2[64 * TR_T];
  alignas(16) float a3[64 * TR_T];
  alignas(16) float d[64 * TR_T];                    // back-propagated error
  alignas(16) float og[PHX_MLP_OUT][TR_T];           // dL/d(outputs)
  alignas(16) float y[TR_T];
  alignas(16) float valid[TR_T];
};
static_assert(sizeof(TrainSmem) <= 227 * 1024, "training tile exceeds shared memory");

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ float gelu_t(float z, float &t) {
  t = tanhf(GELU_C * (z + GELU_A * z * z * z));
  return 0.5f * z * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float t = tanhf(GELU_C * (z + GELU_A * z * z * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * GELU_C * (1.0f + 3.0f * GELU_A * z * z);
}

// Z = WT^T X + b, A = GELU(Z) for a [64][TR_T] tile; WT: [K][64], X: [K][TR_T].
template <int K>
__device__ __forceinline__ void tr_forward(const float *WT, const float *bias, const float *X, float *Z, float *A) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int o0 = ty * 4, s0 = tx * 4;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = bias[o0 + i];
#pragma unroll 8
  for (int k = 0; k < K; k++) {
    const float4 w = *reinterpret_cast<const float4 *>(WT + k * 64 + o0);
    const float4 xv = *reinterpret_cast<const float4 *>(X + k * TR_T + s0);
    const float wv[4] = {w.x, w.y, w.z, w.w}, xx[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(wv[i], xx[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    float4 zv, av;
    float t;
    zv.x = acc[i][0];
    zv.y = acc[i][1];
    zv.z = acc[i][2];
    zv.w = acc[i][3];
    av.x = gelu_t(zv.x, t);
    av.y = gelu_t(zv.y, t);
    av.z = gelu_t(zv.z, t);
    av.w = gelu_t(zv.w, t);
    *reinterpret_cast<float4 *>(Z + (o0 + i) * TR_T + s0) = zv;
    *reinterpret_cast<float4 *>(A + (o0 + i) * TR_T + s0) = av;
  }
}

// Dprev[k][s] = (sum_o W[o][k] D[o][s]) * GELU'(Zprev[k][s]); W: [64][64].
__device__ __forceinline__ void tr_backward(const float *W, const float *D, const float *Zprev, float *Dprev) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int k0 = ty * 4, s0 = tx * 4;
  float acc[4][4] = {};
#pragma unroll 8
  for (int o = 0; o < 64; o++) {
    const float4 w = *reinterpret_cast<const float4 *>(W + o * 64 + k0);
    const float4 dv = *reinterpret_cast<const float4 *>(D + o * TR_T + s0);
    const float wv[4] = {w.x, w.y, w.z, w.w}, dd[4] = {dv.x, dv.y, dv.z, dv.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(wv[i], dd[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int e = (k0 + i) * TR_T + s0 + j;
      Dprev[e] = acc[i][j] * gelu_grad(Zprev[e]);
    }
}

// G[o][k] += sum_s D[o][s] A[k][s] for this thread's 4 x 4 block, with the
// sample index rotated per lane (bank-conflict-free shared reads).
__device__ __forceinline__ void tr_wgrad(const float *D, const float *A, float G[4][4]) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  const int o0 = ty * 4, k0 = tx * 4, rot = tx + 16 * (ty & 1);
#pragma unroll 4
  for (int s = 0; s < TR_T; s++) {
    const int sr = (s + rot) & (TR_T - 1);
    float dv[4], av[4];
#pragma unroll
    for (int i = 0; i < 4; i++) dv[i] = D[(o0 + i) * TR_T + sr];
#pragma unroll
    for (int j = 0; j < 4; j++) av[j] = A[(k0 + j) * TR_T + sr];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) G[i][j] = fmaf(dv[i], av[j], G[i][j]);
  }
}

__device__ __forceinline__ float row_sum_rot(const float *D, int o) {
  float acc = 0.0f;
  for (int s = 0; s < TR_T; s++) acc += D[o * TR_T + ((s + o) & (TR_T - 1))];
  return acc;
}

// Gradient of the mean Gaussian NLL over count samples starting at off
// (x [6][stride], y [stride]); adds inv_batch-weighted sums into grad and
// loss (which the caller zeroes).
__global__ void __launch_bounds__(TR_THREADS) k_mlp_grad(const float *theta, const float *x, const float *y,
                                                         long long stride, long long off, long long count,
                                                         float inv_batch, float *grad, float *loss) {
  extern __shared__ __align__(16) unsigned char tr_dyn[];
  TrainSmem &S = *reinterpret_cast<TrainSmem *>(tr_dyn);
  const int tid = threadIdx.x;
  for (int e = tid; e < 64 * 64; e += TR_THREADS) {
    const int o = e >> 6, k = e & 63;
    const float w2 = bf16r(theta[MLP_OFF_W2 + e]), w3 = bf16r(theta[MLP_OFF_W3 + e]);
    S.W2[e] = w2;
    S.W2T[k * 64 + o] = w2;
    S.W3[e] = w3;
    S.W3T[k * 64 + o] = w3;
  }
  for (int e = tid; e < 64 * PHX_MLP_IN; e += TR_THREADS) {
    const int o = e / PHX_MLP_IN, k = e % PHX_MLP_IN;
    S.W1T[k][o] = bf16r(theta[MLP_OFF_W1 + e]);
  }
  if (tid < PHX_MLP_OUT * 64) S.W4[tid >> 6][tid & 63] = bf16r(theta[MLP_OFF_W4 + tid]);
  if (tid < 64) {
    S.b1[tid] = theta[MLP_OFF_B1 + tid];
    S.b2[tid] = theta[MLP_OFF_B2 + tid];
    S.b3[tid] = theta[MLP_OFF_B3 + tid];
  }
  if (tid < PHX_MLP_OUT) S.b4[tid] = theta[MLP_OFF_B4 + tid];

  float gW2[4][4] = {}, gW3[4][4] = {};
  float gW1[2] = {0.f, 0.f}, gW4 = 0.f, gb1 = 0.f, gb2 = 0.f, gb3 = 0.f, gb4 = 0.f;
  float lsum = 0.f;
  const long long ntiles = (count + TR_T - 1) / TR_T;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    __syncthreads();  // weights staged / previous tile done
    const long long s0 = tile * TR_T;
    for (int e = tid; e < 8 * TR_T; e += TR_THREADS) {
      const int c = e / TR_T, s = e % TR_T;
      const bool ok = c < PHX_MLP_IN && s0 + s < count;
      S.xT[c][s] = ok ? bf16r(x[(long long)c * stride + off + s0 + s]) : 0.0f;
    }
    if (tid < TR_T) {
      const bool ok = s0 + tid < count;
      S.y[tid] = ok ? y[off + s0 + tid] : 0.0f;
      S.valid[tid] = ok ? 1.0f : 0.0f;
    }
    __syncthreads();
    tr_forward<PHX_MLP_IN>(&S.W1T[0][0], S.b1, &S.xT[0][0], S.z1, S.a1);
    __syncthreads();
    tr_forward<64>(S.W2T, S.b2, S.a1, S.z2, S.a2);
    __syncthreads();
    tr_forward<64>(S.W3T, S.b3, S.a2, S.z3, S.a3);
    __syncthreads();
    if (tid < TR_T) {  // outputs and dL/d(outputs) of sample tid
      float o[PHX_MLP_OUT];
      for (int c = 0; c < PHX_MLP_OUT; c++) {
        float acc = S.b4[c];
        for (int k = 0; k < 64; k++) acc = fmaf(S.W4[c][k], S.a3[k * TR_T + tid], acc);
        o[c] = acc;
      }
      const float v = S.valid[tid];
      const float e = S.y[tid] - o[0];
      const float s2 = expf(-2.0f * o[1]);
      lsum += v * inv_batch * (0.5f * e * e * s2 + o[1]);
      S.og[0][tid] = v * inv_batch * (-e * s2);
      S.og[1][tid] = v * inv_batch * (1.0f - e * e * s2);
    }
    __syncthreads();
    for (int e = tid; e < 64 * TR_T; e += TR_THREADS) {  // delta of layer 3
      const int k = e / TR_T, s = e % TR_T;
      S.d[e] = (S.W4[0][k] * S.og[0][s] + S.W4[1][k] * S.og[1][s]) * gelu_grad(S.z3[e]);
    }
    if (tid < PHX_MLP_OUT * 64) {  // W4: o = tid / 64, k = tid % 64
      const int o = tid >> 6, k = tid & 63;
      for (int s = 0; s < TR_T; s++) {
        const int sr = (s + k) & (TR_T - 1);
        gW4 = fmaf(S.og[o][sr], S.a3[k * TR_T + sr], gW4);
      }
    }
    if (tid < PHX_MLP_OUT)
      for (int s = 0; s < TR_T; s++) gb4 += S.og[tid][s];
    __syncthreads();
    tr_wgrad(S.d, S.a2, gW3);
    if (tid < 64) gb3 += row_sum_rot(S.d, tid);
    tr_backward(S.W3, S.d, S.z2, S.z3);  // delta of layer 2 into z3 (no longer needed)
    __syncthreads();
    tr_wgrad(S.z3, S.a1, gW2);
    if (tid < 64) gb2 += row_sum_rot(S.z3, tid);
    tr_backward(S.W2, S.z3, S.z1, S.d);  // delta of layer 1
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int e = tid + r * TR_THREADS;
      if (e < 64 * PHX_MLP_IN) {
        const int o = e / PHX_MLP_IN, k = e % PHX_MLP_IN;
        float acc = 0.f;
        for (int s = 0; s < TR_T; s++) {
          const int sr = (s + o) & (TR_T - 1);
          acc = fmaf(S.d[o * TR_T + sr], S.xT[k][sr], acc);
        }
        gW1[r] += acc;
      }
    }
    if (tid < 64) gb1 += row_sum_rot(S.d, tid);
  }
  // one global add per parameter and CTA
  const int ty = tid >> 4, tx = tid & 15;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int e = (ty * 4 + i) * 64 + tx * 4 + j;
      atomicAdd(grad + MLP_OFF_W2 + e, gW2[i][j]);
      atomicAdd(grad + MLP_OFF_W3 + e, gW3[i][j]);
    }
  for (int r = 0; r < 2; r++) {
    const int e = tid + r * TR_THREADS;
    if (e < 64 * PHX_MLP_IN) atomicAdd(grad + MLP_OFF_W1 + e, gW1[r]);
  }
  if (tid < PHX_MLP_OUT * 64) atomicAdd(grad + MLP_OFF_W4 + tid, gW4);
  if (tid < 64) {
    atomicAdd(grad + MLP_OFF_B1 + tid, gb1);
    atomicAdd(grad + MLP_OFF_B2 + tid, gb2);
    atomicAdd(grad + MLP_OFF_B3 + tid, gb3);
  }
  if (tid < PHX_MLP_OUT) atomicAdd(grad + MLP_OFF_B4 + tid, gb4);
  if (tid < 32) {  // samples were owned by threads 0..63: two warps
    for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (tid == 0) atomicAdd(loss, lsum);
  } else if (tid < 64) {
    for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (tid == 32) atomicAdd(loss, lsum);
  }
}

void launch_mlp_grad(const float *theta, const float *x, const float *y, long long stride, long long off,
                     long long count, float inv_batch, float *grad, float *loss, cudaStream_t s) {
  if (count <= 0) return;
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
  }
  long long grid = (count + TR_T - 1) / TR_T;
  if (grid > nsm) grid = nsm;
  k_mlp_grad<<<(unsigned)grid, TR_THREADS, sizeof(TrainSmem), s>>>(theta, x, y, stride, off, count, inv_batch,
                                                                   grad, loss);
}

// AdamW with decoupled weight decay on the weight matrices (not the
// biases); c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t).  Zeroes grad.
__global__ void k_mlp_adamw(float *theta, float *grad, float *m, float *v, float lr, float b1, float b2, float eps,
                            float wd, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= PHX_MLP_NPARAM) return;
  const bool is_w = i < MLP_OFF_B1 || (i >= MLP_OFF_W2 && i < MLP_OFF_B2) || (i >= MLP_OFF_W3 && i < MLP_OFF_B3) ||
                    (i >= MLP_OFF_W4 && i < MLP_OFF_B4);
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float th = theta[i];
  theta[i] = th - lr * ((mi * c1) / (sqrtf(vi * c2) + eps) + (is_w ? wd : 0.0f) * th);
  grad[i] = 0.0f;
}

void launch_mlp_adamw(float *theta, float *grad, float *m, float *v, float lr, float b1, float b2, float eps,
                      float wd, float c1, float c2, cudaStream_t s) {
  k_mlp_adamw<<<(PHX_MLP_NPARAM + 255) / 256, 256, 0, s>>>(theta, grad, m, v, lr, b1, b2, eps, wd, c1, c2);
}

}  // namespace phx
