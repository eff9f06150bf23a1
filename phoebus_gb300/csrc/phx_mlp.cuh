// phx_mlp.cuh -- the learned con2prim start on the device (no reference
// counterpart): packed BF16 weights and the warp-level tensor-core forward
// pass used inside the con2prim kernels.
//
// Network 6 -> 64 -> 64 -> 64 -> 2 with GELU (tanh form).  FP32 master
// parameters (phx_fluid.h, PHX_MLP_NPARAM) in the order W1[64][6], b1,
// W2[64][64], b2, W3[64][64], b3, W4[2][64], b4 (weights [out][in]).
//
// Inference: one warp evaluates 32 zones as two 16-row tiles with
// mma.sync.m16n8k16 (BF16 operands, FP32 accumulate).  The weights are
// pre-packed in the B-fragment order of that instruction (per n-tile, k-step
// and lane one 8-byte pair), so a lane loads each fragment with one shared
// memory load; the accumulator fragments of one layer are the A fragments of
// the next (after GELU and BF16 rounding), so activations never leave
// registers.
#pragma once
#include <cuda_bf16.h>

#include "phx_bulk.cuh"
#include "phx_kernels.cuh"

namespace phx {

constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + PHX_MLP_HID * PHX_MLP_IN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + PHX_MLP_HID;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + PHX_MLP_HID * PHX_MLP_HID;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + PHX_MLP_HID;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + PHX_MLP_HID * PHX_MLP_HID;
constexpr int MLP_OFF_W4 = MLP_OFF_B3 + PHX_MLP_HID;
constexpr int MLP_OFF_B4 = MLP_OFF_W4 + PHX_MLP_OUT * PHX_MLP_HID;
static_assert(MLP_OFF_B4 + PHX_MLP_OUT == PHX_MLP_NPARAM, "parameter layout");

// B fragments: layer 1 (K 6 -> 16, N 64): 8 n-tiles x 1 k-step; layers 2, 3
// (K 64, N 64): 8 x 4; layer 4 (K 64, N 2 -> 8): 1 x 4.  32 lanes each.
struct MlpPacked {
  uint2 w1[8 * 1 * 32];
  uint2 w2[8 * 4 * 32];
  uint2 w3[8 * 4 * 32];
  uint2 w4[1 * 4 * 32];
  float b1[64], b2[64], b3[64], b4[8];
  // input box of the learned start: a cold zone whose features fall outside
  // [xlo, xhi] (the training set's range, widened) gets no bracket and keeps
  // the reference's start; (-inf, inf) when no box is set
  float xlo[8], xhi[8];
};
static_assert(sizeof(MlpPacked) % 16 == 0, "bulk copies move multiples of 16 bytes");

// Half-width of the learned bracket in standard deviations of ln(mu).
constexpr float MLP_BRACKET_K = 3.0f;

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// GELU, tanh form, with the hardware tanh approximation.
__device__ __forceinline__ float gelu_fast(float z) {
  const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return 0.5f * z * (1.0f + t);
}

// Accumulator fragments C[mt][nt] of a 64-wide layer -> GELU -> A fragments
// A[mt][ks] of the next layer (k-step ks spans n-tiles 2ks and 2ks+1).
__device__ __forceinline__ void mlp_act_to_a(const float C[2][8][4], uint32_t A[2][4][4]) {
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
      const float *c0 = C[mt][2 * ks], *c1 = C[mt][2 * ks + 1];
      A[mt][ks][0] = pack_bf16x2(gelu_fast(c0[0]), gelu_fast(c0[1]));
      A[mt][ks][1] = pack_bf16x2(gelu_fast(c0[2]), gelu_fast(c0[3]));
      A[mt][ks][2] = pack_bf16x2(gelu_fast(c1[0]), gelu_fast(c1[1]));
      A[mt][ks][3] = pack_bf16x2(gelu_fast(c1[2]), gelu_fast(c1[3]));
    }
}

__device__ __forceinline__ void mlp_hidden(const uint2 *W, const float *bias, const uint32_t A[2][4][4],
                                           float C[2][8][4], int lane) {
  const int tig = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const float bx = bias[nt * 8 + tig * 2], by = bias[nt * 8 + tig * 2 + 1];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      C[mt][nt][0] = bx;
      C[mt][nt][1] = by;
      C[mt][nt][2] = bx;
      C[mt][nt][3] = by;
    }
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
      const uint2 bf = W[(nt * 4 + ks) * 32 + lane];
      mma_bf16_16816(C[0][nt], A[0][ks], bf);
      mma_bf16_16816(C[1][nt], A[1][ks], bf);
    }
  }
}

// Forward pass for the 32 zones of a warp (lane L owns zone L).  f: this
// lane's 6 features.  xs: 128 words and os: 64 floats of per-warp shared
// scratch.  Returns this lane's outputs (o0 = ln mu, o1 = ln sigma).
__device__ __forceinline__ void mlp_warp_forward(const MlpPacked &S, const float f[6], uint32_t *xs, float *os,
                                                 float &o0, float &o1) {
  const int lane = threadIdx.x & 31, r = lane >> 2, tig = lane & 3;
  xs[lane * 4 + 0] = pack_bf16x2(f[0], f[1]);
  xs[lane * 4 + 1] = pack_bf16x2(f[2], f[3]);
  xs[lane * 4 + 2] = pack_bf16x2(f[4], f[5]);
  xs[lane * 4 + 3] = 0u;
  __syncwarp();
  uint32_t A[2][4][4];
  float C[2][8][4];
  {  // layer 1: K = 16 (6 features, zero padded), one k-step
    uint32_t A1[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      A1[mt][0] = xs[(mt * 16 + r) * 4 + tig];
      A1[mt][1] = xs[(mt * 16 + r + 8) * 4 + tig];
      A1[mt][2] = 0u;
      A1[mt][3] = 0u;
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const float bx = S.b1[nt * 8 + tig * 2], by = S.b1[nt * 8 + tig * 2 + 1];
      const uint2 bf = S.w1[nt * 32 + lane];
#pragma unroll
      for (int mt = 0; mt < 2; mt++) {
        C[mt][nt][0] = bx;
        C[mt][nt][1] = by;
        C[mt][nt][2] = bx;
        C[mt][nt][3] = by;
        mma_bf16_16816(C[mt][nt], A1[mt], bf);
      }
    }
  }
  mlp_act_to_a(C, A);
  mlp_hidden(S.w2, S.b2, A, C, lane);
  mlp_act_to_a(C, A);
  mlp_hidden(S.w3, S.b3, A, C, lane);
  mlp_act_to_a(C, A);
  float C4[2][4];
  {
    const float bx = S.b4[tig * 2], by = S.b4[tig * 2 + 1];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      C4[mt][0] = bx;
      C4[mt][1] = by;
      C4[mt][2] = bx;
      C4[mt][3] = by;
    }
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
      const uint2 bf = S.w4[ks * 32 + lane];
      mma_bf16_16816(C4[0], A[0][ks], bf);
      mma_bf16_16816(C4[1], A[1][ks], bf);
    }
  }
  if (tig == 0) {  // columns 0, 1 of rows r and r + 8 of each tile
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      os[(mt * 16 + r) * 2 + 0] = C4[mt][0];
      os[(mt * 16 + r) * 2 + 1] = C4[mt][1];
      os[(mt * 16 + r + 8) * 2 + 0] = C4[mt][2];
      os[(mt * 16 + r + 8) * 2 + 1] = C4[mt][3];
    }
  }
  __syncwarp();
  o0 = os[lane * 2];
  o1 = os[lane * 2 + 1];
  __syncwarp();
}

// True when all six features lie inside the network's input box (NaN: no).
__device__ __forceinline__ bool mlp_in_box(const MlpPacked &S, const float f[6]) {
  bool in = true;
#pragma unroll
  for (int c = 0; c < 6; c++) in = in && f[c] >= S.xlo[c] && f[c] <= S.xhi[c];
  return in;
}

// (m, lo, hi) in [0, 1] from the outputs: m = e^{o0}, half-width
// K e^{o1} in ln(mu), clipped at 1.  Non-finite outputs give a NaN bracket,
// which the root find does not try.
__device__ __forceinline__ void mlp_bracket(float o0, float o1, double lb[3]) {
  if (!(isfinite(o0) && isfinite(o1))) {
    lb[0] = lb[1] = lb[2] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const float w = MLP_BRACKET_K * expf(o1);
  lb[0] = (double)fminf(expf(o0), 1.0f);
  lb[1] = (double)fminf(expf(o0 - w), 1.0f);
  lb[2] = (double)fminf(expf(o0 + w), 1.0f);
}

// Bulk-copy the packed weights into shared memory: thread 0 issues one
// cp.async.bulk completing on bar, every thread polls the mbarrier a bounded
// number of times, and the block agrees on the outcome (__syncthreads_and).
// On a timeout the copy gets a second bounded wait before the block gives up
// with ERR_TIMEOUT; every thread returns the same value.
__device__ __forceinline__ bool mlp_stage_weights(MlpPacked *dst, const MlpPacked *src, uint64_t *bar,
                                                  unsigned int *err) {
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(bar, (unsigned)sizeof(MlpPacked));
    bulk_g2s(dst, src, (unsigned)sizeof(MlpPacked), bar);
  }
  return mbar_wait_block(bar, 0u, MBAR_SPIN_LIMIT, err);
}

}  // namespace phx
