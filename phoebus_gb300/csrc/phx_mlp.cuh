// phx_mlp.cuh -- the learned con2prim start on the device (no reference
// counterpart): packed BF16 weights and the CTA-level tensor-core forward
// pass used inside the con2prim kernels.
//
// Network 6 -> 64 -> 64 -> 64 -> 2 with GELU (tanh form).  FP32 master
// parameters (phx_fluid.h, PHX_MLP_NPARAM) in the order W1[64][6], b1,
// W2[64][64], b2, W3[64][64], b3, W4[2][64], b4 (weights [out][in]).
//
// Inference: a CTA of 128 threads evaluates 128 zones as one M = 128 tile on
// the fifth-generation tensor cores.  Thread t writes its zone's layer input
// as row t of a BF16 operand tile in shared memory; one thread issues
// tcgen05.mma (kind::f16: BF16 operands, FP32 accumulate) with the layer's
// weights as the second operand, also in shared memory, and the accumulator
// (128 lanes x 64 FP32 columns) lands in tensor memory; tcgen05.commit
// arrives on an mbarrier when the products are done.  Each warp then reads
// its 32 lanes (rows) back with tcgen05.ld, adds the bias, applies GELU and
// writes the next layer's BF16 input tile.  Layer 1 is one K = 16 product
// (6 features, zero padded), layers 2 and 3 four K = 16 steps each, layer 4
// four steps with N = 16 (2 outputs, zero padded).
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

// Byte offset of element (r, k) of a BF16 matrix with K columns in the
// canonical K-major layout without swizzling that tcgen05.mma reads through
// a shared-memory descriptor: 8-row x 16-byte core matrices, the core
// matrices of one 8-row group adjacent along K (128 bytes apart: the
// descriptor's leading-dimension offset), the 8-row groups K * 16 bytes apart
// (its stride-dimension offset).
__host__ __device__ constexpr int kmaj_off(int r, int k, int K) {
  return (r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Weights as BF16 bit patterns in that layout (rows = output features,
// columns = input features), biases and the input box in FP32.
struct MlpPacked {
  alignas(128) uint16_t w1[64 * 16];  // N 64 x K 16 (6 inputs, zero padded)
  alignas(128) uint16_t w2[64 * 64];
  alignas(128) uint16_t w3[64 * 64];
  alignas(128) uint16_t w4[16 * 64];  // N 16 (2 outputs, zero padded) x K 64
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

// GELU, tanh form, with the hardware tanh approximation.
__device__ __forceinline__ float gelu_fast(float z) {
  const float u = 0.7978845608028654f * (z + 0.044715f * z * z * z);
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return 0.5f * z * (1.0f + t);
}

// ------------------------------------------------ tensor-core forward pass
// TMEM columns of the accumulator: 64 FP32 columns x 128 lanes.  A CTA of the
// inference kernels takes more than 1/8 of an SM's shared memory, so at most
// 8 are resident and their 8 x 64 columns fit the SM's 512.
constexpr uint32_t MLP_TMEM_COLS = 64;

// Per-CTA scratch: the BF16 layer-input tile (M 128 x K 64; layer 1 uses the
// K 16 layout in its first 4 KB), the MMA-completion mbarrier and the TMEM
// base address tcgen05.alloc returns.
struct MlpTile {
  alignas(128) uint16_t a[128 * 64];
  alignas(8) uint64_t bar;
  uint32_t tmem;
  uint32_t pad;
};

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading-
// dimension byte offset >> 4 (bits 16-29, here 128: core matrices adjacent
// along K), stride-dimension byte offset >> 4 (bits 32-45), the descriptor
// version 1 in bits 46-48, base offset 0, no swizzling (bits 61-63 = 0).
__device__ __forceinline__ uint64_t mlp_desc(const void *p, uint32_t sbo) {
  return (uint64_t)((smem_u32(p) & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 = 8 (M = 128) in bits 24-28.
__host__ __device__ constexpr uint32_t mlp_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mlp_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mlp_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (thread = lane),
// waited for inside the same statement.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float v[2]) {
  uint32_t r0, r1;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r0), "=r"(r1)
      : "r"(taddr)
      : "memory");
  v[0] = __uint_as_float(r0);
  v[1] = __uint_as_float(r1);
}

// CTA entry: thread 0 initialises the mbarrier, warp 0 allocates the TMEM
// columns; every thread then reads the base address.
__device__ __forceinline__ void mlp_tc_init(MlpTile *T) {
  if (threadIdx.x == 0) {
    mbar_init(&T->bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&T->tmem)),
                 "r"(MLP_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}
// CTA exit (every thread, after its last tcgen05.ld): warp 0 frees the columns.
__device__ __forceinline__ void mlp_tc_finish(MlpTile *T) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(T->tmem), "r"(MLP_TMEM_COLS)
                 : "memory");
}

// The layer input written by every thread becomes visible to the tensor
// cores (async proxy) and every thread's TMEM reads are complete; then thread
// 0 issues `nk` K = 16 steps of [A | a_sbo] x [W | w_sbo] into the TMEM
// columns and commits them to the mbarrier; every thread waits (bounded) for
// that phase.  False, with ERR_TIMEOUT set, when the wait gave up.
__device__ __forceinline__ bool mlp_tc_layer(MlpTile *T, const uint16_t *W, int nk, uint32_t a_sbo, uint32_t w_sbo,
                                             uint32_t idesc, unsigned &phase, unsigned int *err) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    for (int s = 0; s < nk; s++)
      mlp_mma(T->tmem, mlp_desc(T->a + s * 128, a_sbo), mlp_desc(W + s * 128, w_sbo), idesc, s > 0 ? 1u : 0u);
    mlp_commit(&T->bar);
  }
  const bool ok = mbar_wait_block(&T->bar, phase, MBAR_SPIN_LIMIT, err);
  phase ^= 1u;
  tc_fence_after();
  return ok;
}

// This thread's 64 accumulator columns + bias -> GELU -> BF16 row `row` of
// the next layer's K 64 input tile.
__device__ __forceinline__ void mlp_tc_activate(MlpTile *T, const float *bias, int row) {
  const uint32_t lane_base = (uint32_t)((threadIdx.x >> 5) * 32) << 16;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    float v[32];
    tmem_ld32(T->tmem + lane_base + (uint32_t)(32 * h), v);
#pragma unroll
    for (int g = 0; g < 4; g++) {
      uint4 q;
      const float *c = v + 8 * g;
      const float *b = bias + 32 * h + 8 * g;
      q.x = pack_bf16x2(gelu_fast(c[0] + b[0]), gelu_fast(c[1] + b[1]));
      q.y = pack_bf16x2(gelu_fast(c[2] + b[2]), gelu_fast(c[3] + b[3]));
      q.z = pack_bf16x2(gelu_fast(c[4] + b[4]), gelu_fast(c[5] + b[5]));
      q.w = pack_bf16x2(gelu_fast(c[6] + b[6]), gelu_fast(c[7] + b[7]));
      *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(T->a) + kmaj_off(row, 32 * h + 8 * g, 64)) = q;
    }
  }
}

// Forward pass of the CTA's 128 zones (thread t owns zone t: f its six
// features).  Every thread of the CTA calls it.  Returns this thread's
// outputs (o0 = ln mu, o1 = ln sigma); false, with ERR_TIMEOUT set, when a
// product did not complete within the bounded wait (every thread returns the
// same value; the caller stops using the network).
__device__ __forceinline__ bool mlp_cta_forward(const MlpPacked &S, MlpTile *T, const float f[6], unsigned &phase,
                                                unsigned int *err, float &o0, float &o1) {
  const int t = threadIdx.x;
  unsigned char *a = reinterpret_cast<unsigned char *>(T->a);
  uint4 x0, x1 = make_uint4(0u, 0u, 0u, 0u);
  x0.x = pack_bf16x2(f[0], f[1]);
  x0.y = pack_bf16x2(f[2], f[3]);
  x0.z = pack_bf16x2(f[4], f[5]);
  x0.w = 0u;
  *reinterpret_cast<uint4 *>(a + kmaj_off(t, 0, 16)) = x0;
  *reinterpret_cast<uint4 *>(a + kmaj_off(t, 8, 16)) = x1;
  if (!mlp_tc_layer(T, S.w1, 1, 16 * 16, 16 * 16, mlp_idesc(64), phase, err)) return false;
  mlp_tc_activate(T, S.b1, t);
  if (!mlp_tc_layer(T, S.w2, 4, 64 * 16, 64 * 16, mlp_idesc(64), phase, err)) return false;
  mlp_tc_activate(T, S.b2, t);
  if (!mlp_tc_layer(T, S.w3, 4, 64 * 16, 64 * 16, mlp_idesc(64), phase, err)) return false;
  mlp_tc_activate(T, S.b3, t);
  if (!mlp_tc_layer(T, S.w4, 4, 64 * 16, 64 * 16, mlp_idesc(16), phase, err)) return false;
  float o[2];
  tmem_ld2(T->tmem + ((uint32_t)((t >> 5) * 32) << 16), o);
  o0 = o[0] + S.b4[0];
  o1 = o[1] + S.b4[1];
  return true;
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
