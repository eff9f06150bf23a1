// phx_bulk.cuh -- bulk global->shared copies (cp.async.bulk) completing on
// an mbarrier, with a bounded wait.
#pragma once
#include <cstdint>

namespace phx {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Upper bound on mbarrier polls before a kernel reports ERR_TIMEOUT.  Each
// try_wait may itself suspend for a while, so the bound is kept at ~1e6
// polls (a bulk copy completes within microseconds).
constexpr long long MBAR_SPIN_LIMIT = 1ll << 20;
// The sticky error bit a timed-out wait sets (phx_kernels.cuh: ERR_TIMEOUT).
constexpr unsigned int MBAR_ERR_TIMEOUT = 4u;

// Block-wide bounded wait for phase `phase` of bar.  Every thread polls at
// most `limit` times and the block agrees on the outcome
// (__syncthreads_and).  When the phase did not complete, every thread waits
// once more (again at most `limit` polls) for copies that may still be in
// flight, thread 0 sets MBAR_ERR_TIMEOUT in *err, and every thread returns
// false: the caller returns without touching the staged data.
__device__ __forceinline__ bool mbar_wait_block(uint64_t *bar, unsigned phase, long long limit, unsigned int *err) {
  bool done = false;
  for (long long spins = 0; spins < limit && !done; spins++) done = mbar_try_wait(bar, phase);
  if (__syncthreads_and(done)) return true;
  for (long long spins = 0; spins < limit && !done; spins++) done = mbar_try_wait(bar, phase);
  if (threadIdx.x == 0) atomicOr(err, MBAR_ERR_TIMEOUT);
  __syncthreads();
  return false;
}

}  // namespace phx
