// Device helpers of the bulk-copy staged step kernels (box_tma.cu,
// box_rows.cu): mbarriers with bounded waits, 1D bulk copies (TMA) between
// global and shared memory in both directions, the proxy fence and the
// consumer-warp barrier, and a fixed-divisor division.  Inline PTX for
// sm_103a.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lbm {

constexpr uint64_t kDrainLimitNs = 500000000ull;  // 0.5 s for each copy in flight after a wait gave up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait for phase `parity` of the barrier, giving up after limit_ns
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
  if(mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while(!mbar_try_wait(bar, parity))
    if(global_ns() - t0 > limit_ns) return false;
  return true;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst), "l"(src),
               "r"(bytes), "r"(bar)
               : "memory");
}

// shared -> global bulk copy (bulk-group completion); both addresses and the
// size are multiples of 16 bytes
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// all but the newest N bulk groups of this thread have finished reading shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// all bulk groups of this thread are complete (their writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// generic-proxy writes to shared memory become visible to later bulk copies
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// barrier 1 over the first `count` threads after warp 0 (the consumer warps)
__device__ __forceinline__ void consumers_sync(int count) { asm volatile("barrier.cta.sync 1, %0;" ::"r"(count) : "memory"); }
// the same barrier, returning whether `pred` held in every consumer thread
__device__ __forceinline__ bool consumers_all(bool pred, int count) {
  uint32_t out;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "barrier.cta.red.and.pred p, 1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(out)
      : "r"(static_cast<uint32_t>(pred)), "r"(count)
      : "memory");
  return out != 0;
}

// n / d for n < 2^31 by multiply-high (Granlund-Montgomery, round-up
// multiplier): d fixed per launch, m and l set on the host
struct FastDiv {
  uint32_t d, m;
  int      l;
};

inline FastDiv make_fastdiv(uint32_t d) {
  int l = 0;
  while((uint64_t(1) << l) < d) ++l;
  const uint64_t m = ((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d + 1;
  return FastDiv{d, static_cast<uint32_t>(m), l};
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) { return (__umulhi(n, f.m) + n) >> f.l; }


}  // namespace lbm
