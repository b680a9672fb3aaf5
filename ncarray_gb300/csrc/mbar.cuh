// Bounded mbarrier waits shared by the hand-written kernels (bulk-copy and
// TMA pipelines). A wait that does not complete within its limit returns
// false; the caller records NCA_ERR_TIMEOUT and stops instead of hanging.
#pragma once
#include <cstdint>

namespace nca_dev {

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// true once the phase of parity `parity` of the mbarrier at shared address bar has completed
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
  return ok != 0;
}

// waits at most limit_ns of %globaltimer; the clock is read only when the first try fails
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try(bar, parity)) return true;
    if (gtimer() - t0 > limit_ns) return false;
  }
}

}  // namespace nca_dev
