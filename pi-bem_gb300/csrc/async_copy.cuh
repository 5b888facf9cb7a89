// Shared-memory barriers and bulk asynchronous copies (inline PTX, sm_90 and
// later): mbarrier init / arrive / expect-tx / try-wait and the global ->
// shared cp.async.bulk that completes its bytes on an mbarrier.
#pragma once

#include <cstdint>

namespace pibem
{
  __device__ inline uint32_t smem_u32(const void *p)
  {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
  }

  __device__ inline bool mbar_try(uint32_t addr, uint32_t parity)
  {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(addr), "r"(parity)
                 : "memory");
    return done != 0;
  }

  // Wait for the phase with the given parity, at most `limit` polls.
  __device__ inline bool mbar_wait_bounded(uint32_t addr, uint32_t parity, long limit)
  {
    for (long it = 0; it < limit; ++it)
      if (mbar_try(addr, parity))
        return true;
    return false;
  }

  __device__ inline void mbar_init(uint32_t addr, uint32_t count)
  {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(addr), "r"(count) : "memory");
  }

  __device__ inline void mbar_init_fence()
  {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  __device__ inline void mbar_arrive(uint32_t addr)
  {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" : : "r"(addr) : "memory");
  }

  __device__ inline void mbar_arrive_expect_tx(uint32_t addr, uint32_t bytes)
  {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :
                 : "r"(addr), "r"(bytes)
                 : "memory");
  }

  // global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
  __device__ inline void bulk_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar)
  {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :
                 : "r"(dst), "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
  }
} // namespace pibem
