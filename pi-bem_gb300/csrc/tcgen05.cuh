// 5th-generation tensor-core helpers (inline PTX, sm_100-class): the
// 128-byte-swizzled K-major shared-memory layout and its matrix descriptor,
// MMA completion to an mbarrier, and 32-lane tensor-memory loads.
#pragma once

#include <cstdint>

namespace pibem
{
  // Byte offset of element (row, k) of a 128-byte-swizzled K-major tile of
  // 4-byte elements (0 <= k < 32): 8-row atoms of 1024 bytes, row r of an
  // atom at r * 128, 16-byte chunk c of the row at position c ^ (r & 7).
  __host__ __device__ inline uint32_t sw128_off(int row, int k)
  {
    return uint32_t((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 2) ^ row) & 7) << 4) +
                    (k & 3) * 4);
  }

  // Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
  // 1024 bytes apart (stride byte offset); the leading byte offset is unused
  // for swizzled K-major operands.  A K-step of 8 TF32 values inside the
  // 128-byte line advances the start address by 32 bytes.
  __device__ inline uint64_t smem_desc_sw128(uint32_t saddr)
  {
    uint64_t d = 0;
    d |= uint64_t((saddr >> 4) & 0x3FFFu);
    d |= uint64_t(1) << 16;         // leading byte offset (unused), 16 bytes
    d |= uint64_t(1024 >> 4) << 32; // stride byte offset
    d |= uint64_t(1) << 46;         // descriptor version of sm_100-class tensor cores
    d |= uint64_t(2) << 61;         // swizzle mode: 128 bytes
    return d;                       // base offset 0 (atoms are 1024-byte aligned)
  }

  __device__ inline void mma_commit(uint32_t mbar)
  {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :
                 : "r"(mbar)
                 : "memory");
  }

  __device__ inline void tmem_ld32(uint32_t taddr, float (&v)[32])
  {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                   "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                   "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                   "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j)
      v[j] = __uint_as_float(r[j]);
  }

  // 32 columns of the warp's 32 lanes, without waiting (tcgen05.wait::ld
  // before the registers are used)
  __device__ inline void tmem_ld32_nowait(uint32_t taddr, uint32_t (&r)[32])
  {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                   "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                   "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                   "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
  }

  // The same layout for 2-byte elements (0 <= k < 64, 8 per 16-byte chunk).
  __host__ __device__ inline uint32_t sw128_off_b16(int row, int k)
  {
    return uint32_t((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 3) ^ row) & 7) << 4) +
                    (k & 7) * 2);
  }
} // namespace pibem
