// Tensor-core batched translation GEMM (M2L, M2M, L2L) of the FP32 operator,
// on the 5th-generation tensor cores: tcgen05.mma kind::tf32, accumulators in
// tensor memory, operator tiles staged by bulk TMA copies (cp.async.bulk).
//
// For one chunk of pairs sharing an operator T (K x K, scaled real form):
//     Y[row][k_out] = sum_{k_in} E[src(row)][k_in] T[k_out][k_in]
// with row = (pair, rhs); the rows of a chunk are consecutive in Y.  A tile is
// 128 rows:
//     A (M = 128 rows x K_in)  source expansions, gathered into shared memory
//     B (N = K_out x K_in)     operator, pre-laid-out image copied by TMA
//     D (128 x N) fp32         tensor memory
// FP32 accuracy from TF32 products by splitting both operands,
//     x = hi + lo (hi = TF32 rounding of x),   A B ~ Ah Bh + Al Bh + Ah Bl,
// all three products accumulated into the same FP32 accumulator.
//
// Persistent, warp-specialised pipeline (one block per SM, 13 warps):
//   warps 0-7  producers, two groups of 4 warps filling alternate stages: per
//              K chunk of 32, gather the 128 rows of A with coalesced loads
//              (lane = k, all 32 rows of a warp in flight), split hi/lo and
//              store them in the 128-byte-swizzled K-major layout (a row's 32
//              values fill one 128-byte line, 16-byte chunks XOR-permuted by
//              row & 7, so the stores are free of bank conflicts); the group's
//              first thread copies the chunk's B hi/lo images with
//              cp.async.bulk.  TC_STAGES-deep ring.
//   warp 12    one thread issues the MMAs (4 K-steps x 3 products per chunk)
//              into one of two tensor-memory accumulators and commits.
//   warps 8-11 epilogue: tcgen05.ld of the accumulator (warp 8+q reads lanes
//              32q..32q+31), staged per warp through shared memory and written
//              as contiguous 128-byte row segments.
// The accumulator double buffer lets the epilogue of tile i overlap the MMAs
// of tile i+1, and the stage ring lets the gathers run ahead of the MMAs.
//
// Every wait is bounded: on timeout a role records the failure in *err, raises
// a shared abort flag (so the other roles stop waiting), waits (bounded) for
// its copies and MMAs in flight, and the block frees its tensor memory and
// returns; the host turns the flag into PIBEM_ETIMEDOUT.
#include <algorithm>
#include <cstdint>
#include <cstring>

#include "async_copy.cuh"
#include "tcgen05.cuh"
#include "kernels.h"
#include "pdl.cuh"

namespace pibem
{
  namespace
  {
    constexpr int      TC_ROWS       = 128;
    constexpr int      TC_KC         = 32;  // K values per stage: one 128-byte line of TF32
    constexpr int      TC_GROUP      = 128; // producer group: 4 warps, one row per lane
    constexpr int      TC_EPI_WARP0  = 8;   // warps 8-11
    constexpr int      TC_MMA_WARP   = 12;
    constexpr int      TC_THREADS    = 13 * 32;
    constexpr int      TC_EPI_LD     = 33;  // staging row stride (floats)
    constexpr int      TC_ACC_COLS   = 128; // tensor-memory columns per accumulator (N <= 128)
    constexpr uint32_t TC_TMEM_COLS  = 2 * TC_ACC_COLS;
    constexpr uint32_t TC_A_BYTES    = TC_ROWS * TC_KC * 4; // 16 KB
    constexpr long     TC_SPIN_LIMIT = 1L << 26;

    __device__ inline float tf32_hi(float x)
    {
      uint32_t r;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
      return __uint_as_float(r);
    }

    // Bounded wait; gives up early once another role has raised the abort flag.
    __device__ inline bool mbar_wait(uint32_t addr, uint32_t parity, const volatile int *abort)
    {
      for (long it = 0; it < TC_SPIN_LIMIT; ++it)
        {
          if (mbar_try(addr, parity))
            return true;
          if ((it & 1023) == 1023 && *abort)
            return false;
        }
      return false;
    }

    // Bounded wait that ignores the abort flag (draining copies / MMAs in flight).
    __device__ inline void mbar_drain(uint32_t addr, uint32_t parity)
    {
      for (long it = 0; it < TC_SPIN_LIMIT; ++it)
        if (mbar_try(addr, parity))
          return;
    }

    __device__ inline void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    uint32_t accumulate)
    {
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "setp.ne.b32 p, %4, 0;\n\t"
                   "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                   :
                   : "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                   : "memory");
    }

    __host__ __device__ inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

    // a[s] = v / a[s] with s a run-time stage index: the loop over the
    // compile-time indices keeps the array in registers (no local memory)
    template <typename V, int N>
    __device__ __forceinline__ void put(V (&a)[N], int s, V v)
    {
#pragma unroll
      for (int j = 0; j < N; ++j)
        if (j == s)
          a[j] = v;
    }
    template <typename V, int N>
    __device__ __forceinline__ V get(const V (&a)[N], int s)
    {
      V v = a[0];
#pragma unroll
      for (int j = 1; j < N; ++j)
        if (j == s)
          v = a[j];
      return v;
    }

    // Shared-memory layout, byte offsets from the 1024-byte aligned base:
    // stages x [A hi | A lo | B hi | B lo], epilogue staging (per epilogue warp
    // the largest of a 32 x 33 column-chunk tile, its 32 rows x K row-major + 4
    // floats of alignment shift, and 32 rows of round_up(K, 4)), mbarriers.
    struct TcLayout
    {
      uint32_t b_bytes, stage_bytes, epi, epi_warp_floats, bars, total;
      __host__ __device__ TcLayout(int Np, int K, int stages)
      {
        b_bytes         = uint32_t(Np) * 128;
        stage_bytes     = 2 * TC_A_BYTES + 2 * b_bytes;
        epi             = uint32_t(stages) * stage_bytes;
        epi_warp_floats = uint32_t(round_up(32 * K + 4, 4));
        if (epi_warp_floats < 32 * TC_EPI_LD)
          epi_warp_floats = uint32_t(round_up(32 * TC_EPI_LD, 4));
        if (epi_warp_floats < uint32_t(32 * round_up(K, 4))) // scattered rows of round_up(K, 4)
          epi_warp_floats = uint32_t(32 * round_up(K, 4));
        bars  = epi + 4 * epi_warp_floats * 4;
        total = bars + (2 * uint32_t(stages) + 5) * 8;
      }
    };

    // ALL_LEVELS_M2L only names the instantiation used for the batched M2L of all
    // levels (so that profilers can select it); the code is the same.  TC_STAGES:
    // depth of the stage ring (3, or 2 where shared memory is short, p = 10).
    template <bool ALL_LEVELS_M2L, int TC_STAGES>
    __global__ void __launch_bounds__(TC_THREADS, 1)
      tc_gemm_kernel(int R, int K, int Np, int nkc, int chunk0, int n_chunks,
                     const int32_t *__restrict__ ch_start, const int32_t *__restrict__ ch_cnt,
                     const int32_t *__restrict__ ch_op, const int32_t *__restrict__ q_src,
                     const float *__restrict__ images, const float *__restrict__ E,
                     float *__restrict__ Y, const int32_t *__restrict__ yslot, int ldy,
                     int *__restrict__ err)
    {
      pdl_entry();
      extern __shared__ uint8_t smem_raw[];
      __shared__ uint32_t       tmem_slot;
      __shared__ volatile int   abort_flag;
      const TcLayout  lay(Np, K, TC_STAGES);
      const uint32_t  raw   = smem_u32(smem_raw);
      const uint32_t  base  = (raw + 1023u) & ~1023u;
      uint8_t        *gbase = smem_raw + (base - raw);
      const int       tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
      const uint32_t  bar0 = base + lay.bars;
      // mbarriers: full[s] (producers + copy bytes), empty[s] (MMA commit),
      // tfull[a] (MMA commit), tempty[a] (epilogue threads), drain (MMA commit)
      auto full   = [&](int s) { return bar0 + 8u * uint32_t(s); };
      auto empty  = [&](int s) { return bar0 + 8u * uint32_t(TC_STAGES + s); };
      auto tfull  = [&](int a) { return bar0 + 8u * uint32_t(2 * TC_STAGES + a); };
      auto tempty = [&](int a) { return bar0 + 8u * uint32_t(2 * TC_STAGES + 2 + a); };
      const uint32_t drain = bar0 + 8u * uint32_t(2 * TC_STAGES + 4);
      // each block takes a contiguous range of chunks: consecutive chunks mostly
      // share their operator, so a stage can keep its B tile (see the producers)
      const int ch_lo = chunk0 + int(int64_t(n_chunks) * blockIdx.x / gridDim.x);
      const int ch_hi = chunk0 + int(int64_t(n_chunks) * (blockIdx.x + 1) / gridDim.x);
      const size_t   op_img_floats = size_t(nkc) * Np * TC_KC; // one half of an operator image

      if (tid == 0)
        {
          abort_flag = 0;
          for (int s = 0; s < TC_STAGES; ++s)
            {
              mbar_init(full(s), TC_GROUP + 1);
              mbar_init(empty(s), 1);
            }
          for (int a = 0; a < 2; ++a)
            {
              mbar_init(tfull(a), 1);
              mbar_init(tempty(a), 4 * 32);
            }
          mbar_init(drain, 1);
          asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
      if (warp == 0)
        {
          asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                       :
                       : "r"(smem_u32(&tmem_slot)), "r"(TC_TMEM_COLS)
                       : "memory");
          asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tmem = tmem_slot;
      bool           ok   = true;

      auto fail = [&]() {
        if (ok)
          {
            ok         = false;
            abort_flag = 1;
            atomicExch(err, 1);
          }
      };

      if (warp < 8)
        {
          // ---------------- producers ----------------
          // Two groups of 4 warps fill alternate stages (group g takes the
          // stage iterations it with it % 2 == g), so two gathers are in flight;
          // warp w of a group owns tile rows 32 (w % 4) .. 32 (w % 4) + 31.
          const int grp = warp >> 2, gw = warp & 3, gtid = tid & (TC_GROUP - 1);
          int  it = 0;
          // (operator, K chunk) whose B images each stage holds after the
          // iterations so far (-1: none).  The copy decision is a function of
          // the iteration sequence alone, which both groups walk in full, so
          // both keep the same record, including the stages the other group
          // fills; a copy is skipped when the stage already holds the tile.
          int  held_op[TC_STAGES], held_kc[TC_STAGES];
#pragma unroll
          for (int s = 0; s < TC_STAGES; ++s)
            held_op[s] = held_kc[s] = -1;
          bool inflight[TC_STAGES];
          int  inflight_par[TC_STAGES];
#pragma unroll
          for (int s = 0; s < TC_STAGES; ++s)
            {
              inflight[s]     = false;
              inflight_par[s] = 0;
            }
          for (int ch = ch_lo; ok && ch < ch_hi; ++ch)
            {
              const int    start = ch_start[ch], rows_total = ch_cnt[ch] * R, op = ch_op[ch];
              const float *Bhi   = images + size_t(op) * 2 * op_img_floats;
              const float *Blo   = Bhi + op_img_floats;
              for (int t0 = 0; ok && t0 < rows_total; t0 += TC_ROWS)
                {
                  // source offset of row t0 + 32 gw + lane (-1: padding row); the
                  // host checks that every offset fits in 32 bits
                  int32_t my_src = -1;
                  {
                    const int i = t0 + 32 * gw + lane;
                    if (i < rows_total)
                      {
                        const int q = start + i / R, r = i - (i / R) * R;
                        my_src      = (q_src[q] * R + r) * K;
                      }
                  }
                  // every lane holds the offsets of the warp's 32 rows for all
                  // the tile's K chunks (one shuffle per row per tile)
                  int32_t srcs[32];
#pragma unroll
                  for (int u = 0; u < 32; ++u)
                    srcs[u] = __shfl_sync(0xffffffffu, my_src, u);
                  for (int kc = 0; kc < nkc; ++kc, ++it)
                    {
                      const int s = it % TC_STAGES, use = it / TC_STAGES;
                      if ((it & 1) != grp)
                        {
                          put(held_op, s, op); // the other group's iteration
                          put(held_kc, s, kc);
                          continue;
                        }
                      if (use > 0 && !mbar_wait(empty(s), uint32_t(use - 1) & 1u, &abort_flag))
                        {
                          fail();
                          break;
                        }
                      put(inflight, s, false);
                      const uint32_t st = base + uint32_t(s) * lay.stage_bytes;
                      if (gtid == 0)
                        {
                          if (get(held_op, s) == op && get(held_kc, s) == kc)
                            mbar_arrive(full(s)); // the stage already holds this B tile
                          else
                            {
                              mbar_arrive_expect_tx(full(s), 2 * lay.b_bytes);
                              bulk_copy(st + 2 * TC_A_BYTES, Bhi + size_t(kc) * Np * TC_KC,
                                        lay.b_bytes, full(s));
                              bulk_copy(st + 2 * TC_A_BYTES + lay.b_bytes,
                                        Blo + size_t(kc) * Np * TC_KC, lay.b_bytes, full(s));
                              put(inflight, s, true);
                              put(inflight_par, s, use & 1);
                            }
                        }
                      put(held_op, s, op);
                      put(held_kc, s, kc);
                      // all 32 row loads of the warp in flight at once (coalesced:
                      // lane = k), then split and store
                      const int   k    = kc * TC_KC + lane;
                      const bool k_ok = k < K;
                      float      x[32];
#pragma unroll
                      for (int u = 0; u < 32; ++u)
                        {
                          x[u] = (srcs[u] >= 0 && k_ok) ? E[srcs[u] + k] : 0.0f;
                        }
                      // stores by shared-window address (st.shared), hi then lo
                      const uint32_t a_hi = st + uint32_t(32 * gw) * 128u;
#pragma unroll
                      for (int u = 0; u < 32; ++u)
                        {
                          const uint32_t o = a_hi + sw128_off(u, lane);
                          const float    h = tf32_hi(x[u]);
                          asm volatile("st.shared.f32 [%0], %1;" : : "r"(o), "f"(h) : "memory");
                          asm volatile("st.shared.f32 [%0], %1;"
                                       :
                                       : "r"(o + TC_A_BYTES), "f"(x[u] - h)
                                       : "memory");
                        }
                      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                      mbar_arrive(full(s));
                    }
                }
            }
          if (!ok && gtid == 0)
            for (int s = 0; s < TC_STAGES; ++s)
              if (inflight[s])
                mbar_drain(full(s), uint32_t(inflight_par[s]));
        }
      else if (warp == TC_MMA_WARP)
        {
          // ---------------- MMA issuer ----------------
          if (lane == 0)
            {
              // D f32, A/B tf32, both K-major, N = Np, M = 128
              const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) |
                                     (uint32_t(Np >> 3) << 17) | (uint32_t(TC_ROWS >> 4) << 24);
              int  it = 0, tile = 0;
              bool issued = false;
              for (int ch = ch_lo; ok && ch < ch_hi; ++ch)
                {
                  const int rows_total = ch_cnt[ch] * R;
                  for (int t0 = 0; ok && t0 < rows_total; t0 += TC_ROWS, ++tile)
                    {
                      const int a = tile & 1, use_a = tile >> 1;
                      if (use_a > 0 &&
                          !mbar_wait(tempty(a), uint32_t(use_a - 1) & 1u, &abort_flag))
                        {
                          fail();
                          break;
                        }
                      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                      const uint32_t d = tmem + uint32_t(a * TC_ACC_COLS);
                      for (int kc = 0; kc < nkc; ++kc, ++it)
                        {
                          const int s = it % TC_STAGES;
                          if (!mbar_wait(full(s), uint32_t(it / TC_STAGES) & 1u, &abort_flag))
                            {
                              fail();
                              break;
                            }
                          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                          const uint32_t st = base + uint32_t(s) * lay.stage_bytes;
                          const uint32_t ah = st, al = st + TC_A_BYTES, bh = st + 2 * TC_A_BYTES,
                                         bl = bh + lay.b_bytes;
#pragma unroll
                          for (int ks = 0; ks < TC_KC / 8; ++ks)
                            {
                              const uint32_t off = uint32_t(ks) * 32;
                              const uint64_t dah = smem_desc_sw128(ah + off),
                                             dal = smem_desc_sw128(al + off),
                                             dbh = smem_desc_sw128(bh + off),
                                             dbl = smem_desc_sw128(bl + off);
                              mma_tf32(d, dah, dbh, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
                              mma_tf32(d, dal, dbh, idesc, 1u);
                              mma_tf32(d, dah, dbl, idesc, 1u);
                            }
                          mma_commit(empty(s)); // frees the stage once these MMAs are done
                          issued = true;
                        }
                      if (!ok)
                        break;
                      mma_commit(tfull(a)); // accumulator complete
                    }
                }
              if (!ok && issued)
                {
                  // bounded wait until every MMA issued above has completed
                  mma_commit(drain);
                  mbar_drain(drain, 0);
                }
            }
        }
      else
        {
          // ---------------- epilogue (warps 8-11) ----------------
          // Odd K (even p): the warp stages its 32 rows x K row-major in shared
          // memory (conflict-free: lane = row, K odd) at the alignment of their
          // place in Y, and one thread stores the 16-byte aligned middle of the
          // contiguous block with a bulk copy (cp.async.bulk, shared -> global);
          // the < 4 floats at either end by plain stores.  Even K: 32-column
          // chunks through a 32 x 33 tile, one coalesced row segment per store.
          const int      q     = warp - TC_EPI_WARP0;
          float         *stg   = reinterpret_cast<float *>(gbase + lay.epi) + size_t(q) * lay.epi_warp_floats;
          const uint32_t stg_s = base + lay.epi + uint32_t(q) * lay.epi_warp_floats * 4u;
          const bool     bulk  = (K & 1) != 0;
          bool           pending = false; // a bulk store of this warp may still read stg
          int            tile    = 0;
          for (int ch = ch_lo; ok && ch < ch_hi; ++ch)
            {
              const int start = ch_start[ch], rows_total = ch_cnt[ch] * R;
              for (int t0 = 0; ok && t0 < rows_total; t0 += TC_ROWS, ++tile)
                {
                  const int a = tile & 1;
                  if (!mbar_wait(tfull(a), uint32_t(tile >> 1) & 1u, &abort_flag))
                    {
                      fail();
                      break;
                    }
                  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                  const int row0   = t0 + 32 * q;
                  const int nvalid = min(32, rows_total - row0);
                  float    *ybase  = Y + (int64_t(start) * R + row0) * K;
                  if (yslot)
                    {
                      // rows to their slots: lane i stages row i (ldy values,
                      // zero beyond K) and copies it with one bulk store
                      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                      __syncwarp();
                      for (int c0 = 0; c0 < Np; c0 += 32)
                        {
                          float v[32];
                          tmem_ld32(tmem + (uint32_t(32 * q) << 16) + uint32_t(a * TC_ACC_COLS + c0), v);
#pragma unroll
                          for (int j = 0; j < 32; ++j)
                            if (c0 + j < ldy)
                              stg[lane * ldy + c0 + j] = c0 + j < K ? v[j] : 0.0f;
                        }
                      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                      __syncwarp();
                      if (lane < nvalid)
                        {
                          const int row = row0 + lane, pq = start + row / R, r = row - (row / R) * R;
                          float    *dst = Y + (int64_t(yslot[pq]) * R + r) * ldy;
                          asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                                       :
                                       : "l"(dst), "r"(stg_s + uint32_t(lane * ldy) * 4u),
                                         "r"(uint32_t(ldy) * 4u)
                                       : "memory");
                          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                        }
                    }
                  else if (bulk)
                    {
                      if (pending)
                        {
                          if (lane == 0)
                            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                          __syncwarp();
                          pending = false;
                        }
                      const int shift = int((reinterpret_cast<uintptr_t>(ybase) >> 2) & 3u);
                      for (int c0 = 0; c0 < Np; c0 += 32)
                        {
                          float v[32];
                          tmem_ld32(tmem + (uint32_t(32 * q) << 16) + uint32_t(a * TC_ACC_COLS + c0), v);
#pragma unroll
                          for (int j = 0; j < 32; ++j)
                            if (c0 + j < K)
                              stg[shift + lane * K + c0 + j] = v[j];
                        }
                      if (nvalid > 0)
                        {
                          const int nfl  = nvalid * K;
                          const int head = min((4 - shift) & 3, nfl);
                          const int nvec = (nfl - head) >> 2; // 16-byte units
                          const int tl0  = head + 4 * nvec;
                          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                          __syncwarp();
                          if (lane < head)
                            ybase[lane] = stg[shift + lane];
                          if (lane < nfl - tl0)
                            ybase[tl0 + lane] = stg[shift + tl0 + lane];
                          if (nvec > 0 && lane == 0)
                            {
                              asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                                           :
                                           : "l"(ybase + head),
                                             "r"(stg_s + uint32_t(shift + head) * 4u),
                                             "r"(uint32_t(nvec) * 16u)
                                           : "memory");
                              asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                            }
                          pending = nvec > 0;
                        }
                    }
                  else
                    for (int c0 = 0; c0 < Np; c0 += 32)
                      {
                        float v[32];
                        tmem_ld32(tmem + (uint32_t(32 * q) << 16) + uint32_t(a * TC_ACC_COLS + c0), v);
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                          stg[lane * TC_EPI_LD + j] = v[j];
                        __syncwarp();
                        const int col = c0 + lane;
                        if (col < K)
                          for (int r = 0; r < nvalid; ++r)
                            ybase[int64_t(r) * K + col] = stg[r * TC_EPI_LD + lane];
                        __syncwarp();
                      }
                  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                  mbar_arrive(tempty(a));
                }
            }
          asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); // bulk stores complete
        }

      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :
                     : "r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
    }

    inline float tf32_round_host(float x)
    {
      uint32_t b;
      std::memcpy(&b, &x, 4);
      b = (b + 0x1000u) & ~0x1FFFu; // round to nearest, ties away from zero, 10-bit mantissa
      float r;
      std::memcpy(&r, &b, 4);
      return r;
    }
  } // namespace

  TcGeometry tc_geometry(int K)
  {
    TcGeometry g;
    g.K  = K;
    g.Kp = round_up(K, TC_KC);
    g.Np = round_up(K, 16);
    for (g.stages = 3; g.stages >= 2; --g.stages)
      {
        const TcLayout lay(g.Np, K, g.stages);
        g.smem = size_t(lay.total) + 1024; // + alignment slack of the dynamic base
        if (g.smem <= 220 * 1024)
          break;
      }
    g.ok = K >= 1 && g.Np <= TC_ACC_COLS && g.stages >= 2 && g.smem <= 220 * 1024;
    return g;
  }

  // Image of one operator half: Kp / 32 chunks of [Np rows][32 k] in the swizzled
  // K-major layout, zero beyond K; the hi and lo halves one after the other.
  void build_tc_images(const std::vector<double> &ops_out_in, int nops, int K,
                       std::vector<float> &img)
  {
    const TcGeometry g     = tc_geometry(K);
    const int        nkc   = g.Kp / TC_KC;
    const size_t     chunk = size_t(g.Np) * TC_KC; // floats
    const size_t     half  = size_t(nkc) * chunk;
    img.assign(size_t(nops) * 2 * half, 0.0f);
    for (int o = 0; o < nops; ++o)
      {
        float *hi = img.data() + size_t(o) * 2 * half, *lo = hi + half;
        for (int n = 0; n < K; ++n)
          for (int k = 0; k < K; ++k)
            {
              const double v  = ops_out_in[size_t(o) * K * K + size_t(n) * K + k];
              const float  h  = tf32_round_host(float(v));
              const float  l  = float(v - double(h));
              const size_t at = size_t(k / TC_KC) * chunk + sw128_off(n, k % TC_KC) / 4;
              hi[at]          = h;
              lo[at]          = l;
            }
      }
  }

  void launch_tc_gemm(const OperatorDev<float> &op, int R, int c0, int c1, const float *E, float *Y,
                      const int32_t *yslot, int ldy, int *err, cudaStream_t s)
  {
    if (yslot && ldy != round_up(op.K, 4))
      throw Error(PIBEM_EINVAL, "tensor-core translations: slot rows must hold round_up(K, 4) values");
    if (c1 <= c0)
      return;
    int dev = 0, n_sm = 0;
    PIBEM_CUDA(cudaGetDevice(&dev));
    PIBEM_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    TcGeometry g = tc_geometry(op.K);
    if (op.tc_stages == 2 && g.stages == 3)
      {
        // two stages asked for (a tuning choice): the smaller layout
        const TcLayout lay(g.Np, op.K, 2);
        g.stages = 2;
        g.smem   = size_t(lay.total) + 1024;
      }
    const int nch = c1 - c0;
    if (int64_t(op.n_boxes) * R * op.K >= (int64_t(1) << 31))
      throw Error(PIBEM_EINVAL, "too many right-hand sides for the tensor-core translations "
                                "(expansion offsets exceed 32 bits); use the CUDA-core engine");
    const bool all = c0 == 0 && c1 == op.m2l_chunk_end;
    auto       fn  = g.stages == 3 ? (all ? tc_gemm_kernel<true, 3> : tc_gemm_kernel<false, 3>)
                                   : (all ? tc_gemm_kernel<true, 2> : tc_gemm_kernel<false, 2>);
    raise_smem_limit(reinterpret_cast<const void *>(fn), g.smem);
    launch_pdl(fn, std::min(nch, std::max(n_sm, 1)), TC_THREADS, g.smem, s,
      R, op.K, g.Np, g.Kp / TC_KC, c0, nch, op.ch_start, op.ch_cnt, op.ch_op, op.q_src,
      op.tc_images, E, Y, yslot, ldy, err);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
} // namespace pibem
