// FP64-accurate translation GEMM on the tensor cores: the product Y = T E of
// the FP64-accurate operator (about 47 significant bits, like the float-float
// CUDA-core GEMM it replaces) computed from exact BF16 products, an
// Ozaki-type splitting, with tcgen05.mma kind::f16.
//
// Every expansion row (box, rhs) is scaled by a power of two 2^-e_r so that
// its largest entry is below 1 in magnitude, and written as six signed digits
//     x 2^-e_r = sum_{i<6} d_i 2^-(7 + 8 i) + rest,   |d_i| <= 128, |rest| <= 2^-48,
// each digit times its weight being exact in BF16 (8 significant bits); every
// operator row (output coefficient n) likewise, with its own exponent e_n.
// A product of two slices is exact in FP32 (at most 16 significant bits), and
// the sum over K <= 128 terms of the products of all slice pairs (i, j) with
// the same i + j = g is exact for g <= 3 (at most 4 x 128 x 2^14 < 2^24 units
// of its weight): those groups accumulate exactly in four tensor-memory
// accumulators; the pairs with g = 4, 5 share a fifth (its FP32 rounding is
// below 2^-42 of the result); pairs with g > 5 (below 2^-48) are dropped.
// The epilogue adds the five accumulators in float-float arithmetic and
// scales the (hi, lo) pair by 2^(e_r + e_n).  Per 16 K values: 21 MMAs of
// M = 128 rows, N = 96, K = 16.
//
// Block (160 threads, one per SM, persistent over a contiguous range of
// chunks): warps 0-3 fill a 4-deep ring of A stages (one K chunk of 64 values
// of one slice for the tile's 128 rows, 128-byte-swizzled K-major) from the
// pre-sliced expansions and then run the epilogue; warp 4 copies the
// operator's 12 B slice tiles (2 K chunks x 6 slices, pre-swizzled on the
// host) with one bulk copy when the operator changes and issues the MMAs.
// All waits are bounded; a timeout is recorded in *err and the host reports
// PIBEM_ETIMEDOUT.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "async_copy.cuh"
#include "ffmath.cuh"
#include "kernels.h"
#include "tcgen05.cuh"

namespace pibem
{
  namespace
  {
    constexpr int      OZ_S        = 6;   // slices (digits) per operand
    constexpr int      OZ_G        = 5;   // accumulators: i + j = 0, 1, 2, 3 and 4..5
    constexpr int      OZ_KC       = 64;  // K values per chunk: one 128-byte line of BF16
    constexpr int      OZ_NKC      = 2;   // K chunks (K <= 128)
    constexpr int      OZ_NP       = 96;  // operator rows per tile (N of the MMA; K <= 96)
    constexpr int      OZ_ROWS     = 128; // tile rows (M of the MMA)
    constexpr int      OZ_RING     = 4;   // A stages in flight
    constexpr int      OZ_THREADS  = 160; // warps 0-3 producers / epilogue, warp 4 MMA
    constexpr uint32_t OZ_A_BYTES  = OZ_ROWS * 128;         // 16 KB
    constexpr uint32_t OZ_BT_BYTES = OZ_NP * 128;           // 12 KB per (K chunk, slice)
    constexpr uint32_t OZ_B_BYTES  = OZ_NKC * OZ_S * OZ_BT_BYTES; // 144 KB per operator
    constexpr uint32_t OZ_TMEM_COLS = 512;
    constexpr long     OZ_SPIN     = 1L << 22;

    // shared memory: B (144 KB) | A ring (64 KB) | barriers
    constexpr uint32_t OZ_OFF_A    = OZ_B_BYTES;
    constexpr uint32_t OZ_OFF_BAR  = OZ_OFF_A + OZ_RING * OZ_A_BYTES;
    constexpr uint32_t OZ_SMEM     = OZ_OFF_BAR + 128 + 1024; // 11 barriers; alignment slack

    __host__ __device__ inline int oz_group(int i, int j) { return i + j < 4 ? i + j : 4; }

    // Bounded wait; after a timeout anywhere in the block (abort raised) no
    // further waiting, so a broken pipeline ends quickly (results then wrong,
    // reported through *err).
    __device__ inline bool oz_wait(uint32_t addr, uint32_t parity, int *err, volatile int *abort)
    {
      for (long it = 0; it < OZ_SPIN; ++it)
        {
          if (mbar_try(addr, parity))
            return true;
          if ((it & 255) == 255 && *abort)
            return false;
        }
      *abort = 1;
      atomicExch(err, 1);
      return false;
    }

    __device__ inline void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    uint32_t accumulate)
    {
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "setp.ne.b32 p, %4, 0;\n\t"
                   "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                   :
                   : "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                   : "memory");
    }

    // BF16 bits of a float that BF16 represents exactly (low 16 bits zero)
    __host__ __device__ inline uint16_t bf16_bits(float f)
    {
      uint32_t u;
      memcpy(&u, &f, 4);
      return uint16_t(u >> 16);
    }

    // Digits of the rows of the (hi, lo) expansions E (rows of K values): one
    // warp per row; slices[i][row][128] BF16 (zero beyond K), e_row[row].
    __global__ void oz_slice_rows_kernel(int64_t nrows, int K, const float2 *__restrict__ E,
                                         uint16_t *__restrict__ slices, int *__restrict__ e_row)
    {
      const int64_t row = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
      if (row >= nrows)
        return;
      const int lane = threadIdx.x & 31;
      float2    x[4];
      float     mx = 0.0f;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        {
          const int k = lane + 32 * u;
          x[u]        = k < K ? E[row * K + k] : make_float2(0.0f, 0.0f);
          mx          = fmaxf(mx, fabsf(x[u].x) + fabsf(x[u].y));
        }
      for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      int e = 0;
      if (mx > 0.0f)
        frexpf(mx, &e); // mx < 2^e
      if (lane == 0)
        e_row[row] = e;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        {
          const int k  = lane + 32 * u;
          float     vh = ldexpf(x[u].x, -e), vl = ldexpf(x[u].y, -e);
#pragma unroll
          for (int i = 0; i < OZ_S; ++i)
            {
              const float sc = i == 0 ? 128.0f : 256.0f;
              vh *= sc;
              vl *= sc;
              const float d = rintf(vh);
              const float t = vh - d; // exact
              const float2 r = ff_add(make_float2(t, 0.0f), make_float2(vl, 0.0f));
              vh = r.x;
              vl = r.y;
              slices[(int64_t(i) * nrows + row) * 128 + k] = bf16_bits(ldexpf(d, -(7 + 8 * i)));
            }
        }
    }

    struct OzArgs
    {
      int            R, K, chunk0, n_chunks;
      const int32_t *ch_start, *ch_cnt, *ch_op, *q_src;
      const uint16_t *bimg;   // [op][kc][slice][96 x 64 swizzled]
      const int16_t  *e_col;  // [op][96]
      const uint16_t *aslc;   // [slice][box row][128]
      const int      *e_row;  // [box row]
      int64_t         a_rows; // box rows (n_boxes * R)
      float2         *Y;
      int            *err;
    };

    __global__ void __launch_bounds__(OZ_THREADS, 1) oz_gemm_kernel(OzArgs a)
    {
      extern __shared__ uint8_t smem_raw[];
      __shared__ uint32_t     tmem_slot;
      __shared__ volatile int abort_flag;
      const uint32_t raw  = smem_u32(smem_raw);
      const uint32_t base = (raw + 1023u) & ~1023u;
      const int      tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
      const uint32_t bar0   = base + OZ_OFF_BAR;
      auto a_full  = [&](int s) { return bar0 + 8u * uint32_t(s); };
      auto a_empty = [&](int s) { return bar0 + 8u * uint32_t(OZ_RING + s); };
      const uint32_t b_full = bar0 + 8u * uint32_t(2 * OZ_RING);
      const uint32_t done   = b_full + 8u;
      const uint32_t drain  = done + 8u;
      const int ch_lo = a.chunk0 + int(int64_t(a.n_chunks) * blockIdx.x / gridDim.x);
      const int ch_hi = a.chunk0 + int(int64_t(a.n_chunks) * (blockIdx.x + 1) / gridDim.x);
      const int R = a.R, K = a.K;
      if (tid == 0)
        {
          abort_flag = 0;
          for (int s = 0; s < OZ_RING; ++s)
            {
              mbar_init(a_full(s), 128);
              mbar_init(a_empty(s), 1);
            }
          mbar_init(b_full, 1);
          mbar_init(done, 1);
          mbar_init(drain, 1);
          mbar_init_fence();
        }
      if (warp == 4)
        {
          asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                       :
                       : "r"(smem_u32(&tmem_slot)), "r"(OZ_TMEM_COLS)
                       : "memory");
          asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tmem = tmem_slot;
      // D f32, A and B bf16, both K-major, N = 96, M = 128
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(OZ_NP >> 3) << 17) |
                             (uint32_t(OZ_ROWS >> 4) << 24);
      int  loaded_op = -1, b_loads = 0, tiles = 0;
      long stage = 0; // A stages over all tiles of this block
      bool issued = false, b_pending = false;
      for (int ch = ch_lo; ch < ch_hi; ++ch)
        {
          const int start = a.ch_start[ch], rows_total = a.ch_cnt[ch] * R, op = a.ch_op[ch];
          for (int t0 = 0; t0 < rows_total; t0 += OZ_ROWS, ++tiles)
            {
              if (warp == 4)
                {
                  if (lane == 0)
                    {
                      if (op != loaded_op)
                        {
                          mbar_arrive_expect_tx(b_full, OZ_B_BYTES);
                          bulk_copy(base, a.bimg + size_t(op) * (OZ_B_BYTES / 2), OZ_B_BYTES, b_full);
                          b_pending = !oz_wait(b_full, uint32_t(b_loads) & 1u, a.err, &abort_flag);
                          ++b_loads;
                          loaded_op = op;
                        }
                      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                      int started = 0; // accumulators written in this tile
                      for (int s = 0; s < OZ_NKC * OZ_S; ++s)
                        {
                          const long g_st = stage + s;
                          const int  slot = int(g_st % OZ_RING);
                          oz_wait(a_full(slot), uint32_t(g_st / OZ_RING) & 1u, a.err, &abort_flag);
                          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                          const int      kc = s / OZ_S, i = s % OZ_S;
                          const uint32_t at = base + OZ_OFF_A + uint32_t(slot) * OZ_A_BYTES;
                          for (int j = 0; i + j < OZ_S; ++j)
                            {
                              const int      g  = oz_group(i, j);
                              const uint32_t bt = base + uint32_t(kc * OZ_S + j) * OZ_BT_BYTES;
#pragma unroll
                              for (int ks = 0; ks < OZ_KC / 16; ++ks)
                                {
                                  const uint32_t acc = (((started >> g) & 1) != 0 || ks > 0) ? 1u : 0u;
                                  mma_bf16(tmem + uint32_t(g * OZ_NP), smem_desc_sw128(at + ks * 32),
                                           smem_desc_sw128(bt + ks * 32), idesc, acc);
                                }
                              started |= 1 << g;
                            }
                          mma_commit(a_empty(slot)); // frees the stage once these MMAs are done
                          issued = true;
                        }
                      mma_commit(done); // the tile's accumulators are complete
                    }
                  __syncwarp();
                }
              else
                {
                  // ---------------- producers: one tile row per thread ----------------
                  const int row = t0 + tid;
                  int64_t   src = -1;
                  if (row < rows_total)
                    {
                      const int q = start + row / R, r = row - (row / R) * R;
                      src         = int64_t(a.q_src[q]) * R + r;
                    }
                  // stage s = (K chunk s / 6, slice s % 6); the loads of stage s + 2
                  // are issued before stage s is stored (three stages of the row in
                  // registers), so the L2 latency overlaps the ring waits
                  uint4 buf[3][8];
                  auto  load = [&](int s, uint4(&v)[8]) {
                    const int kc = s / OZ_S, i = s % OZ_S;
                    if (src >= 0)
                      {
                        const uint4 *p = reinterpret_cast<const uint4 *>(
                          a.aslc + (int64_t(i) * a.a_rows + src) * 128 + kc * OZ_KC);
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                          v[c] = __ldg(p + c);
                      }
                    else
#pragma unroll
                      for (int c = 0; c < 8; ++c)
                        v[c] = make_uint4(0u, 0u, 0u, 0u);
                  };
                  load(0, buf[0]);
                  load(1, buf[1]);
#pragma unroll
                  for (int s = 0; s < OZ_NKC * OZ_S; ++s)
                    {
                      if (s + 2 < OZ_NKC * OZ_S)
                        load(s + 2, buf[(s + 2) % 3]);
                      const long g_st = stage + s;
                      const int  slot = int(g_st % OZ_RING);
                      if (g_st >= OZ_RING)
                        oz_wait(a_empty(slot), uint32_t(g_st / OZ_RING - 1) & 1u, a.err, &abort_flag);
                      uint8_t *at = smem_raw + (base - raw) + OZ_OFF_A + size_t(slot) * OZ_A_BYTES;
#pragma unroll
                      for (int c = 0; c < 8; ++c)
                        *reinterpret_cast<uint4 *>(at + sw128_off_b16(tid, 8 * c)) = buf[s % 3][c];
                      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                      mbar_arrive(a_full(slot));
                    }
                  // ---------------- epilogue: row tid of the tile ----------------
                  oz_wait(done, uint32_t(tiles) & 1u, a.err, &abort_flag);
                  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                  const int  q_row = t0 + 32 * warp + lane;
                  const bool valid = q_row < rows_total;
                  int        er    = 0;
                  if (valid)
                    {
                      const int q = start + q_row / R, r = q_row - (q_row / R) * R;
                      er          = a.e_row[int64_t(a.q_src[q]) * R + r];
                    }
                  const int16_t *ec   = a.e_col + size_t(op) * OZ_NP;
                  float2        *yrow = a.Y + (int64_t(start) * R + q_row) * K;
                  for (int c0 = 0; c0 < OZ_NP; c0 += 32)
                    {
                      // the five group sums of 32 columns (five loads, one wait):
                      // g0, g1 and g2, g3 pairwise by TwoSum, the two pairs by
                      // TwoSum, the errors and g4 added last (each below 2^-40 of
                      // the result), one renormalisation
                      uint32_t g[5][32];
#pragma unroll
                      for (int q = 0; q < OZ_G; ++q)
                        tmem_ld32_nowait(tmem + (uint32_t(32 * warp) << 16) + uint32_t(q * OZ_NP + c0), g[q]);
                      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                      if (valid)
#pragma unroll
                        for (int jj = 0; jj < 32; ++jj)
                          {
                            const int n = c0 + jj;
                            if (n >= K)
                              continue;
                            const float g0 = __uint_as_float(g[0][jj]), g1 = __uint_as_float(g[1][jj]);
                            const float g2 = __uint_as_float(g[2][jj]), g3 = __uint_as_float(g[3][jj]);
                            const float g4 = __uint_as_float(g[4][jj]);
                            const float t1 = __fadd_rn(g0, g1), z1 = __fsub_rn(t1, g0);
                            const float e1 = __fadd_rn(__fsub_rn(g0, __fsub_rn(t1, z1)), __fsub_rn(g1, z1));
                            const float t2 = __fadd_rn(g2, g3), z2 = __fsub_rn(t2, g2);
                            const float e2 = __fadd_rn(__fsub_rn(g2, __fsub_rn(t2, z2)), __fsub_rn(g3, z2));
                            const float t  = __fadd_rn(t1, t2), z = __fsub_rn(t, t1);
                            const float d  = __fadd_rn(__fsub_rn(t1, __fsub_rn(t, z)), __fsub_rn(t2, z));
                            const float lo = __fadd_rn(__fadd_rn(e1, __fadd_rn(e2, d)), g4);
                            const float2 r = ff_norm(t, lo);
                            // times 2^(e_r + e_n): a power of two built from its bits
                            // when it is a normal float, else ldexpf
                            const int e = er + ec[n];
                            if (e > -127 && e < 128)
                              {
                                const float sc = __int_as_float((e + 127) << 23);
                                yrow[n] = make_float2(__fmul_rn(r.x, sc), __fmul_rn(r.y, sc));
                              }
                            else
                              yrow[n] = make_float2(ldexpf(r.x, e), ldexpf(r.y, e));
                          }
                    }
                }
              stage += OZ_NKC * OZ_S;
              asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
              __syncthreads(); // accumulators read: the next tile may overwrite them
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            }
        }
      if (warp == 4 && lane == 0)
        {
          if (b_pending) // a copy whose wait gave up: let it land before the block ends
            mbar_wait_bounded(b_full, uint32_t(b_loads - 1) & 1u, OZ_SPIN);
          if (issued)
            {
              mma_commit(drain); // every MMA issued above has completed
              mbar_wait_bounded(drain, 0, OZ_SPIN);
            }
        }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (warp == 4)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :
                     : "r"(tmem), "r"(OZ_TMEM_COLS)
                     : "memory");
    }
  } // namespace

  bool ozaki_ok(int K) { return K >= 1 && K <= OZ_NP; }

  // Host: digits of every operator row (output coefficient), B images and
  // column exponents.  ops_out_in: nops row-major [out][in] K x K operators.
  void build_ozaki_images(const std::vector<double> &ops_out_in, int nops, int K,
                          std::vector<uint16_t> &img, std::vector<int16_t> &e_col)
  {
    img.assign(size_t(nops) * (OZ_B_BYTES / 2), 0);
    e_col.assign(size_t(nops) * OZ_NP, 0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int o = 0; o < nops; ++o)
      for (int n = 0; n < K; ++n)
        {
          const double *t  = &ops_out_in[(size_t(o) * K + n) * K];
          double        mx = 0.0;
          for (int k = 0; k < K; ++k)
            mx = std::max(mx, std::fabs(t[k]));
          int e = 0;
          if (mx > 0.0)
            std::frexp(mx, &e); // mx < 2^e
          e_col[size_t(o) * OZ_NP + n] = int16_t(e);
          for (int k = 0; k < K; ++k)
            {
              double v = std::ldexp(t[k], -e);
              for (int i = 0; i < OZ_S; ++i)
                {
                  v *= (i == 0 ? 128.0 : 256.0);
                  const double d = std::nearbyint(v);
                  v -= d;
                  const int    kc = k / OZ_KC;
                  const size_t at = size_t(o) * (OZ_B_BYTES / 2) +
                                    size_t(kc * OZ_S + i) * (OZ_BT_BYTES / 2) +
                                    sw128_off_b16(n, k % OZ_KC) / 2;
                  img[at] = bf16_bits(float(std::ldexp(d, -(7 + 8 * i))));
                }
            }
        }
  }

  void launch_ozaki_slices(int64_t nrows, int K, const float2 *E, uint16_t *slices, int *e_row,
                           cudaStream_t s)
  {
    if (nrows == 0)
      return;
    oz_slice_rows_kernel<<<unsigned((nrows * 32 + 255) / 256), 256, 0, s>>>(nrows, K, E, slices,
                                                                          e_row);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_ozaki_gemm(const OperatorDev<double> &op, int R, int c0, int c1,
                         const uint16_t *aslc, const int *e_row, int64_t a_rows, float2 *Y,
                         cudaStream_t s)
  {
    if (c1 <= c0)
      return;
    int dev = 0, n_sm = 1;
    PIBEM_CUDA(cudaGetDevice(&dev));
    PIBEM_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    OzArgs a;
    a.R = R, a.K = op.K, a.chunk0 = c0, a.n_chunks = c1 - c0;
    a.ch_start = op.ch_start, a.ch_cnt = op.ch_cnt, a.ch_op = op.ch_op, a.q_src = op.q_src;
    a.bimg = op.oz_images, a.e_col = op.oz_ecol, a.aslc = aslc, a.e_row = e_row;
    a.a_rows = a_rows, a.Y = Y, a.err = op.dev_err;
    raise_smem_limit(reinterpret_cast<const void *>(oz_gemm_kernel), OZ_SMEM);
    oz_gemm_kernel<<<std::min(c1 - c0, n_sm), OZ_THREADS, OZ_SMEM, s>>>(a);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
} // namespace pibem
