// Fused level passes of the FP32 operator, on the CUDA cores:
//
//   M2L sums  L[b]  = sum_{M2L pairs q of b} Y[q]             all levels, one launch
//   L2L       L[b] += T_{oct(b)} L[parent(b)]                  one launch per level
//   M2M       M[P]  = sum_{octant o} T_o M[child_o(P)]          one launch per level
//
// (the reference's ascending pass, bem_fma.cc:2274-2376, and the L2L / M2L part
// of its descending pass, bem_fma.cc:2582-2652.)  The translations of one tree
// level are small (a few thousand K x K matrix-vector products); as batched
// GEMMs followed by a gather they cost two dependent launches per level and a
// round trip of the products through HBM.  Here a block computes complete
// expansions of up to CPB columns (column = (box, right-hand side)).
//
// Threads: groups of KT = 32 ceil(K/32) (at most 128) threads; thread t of a
// group owns output coefficients t, t + KT, ...  Every column's result is
// computed by a fixed sequence of operations that depends on the column's own
// data only (M2M: one octant per group, the eight partial sums added in a
// fixed order; L2L: one thread per output coefficient, k ascending; M2L sums:
// one warp per 32 coefficients, pairs in list order): the same bits whatever
// the number of columns, their grouping into blocks or the other columns of
// the batch.
//
// Where the eight operators of a pass fit in shared memory (K <= 81, p <= 8)
// the M2M and L2L kernels are persistent (one block per SM) and read the
// operators from shared memory, copied there once per launch; otherwise they
// read them through the L1 cache.
#include <algorithm>
#include <cstdint>

#include "async_copy.cuh"
#include "kernels.h"
#include "pdl.cuh"

namespace pibem
{
  namespace
  {
    __host__ __device__ inline int lv_kx(int K) { return (K + 3) / 4 * 4; }

    // acc[c] += sum_{k in [k0, k1)} T[k][ko] X[c][k], k ascending, eight
    // operator loads in flight; T is one operator stored [in][out]
    template <int CPB>
    __device__ __forceinline__ void lv_dot(float (&acc)[CPB], const float *__restrict__ T, int K,
                                           int ko, const float *X, int Kx, int k0, int k1)
    {
      int k = k0;
      for (; k + 8 <= k1; k += 8)
        {
          float t[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            t[u] = __ldg(T + size_t(k + u) * K + ko);
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            {
              const float *x = X + c * Kx + k;
#pragma unroll
              for (int u = 0; u < 8; ++u)
                acc[c] = fmaf(t[u], x[u], acc[c]);
            }
        }
      for (; k < k1; ++k)
        {
          const float t = __ldg(T + size_t(k) * K + ko);
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            acc[c] = fmaf(t, X[c * Kx + k], acc[c]);
        }
    }

    // One level of the upward pass; 8 groups, group o applies the octant-o
    // operator.  Columns c = i * R + r over the level's parents i (par[i],
    // children child8[8 i + o], -1: none).  Shared memory: the children's
    // expansions X[o][CPB][Kx] (zero where a child is missing), then the
    // partial sums P[o][CPB][Kx].
    template <int CPB>
    __global__ void __launch_bounds__(1024)
      m2m_level_kernel(int R, int K, int ncols, const int32_t *__restrict__ par,
                       const int32_t *__restrict__ child8, const float *__restrict__ ops,
                       float *__restrict__ M)
    {
      extern __shared__ float lv_sm[];
      const int Kx = lv_kx(K);
      float    *X  = lv_sm;
      float    *P  = lv_sm + 8 * CPB * Kx;
      const int KT = blockDim.x / 8;
      const int g = threadIdx.x / KT, t = threadIdx.x - g * KT;
      const int c0 = blockIdx.x * CPB, nc = min(CPB, ncols - c0);
      for (int i = threadIdx.x; i < 8 * CPB * Kx; i += blockDim.x)
        {
          const int k = i % Kx, oc = i / Kx, c = oc % CPB, o = oc / CPB;
          float     v = 0.0f;
          if (c < nc && k < K)
            {
              const int col = c0 + c, pi = col / R, r = col - pi * R;
              const int ch  = child8[8 * pi + o];
              if (ch >= 0)
                v = M[(int64_t(ch) * R + r) * K + k];
            }
          X[i] = v;
        }
      bool has = false; // some column of the block has an octant-g child
      for (int c = 0; c < nc; ++c)
        has = has || child8[8 * ((c0 + c) / R) + g] >= 0;
      __syncthreads();
      for (int ko = t; ko < K; ko += KT)
        {
          float acc[CPB];
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            acc[c] = 0.0f;
          if (has)
            lv_dot<CPB>(acc, ops + size_t(g) * K * K, K, ko, X + g * CPB * Kx, Kx, 0, K);
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            P[(g * CPB + c) * Kx + ko] = acc[c];
        }
      __syncthreads();
      if (g == 0)
        for (int ko = t; ko < K; ko += KT)
          for (int c = 0; c < nc; ++c)
            {
              const int col = c0 + c, pi = col / R, r = col - pi * R;
              auto      at  = [&](int o) { return P[(o * CPB + c) * Kx + ko]; };
              const float v = ((at(0) + at(1)) + (at(2) + at(3))) + ((at(4) + at(5)) + (at(6) + at(7)));
              M[(int64_t(par[pi]) * R + r) * K + ko] = v;
            }
    }

    // M2L sums of the boxes of the downward lists, all levels.  The M2L
    // products are target-major: the rows (slot, rhs) of a box's pairs are the
    // slots [beg, end) in list order, rows of Kx = round_up(K, 4) values.  One
    // warp per column c = i * R + r; lane l adds coefficients 4l..4l+3 over
    // the box's rows in order, 16 rows in flight.
    __global__ void __launch_bounds__(256)
      m2l_sum_kernel(int R, int K, int64_t ncols, const int32_t *__restrict__ box,
                     const int32_t *__restrict__ beg, const int32_t *__restrict__ end,
                     const float *__restrict__ Y, float *__restrict__ Lx)
    {
      pdl_entry();
      const int64_t col = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
      if (col >= ncols)
        return;
      const int     lane = threadIdx.x & 31;
      const int     bi = int(col / R), r = int(col - int64_t(bi) * R);
      const int     n4 = lv_kx(K) / 4;
      const int     e0 = beg[bi], e1 = end[bi];
      float4        s  = make_float4(0.f, 0.f, 0.f, 0.f);
      if (lane < n4)
        {
          const float4 *y      = reinterpret_cast<const float4 *>(Y) + (int64_t(e0) * R + r) * n4 + lane;
          const int64_t stride = int64_t(R) * n4;
          int           e      = e0;
          for (; e + 16 <= e1; e += 16)
            {
              float4 v[16];
#pragma unroll
              for (int u = 0; u < 16; ++u)
                v[u] = __ldg(y + int64_t(e - e0 + u) * stride);
#pragma unroll
              for (int u = 0; u < 16; ++u)
                {
                  s.x += v[u].x;
                  s.y += v[u].y;
                  s.z += v[u].z;
                  s.w += v[u].w;
                }
            }
          for (; e < e1; ++e)
            {
              const float4 v = __ldg(y + int64_t(e - e0) * stride);
              s.x += v.x;
              s.y += v.y;
              s.z += v.z;
              s.w += v.w;
            }
          float *o = Lx + (int64_t(box[bi]) * R + r) * K + 4 * lane;
          const float sv[4] = {s.x, s.y, s.z, s.w};
#pragma unroll
          for (int c = 0; c < 4; ++c)
            if (4 * lane + c < K)
              o[c] = sv[c];
        }
    }

    // One level of the downward pass after the M2L sums: L[b] += T_oct L[parent]
    // for the level's boxes with an L2L parent (par[i] >= 0); 4 groups, group g
    // takes input coefficients [K g / 4, K (g + 1) / 4).  Columns c = i * R + r.
    // Shared memory: the parents' expansions X[CPB][Kx], partial sums
    // P[g][CPB][Kx].
    template <int CPB>
    __global__ void __launch_bounds__(512)
      l2l_level_kernel(int R, int K, int ncols, const int32_t *__restrict__ box,
                       const int32_t *__restrict__ par, const uint8_t *__restrict__ oct,
                       const float *__restrict__ ops, float *__restrict__ Lx)
    {
      extern __shared__ float lv_sm[];
      const int Kx = lv_kx(K);
      float    *X  = lv_sm;
      float    *P  = lv_sm + CPB * Kx;
      const int KT = blockDim.x / 4;
      const int g = threadIdx.x / KT, t = threadIdx.x - g * KT;
      const int c0 = blockIdx.x * CPB, nc = min(CPB, ncols - c0);
      for (int i = threadIdx.x; i < CPB * Kx; i += blockDim.x)
        {
          const int k = i % Kx, c = i / Kx;
          float     v = 0.0f;
          if (c < nc && k < K)
            {
              const int col = c0 + c, bi = col / R, r = col - bi * R;
              const int pb  = par[bi];
              if (pb >= 0)
                v = Lx[(int64_t(pb) * R + r) * K + k];
            }
          X[i] = v;
        }
      // one operator for the whole block when its columns share the octant
      // (the boxes of a level are listed by octant); the arithmetic per column
      // is the same either way
      const int o0      = oct[c0 / R];
      bool      uniform = true;
      for (int c = 1; c < nc; ++c)
        uniform = uniform && oct[(c0 + c) / R] == o0;
      __syncthreads();
      const int k0 = K * g / 4, k1 = K * (g + 1) / 4;
      for (int ko = t; ko < K; ko += KT)
        {
          float acc[CPB];
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            acc[c] = 0.0f;
          if (uniform)
            lv_dot<CPB>(acc, ops + size_t(o0) * K * K, K, ko, X, Kx, k0, k1);
          else
#pragma unroll
            for (int c = 0; c < CPB; ++c)
              if (c < nc)
                {
                  float a1[1] = {0.0f};
                  lv_dot<1>(a1, ops + size_t(oct[(c0 + c) / R]) * K * K, K, ko, X + c * Kx, Kx, k0,
                            k1);
                  acc[c] = a1[0];
                }
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            P[(g * CPB + c) * Kx + ko] = acc[c];
        }
      __syncthreads();
      if (g == 0)
        for (int ko = t; ko < K; ko += KT)
          for (int c = 0; c < nc; ++c)
            {
              const int col = c0 + c, bi = col / R, r = col - bi * R;
              if (par[bi] < 0)
                continue;
              auto        at = [&](int q) { return P[(q * CPB + c) * Kx + ko]; };
              const float l  = (at(0) + at(1)) + (at(2) + at(3));
              float      *o  = Lx + (int64_t(box[bi]) * R + r) * K + ko;
              *o             = *o + l;
            }
    }

    __host__ __device__ inline int lv_kk(int K) { return (K * K + 3) / 4 * 4; } // padded operator

    constexpr long LV_SPIN_LIMIT = 1L << 24;

    // Thread 0 starts one bulk copy of n operators (lv_kk(K) floats each,
    // 16-byte aligned) into shared memory, completing on the barrier; the
    // barrier is initialised here and visible after the next __syncthreads.
    __device__ inline void lv_start_ops(float *dst, const float *src, int n, int K, uint64_t *bar)
    {
      if (threadIdx.x == 0)
        {
          const uint32_t b     = smem_u32(bar);
          const uint32_t bytes = uint32_t(n) * uint32_t(lv_kk(K)) * 4u;
          mbar_init(b, 1);
          mbar_init_fence();
          mbar_arrive_expect_tx(b, bytes);
          bulk_copy(smem_u32(dst), src, bytes, b);
        }
    }

    // Every thread waits (bounded) for the operators; false after a timeout,
    // which is recorded in *err.
    __device__ inline bool lv_wait_ops(uint64_t *bar, int *err)
    {
      if (mbar_wait_bounded(smem_u32(bar), 0, LV_SPIN_LIMIT))
        return true;
      atomicExch(err, 1);
      return false;
    }

    // M2M of one level with the eight operators in shared memory; persistent
    // blocks take batches of CPB columns.  8 groups, group o applies octant o.
    // Shared memory: T[8][lv_kk], X[8][CPB][Kx] (children), reused for the
    // partial sums P[8][CPB][Kx].
    template <int CPB>
    __global__ void __launch_bounds__(768, 1)
      m2m_level_smem_kernel(int R, int K, int ncols, const int32_t *__restrict__ par,
                            const int32_t *__restrict__ child8, const float *__restrict__ lvops,
                            float *__restrict__ M, int *__restrict__ err)
    {
      pdl_entry();
      extern __shared__ __align__(16) float lv_sm[];
      __shared__ uint64_t ops_bar;
      const int Kx = lv_kx(K), KK = lv_kk(K);
      float    *Ts = lv_sm;
      float    *X  = lv_sm + 8 * KK;
      const int KT = blockDim.x / 8, nw = blockDim.x >> 5;
      const int g = threadIdx.x / KT, ko = threadIdx.x - g * KT; // KT >= K: one coefficient
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      lv_start_ops(Ts, lvops, 8, K, &ops_bar);
      const float *T     = Ts + g * KK;
      bool         ops_ok = true, waited = false;
      for (int c0 = blockIdx.x * CPB; c0 < ncols; c0 += gridDim.x * CPB)
        {
          const int nc = min(CPB, ncols - c0);
          for (int row = warp; row < 8 * CPB; row += nw)
            {
              const int o = row / CPB, c = row - o * CPB;
              int64_t   src = -1;
              if (c < nc)
                {
                  const int col = c0 + c, pi = col / R, r = col - pi * R;
                  const int ch  = child8[8 * pi + o];
                  if (ch >= 0)
                    src = (int64_t(ch) * R + r) * K;
                }
              for (int k = lane; k < Kx; k += 32)
                X[row * Kx + k] = (src >= 0 && k < K) ? M[src + k] : 0.0f;
            }
          bool has = false; // some column of the batch has an octant-g child
          for (int c = 0; c < nc; ++c)
            has = has || child8[8 * ((c0 + c) / R) + g] >= 0;
          __syncthreads();
          if (!waited)
            {
              ops_ok = lv_wait_ops(&ops_bar, err);
              waited = true;
            }
          float acc[CPB];
#pragma unroll
          for (int c = 0; c < CPB; ++c)
            acc[c] = 0.0f;
          if (has && ops_ok && ko < K)
            {
              const float *x = X + g * CPB * Kx;
              int          k = 0;
              for (; k + 4 <= K; k += 4)
                {
                  float tv[4];
#pragma unroll
                  for (int u = 0; u < 4; ++u)
                    tv[u] = T[(k + u) * K + ko];
#pragma unroll
                  for (int c = 0; c < CPB; ++c)
                    {
                      const float4 xv = *reinterpret_cast<const float4 *>(x + c * Kx + k);
                      acc[c]          = fmaf(tv[0], xv.x, acc[c]);
                      acc[c]          = fmaf(tv[1], xv.y, acc[c]);
                      acc[c]          = fmaf(tv[2], xv.z, acc[c]);
                      acc[c]          = fmaf(tv[3], xv.w, acc[c]);
                    }
                }
              for (; k < K; ++k)
                {
                  const float tv = T[k * K + ko];
#pragma unroll
                  for (int c = 0; c < CPB; ++c)
                    acc[c] = fmaf(tv, x[c * Kx + k], acc[c]);
                }
            }
          __syncthreads(); // X no longer read: it becomes P
          if (ko < K)
#pragma unroll
            for (int c = 0; c < CPB; ++c)
              X[(g * CPB + c) * Kx + ko] = acc[c];
          __syncthreads();
          if (g == 0 && ko < K)
            for (int c = 0; c < nc; ++c)
                {
                  const int col = c0 + c, pi = col / R, r = col - pi * R;
                  auto      at  = [&](int o) { return X[(o * CPB + c) * Kx + ko]; };
                  const float v = ((at(0) + at(1)) + (at(2) + at(3))) + ((at(4) + at(5)) + (at(6) + at(7)));
                  M[(int64_t(par[pi]) * R + r) * K + ko] = v;
                }
          __syncthreads();
        }
      if (!waited) // never leave with the copy in flight
        lv_wait_ops(&ops_bar, err);
    }

    // L2L of one level with its operators in shared memory, after the M2L
    // sums: L[b] += T_oct L[parent] for the boxes with an L2L parent.  Persistent
    // blocks take contiguous column ranges (the boxes are listed by octant, so
    // a range needs the operators of a few octants, copied once); batches of
    // 16 columns, 8 groups, group g computes columns g and g + 8 of a batch,
    // one thread per output coefficient, k ascending.  Shared memory:
    // T[8][lv_kk] (the octants [o_lo, o_hi] of the range), X[16][Kx].
    __global__ void __launch_bounds__(768, 1)
      l2l_level_smem_kernel(int R, int K, int ncols, const int32_t *__restrict__ box,
                            const int32_t *__restrict__ par, const uint8_t *__restrict__ oct,
                            const float *__restrict__ lvops, float *__restrict__ Lx,
                            int *__restrict__ err)
    {
      pdl_entry();
      extern __shared__ __align__(16) float lv_sm[];
      __shared__ uint64_t ops_bar;
      const int Kx = lv_kx(K), KK = lv_kk(K);
      const int lo = int(int64_t(ncols) * blockIdx.x / gridDim.x);
      const int hi = int(int64_t(ncols) * (blockIdx.x + 1) / gridDim.x);
      if (lo >= hi)
        return;
      float    *Ts = lv_sm;
      float    *X  = lv_sm + 8 * KK;
      const int KT = blockDim.x / 8, nw = blockDim.x >> 5;
      const int g = threadIdx.x / KT, t = threadIdx.x - g * KT;
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const int o_lo = oct[lo / R], o_hi = oct[(hi - 1) / R];
      lv_start_ops(Ts, lvops + size_t(o_lo) * KK, o_hi - o_lo + 1, K, &ops_bar);
      bool ops_ok = true, waited = false;
      for (int c0 = lo; c0 < hi; c0 += 16)
        {
          const int nc = min(16, hi - c0);
          for (int c = warp; c < nc; c += nw)
            {
              const int col = c0 + c, bi = col / R, r = col - bi * R;
              const int pb  = par[bi];
              for (int k = lane; k < Kx; k += 32)
                X[c * Kx + k] = (pb >= 0 && k < K) ? Lx[(int64_t(pb) * R + r) * K + k] : 0.0f;
            }
          __syncthreads();
          if (!waited)
            {
              ops_ok = lv_wait_ops(&ops_bar, err);
              waited = true;
            }
          for (int c = g; c < nc; c += 8)
            {
              const int col = c0 + c, bi = col / R, r = col - bi * R;
              if (par[bi] < 0 || !ops_ok)
                continue;
              const float *T = Ts + (oct[bi] - o_lo) * KK;
              const float *x = X + c * Kx;
              for (int ko = t; ko < K; ko += KT)
                {
                  float a = 0.0f;
                  int   k = 0;
                  for (; k + 4 <= K; k += 4)
                    {
                      const float4 xv = *reinterpret_cast<const float4 *>(x + k);
                      a               = fmaf(T[k * K + ko], xv.x, a);
                      a               = fmaf(T[(k + 1) * K + ko], xv.y, a);
                      a               = fmaf(T[(k + 2) * K + ko], xv.z, a);
                      a               = fmaf(T[(k + 3) * K + ko], xv.w, a);
                    }
                  for (; k < K; ++k)
                    a = fmaf(T[k * K + ko], x[k], a);
                  float *o = Lx + (int64_t(box[bi]) * R + r) * K + ko;
                  *o       = *o + a;
                }
            }
          __syncthreads();
        }
      if (!waited)
        lv_wait_ops(&ops_bar, err);
    }

    int lv_kt(int K) { return std::min(128, (K + 31) / 32 * 32); }

    // Columns per block: the most (up to cap) that still give every SM a
    // block; shared memory = floats_per_col * CPB * Kx floats.
    int lv_cpb(int K, int64_t ncols, int floats_per_col, int cap)
    {
      int dev = 0, n_sm = 1;
      PIBEM_CUDA(cudaGetDevice(&dev));
      PIBEM_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
      int cpb = cap;
      while (cpb > 1 && (ncols < int64_t(cpb) * n_sm ||
                         size_t(floats_per_col) * cpb * lv_kx(K) * sizeof(float) > 48 * 1024))
        cpb /= 2;
      return cpb;
    }
  } // namespace

  // the operator pass in shared memory: 8 operators + the larger of the
  // M2M X (8 x 4 columns) and the L2L X (16 columns)
  static size_t lv_smem_bytes(int K)
  {
    return (size_t(8) * lv_kk(K) + size_t(32) * lv_kx(K)) * sizeof(float);
  }
  static bool lv_smem_ok(int K) { return K <= 96 && lv_smem_bytes(K) <= 227 * 1024; }

  static int lv_n_sm()
  {
    int dev = 0, n_sm = 1;
    PIBEM_CUDA(cudaGetDevice(&dev));
    PIBEM_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    return n_sm;
  }

  bool fused_levels_ok(int K, int R)
  {
    return R >= 1 && size_t(16) * lv_kx(K) * sizeof(float) <= 48 * 1024;
  }

  size_t fused_level_ops_floats(int K) { return size_t(16) * lv_kk(K); }

  void launch_m2m_level_fused(const OperatorDev<float> &op, int R, int level, float *M,
                              cudaStream_t s)
  {
    const int a = op.up_box_ptr[level], b = op.up_box_ptr[level + 1];
    if (b <= a)
      return;
    const int K     = op.K;
    const int ncols = (b - a) * R;
    if (op.lv_ops && op.dev_err && lv_smem_ok(K))
      {
        const int    cpb  = ncols >= 4 * lv_n_sm() ? 4 : (ncols >= 2 * lv_n_sm() ? 2 : 1);
        const size_t smem = (size_t(8) * lv_kk(K) + size_t(8) * cpb * lv_kx(K)) * sizeof(float);
        const dim3   grid(unsigned(std::min<int64_t>(lv_n_sm(), (ncols + cpb - 1) / cpb)));
        auto launch = [&](auto kern) {
          raise_smem_limit(reinterpret_cast<const void *>(kern), smem);
          launch_pdl(kern, grid, 8 * lv_kt(K), smem, s, R, K, ncols, op.up_box + a,
                     op.up_child8 + size_t(8) * a, op.lv_ops, M, op.dev_err);
        };
        switch (cpb)
          {
            case 4: launch(m2m_level_smem_kernel<4>); break;
            case 2: launch(m2m_level_smem_kernel<2>); break;
            default: launch(m2m_level_smem_kernel<1>); break;
          }
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
        return;
      }
    const int    cpb   = lv_cpb(K, ncols, 16, 4);
    const size_t smem  = size_t(16) * cpb * lv_kx(K) * sizeof(float);
    const float *ops   = op.ops + size_t(op.lv_op0) * K * K;
    const dim3   grid(unsigned((ncols + cpb - 1) / cpb));
    auto launch = [&](auto kern) {
      kern<<<grid, 8 * lv_kt(K), smem, s>>>(R, K, ncols, op.up_box + a,
                                            op.up_child8 + size_t(8) * a, ops, M);
    };
    switch (cpb)
      {
        case 4: launch(m2m_level_kernel<4>); break;
        case 2: launch(m2m_level_kernel<2>); break;
        default: launch(m2m_level_kernel<1>); break;
      }
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_m2l_sums_fused(const OperatorDev<float> &op, int R, float *Lx, const float *Y,
                             cudaStream_t s)
  {
    const int a = op.down_box_ptr.empty() ? 0 : op.down_box_ptr[1];
    const int b = op.down_box_ptr.empty() ? 0 : op.down_box_ptr.back();
    if (b <= a)
      return;
    const int64_t ncols = int64_t(b - a) * R;
    launch_pdl(m2l_sum_kernel, unsigned((ncols + 7) / 8), 256, 0, s,
      R, op.K, ncols, op.down_box + a, op.down_m2l_beg + a, op.down_m2l_end + a, Y, Lx);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_l2l_level_fused(const OperatorDev<float> &op, int R, int level, float *Lx,
                              cudaStream_t s)
  {
    const int a = op.down_box_ptr[level], b = op.down_box_ptr[level + 1];
    if (b <= a || op.down_l2l_level.empty() || !op.down_l2l_level[level])
      return;
    const int K     = op.K;
    const int ncols = (b - a) * R;
    if (op.lv_ops && op.dev_err && lv_smem_ok(K))
      {
        const size_t smem = lv_smem_bytes(K);
        raise_smem_limit(reinterpret_cast<const void *>(l2l_level_smem_kernel), smem);
        launch_pdl(l2l_level_smem_kernel, unsigned(std::min(lv_n_sm(), ncols)), 8 * lv_kt(K), smem, s,
          R, K, ncols, op.down_box + a, op.down_par + a, op.down_oct + a,
          op.lv_ops + size_t(8) * lv_kk(K), Lx, op.dev_err);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
        return;
      }
    const int    cpb   = lv_cpb(K, ncols, 5, 8);
    const size_t smem  = size_t(5) * cpb * lv_kx(K) * sizeof(float);
    const float *ops   = op.ops + size_t(op.lv_op0 + 8) * K * K;
    const dim3   grid(unsigned((ncols + cpb - 1) / cpb));
    auto launch = [&](auto kern) {
      kern<<<grid, 4 * lv_kt(K), smem, s>>>(R, K, ncols, op.down_box + a, op.down_par + a,
                                            op.down_oct + a, ops, Lx);
    };
    switch (cpb)
      {
        case 8: launch(l2l_level_kernel<8>); break;
        case 4: launch(l2l_level_kernel<4>); break;
        case 2: launch(l2l_level_kernel<2>); break;
        default: launch(l2l_level_kernel<1>); break;
      }
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
} // namespace pibem
