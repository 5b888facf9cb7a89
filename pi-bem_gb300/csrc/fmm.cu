// FMM operator kernels, one pass of BEMFMA::generate_multipole_expansions +
// multipole_matr_vect_products (source/bem_fma.cc:1971-3072) for R right-hand
// sides at once, in FP64 or FP32 (template parameter T):
//   near-field leaf-block SpMV          (prec_*_matrix.vmult, bem_fma.cc:2408-2409)
//   P2M apply from precomputed tables   (bem_fma.cc:2064-2114)
//   M2M, level by level upwards         (bem_fma.cc:2274-2376)
//   L2L + M2L, level by level downwards (bem_fma.cc:2582-2652)
//   M2P for deeper non-interaction boxes (bem_fma.cc:2664-2704)
//   L2P at the nodes of childless boxes (bem_fma.cc:2959-2986)
// Expansions are laid out [box][rhs][k] with K = (p+1)^2 scaled reals.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <type_traits>

#include "devmath.cuh"
#include "ffmath.cuh"
#include "kernels.h"
#include "pdl.cuh"

namespace pibem
{
  namespace
  {
    constexpr int RC = 4; // rhs columns handled per register block in the SpMVs

    template <typename T>
    __device__ inline T warp_sum(T v)
    {
      for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
      return v;
    }

    // a * b + c with one rounding (no dependence on the compiler's contraction)
    __device__ __forceinline__ float  fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

    // s + a . x for 4 values, with the rounding steps spelled out so that every
    // code path (one column or several) computes a column bit-for-bit alike.
    __device__ inline float dot4_acc(float s, const float (&a)[4], const float *x)
    {
      float d = __fmul_rn(a[0], x[0]);
      d       = __fmaf_rn(a[1], x[1], d);
      d       = __fmaf_rn(a[2], x[2], d);
      d       = __fmaf_rn(a[3], x[3], d);
      return __fadd_rn(s, d);
    }
    __device__ inline double dot4_acc(double s, const double (&a)[4], const double *x)
    {
      double d = __dmul_rn(a[0], x[0]);
      d        = __fma_rn(a[1], x[1], d);
      d        = __fma_rn(a[2], x[2], d);
      d        = __fma_rn(a[3], x[3], d);
      return __dadd_rn(s, d);
    }

    // 4-wide loads from 16-byte aligned rows.
    __device__ inline void load4(const float *p, float (&v)[4])
    {
      const float4 t = *reinterpret_cast<const float4 *>(p);
      v[0] = t.x;
      v[1] = t.y;
      v[2] = t.z;
      v[3] = t.w;
    }
    __device__ inline void load4(const double *p, double (&v)[4])
    {
      const double2 a = *reinterpret_cast<const double2 *>(p);
      const double2 b = *reinterpret_cast<const double2 *>(p + 2);
      v[0] = a.x;
      v[1] = a.y;
      v[2] = b.x;
      v[3] = b.y;
    }

    // Near-field leaf-block SpMV: one block per childless box.  The x entries of
    // the block's columns are gathered once into shared memory (rb rhs at a
    // time, zero in the row padding), then each warp streams whole rows of the
    // dense leaf block with 16-byte loads (rows padded to 4 values).
    template <typename T, bool ONE_COL>
    __global__ void __launch_bounds__(256)
      near_leaf_kernel(int R, int rb, int N, const int64_t *__restrict__ nrow_ptr,
                       const int64_t *__restrict__ ncol_ptr, const int64_t *__restrict__ nval_ptr,
                       const int32_t *__restrict__ nrows, const int32_t *__restrict__ ncols,
                       const T *__restrict__ vals, const T *__restrict__ x, T *__restrict__ y,
                       bool acc)
    {
      pdl_entry();
      extern __shared__ __align__(16) unsigned char smem_raw[];
      T            *sx   = reinterpret_cast<T *>(smem_raw); // [rb][ld]
      const int     leaf = blockIdx.x;
      const int64_t c0 = ncol_ptr[leaf], nc = ncol_ptr[leaf + 1] - c0;
      const int64_t ld = (nc + 3) / 4 * 4;
      const int64_t r0 = nrow_ptr[leaf], nr = nrow_ptr[leaf + 1] - r0;
      const T      *V    = vals + nval_ptr[leaf];
      const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      const int     n4   = int(ld / 4);
      for (int ra = 0; ra < R; ra += rb)
        {
          const int rc = min(rb, R - ra);
          __syncthreads();
          for (int64_t i = threadIdx.x; i < rc * ld; i += blockDim.x)
            {
              const int64_t r = i / ld, c = i - r * ld;
              sx[i]           = c < nc ? x[(ra + r) * int64_t(N) + ncols[c0 + c]] : T(0);
            }
          __syncthreads();
          for (int64_t row = warp; row < nr; row += nw)
            {
              const T  *v    = V + row * ld;
              const int node = nrows[r0 + row];
              if (ONE_COL)
                {
                  // one column: several 16-byte loads of the row in flight per lane
                  T s0 = T(0);
#pragma unroll 4
                  for (int j = lane; j < n4; j += 32)
                    {
                      T a[4];
                      load4(v + 4 * j, a);
                      s0 = dot4_acc(s0, a, sx + 4 * j);
                    }
                  const T t = warp_sum(s0);
                  if (lane == 0)
                    {
                      T &o = y[ra * int64_t(N) + node];
                      o    = acc ? o + t : t;
                    }
                  continue;
                }
              for (int rq = 0; rq < rc; rq += 4)
                {
                  T s[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll 2
                  for (int j = lane; j < n4; j += 32)
                    {
                      T a[4];
                      load4(v + 4 * j, a);
#pragma unroll
                      for (int rr = 0; rr < 4; ++rr)
                        if (rq + rr < rc)
                          s[rr] = dot4_acc(s[rr], a, sx + (rq + rr) * ld + 4 * j);
                    }
#pragma unroll
                  for (int rr = 0; rr < 4; ++rr)
                    if (rq + rr < rc)
                      {
                        const T t = warp_sum(s[rr]);
                        if (lane == 0)
                          {
                            T &o = y[(ra + rq + rr) * int64_t(N) + node];
                            o    = acc ? o + t : t;
                          }
                      }
                }
            }
        }
    }

    // 4-byte asynchronous global -> shared copy (cp.async, L1-allocating)
    __device__ inline void cp_async4(void *dst, const void *src)
    {
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                   "l"(src)
                   : "memory");
    }
    __device__ inline void cp_async8(void *dst, const void *src)
    {
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                   "l"(src)
                   : "memory");
    }
    __device__ inline void cp_async_x(float *dst, const float *src) { cp_async4(dst, src); }
    __device__ inline void cp_async_x(double *dst, const double *src) { cp_async8(dst, src); }

    // Near-field SpMV for one column where near_leaf_sched_kernel's shared
    // memory would not fit (more than about 14,500 columns in a leaf in FP32,
    // 9,600 in FP64),
    // software-pipelined: persistent blocks
    // take leaves L, L + gridDim.x, ... (the grid works through the leaves in
    // ascending windows.  Measured on GB300, 98k spheroid: 80 us; contiguous
    // leaf ranges of equal bytes per block 125 us; an L2 prefetch of the leaves
    // ahead with cp.async.bulk.prefetch 89-92 us; a dynamic schedule drawing
    // leaves from an atomic counter 89 us); while the warps stream the rows of a
    // leaf, the x entries of the block's next leaf are gathered into the other
    // half of a double buffer with cp.async.  A row is computed exactly as in
    // near_leaf_kernel (same chunks per lane, same order, same butterfly).
    // Shared memory: 2 x ld_max values.
    template <typename T>
    __global__ void __launch_bounds__(256)
      near_leaf_pipe_kernel(int n_leaves, int ld_max, const int64_t *__restrict__ nrow_ptr,
                            const int64_t *__restrict__ ncol_ptr,
                            const int64_t *__restrict__ nval_ptr, const int32_t *__restrict__ nrows,
                            const int32_t *__restrict__ ncols, const T *__restrict__ vals,
                            const T *__restrict__ x, T *__restrict__ y, bool acc)
    {
      pdl_entry();
      extern __shared__ __align__(16) unsigned char smem_raw[];
      T        *sxb  = reinterpret_cast<T *>(smem_raw); // [2][ld_max]
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      // gather of leaf l into buffer b: cp.async for the columns, zeros in the padding
      auto gather = [&](int l, int b) {
        const int64_t c0 = ncol_ptr[l], nc = ncol_ptr[l + 1] - c0;
        const int64_t ld = (nc + 3) / 4 * 4;
        T            *sx = sxb + int64_t(b) * ld_max;
        for (int64_t c = threadIdx.x; c < ld; c += blockDim.x)
          if (c < nc)
            cp_async_x(sx + c, x + ncols[c0 + c]);
          else
            sx[c] = T(0);
        asm volatile("cp.async.commit_group;" ::: "memory");
      };
      int leaf = blockIdx.x, buf = 0;
      if (leaf >= n_leaves)
        return;
      gather(leaf, 0);
      for (; leaf < n_leaves; leaf += gridDim.x, buf ^= 1)
        {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
          __syncthreads(); // this leaf's x is in place; the other buffer is free
          const int next = leaf + gridDim.x;
          if (next < n_leaves)
            gather(next, buf ^ 1);
          const T      *sx = sxb + int64_t(buf) * ld_max;
          const int64_t c0 = ncol_ptr[leaf], nc = ncol_ptr[leaf + 1] - c0;
          const int64_t ld = (nc + 3) / 4 * 4;
          const int     n4 = int(ld / 4);
          const int64_t r0 = nrow_ptr[leaf], nr = nrow_ptr[leaf + 1] - r0;
          const T      *V  = vals + nval_ptr[leaf];
          // two rows per warp at a time (rows row and row + nw), four 16-byte
          // loads of each in flight per lane
          for (int64_t row = warp; row < nr; row += 2 * nw)
            {
              const bool two = row + nw < nr;
              const T   *v0  = V + row * ld;
              const T   *v1  = V + (two ? row + nw : row) * ld;
              T          s0 = T(0), s1 = T(0);
#pragma unroll 4
              for (int j = lane; j < n4; j += 32)
                {
                  T a0[4], a1[4];
                  load4(v0 + 4 * j, a0);
                  load4(v1 + 4 * j, a1);
                  s0 = dot4_acc(s0, a0, sx + 4 * j);
                  s1 = dot4_acc(s1, a1, sx + 4 * j);
                }
              const T t0 = warp_sum(s0), t1 = warp_sum(s1);
              if (lane == 0)
                {
                  T &o0 = y[nrows[r0 + row]];
                  o0    = acc ? o0 + t0 : t0;
                  if (two)
                    {
                      T &o1 = y[nrows[r0 + row + nw]];
                      o1    = acc ? o1 + t1 : t1;
                    }
                }
            }
        }
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }

    __device__ inline void cp_async16(void *dst, const void *src)
    {
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                   "l"(src)
                   : "memory");
    }

    // Schedule position of the t-th leaf of block b: snake order over the G
    // blocks (b, 2G-1-b, 2G+b, ...), so that with the leaves sorted by bytes
    // every block streams about the same amount.
    __device__ __forceinline__ int64_t near_sched_pos(int b, int t, int G)
    {
      return int64_t(t) * G + ((t & 1) ? G - 1 - b : b);
    }

    // 16-byte streaming loads that do not allocate in L1
    __device__ inline void load4_na(const float *p, float (&v)[4])
    {
      asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
          : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
          : "l"(p));
    }
    __device__ inline void load4_na(const double *p, double (&v)[4])
    {
      asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v[0]), "=d"(v[1]) : "l"(p));
      asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v[2]), "=d"(v[3]) : "l"(p + 2));
    }
    template <bool NA, typename T>
    __device__ __forceinline__ void load4v(const T *p, T (&v)[4])
    {
      if constexpr (NA)
        load4_na(p, v);
      else
        load4(p, v);
    }

    // Near-field SpMV for one column: persistent blocks over a schedule of the
    // leaves sorted by value bytes (record per leaf: value offset, column
    // offset, row offset, rows | columns << 32), three stages deep.  While the
    // warps stream the rows of the block's leaf t, the block has one cp.async
    // group in flight holding the x entries of its leaf t+1 (gathered through
    // the column ids already in shared memory), the column ids of leaf t+2 and
    // the schedule record of leaf t+3, so that inside a leaf only the row
    // values are waited for.  Rows: two per warp at a time, the 16-byte loads of NB
    // chunks per lane and row issued before any is used (NA: loads that do not
    // allocate in L1).  A row is computed exactly as in near_leaf_kernel (same
    // chunks per lane, same order, same butterfly), so the leaf order and the
    // block shape do not change a bit of y.
    // Shared memory: 128 bytes of records, 2 x ld_max column ids, 2 x ld_max x.
    template <typename T, int NB, int BS, bool NA>
    __global__ void __launch_bounds__(BS)
      near_leaf_sched_kernel(int n_leaves, int ld_max, const int64_t *__restrict__ sched,
                             const int32_t *__restrict__ nrows, const int32_t *__restrict__ ncols,
                             const T *__restrict__ vals, const T *__restrict__ x,
                             T *__restrict__ y, bool acc)
    {
      pdl_entry();
      extern __shared__ __align__(16) unsigned char smem_raw[];
      int64_t  *srec = reinterpret_cast<int64_t *>(smem_raw);       // [4][4]
      int32_t  *sid  = reinterpret_cast<int32_t *>(smem_raw + 128); // [2][ld_max]
      T        *sxb  = reinterpret_cast<T *>(smem_raw + 128 + size_t(8) * ld_max); // [2][ld_max]
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      const int G = gridDim.x, b = blockIdx.x;
      auto valid = [&](int t) { return near_sched_pos(b, t, G) < n_leaves; };
      auto rec   = [&](int t) { return srec + 4 * (t & 3); };
      // schedule record of leaf t (threads 0 and 1, 16 bytes each)
      auto fetch_rec = [&](int t) {
        if (threadIdx.x < 2 && valid(t))
          cp_async16(rec(t) + 2 * threadIdx.x, sched + 4 * near_sched_pos(b, t, G) + 2 * threadIdx.x);
      };
      // column ids of leaf t (its record in place)
      auto fetch_ids = [&](int t) {
        const int64_t c0 = rec(t)[1];
        const int     nc = int(uint64_t(rec(t)[3]) >> 32);
        int32_t      *d  = sid + (t & 1) * ld_max;
        for (int c = threadIdx.x; c < nc; c += blockDim.x)
          cp_async4(d + c, ncols + c0 + c);
      };
      // x entries of leaf t (its column ids in place), zeros in the padding
      auto gather_x = [&](int t) {
        const int      nc = int(uint64_t(rec(t)[3]) >> 32), ld = (nc + 3) & ~3;
        const int32_t *si = sid + (t & 1) * ld_max;
        T             *d  = sxb + (t & 1) * ld_max;
        for (int c = threadIdx.x; c < ld; c += blockDim.x)
          if (c < nc)
            cp_async_x(d + c, x + si[c]);
          else
            d[c] = T(0);
      };
      if (!valid(0))
        return;
      fetch_rec(0);
      fetch_rec(1);
      fetch_rec(2);
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      __syncthreads();
      fetch_ids(0);
      if (valid(1))
        fetch_ids(1);
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      __syncthreads();
      gather_x(0);
      asm volatile("cp.async.commit_group;" ::: "memory");
      for (int t = 0; valid(t); ++t)
        {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
          __syncthreads(); // leaf t's x, leaf t+1's ids, records t..t+2 in place
          if (valid(t + 1))
            gather_x(t + 1);
          if (valid(t + 2))
            fetch_ids(t + 2);
          fetch_rec(t + 3);
          asm volatile("cp.async.commit_group;" ::: "memory");
          const int64_t *r  = rec(t);
          const T       *V  = vals + r[0];
          const int64_t  r0 = r[2];
          const int      nr = int(uint32_t(uint64_t(r[3]))), nc = int(uint64_t(r[3]) >> 32);
          const int      ld = (nc + 3) & ~3, n4 = ld >> 2;
          const T       *sx = sxb + (t & 1) * ld_max;
          for (int row = warp; row < nr; row += 2 * nw)
            {
              const bool two = row + nw < nr;
              int        o0 = 0, o1 = 0;
              if (lane == 0)
                {
                  o0 = nrows[r0 + row];
                  o1 = two ? nrows[r0 + row + nw] : o0;
                }
              const T *v0 = V + int64_t(row) * ld;
              const T *v1 = V + int64_t(two ? row + nw : row) * ld;
              T        s0 = T(0), s1 = T(0);
              for (int jb = lane; jb < n4; jb += 32 * NB)
                {
                  T a0[NB][4], a1[NB][4];
#pragma unroll
                  for (int k = 0; k < NB; ++k)
                    if (jb + 32 * k < n4)
                      {
                        load4v<NA>(v0 + 4 * (jb + 32 * k), a0[k]);
                        if (two)
                          load4v<NA>(v1 + 4 * (jb + 32 * k), a1[k]);
                      }
#pragma unroll
                  for (int k = 0; k < NB; ++k)
                    if (jb + 32 * k < n4)
                      {
                        s0 = dot4_acc(s0, a0[k], sx + 4 * (jb + 32 * k));
                        if (two)
                          s1 = dot4_acc(s1, a1[k], sx + 4 * (jb + 32 * k));
                      }
                }
              const T t0 = warp_sum(s0), t1 = warp_sum(s1);
              if (lane == 0)
                {
                  T &y0 = y[o0];
                  y0    = acc ? y0 + t0 : t0;
                  if (two)
                    {
                      T &y1 = y[o1];
                      y1    = acc ? y1 + t1 : t1;
                    }
                }
            }
        }
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }

    // FP64-accurate near-field SpMV for one column on the FP32 pipes: the
    // values and x as (hi, lo) FP32 pairs (8 bytes a value, as FP64), every
    // product split exactly (TwoProduct) with its cross terms, the row sums
    // carried with TwoSum; about 11 FP32 instructions per value, so the kernel
    // streams at HBM speed where FP64 FMA (1/58 of the FP32 rate) could not.
    // Same structure as near_leaf_pipe_kernel: persistent blocks, the next
    // leaf's x gathered with cp.async while the warps stream two rows each.
    // y[row] = hi + lo in FP64 (acc: added).
    __global__ void __launch_bounds__(256)
      near_leaf_ff_kernel(int n_leaves, int ld_max,
                          const int64_t *__restrict__ nrow_ptr,
                          const int64_t *__restrict__ ncol_ptr, const int64_t *__restrict__ nval_ptr,
                          const int32_t *__restrict__ nrows, const int32_t *__restrict__ ncols,
                          const float2 *__restrict__ vals, const float2 *__restrict__ x,
                          double *__restrict__ y, bool acc)
    {
      extern __shared__ __align__(16) unsigned char smem_raw[];
      float2   *sxb  = reinterpret_cast<float2 *>(smem_raw); // [2][ld_max]
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      auto gather = [&](int l, int b) {
        const int64_t c0 = ncol_ptr[l], nc = ncol_ptr[l + 1] - c0;
        const int64_t ld = (nc + 3) / 4 * 4;
        float2       *sx = sxb + int64_t(b) * ld_max;
        for (int64_t c = threadIdx.x; c < ld; c += blockDim.x)
          if (c < nc)
            cp_async8(reinterpret_cast<double *>(sx + c), reinterpret_cast<const double *>(x + ncols[c0 + c]));
          else
            sx[c] = make_float2(0.f, 0.f);
        asm volatile("cp.async.commit_group;" ::: "memory");
      };
      int leaf = blockIdx.x, buf = 0;
      if (leaf >= n_leaves)
        return;
      gather(leaf, 0);
      for (; leaf < n_leaves; leaf += gridDim.x, buf ^= 1)
        {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
          __syncthreads();
          const int next = leaf + gridDim.x;
          if (next < n_leaves)
            gather(next, buf ^ 1);
          const float2 *sx = sxb + int64_t(buf) * ld_max;
          const int64_t c0 = ncol_ptr[leaf], nc = ncol_ptr[leaf + 1] - c0;
          const int64_t ld = (nc + 3) / 4 * 4;
          const int     n4 = int(ld / 4);
          const int64_t r0 = nrow_ptr[leaf], nr = nrow_ptr[leaf + 1] - r0;
          const float2 *V  = vals + nval_ptr[leaf];
          for (int64_t row = warp; row < nr; row += 2 * nw)
            {
              const bool    two = row + nw < nr;
              const float2 *v0  = V + row * ld;
              const float2 *v1  = V + (two ? row + nw : row) * ld;
              float         h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
#pragma unroll 2
              for (int j = lane; j < n4; j += 32)
                {
                  const float4 a0 = *reinterpret_cast<const float4 *>(v0 + 4 * j);
                  const float4 b0 = *reinterpret_cast<const float4 *>(v0 + 4 * j + 2);
                  const float4 a1 = *reinterpret_cast<const float4 *>(v1 + 4 * j);
                  const float4 b1 = *reinterpret_cast<const float4 *>(v1 + 4 * j + 2);
                  const float2 x0 = sx[4 * j], x1 = sx[4 * j + 1], x2 = sx[4 * j + 2], x3 = sx[4 * j + 3];
                  ff_mac(h0, l0, make_float2(a0.x, a0.y), x0);
                  ff_mac(h0, l0, make_float2(a0.z, a0.w), x1);
                  ff_mac(h0, l0, make_float2(b0.x, b0.y), x2);
                  ff_mac(h0, l0, make_float2(b0.z, b0.w), x3);
                  ff_mac(h1, l1, make_float2(a1.x, a1.y), x0);
                  ff_mac(h1, l1, make_float2(a1.z, a1.w), x1);
                  ff_mac(h1, l1, make_float2(b1.x, b1.y), x2);
                  ff_mac(h1, l1, make_float2(b1.z, b1.w), x3);
                }
              float2 t0 = ff_norm(h0, l0), t1 = ff_norm(h1, l1);
              for (int o = 16; o > 0; o >>= 1)
                {
                  t0 = ff_add(t0, make_float2(__shfl_xor_sync(0xffffffffu, t0.x, o),
                                              __shfl_xor_sync(0xffffffffu, t0.y, o)));
                  t1 = ff_add(t1, make_float2(__shfl_xor_sync(0xffffffffu, t1.x, o),
                                              __shfl_xor_sync(0xffffffffu, t1.y, o)));
                }
              if (lane == 0)
                {
                  double &o0 = y[nrows[r0 + row]];
                  o0         = acc ? __dadd_rn(o0, ff_join(t0)) : ff_join(t0);
                  if (two)
                    {
                      double &o1 = y[nrows[r0 + row + nw]];
                      o1         = acc ? __dadd_rn(o1, ff_join(t1)) : ff_join(t1);
                    }
                }
            }
        }
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }

    // P2M apply: M^[leaf][r][k] = sum_rows w(row, r) T[row][k] x_r[dof(row)],
    // w selecting the double layer (Ker1), the single layer (Ker2) or the
    // combined system strengths.  One warp per leaf, 8 leaves per block: lane l
    // owns coefficients 4l..4l+3 (table rows padded to K4 values); the rows'
    // weights are gathered 32 at a time (lane j: row j) and broadcast by
    // shuffles; eight table rows in flight; the rows are summed in order.
    // COMBINED: every column uses the combined strengths, read from the table
    // Tc = (Dirichlet dof ? -T2 : T1) made at set_bc (one table row per row
    // instead of two); T1 is then Tc and T2 is unused.
    // RC: columns per pass (1 for one right-hand side, else 4).
    template <typename T, bool COMBINED, int RC>
    __global__ void __launch_bounds__(256)
      p2m_apply_kernel(int n_leaves, int R, int K, int N, const int64_t *__restrict__ prow_ptr,
                       const int32_t *__restrict__ pleaf_box, const int32_t *__restrict__ prow_dof,
                       const T *__restrict__ T1, const T *__restrict__ T2,
                       const uint8_t *__restrict__ dir, const uint8_t *__restrict__ modes,
                       const T *__restrict__ x, T *__restrict__ M)
    {
      pdl_entry();
      const int leaf = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
      if (leaf >= n_leaves)
        return;
      const int     K4  = (K + 3) / 4 * 4;
      const int64_t box = pleaf_box[leaf];
      const int64_t rb = prow_ptr[leaf], re = prow_ptr[leaf + 1];
      const bool    act = 4 * lane < K4;
      for (int rq = 0; rq < R; rq += RC)
        {
          const int rc = min(RC, R - rq);
          T         acc[RC][4];
#pragma unroll
          for (int a = 0; a < RC; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
              acc[a][b] = T(0);
          for (int64_t b0 = rb; b0 < re; b0 += 32)
            {
              const int nb = re - b0 < 32 ? int(re - b0) : 32;
              T         w1[RC], w2[RC];
#pragma unroll
              for (int rr = 0; rr < RC; ++rr)
                w1[rr] = w2[rr] = T(0);
              if (lane < nb)
                {
                  const int  dof = prow_dof[b0 + lane];
                  const bool d   = dir[dof] != 0;
#pragma unroll
                  for (int rr = 0; rr < RC; ++rr)
                    if (rr < rc)
                      {
                        const T xv = x[int64_t(rq + rr) * N + dof];
                        if constexpr (COMBINED)
                          w1[rr] = xv;
                        else
                          {
                            const uint8_t mode = modes[rq + rr];
                            const bool    dd   = mode == MODE_SWAPPED ? !d : d;
                            w1[rr] = mode == MODE_KER2 ? T(0) : (mode == MODE_KER1 ? xv : (dd ? T(0) : xv));
                            w2[rr] = mode == MODE_KER1 ? T(0) : (mode == MODE_KER2 ? xv : (dd ? -xv : T(0)));
                          }
                      }
                }
              for (int j0 = 0; j0 < nb; j0 += 8)
                {
                  T t1[8][4], t2[8][4];
#pragma unroll
                  for (int u = 0; u < 8; ++u)
                    if (act && j0 + u < nb)
                      {
                        load4(T1 + (b0 + j0 + u) * K4 + 4 * lane, t1[u]);
                        if constexpr (!COMBINED)
                          load4(T2 + (b0 + j0 + u) * K4 + 4 * lane, t2[u]);
                      }
#pragma unroll
                  for (int u = 0; u < 8; ++u)
                    if (j0 + u < nb)
#pragma unroll
                      for (int rr = 0; rr < RC; ++rr)
                        if (rr < rc)
                          {
                            const T a1 = __shfl_sync(0xffffffffu, w1[rr], j0 + u);
                            if constexpr (COMBINED)
                              {
#pragma unroll
                                for (int c = 0; c < 4; ++c)
                                  acc[rr][c] += a1 * t1[u][c];
                              }
                            else
                              {
                                const T a2 = __shfl_sync(0xffffffffu, w2[rr], j0 + u);
#pragma unroll
                                for (int c = 0; c < 4; ++c)
                                  acc[rr][c] += a1 * t1[u][c] + a2 * t2[u][c];
                              }
                          }
                }
            }
          if (act)
#pragma unroll
            for (int rr = 0; rr < RC; ++rr)
              if (rr < rc)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                  if (4 * lane + c < K)
                    M[(box * R + rq + rr) * K + 4 * lane + c] = acc[rr][c];
        }
    }

    // Batched translation GEMM.  Scaled operators do not depend on the level:
    // M2L depends only on the integer source-target offset, M2M / L2L only on
    // the child octant.  Pairs sharing an operator are cut into chunks of <= 128;
    // block (c, t) computes  Y[q] = T_op(c) E[src(q)]  for columns 64t..64t+63 of
    // chunk c (column = (pair, rhs)), with the operator staged in shared memory
    // (CUDA-core FMA, 16x16 threads, KI x 4 outputs per thread, KI = ceil(K/16)
    // so that no thread computes rows beyond K).
    constexpr int GB_COLS = 64;
    constexpr int GB_LDB  = GB_COLS + 1;

    template <typename T, int KI>
    __global__ void __launch_bounds__(256, 2)
      trans_gemm_kernel(int R, int K, int chunk0, const int32_t *__restrict__ chunk_start,
                        const int32_t *__restrict__ chunk_cnt, const int32_t *__restrict__ chunk_off,
                        const int32_t *__restrict__ q_src, const T *__restrict__ ops,
                        const T *__restrict__ M, T *__restrict__ Y,
                        const int32_t *__restrict__ yslot, int ldy)
    {
      extern __shared__ unsigned char smem_raw[];
      T        *sT    = reinterpret_cast<T *>(smem_raw); // [K][K] in-major
      T        *sB    = sT + K * K;                      // [K][GB_LDB]
      const int ch    = chunk0 + blockIdx.x;
      const int start = chunk_start[ch], ncols = chunk_cnt[ch] * R;
      const int c0    = blockIdx.y * GB_COLS;
      if (c0 >= ncols)
        return;
      const int nc = min(GB_COLS, ncols - c0);
      const T  *op = ops + int64_t(chunk_off[ch]) * K * K;
      for (int i = threadIdx.x; i < K * K; i += blockDim.x)
        sT[i] = op[i];
      for (int idx = threadIdx.x; idx < nc * K; idx += blockDim.x)
        {
          const int     c  = idx / K, ki = idx - c * K;
          const int     cg = c0 + c;
          const int64_t q  = start + cg / R;
          const int     r  = cg % R;
          sB[ki * GB_LDB + c] = M[(int64_t(q_src[q]) * R + r) * K + ki];
        }
      __syncthreads();
      // rows ko = row0 + tx + 16 i of this block (row0 > 0 when the rows are split
      // over blockIdx.z for launches with few blocks)
      const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4, row0 = blockIdx.z * 16 * KI;
      T         acc[KI][4];
#pragma unroll
      for (int i = 0; i < KI; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          acc[i][j] = T(0);
      for (int ki = 0; ki < K; ++ki)
        {
          T a[KI], b[4];
#pragma unroll
          for (int i = 0; i < KI; ++i)
            {
              const int ko = row0 + tx + 16 * i;
              a[i]         = ko < K ? sT[ki * K + ko] : T(0);
            }
#pragma unroll
          for (int j = 0; j < 4; ++j)
            b[j] = sB[ki * GB_LDB + ty + 16 * j];
#pragma unroll
          for (int i = 0; i < KI; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
              acc[i][j] = fma_rn(a[i], b[j], acc[i][j]);
        }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        {
          const int c = ty + 16 * j;
          if (c >= nc)
            continue;
          const int     cg = c0 + c;
          const int64_t q  = start + cg / R;
          const int     r  = cg % R;
          const int64_t yr = (yslot ? int64_t(yslot[q]) : q) * R + r; // row of (pair, rhs)
#pragma unroll
          for (int i = 0; i < KI; ++i)
            {
              const int ko = row0 + tx + 16 * i;
              if (ko < K)
                Y[yr * ldy + ko] = acc[i][j];
            }
        }
    }

    __device__ __forceinline__ float2 ff_load(const double *p) { return ff_split(*p); }
    __device__ __forceinline__ float2 ff_load(const float2 *p) { return *p; }
    __device__ __forceinline__ void   ff_store(double *p, float h, float l) { *p = __dadd_rn(double(h), double(l)); }
    __device__ __forceinline__ void   ff_store(float2 *p, float h, float l) { *p = ff_norm(h, l); }

    // The translation GEMM of the FP64 operator in float-float arithmetic on
    // the FP32 pipes: operator pre-split into (hi, lo) pairs; expansions and
    // products either FP64 (split on load, joined on store) or already in
    // (hi, lo) form (IO = float2: no FP64 instruction at all).  Thread (tx, ty)
    // of TX x (64 / CJ) computes rows row0 + tx + TX i (i < RI) and columns
    // ty + (64 / CJ) j (j < CJ) of a 64-column block of chunk c; TX RI >= K
    // rows with TX = ceil(K / RI), so at most RI - 1 rows are padding.
    template <int RI, int CJ, typename IO>
    __global__ void __launch_bounds__(256, 2)
      ff_gemm_kernel(int R, int K, int TX, int chunk0, const int32_t *__restrict__ chunk_start,
                     const int32_t *__restrict__ chunk_cnt, const int32_t *__restrict__ chunk_off,
                     const int32_t *__restrict__ q_src, const float2 *__restrict__ ops,
                     const IO *__restrict__ M, IO *__restrict__ Y)
    {
      extern __shared__ __align__(16) unsigned char smem_raw[];
      float2   *sT    = reinterpret_cast<float2 *>(smem_raw); // [K][K] in-major
      float2   *sB    = sT + K * K;                           // [K][GB_LDB]
      const int ch    = chunk0 + blockIdx.x;
      const int start = chunk_start[ch], ncols = chunk_cnt[ch] * R;
      const int c0    = blockIdx.y * GB_COLS;
      if (c0 >= ncols)
        return;
      const int     nc = min(GB_COLS, ncols - c0);
      const float2 *op = ops + int64_t(chunk_off[ch]) * K * K;
      for (int i = threadIdx.x; i < K * K; i += blockDim.x)
        sT[i] = op[i];
      for (int idx = threadIdx.x; idx < nc * K; idx += blockDim.x)
        {
          const int     c  = idx / K, ki = idx - c * K;
          const int     cg = c0 + c;
          const int64_t q  = start + cg / R;
          const int     r  = cg % R;
          sB[ki * GB_LDB + c] = ff_load(M + (int64_t(q_src[q]) * R + r) * K + ki);
        }
      __syncthreads();
      constexpr int TY = 64 / CJ;
      const int     tx = threadIdx.x % TX, ty = threadIdx.x / TX, row0 = blockIdx.z * TX * RI;
      if (ty >= TY)
        return;
      float sh[RI][CJ], sl[RI][CJ];
#pragma unroll
      for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < CJ; ++j)
          sh[i][j] = sl[i][j] = 0.0f;
      for (int ki = 0; ki < K; ++ki)
        {
          float2 a[RI], b[CJ];
#pragma unroll
          for (int i = 0; i < RI; ++i)
            {
              const int ko = row0 + tx + TX * i;
              a[i]         = ko < K ? sT[ki * K + ko] : make_float2(0.0f, 0.0f);
            }
#pragma unroll
          for (int j = 0; j < CJ; ++j)
            b[j] = sB[ki * GB_LDB + ty + TY * j];
#pragma unroll
          for (int i = 0; i < RI; ++i)
#pragma unroll
            for (int j = 0; j < CJ; ++j)
              ff_mac(sh[i][j], sl[i][j], a[i], b[j]);
        }
#pragma unroll
      for (int j = 0; j < CJ; ++j)
        {
          const int c = ty + TY * j;
          if (c >= nc)
            continue;
          const int     cg = c0 + c;
          const int64_t q  = start + cg / R;
          const int     r  = cg % R;
#pragma unroll
          for (int i = 0; i < RI; ++i)
            {
              const int ko = row0 + tx + TX * i;
              if (ko < K)
                ff_store(Y + (q * R + r) * K + ko, sh[i][j], sl[i][j]);
            }
        }
    }

    // out[box] = sum of the box's (hi, lo) translation products, in list order,
    // in float-float arithmetic; 8 loads in flight.
    __global__ void gather_ff_kernel(int R, int K, const int32_t *__restrict__ boxes,
                                     const int64_t *__restrict__ q_ptr,
                                     const int32_t *__restrict__ q, const float2 *__restrict__ Y,
                                     float2 *__restrict__ out)
    {
      const int64_t b  = boxes[blockIdx.x];
      const int64_t e0 = q_ptr[blockIdx.x], e1 = q_ptr[blockIdx.x + 1];
      const int64_t RK = int64_t(R) * K;
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        {
          float2  acc = make_float2(0.0f, 0.0f);
          int64_t e   = e0;
          for (; e + 8 <= e1; e += 8)
            {
              float2 v[8];
#pragma unroll
              for (int u = 0; u < 8; ++u)
                v[u] = Y[int64_t(q[e + u]) * RK + i];
#pragma unroll
              for (int u = 0; u < 8; ++u)
                acc = ff_add(acc, v[u]);
            }
          for (; e < e1; ++e)
            acc = ff_add(acc, Y[int64_t(q[e]) * RK + i]);
          out[b * RK + i] = acc;
        }
    }

    __global__ void d2ff_kernel(int64_t n, const double *__restrict__ a, float2 *__restrict__ b)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i < n)
        b[i] = ff_split(a[i]);
    }
    __global__ void ff2d_kernel(int64_t n, const float2 *__restrict__ a, double *__restrict__ b)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i < n)
        b[i] = ff_join(a[i]);
    }

    // out[box] = sum of the box's translation products Y[q], in list order.  The
    // loads of 8 consecutive products are issued before they are added (same
    // order of additions), so a thread has 8 L2 reads in flight.
    template <typename T>
    __global__ void gather_kernel(int R, int K, const int32_t *__restrict__ boxes,
                                  const int64_t *__restrict__ q_ptr, const int32_t *__restrict__ q,
                                  const T *__restrict__ Y, T *__restrict__ out)
    {
      const int64_t b  = boxes[blockIdx.x];
      const int64_t e0 = q_ptr[blockIdx.x], e1 = q_ptr[blockIdx.x + 1];
      const int64_t RK = int64_t(R) * K;
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        {
          T       acc = T(0);
          int64_t e   = e0;
          for (; e + 8 <= e1; e += 8)
            {
              T v[8];
#pragma unroll
              for (int u = 0; u < 8; ++u)
                v[u] = Y[int64_t(q[e + u]) * RK + i];
#pragma unroll
              for (int u = 0; u < 8; ++u)
                acc += v[u];
            }
          for (; e < e1; ++e)
            acc += Y[int64_t(q[e]) * RK + i];
          out[b * RK + i] = acc;
        }
    }

    // M2P phase 1: one thread per (pair, collocation node of the pair's target
    // box): scratch[r][item] = multipole of the source box evaluated at the
    // node.  tnodes lists each target box's collocation nodes (tnode_ptr).
    template <typename T>
    __global__ void m2p_eval_kernel(int64_t n_items, int R, int K, int p,
                                    const int64_t *__restrict__ item_ptr,
                                    const int32_t *__restrict__ item_pair,
                                    const int32_t *__restrict__ pair_tgt,
                                    const int32_t *__restrict__ tgt,
                                    const int32_t *__restrict__ src,
                                    const int64_t *__restrict__ tnode_ptr,
                                    const int32_t *__restrict__ tnodes,
                                    const double *__restrict__ xyz,
                                    const double *__restrict__ center,
                                    const double *__restrict__ delta, const T *__restrict__ M,
                                    T *__restrict__ scratch)
    {
      pdl_entry();
      const int64_t it = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (it >= n_items)
        return;
      const int64_t e    = item_pair[it];
      const int64_t s    = src[e];
      const int     node = tnodes[tnode_ptr[pair_tgt[e]] + (it - item_ptr[e])];
      const double  h    = delta[s];
      T             rx, ry, rz, ih;
      if constexpr (std::is_same<T, float>::value)
        {
          // FP32 operator: the offset from the centre in FP64 (no cancellation),
          // scaled in FP32 (GB300's FP64 divide would dominate this kernel)
          ih = __frcp_rn(float(h));
          rx = float(xyz[3 * int64_t(node)] - center[3 * s]) * ih;
          ry = float(xyz[3 * int64_t(node) + 1] - center[3 * s + 1]) * ih;
          rz = float(xyz[3 * int64_t(node) + 2] - center[3 * s + 2]) * ih;
        }
      else
        {
          rx = (xyz[3 * int64_t(node)] - center[3 * s]) / h;
          ry = (xyz[3 * int64_t(node) + 1] - center[3 * s + 1]) / h;
          rz = (xyz[3 * int64_t(node) + 2] - center[3 * s + 2]) / h;
          ih = 1.0 / h;
        }
      for (int r = 0; r < R; ++r)
        scratch[int64_t(r) * n_items + it] =
          eval_expansion_fast<T, T>(M + (s * R + r) * K, p, rx, ry, rz, true) * ih;
    }

    // The table-driven evaluation of eval_expansion_fast (same recurrences, same
    // order of terms) in float-float arithmetic for the FP64-accurate operator:
    // r is the offset from the box centre in box units (pairs), coef the
    // expansion as pairs.  About 90 FP32 instructions per term against the
    // FP64 pipe's 1/58 rate.
    __device__ float2 eval_multipole_ff(const float2 *__restrict__ coef, int p, float2 rx, float2 ry,
                                        float2 rz)
    {
      const float2 rxy2 = ff_add(ff_mul(rx, rx), ff_mul(ry, ry));
      const float2 rho  = ff_sqrt(ff_add(rxy2, ff_mul(rz, rz)));
      const float2 inv  = ff_recip(rho);
      const float2 x    = ff_mul(rz, inv);
      const float2 s    = ff_sqrt(ff_sub(make_float2(1.f, 0.f), ff_mul(x, x)));
      const float2 rxy  = ff_sqrt(rxy2);
      float2       cb = make_float2(1.f, 0.f), sb = make_float2(0.f, 0.f);
      if (rxy.x > 0.f)
        {
          const float2 ir = ff_recip(rxy);
          cb              = ff_mul(rx, ir);
          sb              = ff_mul(ry, ir);
        }
      const float2 step = inv;
      float2       acc = make_float2(0.f, 0.f), pmm = make_float2(1.f, 0.f), rpm = inv;
      float2       cm = make_float2(1.f, 0.f), sm = make_float2(0.f, 0.f);
      for (int m = 0; m <= p; ++m)
        {
          if (m > 0)
            {
              pmm             = ff_mul(pmm, ff_mul(ff_neg(c_leg.ffcmm[m]), s));
              rpm             = ff_mul(rpm, step);
              const float2 c2 = ff_sub(ff_mul(cm, cb), ff_mul(sm, sb));
              sm              = ff_add(ff_mul(sm, cb), ff_mul(cm, sb));
              cm              = c2;
            }
          // 2 cm and -2 sm: exact scalings
          const float2 cr = m == 0 ? make_float2(1.f, 0.f) : make_float2(2.f * cm.x, 2.f * cm.y);
          const float2 ci = m == 0 ? make_float2(0.f, 0.f) : make_float2(-2.f * sm.x, -2.f * sm.y);
          auto term = [&](int n) {
            const int    k0 = n * n + (m == 0 ? 0 : 2 * m - 1);
            const float2 v  = m > 0 ? ff_add(ff_mul(coef[k0], cr), ff_mul(coef[k0 + 1], ci))
                                    : ff_mul(coef[k0], cr);
            return v;
          };
          float2 p0 = pmm, rp = rpm;
          acc       = ff_add(acc, ff_mul(ff_mul(term(m), p0), rp));
          if (m + 1 <= p)
            {
              float2 p1 = ff_mul(ff_mul(x, c_leg.ffcm1[m]), pmm);
              rp        = ff_mul(rp, step);
              acc       = ff_add(acc, ff_mul(ff_mul(term(m + 1), p1), rp));
              for (int n = m + 2; n <= p; ++n)
                {
                  const float2 p2 = ff_sub(ff_mul(ff_mul(c_leg.ffra[n][m], x), p1),
                                           ff_mul(c_leg.ffrb[n][m], p0));
                  p0 = p1;
                  p1 = p2;
                  rp = ff_mul(rp, step);
                  acc = ff_add(acc, ff_mul(ff_mul(term(n), p1), rp));
                }
            }
        }
      return acc;
    }

    // M2P phase 1 of the FP64-accurate operator: as m2p_eval_kernel, from the
    // (hi, lo) multipoles; the offset from the centre is formed in FP64 and
    // split, the scaling by 1 / h in float-float; the value stored in FP64.
    __global__ void m2p_eval_ff_kernel(int64_t n_items, int R, int K, int p,
                                       const int64_t *__restrict__ item_ptr,
                                       const int32_t *__restrict__ item_pair,
                                       const int32_t *__restrict__ pair_tgt,
                                       const int32_t *__restrict__ src,
                                       const int64_t *__restrict__ tnode_ptr,
                                       const int32_t *__restrict__ tnodes,
                                       const double *__restrict__ xyz,
                                       const double *__restrict__ center,
                                       const double *__restrict__ delta,
                                       const float2 *__restrict__ M, double *__restrict__ scratch)
    {
      const int64_t it = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (it >= n_items)
        return;
      const int64_t e    = item_pair[it];
      const int64_t s    = src[e];
      const int     node = tnodes[tnode_ptr[pair_tgt[e]] + (it - item_ptr[e])];
      const float2  ih   = ff_recip(ff_split(delta[s]));
      const float2  rx   = ff_mul(ff_split(__dsub_rn(xyz[3 * int64_t(node)], center[3 * s])), ih);
      const float2  ry   = ff_mul(ff_split(__dsub_rn(xyz[3 * int64_t(node) + 1], center[3 * s + 1])), ih);
      const float2  rz   = ff_mul(ff_split(__dsub_rn(xyz[3 * int64_t(node) + 2], center[3 * s + 2])), ih);
      for (int r = 0; r < R; ++r)
        scratch[int64_t(r) * n_items + it] =
          ff_join(ff_mul(eval_multipole_ff(M + (s * R + r) * K, p, rx, ry, rz), ih));
    }

    // M2P phase 2: one warp per target box, one lane per node of the box: the
    // node's values over the box's sources, added in list order to y.  The
    // items of a target box are contiguous, source-major (item_ptr[e] =
    // item_ptr[e0] + (e - e0) nn), so a node's values sit nn apart; 16 loads
    // in flight.
    template <typename T>
    __global__ void __launch_bounds__(256)
      m2p_sum_kernel(int n_tgt, int R, int N, int64_t n_items, const int64_t *__restrict__ tnode_ptr,
                     const int32_t *__restrict__ tgt, const int64_t *__restrict__ src_ptr,
                     const int64_t *__restrict__ item_ptr, const int32_t *__restrict__ tnodes,
                     const T *__restrict__ scratch, T *__restrict__ y)
    {
      pdl_entry();
      const int ti = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
      if (ti >= n_tgt)
        return;
      const int64_t  nn = tnode_ptr[ti + 1] - tnode_ptr[ti];
      const int64_t  e0 = src_ptr[ti], ns = src_ptr[ti + 1] - e0;
      const int64_t  base = e0 < src_ptr[n_tgt] ? item_ptr[e0] : 0;
      const int32_t *nodes = tnodes + tnode_ptr[ti];
      for (int64_t i = lane; i < nn; i += 32)
        {
          const int node = nodes[i];
          for (int r = 0; r < R; ++r)
            {
              const T *sc  = scratch + int64_t(r) * n_items + base + i;
              T        acc = T(0);
              int64_t  j   = 0;
              for (; j + 16 <= ns; j += 16)
                {
                  T v[16];
#pragma unroll
                  for (int u = 0; u < 16; ++u)
                    v[u] = sc[(j + u) * nn];
#pragma unroll
                  for (int u = 0; u < 16; ++u)
                    acc += v[u];
                }
              for (; j < ns; ++j)
                acc += sc[j * nn];
              y[int64_t(r) * N + node] += acc;
            }
        }
    }

    // L2P: y[r][node] += W[row] . L^[leaf][r] for every row (node of a
    // childless box).  One warp per leaf, 8 leaves per block: lane l multiplies
    // coefficients 4l..4l+3 (W rows padded to K4 values), eight rows in flight;
    // the lanes' products are added by a fixed butterfly, and lane u updates
    // the node of row u of each group of eight.
    template <typename T>
    __global__ void __launch_bounds__(256)
      l2p_kernel(int n_leaves, int R, int K, int N, const int64_t *__restrict__ row_ptr,
                 const int32_t *__restrict__ lleaf_box, const int32_t *__restrict__ nrows,
                 const T *__restrict__ W, const T *__restrict__ Lx, T *__restrict__ y)
    {
      pdl_entry();
      const int leaf = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
      if (leaf >= n_leaves)
        return;
      const int     K4  = (K + 3) / 4 * 4;
      const int64_t box = lleaf_box[leaf];
      const int64_t r0 = row_ptr[leaf], r1 = row_ptr[leaf + 1];
      const bool    act = 4 * lane < K4;
      for (int r = 0; r < R; ++r)
        {
          T l[4] = {T(0), T(0), T(0), T(0)};
          if (act)
            {
              const T *lp = Lx + (box * R + r) * K;
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (4 * lane + c < K)
                  l[c] = lp[4 * lane + c];
            }
          for (int64_t i0 = r0; i0 < r1; i0 += 8)
            {
              T w[8][4];
#pragma unroll
              for (int u = 0; u < 8; ++u)
                if (act && i0 + u < r1)
                  load4(W + (i0 + u) * K4 + 4 * lane, w[u]);
                else
                  w[u][0] = w[u][1] = w[u][2] = w[u][3] = T(0);
              T mine = T(0);
#pragma unroll
              for (int u = 0; u < 8; ++u)
                {
                  T s = (w[u][0] * l[0] + w[u][1] * l[1]) + (w[u][2] * l[2] + w[u][3] * l[3]);
                  s   = warp_sum(s);
                  if (lane == u)
                    mine = s;
                }
              if (lane < 8 && i0 + lane < r1)
                y[int64_t(r) * N + nrows[i0 + lane]] += mine;
            }
        }
    }

    // L2P of the FP64-accurate operator in float-float: as l2p_kernel, from
    // the (hi, lo) locals and (hi, lo) rows of W, products by TwoProduct, the
    // row sums carried with TwoSum and reduced by the same butterfly; y += the
    // sum in FP64.
    __global__ void __launch_bounds__(256)
      l2p_ff_kernel(int n_leaves, int R, int K, int N, const int64_t *__restrict__ row_ptr,
                    const int32_t *__restrict__ lleaf_box, const int32_t *__restrict__ nrows,
                    const float2 *__restrict__ W, const float2 *__restrict__ Lx,
                    double *__restrict__ y)
    {
      const int leaf = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
      if (leaf >= n_leaves)
        return;
      const int     K4  = (K + 3) / 4 * 4;
      const int64_t box = lleaf_box[leaf];
      const int64_t r0 = row_ptr[leaf], r1 = row_ptr[leaf + 1];
      const bool    act = 4 * lane < K4;
      for (int r = 0; r < R; ++r)
        {
          float2 l[4];
#pragma unroll
          for (int c = 0; c < 4; ++c)
            l[c] = make_float2(0.f, 0.f);
          if (act)
            {
              const float2 *lp = Lx + (box * R + r) * K;
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (4 * lane + c < K)
                  l[c] = lp[4 * lane + c];
            }
          for (int64_t i0 = r0; i0 < r1; i0 += 8)
            {
              float2 w[8][4];
#pragma unroll
              for (int u = 0; u < 8; ++u)
                if (act && i0 + u < r1)
                  {
                    const float4 a = *reinterpret_cast<const float4 *>(W + (i0 + u) * K4 + 4 * lane);
                    const float4 b = *reinterpret_cast<const float4 *>(W + (i0 + u) * K4 + 4 * lane + 2);
                    w[u][0] = make_float2(a.x, a.y);
                    w[u][1] = make_float2(a.z, a.w);
                    w[u][2] = make_float2(b.x, b.y);
                    w[u][3] = make_float2(b.z, b.w);
                  }
                else
                  w[u][0] = w[u][1] = w[u][2] = w[u][3] = make_float2(0.f, 0.f);
              double mine = 0.0;
#pragma unroll
              for (int u = 0; u < 8; ++u)
                {
                  float h = 0.f, lo = 0.f;
#pragma unroll
                  for (int c = 0; c < 4; ++c)
                    ff_mac(h, lo, w[u][c], l[c]);
                  float2 t = ff_norm(h, lo);
                  for (int o = 16; o > 0; o >>= 1)
                    t = ff_add(t, make_float2(__shfl_xor_sync(0xffffffffu, t.x, o),
                                              __shfl_xor_sync(0xffffffffu, t.y, o)));
                  if (lane == u)
                    mine = ff_join(t);
                }
              if (lane < 8 && i0 + lane < r1)
                {
                  double &o = y[int64_t(r) * N + nrows[i0 + lane]];
                  o         = __dadd_rn(o, mine);
                }
            }
        }
    }

    inline int tpb_for(int RK) { return RK >= 256 ? 256 : (RK >= 128 ? 128 : 64); }

    int near_sm_count()
    {
      int dev = 0, n_sm = 1;
      PIBEM_CUDA(cudaGetDevice(&dev));
      PIBEM_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
      return n_sm;
    }

  } // namespace

  void launch_l2p_ff(const OperatorDev<double> &op, int R, int N, const float2 *Lff, double *y,
                     cudaStream_t s)
  {
    if (op.n_rows == 0 || op.n_near_leaves == 0)
      return;
    l2p_ff_kernel<<<unsigned((op.n_near_leaves + 7) / 8), 256, 0, s>>>(
      op.n_near_leaves, R, op.K, N, op.nrow_ptr, op.lleaf_box, op.nrows, op.Wff, Lff, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  template <typename T>
  void launch_near_spmv(const OperatorDev<T> &op, int R, int N, const T *vals, const T *x, T *y,
                        bool accumulate, cudaStream_t s)
  {
    if (op.n_near_leaves == 0)
      return;
    const int64_t maxnc = (std::max<int64_t>(op.max_near_cols, 1) + 3) / 4 * 4;
    int           rb    = int(std::max<int64_t>(1, (96 * 1024) / (maxnc * int64_t(sizeof(T)))));
    rb                  = std::min(rb, R);
    const size_t smem   = size_t(rb) * maxnc * sizeof(T);
    const size_t smem_s = 128 + size_t(2) * maxnc * (4 + sizeof(T));
    if (R == 1 && op.near_sched && smem_s <= 227 * 1024)
      {
        // one column: the scheduled three-stage kernel, 4 warps a block, three
        // 4-value chunks per lane and row in flight, loads that do not
        // allocate in L1.  Measured on GB300 (98k spheroid, CUDA events)
        // against near_leaf_pipe_kernel: FP32 79.5 -> 55.6 us (8 warps with two
        // chunks 62 us; 4 warps with two / four / five chunks 67 / 58 / 64 us;
        // one row per warp with six chunks 62 us; a shared-memory carveout of
        // 100 % 66 us), FP64 328 -> 229 us (8 warps with two chunks 265 us; 4
        // warps with one / two chunks 269 / 233 us).
        constexpr int bs   = 128;
        auto          kern = near_leaf_sched_kernel<T, 3, 128, true>;
        if (smem_s > 48 * 1024)
          raise_smem_limit(reinterpret_cast<const void *>(kern), smem_s);
        int per_sm = 0;
        PIBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, bs, smem_s));
        const int grid = std::min(op.n_near_leaves, std::max(per_sm, 1) * near_sm_count());
        launch_pdl(kern, grid, bs, smem_s, s, op.n_near_leaves, int(maxnc), op.near_sched,
                   op.nrows, op.ncols, vals, x, y, accumulate);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
        return;
      }
    if (R == 1)
      {
        // one column: the software-pipelined persistent kernel (a row is
        // computed with the same rounding steps in the same order as below)
        // resident blocks per SM: FP32 6 (40 registers), FP64 4 (64 registers)
        constexpr int MINB  = sizeof(T) == 4 ? NEAR_BLOCKS_PER_SM_F32 : NEAR_BLOCKS_PER_SM_WIDE;
        auto          kern  = near_leaf_pipe_kernel<T>;
        const size_t  smem1 = size_t(2) * maxnc * sizeof(T);
        if (smem1 > 48 * 1024)
          raise_smem_limit(reinterpret_cast<const void *>(kern), smem1);
        const int grid = std::min(op.n_near_leaves, MINB * near_sm_count());
        launch_pdl(kern, grid, 256, smem1, s, op.n_near_leaves, int(maxnc), op.nrow_ptr, op.ncol_ptr,
                                      op.nval_ptr, op.nrows, op.ncols, vals, x, y, accumulate);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
        return;
      }
    auto kern = near_leaf_kernel<T, false>;
    if (smem > 48 * 1024)
      raise_smem_limit(reinterpret_cast<const void *>(kern), smem);
    launch_pdl(kern, op.n_near_leaves, 256, smem, s, R, rb, N, op.nrow_ptr, op.ncol_ptr, op.nval_ptr,
                                             op.nrows, op.ncols, vals, x, y, accumulate);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  bool near_ff_fits(const OperatorDev<double> &op)
  {
    const int64_t maxnc = (std::max<int64_t>(op.max_near_cols, 1) + 3) / 4 * 4;
    return size_t(2) * maxnc * sizeof(float2) <= 227 * 1024;
  }

  void launch_near_spmv_ff(const OperatorDev<double> &op, int R, int N, const float2 *vals,
                           const float2 *xff, double *y, bool accumulate, cudaStream_t s)
  {
    if (op.n_near_leaves == 0)
      return;
    const int64_t maxnc = (std::max<int64_t>(op.max_near_cols, 1) + 3) / 4 * 4;
    const size_t smem1 = size_t(2) * maxnc * sizeof(float2);
    if (smem1 > 48 * 1024)
      raise_smem_limit(reinterpret_cast<const void *>(near_leaf_ff_kernel), smem1);
    // one launch per column: a column's result does not depend on R
    for (int r = 0; r < R; ++r)
      {
        near_leaf_ff_kernel<<<std::min(op.n_near_leaves, NEAR_BLOCKS_PER_SM_WIDE * near_sm_count()),
                              256, smem1, s>>>(
          op.n_near_leaves, int(maxnc), op.nrow_ptr, op.ncol_ptr, op.nval_ptr, op.nrows, op.ncols, vals,
          xff + int64_t(r) * N, y + int64_t(r) * N, accumulate);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
      }
  }

  template <typename T>
  void launch_p2m_apply(const OperatorDev<T> &op, int R, int N, const uint8_t *dir,
                        const uint8_t *modes, const T *x, T *M, bool combined, cudaStream_t s)
  {
    if (op.n_p2m_leaves == 0)
      return;
    const unsigned grid = unsigned((op.n_p2m_leaves + 7) / 8);
    const bool     comb = combined && op.Tc;
    auto launch = [&](auto kern) {
      launch_pdl(kern, grid, 256, 0, s, op.n_p2m_leaves, R, op.K, N, op.prow_ptr, op.pleaf_box, op.prow_dof,
                                comb ? op.Tc : op.T1, op.T2, dir, modes, x, M);
    };
    if (comb)
      R == 1 ? launch(p2m_apply_kernel<T, true, 1>) : launch(p2m_apply_kernel<T, true, 4>);
    else
      R == 1 ? launch(p2m_apply_kernel<T, false, 1>) : launch(p2m_apply_kernel<T, false, 4>);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  // The downward pass of the FP32 operator as fused level passes: target-major
  // M2L products, their sums per box, then L2L level by level.
  static bool fused_down(const OperatorDev<float> &op, int R)
  {
    return op.down_par && op.down_m2l_beg && fused_levels_ok(op.K, R);
  }

  // The float-float translation GEMM for chunks [c0, c1); IO = double (FP64
  // expansions) or float2 ((hi, lo) expansions).  A launch with fewer blocks
  // than ~2 per SM splits the rows over blockIdx.z (16 per block).
  template <typename IO>
  void launch_ff_gemm(const OperatorDev<double> &op, int R, int c0, int c1, const IO *E, IO *Y,
                      cudaStream_t s)
  {
    if (c1 <= c0)
      return;
    const int      K  = op.K;
    const unsigned gx = unsigned(c1 - c0),
                   gy = unsigned((op.max_chunk_pairs * R + GB_COLS - 1) / GB_COLS);
    const bool     split = int64_t(gx) * gy < 256;
    const int      RI    = split ? 1 : std::min(4, (K + 31) / 32);
    const int      TX    = split ? 16 : (K + RI - 1) / RI;
    const int      CJ    = split ? 4 : 8; // columns per thread (split: 16 x 16 threads)
    const dim3     grid(gx, gy, split ? unsigned((K + 15) / 16) : 1u);
    const size_t   smem = (size_t(K) * K + size_t(K) * GB_LDB) * sizeof(float2);
    if (K > 128)
      throw Error(PIBEM_EINVAL, "float-float translations: K = (p+1)^2 above 128");
    auto launch = [&](auto kern) {
      if (smem > 48 * 1024)
        raise_smem_limit(reinterpret_cast<const void *>(kern), smem);
      kern<<<grid, (64 / CJ) * TX, smem, s>>>(R, K, TX, c0, op.ch_start, op.ch_cnt, op.ch_op,
                                              op.q_src, op.ops_ff, E, Y);
    };
    if (CJ == 4)
      launch(ff_gemm_kernel<1, 4, IO>);
    else
      switch (RI)
        {
          case 1: launch(ff_gemm_kernel<1, 8, IO>); break;
          case 2: launch(ff_gemm_kernel<2, 8, IO>); break;
          case 3: launch(ff_gemm_kernel<3, 8, IO>); break;
          default: launch(ff_gemm_kernel<4, 8, IO>); break;
        }
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
  template void launch_ff_gemm<double>(const OperatorDev<double> &, int, int, int, const double *,
                                       double *, cudaStream_t);
  template void launch_ff_gemm<float2>(const OperatorDev<double> &, int, int, int, const float2 *,
                                       float2 *, cudaStream_t);

  // the FP64-accurate tree passes on (hi, lo) expansions
  void launch_upward_level_ff(const OperatorDev<double> &op, int R, int level, float2 *M, float2 *Y,
                              cudaStream_t s)
  {
    launch_ff_gemm<float2>(op, R, op.up_chunk_ptr[level], op.up_chunk_ptr[level + 1], M, Y, s);
    const int a = op.up_box_ptr[level], b = op.up_box_ptr[level + 1];
    if (b > a)
      {
        gather_ff_kernel<<<b - a, R * op.K >= 128 ? 128 : 96, 0, s>>>(
          R, op.K, op.up_box + a, op.up_q_ptr + a, op.up_q, Y, M);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
      }
  }
  void launch_m2l_ff(const OperatorDev<double> &op, int R, const float2 *M, float2 *Y, cudaStream_t s)
  {
    launch_ff_gemm<float2>(op, R, 0, op.m2l_chunk_end, M, Y, s);
  }
  void launch_downward_level_ff(const OperatorDev<double> &op, int R, int level, float2 *Lx,
                                float2 *Y, cudaStream_t s)
  {
    launch_ff_gemm<float2>(op, R, op.down_chunk_ptr[level], op.down_chunk_ptr[level + 1], Lx, Y, s);
    const int a = op.down_box_ptr[level], b = op.down_box_ptr[level + 1];
    if (b > a)
      {
        gather_ff_kernel<<<b - a, R * op.K >= 128 ? 128 : 96, 0, s>>>(
          R, op.K, op.down_box + a, op.down_q_ptr + a, op.down_q, Y, Lx);
        PIBEM_CUDA(cudaGetLastError());
        note_launch();
      }
  }
  void launch_convert_d2ff(int64_t n, const double *a, float2 *b, cudaStream_t s)
  {
    if (n == 0)
      return;
    d2ff_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, a, b);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
  void launch_convert_ff2d(int64_t n, const float2 *a, double *b, cudaStream_t s)
  {
    if (n == 0)
      return;
    ff2d_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, a, b);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  // Y row of (pair q, rhs r): (yslot ? yslot[q] : q) * R + r, rows of ldy values
  template <typename T>
  static void launch_trans_gemm(const OperatorDev<T> &op, int R, int c0, int c1, const T *E, T *Y,
                                cudaStream_t s, const int32_t *yslot = nullptr, int ldy = 0)
  {
    if (c1 <= c0)
      return;
    if (ldy == 0)
      ldy = op.K;
    if constexpr (std::is_same<T, float>::value)
      if (op.tc_images)
        {
          launch_tc_gemm(op, R, c0, c1, E, Y, yslot, ldy, op.tc_err, s);
          return;
        }
    // largest column count of the chunks in [c0, c1): R x (<= 128 pairs).  A
    // launch with fewer blocks than ~2 per SM (the tree's small levels) splits
    // each block's rows over blockIdx.z (16 rows per block) for parallelism.
    const unsigned gx = unsigned(c1 - c0),
                   gy = unsigned((op.max_chunk_pairs * R + GB_COLS - 1) / GB_COLS);
    const bool     split = int64_t(gx) * gy < 256;
    const int      KI    = split ? 1 : (op.K + 15) / 16;
    const dim3     grid(gx, gy, split ? unsigned((op.K + 15) / 16) : 1u);
    if constexpr (std::is_same<T, double>::value)
      if (op.ops_ff)
        {
          launch_ff_gemm<double>(op, R, c0, c1, E, Y, s);
          return;
        }
    const size_t smem = (size_t(op.K) * op.K + size_t(op.K) * GB_LDB) * sizeof(T);
    auto launch = [&](auto kern) {
      if (smem > 48 * 1024)
        raise_smem_limit(reinterpret_cast<const void *>(kern), smem);
      kern<<<grid, 256, smem, s>>>(R, op.K, c0, op.ch_start, op.ch_cnt, op.ch_op, op.q_src, op.ops,
                                   E, Y, yslot, ldy);
    };
    switch (KI)
      {
        case 1: launch(trans_gemm_kernel<T, 1>); break;
        case 2: launch(trans_gemm_kernel<T, 2>); break;
        case 3: launch(trans_gemm_kernel<T, 3>); break;
        case 4: launch(trans_gemm_kernel<T, 4>); break;
        case 5: launch(trans_gemm_kernel<T, 5>); break;
        case 6: launch(trans_gemm_kernel<T, 6>); break;
        case 7: launch(trans_gemm_kernel<T, 7>); break;
        default: launch(trans_gemm_kernel<T, 8>); break;
      }
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  template <typename T>
  static void launch_gather(int R, int K, int nbox, const int32_t *boxes, const int64_t *q_ptr,
                            const int32_t *q, const T *Y, T *out, cudaStream_t s)
  {
    if (nbox <= 0)
      return;
    gather_kernel<T><<<nbox, R * K >= 128 ? 128 : 96, 0, s>>>(R, K, boxes, q_ptr, q, Y, out);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  template <typename T>
  void launch_upward_level(const OperatorDev<T> &op, int R, int level, T *M, T *Y, cudaStream_t s)
  {
    if constexpr (std::is_same<T, float>::value)
      if (op.up_child8 && fused_levels_ok(op.K, R))
        {
          launch_m2m_level_fused(op, R, level, M, s);
          return;
        }
    launch_trans_gemm<T>(op, R, op.up_chunk_ptr[level], op.up_chunk_ptr[level + 1], M, Y, s);
    const int a = op.up_box_ptr[level], b = op.up_box_ptr[level + 1];
    launch_gather<T>(R, op.K, b - a, op.up_box + a, op.up_q_ptr + a, op.up_q, Y, M, s);
  }

  // the M2L products of all levels; for the fused level passes in the
  // target-major order with 16-byte aligned rows (what the M2L sums read)
  template <typename T>
  void launch_m2l_gemm(const OperatorDev<T> &op, int R, const T *M, T *Y, cudaStream_t s)
  {
    if constexpr (std::is_same<T, float>::value)
      if (fused_down(op, R))
        {
          launch_trans_gemm<T>(op, R, 0, op.m2l_chunk_end, M, Y, s, op.m2l_yslot,
                               (op.K + 3) / 4 * 4);
          return;
        }
    launch_trans_gemm<T>(op, R, 0, op.m2l_chunk_end, M, Y, s);
  }

  template <typename T>
  void launch_m2l_sums(const OperatorDev<T> &op, int R, T *Lx, const T *Y, cudaStream_t s)
  {
    if constexpr (std::is_same<T, float>::value)
      if (fused_down(op, R))
        launch_m2l_sums_fused(op, R, Lx, Y, s);
  }

  template <typename T>
  void launch_downward_level(const OperatorDev<T> &op, int R, int level, T *Lx, T *Y,
                             cudaStream_t s)
  {
    if constexpr (std::is_same<T, float>::value)
      if (fused_down(op, R))
        {
          launch_l2l_level_fused(op, R, level, Lx, s);
          return;
        }
    launch_trans_gemm<T>(op, R, op.down_chunk_ptr[level], op.down_chunk_ptr[level + 1], Lx, Y, s);
    const int a = op.down_box_ptr[level], b = op.down_box_ptr[level + 1];
    launch_gather<T>(R, op.K, b - a, op.down_box + a, op.down_q_ptr + a, op.down_q, Y, Lx, s);
  }

  template <typename T>
  void launch_m2p(const OperatorDev<T> &op, const TreeDev &td, int R, int N, const T *M, T *y,
                  cudaStream_t s)
  {
    if (op.n_m2p_tgt == 0)
      return;
    launch_pdl(m2p_eval_kernel<T>, unsigned((op.n_m2p_items + 127) / 128), 128, 0, s, 
      op.n_m2p_items, R, op.K, op.p, op.m2p_item_ptr, op.m2p_item_pair, op.m2p_pair_tgt,
      op.m2p_tgt, op.m2p_src, op.m2p_tnode_ptr, op.m2p_tnodes, td.xyz, td.center, td.delta, M,
      op.m2p_scratch);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
    launch_pdl(m2p_sum_kernel<T>, unsigned((op.n_m2p_tgt + 7) / 8), 256, 0, s, 
      op.n_m2p_tgt, R, N, op.n_m2p_items, op.m2p_tnode_ptr, op.m2p_tgt, op.m2p_src_ptr,
      op.m2p_item_ptr, op.m2p_tnodes, op.m2p_scratch, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_m2p_ff(const OperatorDev<double> &op, const TreeDev &td, int R, int N, const float2 *Mff,
                     double *y, cudaStream_t s)
  {
    if (op.n_m2p_tgt == 0)
      return;
    m2p_eval_ff_kernel<<<unsigned((op.n_m2p_items + 127) / 128), 128, 0, s>>>(
      op.n_m2p_items, R, op.K, op.p, op.m2p_item_ptr, op.m2p_item_pair, op.m2p_pair_tgt, op.m2p_src,
      op.m2p_tnode_ptr, op.m2p_tnodes, td.xyz, td.center, td.delta, Mff, op.m2p_scratch);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
    m2p_sum_kernel<double><<<unsigned((op.n_m2p_tgt + 7) / 8), 256, 0, s>>>(
      op.n_m2p_tgt, R, N, op.n_m2p_items, op.m2p_tnode_ptr, op.m2p_tgt, op.m2p_src_ptr,
      op.m2p_item_ptr, op.m2p_tnodes, op.m2p_scratch, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void ensure_fmm_tables(int device, cudaStream_t s)
  {
    static bool       done[64] = {};
    static std::mutex mu; // handles may be set up from several host threads
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 64 || done[device])
      return;
    LegendreTables t;
    fill_legendre_tables(t);
    PIBEM_CUDA(cudaMemcpyToSymbolAsync(c_leg, &t, sizeof(t), 0, cudaMemcpyHostToDevice, s));
    PIBEM_CUDA(cudaStreamSynchronize(s));
    done[device] = true;
  }

  template <typename T>
  void launch_l2p(const OperatorDev<T> &op, int R, int N, const T *Lx, T *y, cudaStream_t s)
  {
    if (op.n_rows == 0 || op.n_near_leaves == 0)
      return;
    launch_pdl(l2p_kernel<T>, unsigned((op.n_near_leaves + 7) / 8), 256, 0, s, 
      op.n_near_leaves, R, op.K, N, op.nrow_ptr, op.lleaf_box, op.nrows, op.W, Lx, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

#define PIBEM_INSTANTIATE(T)                                                                      \
  template void launch_near_spmv<T>(const OperatorDev<T> &, int, int, const T *, const T *, T *, \
                                    bool, cudaStream_t);                                         \
  template void launch_p2m_apply<T>(const OperatorDev<T> &, int, int, const uint8_t *,           \
                                    const uint8_t *, const T *, T *, bool, cudaStream_t);        \
  template void launch_upward_level<T>(const OperatorDev<T> &, int, int, T *, T *, cudaStream_t); \
  template void launch_m2l_gemm<T>(const OperatorDev<T> &, int, const T *, T *, cudaStream_t);    \
  template void launch_m2l_sums<T>(const OperatorDev<T> &, int, T *, const T *, cudaStream_t);    \
  template void launch_downward_level<T>(const OperatorDev<T> &, int, int, T *, T *,             \
                                         cudaStream_t);                                          \
  template void launch_m2p<T>(const OperatorDev<T> &, const TreeDev &, int, int, const T *, T *, \
                              cudaStream_t);                                                     \
  template void launch_l2p<T>(const OperatorDev<T> &, int, int, const T *, T *, cudaStream_t);
  PIBEM_INSTANTIATE(double)
  PIBEM_INSTANTIATE(float)
} // namespace pibem
