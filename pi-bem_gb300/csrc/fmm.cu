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
#include "devmath.cuh"
#include "kernels.h"

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

    template <typename T>
    __global__ void near_spmv_kernel(int64_t n_rows, int R, int N, const int32_t *__restrict__ row_leaf,
                                     const int64_t *__restrict__ nrow_ptr,
                                     const int64_t *__restrict__ ncol_ptr,
                                     const int64_t *__restrict__ nval_ptr,
                                     const int32_t *__restrict__ nrows,
                                     const int32_t *__restrict__ ncols,
                                     const T *__restrict__ vals, const T *__restrict__ x,
                                     T *__restrict__ y, bool acc)
    {
      const int64_t row  = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
      const int     lane = threadIdx.x & 31;
      if (row >= n_rows)
        return;
      const int     leaf = row_leaf[row];
      const int64_t r    = row - nrow_ptr[leaf];
      const int64_t c0   = ncol_ptr[leaf];
      const int64_t nc   = ncol_ptr[leaf + 1] - c0;
      const T      *v    = vals + nval_ptr[leaf] + r * nc;
      const int     node = nrows[row];
      for (int r0 = 0; r0 < R; r0 += RC)
        {
          T s[RC];
#pragma unroll
          for (int j = 0; j < RC; ++j)
            s[j] = T(0);
          for (int64_t c = lane; c < nc; c += 32)
            {
              const T   a   = v[c];
              const int col = ncols[c0 + c];
#pragma unroll
              for (int j = 0; j < RC; ++j)
                if (r0 + j < R)
                  s[j] += a * x[int64_t(r0 + j) * N + col];
            }
#pragma unroll
          for (int j = 0; j < RC; ++j)
            s[j] = warp_sum(s[j]);
          if (lane == 0)
            for (int j = 0; j < RC && r0 + j < R; ++j)
              {
                T &o = y[int64_t(r0 + j) * N + node];
                o    = acc ? o + s[j] : s[j];
              }
        }
    }

    template <typename T>
    __global__ void p2m_apply_kernel(int R, int K, int N, const int64_t *__restrict__ prow_ptr,
                                     const int32_t *__restrict__ pleaf_box,
                                     const int32_t *__restrict__ prow_dof,
                                     const T *__restrict__ T1, const T *__restrict__ T2,
                                     const uint8_t *__restrict__ dir,
                                     const uint8_t *__restrict__ modes, const T *__restrict__ x,
                                     T *__restrict__ M)
    {
      const int     leaf = blockIdx.x;
      const int64_t box  = pleaf_box[leaf];
      const int64_t rb = prow_ptr[leaf], re = prow_ptr[leaf + 1];
      for (int idx = threadIdx.x; idx < R * K; idx += blockDim.x)
        {
          const int     r    = idx / K;
          const int     k    = idx - r * K;
          const uint8_t mode = modes[r];
          T             acc  = T(0);
          for (int64_t row = rb; row < re; ++row)
            {
              const int dof = prow_dof[row];
              const T   xv  = x[int64_t(r) * N + dof];
              if (mode == MODE_KER1)
                acc += T1[row * K + k] * xv;
              else if (mode == MODE_KER2)
                acc += T2[row * K + k] * xv;
              else
                acc += dir[dof] ? -T2[row * K + k] * xv : T1[row * K + k] * xv;
            }
          M[(box * R + r) * K + k] = acc;
        }
    }

    // Generic translation: out[t] (= or +=) sum over sources s of op[s] * in[s]
    // for one target box per block.  Four warps share the target's sources
    // (warp w takes sources w, w+4, ...); each lane owns output rows
    // k = lane + 32 j; the four partial sums are added in a fixed order, so the
    // result does not depend on scheduling.  ops are stored [op][in][out].
    //   SRC_CSR:      M2L, sources and offset ids from a per-target list
    //   SRC_CHILDREN: M2M, sources = children, op = child octant
    //   SRC_PARENT:   L2L, source = parent, op = own octant
    enum
    {
      SRC_CSR      = 0,
      SRC_CHILDREN = 1,
      SRC_PARENT   = 2
    };
    constexpr int TW  = 4; // warps per block
    constexpr int KPL = 4; // output rows per lane (K <= 128)
    constexpr int RCH = 4; // rhs columns per register block

    template <typename T, int MODE, bool ACCUM>
    __global__ void __launch_bounds__(TW * 32)
      translate_kernel(int R, int K, const int32_t *__restrict__ targets,
                       const int64_t *__restrict__ src_ptr, const int32_t *__restrict__ src,
                       const int32_t *__restrict__ opid, const int32_t *__restrict__ child_first,
                       const int32_t *__restrict__ nchild, const int32_t *__restrict__ digit,
                       const int32_t *__restrict__ parent, const T *__restrict__ ops,
                       const T *__restrict__ in, T *__restrict__ out)
    {
      extern __shared__ unsigned char smem_raw[];
      T            *sSrc = reinterpret_cast<T *>(smem_raw);   // [TW][RCH][K]
      T            *sAcc = sSrc + TW * RCH * K;               // [TW][RCH][K]
      const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const int64_t t    = targets[blockIdx.x];
      int64_t       e0, e1;
      if (MODE == SRC_CSR)
        {
          e0 = src_ptr[blockIdx.x];
          e1 = src_ptr[blockIdx.x + 1];
        }
      else if (MODE == SRC_CHILDREN)
        {
          e0 = child_first[t];
          e1 = e0 + nchild[t];
        }
      else
        {
          e0 = 0;
          e1 = 1;
        }
      T *mySrc = sSrc + warp * RCH * K;
      for (int r0 = 0; r0 < R; r0 += RCH)
        {
          const int rc = min(RCH, R - r0);
          T         acc[RCH][KPL];
#pragma unroll
          for (int r = 0; r < RCH; ++r)
#pragma unroll
            for (int j = 0; j < KPL; ++j)
              acc[r][j] = T(0);
          for (int64_t e = e0 + warp; e < e1; e += TW)
            {
              int64_t sb;
              int     o;
              if (MODE == SRC_CSR)
                {
                  sb = src[e];
                  o  = opid[e];
                }
              else if (MODE == SRC_CHILDREN)
                {
                  sb = e;
                  o  = digit[e];
                }
              else
                {
                  sb = parent[t];
                  o  = digit[t];
                }
              const T *ip = in + (sb * R + r0) * K;
              for (int i = lane; i < rc * K; i += 32)
                mySrc[i] = ip[i];
              __syncwarp();
              const T *op = ops + int64_t(o) * K * K;
              for (int ki = 0; ki < K; ++ki)
                {
                  T w[KPL];
#pragma unroll
                  for (int j = 0; j < KPL; ++j)
                    {
                      const int ko = lane + 32 * j;
                      w[j]         = ko < K ? op[int64_t(ki) * K + ko] : T(0);
                    }
#pragma unroll
                  for (int r = 0; r < RCH; ++r)
                    if (r < rc)
                      {
                        const T m = mySrc[r * K + ki];
#pragma unroll
                        for (int j = 0; j < KPL; ++j)
                          acc[r][j] += w[j] * m;
                      }
                }
              __syncwarp();
            }
          T *myAcc = sAcc + warp * RCH * K;
#pragma unroll
          for (int r = 0; r < RCH; ++r)
#pragma unroll
            for (int j = 0; j < KPL; ++j)
              {
                const int ko = lane + 32 * j;
                if (r < rc && ko < K)
                  myAcc[r * K + ko] = acc[r][j];
              }
          __syncthreads();
          for (int i = threadIdx.x; i < rc * K; i += blockDim.x)
            {
              T v = sAcc[i];
              for (int w = 1; w < TW; ++w)
                v += sAcc[w * RCH * K + i];
              T *o = out + (t * R + r0) * K + i;
              *o   = ACCUM ? *o + v : v;
            }
          __syncthreads();
        }
    }

    // M2P phase 1: one thread per (pair, node of the pair's target box):
    // scratch[r][item] = multipole of the source box evaluated at the node.
    template <typename T>
    __global__ void m2p_eval_kernel(int64_t n_items, int64_t n_pairs, int R, int K, int p,
                                    const int64_t *__restrict__ item_ptr,
                                    const int32_t *__restrict__ pair_tgt,
                                    const int32_t *__restrict__ tgt,
                                    const int32_t *__restrict__ src,
                                    const int32_t *__restrict__ nbeg,
                                    const int32_t *__restrict__ node_sorted,
                                    const double *__restrict__ xyz,
                                    const double *__restrict__ center,
                                    const double *__restrict__ delta, const T *__restrict__ M,
                                    T *__restrict__ scratch)
    {
      const int64_t it = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (it >= n_items)
        return;
      int64_t lo = 0, hi = n_pairs - 1;
      while (lo < hi)
        {
          int64_t mid = (lo + hi + 1) >> 1;
          if (item_ptr[mid] <= it)
            lo = mid;
          else
            hi = mid - 1;
        }
      const int64_t e    = lo;
      const int64_t t    = tgt[pair_tgt[e]];
      const int64_t s    = src[e];
      const int     node = node_sorted[nbeg[t] + (it - item_ptr[e])];
      const double  h    = delta[s];
      const T       rx   = T((xyz[3 * int64_t(node)] - center[3 * s]) / h);
      const T       ry   = T((xyz[3 * int64_t(node) + 1] - center[3 * s + 1]) / h);
      const T       rz   = T((xyz[3 * int64_t(node) + 2] - center[3 * s + 2]) / h);
      const T       ih   = T(1.0 / h);
      for (int r = 0; r < R; ++r)
        scratch[int64_t(r) * n_items + it] =
          eval_expansion_fast<T, T>(M + (s * R + r) * K, p, rx, ry, rz, true) * ih;
    }

    // M2P phase 2: one thread per (target box node): fixed-order sum over the
    // box's sources, added to y.
    template <typename T>
    __global__ void m2p_sum_kernel(int64_t n_tnodes, int n_tgt, int R, int N, int64_t n_items,
                                   const int64_t *__restrict__ tnode_ptr,
                                   const int32_t *__restrict__ tgt,
                                   const int64_t *__restrict__ src_ptr,
                                   const int64_t *__restrict__ item_ptr,
                                   const int32_t *__restrict__ nbeg,
                                   const int32_t *__restrict__ node_sorted,
                                   const T *__restrict__ scratch, T *__restrict__ y)
    {
      const int64_t tn = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (tn >= n_tnodes)
        return;
      int lo = 0, hi = n_tgt - 1;
      while (lo < hi)
        {
          int mid = (lo + hi + 1) >> 1;
          if (tnode_ptr[mid] <= tn)
            lo = mid;
          else
            hi = mid - 1;
        }
      const int64_t i    = tn - tnode_ptr[lo];
      const int     node = node_sorted[nbeg[tgt[lo]] + i];
      for (int r = 0; r < R; ++r)
        {
          T acc = T(0);
          for (int64_t e = src_ptr[lo]; e < src_ptr[lo + 1]; ++e)
            acc += scratch[int64_t(r) * n_items + item_ptr[e] + i];
          y[int64_t(r) * N + node] += acc;
        }
    }

    template <typename T>
    __global__ void l2p_kernel(int64_t n_rows, int R, int K, int N,
                               const int32_t *__restrict__ row_leaf,
                               const int32_t *__restrict__ lleaf_box,
                               const int32_t *__restrict__ nrows, const T *__restrict__ W,
                               const T *__restrict__ Lx, T *__restrict__ y)
    {
      const int64_t row  = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
      const int     lane = threadIdx.x & 31;
      if (row >= n_rows)
        return;
      const int64_t box  = lleaf_box[row_leaf[row]];
      const int     node = nrows[row];
      const T      *w    = W + row * K;
      for (int r = 0; r < R; ++r)
        {
          const T *l = Lx + (box * R + r) * K;
          T        s = T(0);
          for (int k = lane; k < K; k += 32)
            s += w[k] * l[k];
          s = warp_sum(s);
          if (lane == 0)
            y[int64_t(r) * N + node] += s;
        }
    }

    inline int tpb_for(int RK) { return RK >= 256 ? 256 : (RK >= 128 ? 128 : 64); }
  } // namespace

  template <typename T>
  void launch_near_spmv(const OperatorDev<T> &op, int R, int N, const T *vals, const T *x, T *y,
                        bool accumulate, cudaStream_t s)
  {
    if (op.n_rows == 0)
      return;
    const int64_t threads = op.n_rows * 32;
    near_spmv_kernel<T><<<unsigned((threads + 255) / 256), 256, 0, s>>>(
      op.n_rows, R, N, op.row_leaf, op.nrow_ptr, op.ncol_ptr, op.nval_ptr, op.nrows, op.ncols, vals,
      x, y, accumulate);
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T>
  void launch_p2m_apply(const OperatorDev<T> &op, int R, int N, const uint8_t *dir,
                        const uint8_t *modes, const T *x, T *M, cudaStream_t s)
  {
    if (op.n_p2m_leaves == 0)
      return;
    p2m_apply_kernel<T><<<op.n_p2m_leaves, tpb_for(R * op.K), 0, s>>>(
      R, op.K, N, op.prow_ptr, op.pleaf_box, op.prow_dof, op.T1, op.T2, dir, modes, x, M);
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T, int MODE, bool ACCUM>
  static void launch_translate(int nt, int R, int K, const int32_t *targets, const int64_t *src_ptr,
                               const int32_t *src, const int32_t *opid, const TreeDev &td,
                               const T *ops, const T *in, T *out, cudaStream_t s)
  {
    if (nt <= 0)
      return;
    const size_t smem = size_t(2) * TW * RCH * K * sizeof(T);
    auto         fn   = translate_kernel<T, MODE, ACCUM>;
    if (smem > 48 * 1024)
      PIBEM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    fn<<<nt, TW * 32, smem, s>>>(R, K, targets, src_ptr, src, opid, td.child_first, td.nchild,
                                 td.digit, td.parent, ops, in, out);
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T>
  void launch_m2m_level(const OperatorDev<T> &op, const TreeDev &td, int R, int parent_level, T *M,
                        cudaStream_t s)
  {
    const int a = op.parents_level_ptr[parent_level], b = op.parents_level_ptr[parent_level + 1];
    launch_translate<T, SRC_CHILDREN, false>(b - a, R, op.K, op.parents + a, nullptr, nullptr,
                                             nullptr, td, op.m2m_ops, M, M, s);
  }

  template <typename T>
  void launch_l2l_level(const OperatorDev<T> &op, const TreeDev &td, int R, int level, T *Lx,
                        cudaStream_t s)
  {
    const int a = op.l2l_level_ptr[level], b = op.l2l_level_ptr[level + 1];
    launch_translate<T, SRC_PARENT, false>(b - a, R, op.K, op.l2l_box + a, nullptr, nullptr,
                                           nullptr, td, op.l2l_ops, Lx, Lx, s);
  }

  template <typename T>
  void launch_m2l_level(const OperatorDev<T> &op, int R, int level, const T *M, T *Lx,
                        cudaStream_t s)
  {
    const int a = op.m2l_level_ptr[level], b = op.m2l_level_ptr[level + 1];
    TreeDev   none;
    launch_translate<T, SRC_CSR, true>(b - a, R, op.K, op.m2l_tgt + a, op.m2l_src_ptr + a,
                                       op.m2l_src, op.m2l_off, none, op.m2l_ops, M, Lx, s);
  }

  template <typename T>
  void launch_m2p(const OperatorDev<T> &op, const TreeDev &td, int R, int N, const T *M, T *y,
                  cudaStream_t s)
  {
    if (op.n_m2p_tgt == 0)
      return;
    m2p_eval_kernel<T><<<unsigned((op.n_m2p_items + 127) / 128), 128, 0, s>>>(
      op.n_m2p_items, op.n_m2p_pairs, R, op.K, op.p, op.m2p_item_ptr, op.m2p_pair_tgt, op.m2p_tgt,
      op.m2p_src, td.nbeg, td.node_sorted, td.xyz, td.center, td.delta, M, op.m2p_scratch);
    PIBEM_CUDA(cudaGetLastError());
    m2p_sum_kernel<T><<<unsigned((op.n_m2p_tnodes + 127) / 128), 128, 0, s>>>(
      op.n_m2p_tnodes, op.n_m2p_tgt, R, N, op.n_m2p_items, op.m2p_tnode_ptr, op.m2p_tgt,
      op.m2p_src_ptr, op.m2p_item_ptr, td.nbeg, td.node_sorted, op.m2p_scratch, y);
    PIBEM_CUDA(cudaGetLastError());
  }

  void ensure_fmm_tables(int device, cudaStream_t s)
  {
    static bool done[64] = {};
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
    if (op.n_rows == 0)
      return;
    const int64_t threads = op.n_rows * 32;
    l2p_kernel<T><<<unsigned((threads + 255) / 256), 256, 0, s>>>(
      op.n_rows, R, op.K, N, op.row_leaf, op.lleaf_box, op.nrows, op.W, Lx, y);
    PIBEM_CUDA(cudaGetLastError());
  }

#define PIBEM_INSTANTIATE(T)                                                                      \
  template void launch_near_spmv<T>(const OperatorDev<T> &, int, int, const T *, const T *, T *, \
                                    bool, cudaStream_t);                                         \
  template void launch_p2m_apply<T>(const OperatorDev<T> &, int, int, const uint8_t *,           \
                                    const uint8_t *, const T *, T *, cudaStream_t);              \
  template void launch_m2m_level<T>(const OperatorDev<T> &, const TreeDev &, int, int, T *,      \
                                    cudaStream_t);                                               \
  template void launch_l2l_level<T>(const OperatorDev<T> &, const TreeDev &, int, int, T *,      \
                                    cudaStream_t);                                               \
  template void launch_m2l_level<T>(const OperatorDev<T> &, int, int, const T *, T *,            \
                                    cudaStream_t);                                               \
  template void launch_m2p<T>(const OperatorDev<T> &, const TreeDev &, int, int, const T *, T *, \
                              cudaStream_t);                                                     \
  template void launch_l2p<T>(const OperatorDev<T> &, int, int, const T *, T *, cudaStream_t);
  PIBEM_INSTANTIATE(double)
  PIBEM_INSTANTIATE(float)
} // namespace pibem
