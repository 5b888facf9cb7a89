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

    // out[box] (=|+=) sum_src op[src_op]^T-contract in[src]; shared by M2M, L2L, M2L.
    // ops are stored [op][in][out].
    template <typename T>
    __device__ inline void accumulate_translation(int R, int K, const T *__restrict__ op,
                                                  const T *__restrict__ sIn, T *__restrict__ sOut)
    {
      for (int idx = threadIdx.x; idx < R * K; idx += blockDim.x)
        {
          const int r  = idx / K;
          const int ko = idx - r * K;
          const T  *in = sIn + r * K;
          T         a0 = T(0), a1 = T(0);
          int       ki = 0;
          for (; ki + 1 < K; ki += 2)
            {
              a0 += op[int64_t(ki) * K + ko] * in[ki];
              a1 += op[int64_t(ki + 1) * K + ko] * in[ki + 1];
            }
          if (ki < K)
            a0 += op[int64_t(ki) * K + ko] * in[ki];
          sOut[idx] += a0 + a1;
        }
    }

    template <typename T>
    __global__ void m2m_kernel(int R, int K, const int32_t *__restrict__ parents,
                               const int32_t *__restrict__ child_first,
                               const int32_t *__restrict__ nchild,
                               const int32_t *__restrict__ digit, const T *__restrict__ ops,
                               T *__restrict__ M)
    {
      extern __shared__ unsigned char smem_raw[];
      T            *sIn  = reinterpret_cast<T *>(smem_raw);
      T            *sOut = sIn + R * K;
      const int64_t P    = parents[blockIdx.x];
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        sOut[i] = T(0);
      const int c0 = child_first[P], nc = nchild[P];
      for (int c = 0; c < nc; ++c)
        {
          __syncthreads();
          const int64_t ch = c0 + c;
          for (int i = threadIdx.x; i < R * K; i += blockDim.x)
            sIn[i] = M[ch * R * K + i];
          __syncthreads();
          accumulate_translation(R, K, ops + int64_t(digit[ch]) * K * K, sIn, sOut);
        }
      __syncthreads();
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        M[P * R * K + i] = sOut[i];
    }

    template <typename T>
    __global__ void l2l_kernel(int R, int K, const int32_t *__restrict__ boxes,
                               const int32_t *__restrict__ parent,
                               const int32_t *__restrict__ digit, const T *__restrict__ ops,
                               T *__restrict__ Lx)
    {
      extern __shared__ unsigned char smem_raw[];
      T            *sIn  = reinterpret_cast<T *>(smem_raw);
      T            *sOut = sIn + R * K;
      const int64_t b    = boxes[blockIdx.x];
      const int64_t P    = parent[b];
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        {
          sIn[i]  = Lx[P * R * K + i];
          sOut[i] = T(0);
        }
      __syncthreads();
      accumulate_translation(R, K, ops + int64_t(digit[b]) * K * K, sIn, sOut);
      __syncthreads();
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        Lx[b * R * K + i] = sOut[i];
    }

    template <typename T>
    __global__ void m2l_kernel(int R, int K, const int32_t *__restrict__ tgt,
                               const int64_t *__restrict__ src_ptr,
                               const int32_t *__restrict__ src, const int32_t *__restrict__ off,
                               const T *__restrict__ ops, const T *__restrict__ M,
                               T *__restrict__ Lx)
    {
      extern __shared__ unsigned char smem_raw[];
      T            *sIn  = reinterpret_cast<T *>(smem_raw);
      T            *sOut = sIn + R * K;
      const int     ti   = blockIdx.x;
      const int64_t t    = tgt[ti];
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        sOut[i] = T(0);
      for (int64_t e = src_ptr[ti]; e < src_ptr[ti + 1]; ++e)
        {
          __syncthreads();
          const int64_t s = src[e];
          for (int i = threadIdx.x; i < R * K; i += blockDim.x)
            sIn[i] = M[s * R * K + i];
          __syncthreads();
          accumulate_translation(R, K, ops + int64_t(off[e]) * K * K, sIn, sOut);
        }
      __syncthreads();
      for (int i = threadIdx.x; i < R * K; i += blockDim.x)
        Lx[t * R * K + i] += sOut[i];
    }

    template <typename T>
    __global__ void m2p_kernel(int R, int K, int p, int N, const int32_t *__restrict__ tgt,
                               const int64_t *__restrict__ src_ptr,
                               const int32_t *__restrict__ src, const int32_t *__restrict__ nbeg,
                               const int32_t *__restrict__ nend,
                               const int32_t *__restrict__ node_sorted,
                               const double *__restrict__ xyz, const double *__restrict__ center,
                               const double *__restrict__ delta, const T *__restrict__ M,
                               T *__restrict__ y)
    {
      const int64_t t  = tgt[blockIdx.x];
      const int     n0 = nbeg[t], nn = nend[t] - n0;
      for (int idx = threadIdx.x; idx < nn * R; idx += blockDim.x)
        {
          const int node = node_sorted[n0 + idx % nn];
          const int r    = idx / nn;
          T         acc  = T(0);
          for (int64_t e = src_ptr[blockIdx.x]; e < src_ptr[blockIdx.x + 1]; ++e)
            {
              const int64_t s  = src[e];
              const double  h  = delta[s];
              const T       rx = T((xyz[3 * int64_t(node)] - center[3 * s]) / h);
              const T       ry = T((xyz[3 * int64_t(node) + 1] - center[3 * s + 1]) / h);
              const T       rz = T((xyz[3 * int64_t(node) + 2] - center[3 * s + 2]) / h);
              acc += eval_expansion<T, T>(M + (s * R + r) * K, p, rx, ry, rz, true) / T(h);
            }
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

  template <typename T>
  static void set_smem(const void *fn, size_t bytes)
  {
    if (bytes > 48 * 1024)
      PIBEM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
  }

  template <typename T>
  void launch_m2m_level(const OperatorDev<T> &op, const TreeDev &td, int R, int parent_level, T *M,
                        cudaStream_t s)
  {
    const int a = op.parents_level_ptr[parent_level], b = op.parents_level_ptr[parent_level + 1];
    if (b <= a)
      return;
    size_t smem = size_t(2) * R * op.K * sizeof(T);
    set_smem<T>((const void *)m2m_kernel<T>, smem);
    m2m_kernel<T><<<b - a, tpb_for(R * op.K), smem, s>>>(R, op.K, op.parents + a, td.child_first,
                                                         td.nchild, td.digit, op.m2m_ops, M);
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T>
  void launch_l2l_level(const OperatorDev<T> &op, const TreeDev &td, int R, int level, T *Lx,
                        cudaStream_t s)
  {
    const int a = op.l2l_level_ptr[level], b = op.l2l_level_ptr[level + 1];
    if (b <= a)
      return;
    size_t smem = size_t(2) * R * op.K * sizeof(T);
    set_smem<T>((const void *)l2l_kernel<T>, smem);
    l2l_kernel<T><<<b - a, tpb_for(R * op.K), smem, s>>>(R, op.K, op.l2l_box + a, td.parent,
                                                         td.digit, op.l2l_ops, Lx);
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T>
  void launch_m2l_level(const OperatorDev<T> &op, int R, int level, const T *M, T *Lx,
                        cudaStream_t s)
  {
    const int a = op.m2l_level_ptr[level], b = op.m2l_level_ptr[level + 1];
    if (b <= a)
      return;
    size_t smem = size_t(2) * R * op.K * sizeof(T);
    set_smem<T>((const void *)m2l_kernel<T>, smem);
    m2l_kernel<T><<<b - a, tpb_for(R * op.K), smem, s>>>(R, op.K, op.m2l_tgt + a,
                                                         op.m2l_src_ptr + a, op.m2l_src,
                                                         op.m2l_off, op.m2l_ops, M, Lx);
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T>
  void launch_m2p(const OperatorDev<T> &op, const TreeDev &td, int R, int N, const T *M, T *y,
                  cudaStream_t s)
  {
    if (op.n_m2p_tgt == 0)
      return;
    m2p_kernel<T><<<op.n_m2p_tgt, 64, 0, s>>>(R, op.K, op.p, N, op.m2p_tgt, op.m2p_src_ptr,
                                              op.m2p_src, td.nbeg, td.nend, td.node_sorted,
                                              td.xyz, td.center, td.delta, M, y);
    PIBEM_CUDA(cudaGetLastError());
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
