// Vector kernels of the device-resident GMRES (FP64 Arnoldi with classical
// Gram-Schmidt applied twice) and of the BEMProblem wrappers (masks, rhs,
// system matrix).  Reductions are two-stage with a fixed order, so results do
// not depend on scheduling.
#include <algorithm>

#include "krylov.h"
#include "pdl.cuh"

namespace pibem
{
  namespace
  {
    constexpr int kDotBlock = 256;

    // partial[(r * nblk + blk) * ncols + i] = sum over the block's rows of V[r][i][t] w[r][t].
    // Warp k of the block takes columns k, k + 8, ...; its lanes stride over the
    // block's rows (coalesced; the w slice is re-read from L1) and the warp sum is
    // reduced in a fixed order, so the columns proceed in parallel without block
    // barriers.
    __global__ void dots_partial_kernel(int64_t n, int ncols, int64_t ldv, int64_t ldr,
                                        const double *__restrict__ V,
                                        const double *__restrict__ w, int nblk,
                                        double *__restrict__ partial)
    {
      const int     r     = blockIdx.y;
      const int     blk   = blockIdx.x;
      const double *Vr    = V + int64_t(r) * ldr;
      const double *wr    = w + int64_t(r) * n;
      const int64_t chunk = (n + nblk - 1) / nblk;
      const int64_t t0 = int64_t(blk) * chunk, t1 = min(n, t0 + chunk);
      const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      for (int i = warp; i < ncols; i += nw)
        {
          const double *v = Vr + int64_t(i) * ldv;
          double        s = 0;
#pragma unroll 8
          for (int64_t t = t0 + lane; t < t1; t += 32)
            s += v[t] * wr[t];
          for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
          if (lane == 0)
            partial[(int64_t(r) * nblk + blk) * ncols + i] = s;
        }
    }

    // one warp per output: lanes stride over the block partials, fixed-order tree
    __global__ void dots_final_kernel(int R, int ncols, int nblk, const double *__restrict__ partial,
                                      double *__restrict__ out)
    {
      const int idx  = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
      const int lane = threadIdx.x & 31;
      if (idx >= R * ncols)
        return;
      const int r = idx / ncols, i = idx % ncols;
      double    s = 0;
      for (int b = lane; b < nblk; b += 32)
        s += partial[(int64_t(r) * nblk + b) * ncols + i];
      for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0)
        out[idx] = s;
    }

    // w[r][t] -= sum_i V[r][i][t] h[r][i]   (h on the device, layout [r][ldh])
    //   (jvec non-null: column r takes ncols = jvec[r]; sel non-null: selected
    //   columns only)
    __global__ void gemv_sub_kernel(int64_t n, int R, int ncols, int64_t ldv, int64_t ldr,
                                    const double *__restrict__ V, const double *__restrict__ h,
                                    int ldh, double *__restrict__ w, double sign,
                                    const int *__restrict__ jvec, const int *__restrict__ sel)
    {
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      int64_t r = idx / n, t = idx % n;
      if (sel && !sel[r])
        return;
      if (jvec)
        ncols = jvec[r];
      double  s = 0;
#pragma unroll 8
      for (int i = 0; i < ncols; ++i)
        s += V[r * ldr + int64_t(i) * ldv + t] * h[r * ldh + i];
      w[idx] -= sign * s;
    }

    // One Gram-Schmidt step of the Arnoldi process in one launch per pass, with
    // the same arithmetic as dots_partial + dots_final and gemv_sub:
    //   MODE 0: out[r][i]  = V[r][i] . w[r]                      (i < ncols)
    //   MODE 1: w[r] -= sum_i V[r][i] hin[r][i], then out[r][i] = V[r][i] . w[r]
    //   MODE 2: w[r] -= sum_i V[r][i] hin[r][i], then out[r][0] = w[r] . w[r]
    // Block blk of row r owns rows [blk chunk, (blk + 1) chunk) of every vector:
    // it updates them (threads stride over the rows, the sum over i in order),
    // then forms its partial dots (warp k takes outputs k, k + 8, ...; lanes
    // stride over the rows; fixed shuffle tree).  The last block of row r to
    // finish (a ticket taken after a fence) adds the nblk partials of each
    // output in the fixed order of dots_final and resets the ticket, so the
    // result does not depend on which block is last.
    //   jvec (may be null): per-column Arnoldi step j = jvec[r] read on the
    //   device (the pass takes ncols = j + 1 basis vectors; j < 0: the column
    //   is idle and its blocks return); out holds ldo values per column r.
    template <int MODE>
    __global__ void __launch_bounds__(256)
      cgs_step_kernel(int64_t n, int ncols, int64_t ldv, int64_t ldr, const double *__restrict__ V,
                      const double *__restrict__ hin, int ldh, double *__restrict__ w, int nblk,
                      double *__restrict__ partial, int *__restrict__ ticket,
                      double *__restrict__ out, const int *__restrict__ jvec, int ldo)
    {
      pdl_entry();
      if (jvec)
        {
          const int j = jvec[blockIdx.y];
          if (j < 0)
            return;
          ncols = j + 1;
        }
      const int     r     = blockIdx.y;
      const int     blk   = blockIdx.x;
      const double *Vr    = V + int64_t(r) * ldr;
      double       *wr    = w + int64_t(r) * n;
      const int64_t chunk = (n + nblk - 1) / nblk;
      const int64_t t0 = int64_t(blk) * chunk, t1 = min(n, t0 + chunk);
      const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      if constexpr (MODE > 0)
        {
          const double *hr = hin + int64_t(r) * ldh;
          for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x)
            {
              double s = 0;
#pragma unroll 8
              for (int i = 0; i < ncols; ++i)
                s += Vr[int64_t(i) * ldv + t] * hr[i];
              wr[t] -= s;
            }
          __syncthreads(); // the block's w rows are updated (visible to the block)
        }
      const int nout = MODE == 2 ? 1 : ncols;
      // partial sums of column r: per block pstride values (with jvec the
      // columns have different output counts, so a fixed stride, ldo, keeps
      // their regions apart)
      const int pstride = jvec ? ldo : nout;
      for (int i = warp; i < nout; i += nw)
        {
          const double *v = MODE == 2 ? wr : Vr + int64_t(i) * ldv;
          double        s = 0;
#pragma unroll 8
          for (int64_t t = t0 + lane; t < t1; t += 32)
            s += v[t] * wr[t];
          for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
          if (lane == 0)
            partial[(int64_t(r) * nblk + blk) * pstride + i] = s;
        }
      __threadfence();
      __syncthreads();
      __shared__ int last;
      if (threadIdx.x == 0)
        last = atomicAdd(ticket + r, 1) == nblk - 1;
      __syncthreads();
      if (!last)
        return;
      __threadfence();
      for (int i = warp; i < nout; i += nw)
        {
          double s = 0;
          for (int b = lane; b < nblk; b += 32)
            s += __ldcg(partial + (int64_t(r) * nblk + b) * pstride + i);
          for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
          if (lane == 0)
            out[int64_t(r) * ldo + i] = s;
        }
      if (threadIdx.x == 0)
        ticket[r] = 0;
    }

    // V[r][j+1] = w[r] / hn[r]  (hn > 0), else 0; with jvec the output column
    // is basis vector jvec[r] + 1 of out (jvec[r] < 0: column skipped); with sel
    // only the columns with sel[r] != 0; with z the value is also written to z[r]
    __global__ void normalize_kernel(int64_t n, int R, const double *__restrict__ w,
                                     const double *__restrict__ nrm, double *__restrict__ out,
                                     int64_t ldr, const int *__restrict__ jvec,
                                     double *__restrict__ z, const int *__restrict__ sel)
    {
      pdl_entry();
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      int64_t r = idx / n, t = idx % n;
      if (sel && !sel[r])
        return;
      int64_t off = 0;
      if (jvec)
        {
          if (jvec[r] < 0)
            return;
          off = int64_t(jvec[r] + 1) * n;
        }
      double       h = sqrt(nrm[r]);
      const double v = h > 0 ? w[idx] / h : 0.0;
      out[r * ldr + off + t] = v;
      if (z)
        z[idx] = v;
    }

    // ---- device-driven GMRES cycles, one state per column (slot) -------------
    // Per column r: Hessenberg H[r] ((m+1) x m, entry (i, j) at i m + j), Givens
    // cosines / sines cs[r], sn[r] (m), g[r] (m+1), jvec[r] (the column's next
    // Arnoldi step; -1: the column takes no part), kdone[r] (-1, or the step
    // count after which the column met its tolerance), its[r] / maxit[r]
    // (iterations so far / limit), bn[r], tol[r] (stopping test |g_{j+1}| /
    // bn <= tol).  hb: [h1 (R x L) | h2 (R x L) | |w|^2 (R)], L = m + 1, the two
    // Gram-Schmidt passes' coefficients and the norm of a step.  ctl[0]: 1 while
    // the steps go on; ctl[1]: steps run; ctl[2]: most steps before the host is
    // back (a quantum); ctl[3]: 1 to stop at the first column that ends its
    // cycle, 0 to go on until every column has ended its cycle.

    // cycle start of the selected columns: g[r] = (beta_r, 0, ...) with beta_r =
    // sqrt(nrm2[r]), jvec[r] = 0, kdone[r] = -1
    __global__ void gmres_cycle_init_kernel(int R, int L, const int *__restrict__ sel,
                                            const double *__restrict__ nrm2, double *__restrict__ g,
                                            int *__restrict__ kdone, int *__restrict__ jvec)
    {
      for (int r = threadIdx.x; r < R; r += blockDim.x)
        if (sel[r])
          {
            g[int64_t(r) * L] = sqrt(nrm2[r]);
            kdone[r]          = -1;
            jvec[r]           = 0;
          }
    }

    // Step j = jvec[r] of every active column: the Hessenberg column, its Givens
    // rotation and the stopping test (|g_{j+1}| / bn <= tol, or a zero
    // subdiagonal); then jvec and the iteration count advance.  A column ends its
    // cycle when it meets its tolerance, after m steps or at its iteration
    // limit (jvec = -2 - steps: no more steps); when the steps stop (see ctl),
    // ctl[0] = 0 and, in a graph, the loop's condition is cleared.
    __global__ void gmres_givens_kernel(int R, int m, const double *__restrict__ hb,
                                        double *__restrict__ H, double *__restrict__ cs,
                                        double *__restrict__ sn, double *__restrict__ g,
                                        int *__restrict__ kdone, int *__restrict__ jvec,
                                        int *__restrict__ its, const int *__restrict__ maxit,
                                        const double *__restrict__ bn,
                                        const double *__restrict__ tol, int *__restrict__ ctl,
                                        cudaGraphConditionalHandle cond, int use_cond)
    {
      pdl_entry();
      const int L = m + 1;
      __shared__ int ended, active, alive;
      if (threadIdx.x == 0)
        ended = active = alive = 0;
      __syncthreads();
      for (int r = threadIdx.x; r < R; r += blockDim.x)
        {
          const int j = jvec[r];
          if (j < 0)
            continue;
          active = 1;
          double       *Hc = H + int64_t(r) * L * m;
          const double *h1 = hb + int64_t(r) * L, *h2 = hb + int64_t(R) * L + int64_t(r) * L;
          for (int i = 0; i <= j; ++i)
            Hc[int64_t(i) * m + j] = h1[i] + h2[i];
          Hc[int64_t(j + 1) * m + j] = sqrt(hb[2 * int64_t(R) * L + r]);
          double *c = cs + int64_t(r) * m, *sv = sn + int64_t(r) * m, *gg = g + int64_t(r) * L;
          for (int i = 0; i < j; ++i)
            {
              const double a0 = Hc[int64_t(i) * m + j], a1 = Hc[int64_t(i + 1) * m + j];
              Hc[int64_t(i) * m + j]     = c[i] * a0 + sv[i] * a1;
              Hc[int64_t(i + 1) * m + j] = -sv[i] * a0 + c[i] * a1;
            }
          const double a = Hc[int64_t(j) * m + j], bb = Hc[int64_t(j + 1) * m + j];
          const double d = hypot(a, bb);
          c[j]           = d > 0 ? a / d : 1.0;
          sv[j]          = d > 0 ? bb / d : 0.0;
          Hc[int64_t(j) * m + j]     = d;
          Hc[int64_t(j + 1) * m + j] = 0;
          gg[j + 1]                  = -sv[j] * gg[j];
          gg[j]                      = c[j] * gg[j];
          const int it               = its[r] + 1;
          its[r]                     = it;
          if (fabs(gg[j + 1]) / bn[r] <= tol[r] || bb == 0.0)
            kdone[r] = j + 1;
          if (kdone[r] >= 0 || j + 1 >= m || it >= maxit[r])
            {
              // the column ends its cycle: it takes no more steps (jvec
              // -2 - steps until the host has used it)
              jvec[r] = -2 - (j + 1);
              ended   = 1;
            }
          else
            {
              jvec[r] = j + 1;
              alive   = 1;
            }
        }
      __syncthreads();
      if (threadIdx.x == 0)
        {
          const int steps = ctl[1] + 1; // steps run since the host set ctl
          // the steps go on while some column is in its cycle, for at most
          // ctl[2] steps, and with ctl[3] set only until the first column ends
          // its cycle (every active column ends its cycle within m steps)
          const int stop = !alive || (ended && ctl[3]) || steps >= ctl[2];
          ctl[0]          = !stop;
          ctl[1]          = steps;
          if (use_cond && stop)
            cudaGraphSetConditional(cond, 0);
        }
    }

    // End of a column's cycle: y[r] solves its triangular system of k steps (k =
    // kdone[r] if it met its tolerance, else jvec[r]); y[r][i] = 0 for i >= k.
    // Selected columns only.
    __global__ void gmres_lsq_kernel(int R, int m, const int *__restrict__ sel,
                                     const double *__restrict__ H, const double *__restrict__ g,
                                     const int *__restrict__ kdone, const int *__restrict__ jvec,
                                     double *__restrict__ y)
    {
      const int L = m + 1;
      for (int r = threadIdx.x; r < R; r += blockDim.x)
        {
          if (!sel[r])
            continue;
          const int     k  = kdone[r] < 0 ? jvec[r] : kdone[r];
          const double *Hc = H + int64_t(r) * L * m;
          const double *gg = g + int64_t(r) * L;
          double       *yr = y + int64_t(r) * L;
          for (int i = k; i < L; ++i)
            yr[i] = 0.0;
          for (int i = k - 1; i >= 0; --i)
            {
              double sum = gg[i];
              for (int jj = i + 1; jj < k; ++jj)
                sum -= Hc[int64_t(i) * m + jj] * yr[jj];
              yr[i] = sum / Hc[int64_t(i) * m + i];
            }
        }
    }

    // dst[k] = src[cols[k]] (n values a column; source column stride lds)
    __global__ void gather_cols_kernel(int64_t n, int Rc, const int *__restrict__ cols,
                                       const double *__restrict__ src, int64_t lds,
                                       double *__restrict__ dst)
    {
      pdl_entry();
      const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * Rc)
        return;
      const int64_t k = idx / n, t = idx - k * n;
      dst[idx]        = src[int64_t(cols[k]) * lds + t];
    }
    // dst[cols[k]] = src[k]
    __global__ void scatter_cols_kernel(int64_t n, int Rc, const int *__restrict__ cols,
                                        const double *__restrict__ src, double *__restrict__ dst,
                                        int64_t ldd)
    {
      pdl_entry();
      const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * Rc)
        return;
      const int64_t k = idx / n, t = idx - k * n;
      dst[int64_t(cols[k]) * ldd + t] = src[idx];
    }

    // dst[k] = float(src[cols[k]]) and dst[cols[k]] = double(src[k]): the
    // gather / scatter of the active columns fused with the FP32 operator's
    // input and output conversions
    __global__ void gather_d2f_kernel(int64_t n, int Rc, const int *__restrict__ cols,
                                      const double *__restrict__ src, float *__restrict__ dst)
    {
      pdl_entry();
      const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * Rc)
        return;
      const int64_t k = idx / n, t = idx - k * n;
      dst[idx]        = float(src[int64_t(cols[k]) * n + t]);
    }
    __global__ void f2d_scatter_kernel(int64_t n, int Rc, const int *__restrict__ cols,
                                       const float *__restrict__ src, double *__restrict__ dst)
    {
      pdl_entry();
      const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * Rc)
        return;
      const int64_t k = idx / n, t = idx - k * n;
      dst[int64_t(cols[k]) * n + t] = double(src[idx]);
    }

    // y[r] = a x[r] + b y[r] for the selected columns
    __global__ void axpby_sel_kernel(int64_t n, int R, const int *__restrict__ sel, double a,
                                     const double *__restrict__ x, double b, double *__restrict__ y)
    {
      const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R || !sel[idx / n])
        return;
      y[idx] = a * x[idx] + b * y[idx];
    }

    __global__ void axpby_kernel(int64_t n, double a, const double *__restrict__ x, double b,
                                 double *__restrict__ y)
    {
      int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i < n)
        y[i] = a * x[i] + b * y[i];
    }

    __global__ void d2f_kernel(int64_t n, const double *__restrict__ a, float *__restrict__ b)
    {
      pdl_entry();
      int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i < n)
        b[i] = float(a[i]);
    }
    __global__ void f2d_kernel(int64_t n, const float *__restrict__ a, double *__restrict__ b)
    {
      pdl_entry();
      int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i < n)
        b[i] = double(a[i]);
    }

    // S = N where the column dof is Neumann, -D where Dirichlet, + alpha on the
    // diagonal of Neumann rows (BEMProblem::vmult FMA branch, bem_problem.cc:1199-1209,
    // as one matrix like BEMFMA's init_preconditioner, bem_fma.cc:952-962).
    __global__ void system_matrix_kernel(int64_t n_vals, int n_leaves,
                                         const int64_t *__restrict__ val_ptr,
                                         const int64_t *__restrict__ col_ptr,
                                         const int64_t *__restrict__ row_ptr,
                                         const int32_t *__restrict__ rows,
                                         const int32_t *__restrict__ cols,
                                         const uint8_t *__restrict__ dir,
                                         const double *__restrict__ alpha,
                                         const double *__restrict__ Nv,
                                         const double *__restrict__ Dv, double *__restrict__ S,
                                         float *__restrict__ S32)
    {
      int64_t vi = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (vi >= n_vals)
        return;
      int lo = 0, hi = n_leaves - 1;
      while (lo < hi)
        {
          int mid = (lo + hi + 1) >> 1;
          if (val_ptr[mid] <= vi)
            lo = mid;
          else
            hi = mid - 1;
        }
      const int64_t nc  = col_ptr[lo + 1] - col_ptr[lo];
      const int64_t ld  = (nc + 3) / 4 * 4;
      const int64_t loc = vi - val_ptr[lo];
      if (loc % ld >= nc)
        {
          S[vi] = 0.0;
          if (S32)
            S32[vi] = 0.0f;
          return;
        }
      const int row = rows[row_ptr[lo] + loc / ld];
      const int col = cols[col_ptr[lo] + loc % ld];
      double        v   = dir[col] ? -Dv[vi] : Nv[vi];
      if (row == col && !dir[row])
        v += alpha[row];
      S[vi] = v;
      if (S32)
        S32[vi] = float(v);
    }

    // rhs = -(outN + alpha*(tmp.dir)) + outD  (BEMProblem::compute_rhs, bem_problem.cc:1240-1258)
    __global__ void rhs_combine_kernel(int64_t n, int R, const double *__restrict__ tmp,
                                       const uint8_t *__restrict__ dir,
                                       const double *__restrict__ alpha,
                                       const double *__restrict__ oN, const double *__restrict__ oD,
                                       double *__restrict__ rhs)
    {
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      int64_t t  = idx % n;
      double  sp = dir[t] ? tmp[idx] : 0.0;
      rhs[idx]   = -(oN[idx] + alpha[t] * sp) + oD[idx];
    }

    // split tmp_rhs into (tmp.dir, tmp.neu)
    __global__ void split_masks_kernel(int64_t n, int R, const double *__restrict__ tmp,
                                       const uint8_t *__restrict__ dir, double *__restrict__ a,
                                       double *__restrict__ b)
    {
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      int64_t t = idx % n;
      a[idx]    = dir[t] ? tmp[idx] : 0.0;
      b[idx]    = dir[t] ? 0.0 : tmp[idx];
    }

    // scatter: phi(i) = sol(i) on Neumann nodes, dphi_dn(i) = sol(i) on Dirichlet nodes
    __global__ void scatter_kernel(int64_t n, int R, const double *__restrict__ sol,
                                   const uint8_t *__restrict__ dir, double *__restrict__ phi,
                                   double *__restrict__ dphi)
    {
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      int64_t t = idx % n;
      if (dir[t])
        dphi[idx] = sol[idx];
      else
        phi[idx] = sol[idx];
    }

    __global__ void add_scalar_kernel(int64_t n, int R, const double *__restrict__ shift,
                                      double *__restrict__ x)
    {
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      x[idx] += shift[idx / n];
    }

    // x[r] += -sqrt(nrm2[r])  (the pure-Neumann shift v - ||v||)
    __global__ void sub_norm_kernel(int64_t n, int R, const double *__restrict__ nrm2,
                                    double *__restrict__ x)
    {
      int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      x[idx] += -sqrt(nrm2[idx / n]);
    }

    // z[node] = sum_c Pinv[leaf][r][c] v[rows_c]  (leaf-block Jacobi, right
    // preconditioner), in the precision P of the stored inverses: FP32 for the
    // mixed path's inner solves (GB300's FP64 rate is 1/58 of its FP32 rate),
    // FP64 for the plain FP64 path (whose GMRES would otherwise see the FP32
    // rounding as a nonlinearity near its 1e-8 target).  One warp per leaf, 8
    // per block: the leaf's v entries are gathered into the warp's shared
    // slice, lane i computes rows i, i + 32, ... with c ascending; the blocks
    // are stored column-major (entry (r, c) at c * nr + r), so a column is read
    // across the lanes.
    template <typename P>
    __global__ void __launch_bounds__(256)
      block_apply_kernel(int n_leaves, int max_rows, int R, int64_t n, int64_t ldv,
                         const int64_t *__restrict__ row_ptr, const int64_t *__restrict__ blk_ptr,
                         const int32_t *__restrict__ rows, const P *__restrict__ Pinv,
                         const double *__restrict__ v, double *__restrict__ z,
                         const double *__restrict__ nrm2, double *__restrict__ vout, int64_t ldo,
                         const int *__restrict__ jvec, const int *__restrict__ sel)
    {
      pdl_entry();
      extern __shared__ __align__(8) unsigned char sv_raw[];
      P        *sv_all = reinterpret_cast<P *>(sv_raw);
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const int leaf = blockIdx.x * 8 + warp;
      if (leaf >= n_leaves)
        return;
      P            *sv = sv_all + int64_t(warp) * max_rows;
      const int64_t r0 = row_ptr[leaf];
      const int     nr = int(row_ptr[leaf + 1] - r0);
      const P      *B  = Pinv + blk_ptr[leaf];
      for (int rr = 0; rr < R; ++rr)
        {
          if (sel && !sel[rr])
            continue;
          int64_t vo = int64_t(rr) * ldo; // output column (basis vector jvec[rr] + 1 with jvec)
          if (jvec)
            {
              if (jvec[rr] < 0)
                continue;
              vo += int64_t(jvec[rr] + 1) * n;
            }
          if (nrm2)
            {
              // the Arnoldi normalisation fused in (as normalize_kernel):
              // vout = v / |v|, then z = P^-1 vout
              const double h = sqrt(nrm2[rr]);
              for (int c = lane; c < nr; c += 32)
                {
                  const int64_t row = rows[r0 + c];
                  const double  vn  = h > 0 ? v[int64_t(rr) * ldv + row] / h : 0.0;
                  vout[vo + row] = vn;
                  sv[c]          = P(vn);
                }
            }
          else
            for (int c = lane; c < nr; c += 32)
              sv[c] = P(v[int64_t(rr) * ldv + rows[r0 + c]]);
          __syncwarp();
          for (int i = lane; i - lane < nr; i += 32)
            {
              P s = P(0);
              if (i < nr)
                {
                  int c = 0;
                  for (; c + 8 <= nr; c += 8)
                    {
                      P p[8];
#pragma unroll
                      for (int u = 0; u < 8; ++u)
                        p[u] = B[int64_t(c + u) * nr + i];
#pragma unroll
                      for (int u = 0; u < 8; ++u)
                        s = fma(p[u], sv[c + u], s);
                    }
                  for (; c < nr; ++c)
                    s = fma(B[int64_t(c) * nr + i], sv[c], s);
                  z[int64_t(rr) * n + rows[r0 + i]] = double(s);
                }
            }
          __syncwarp();
        }
    }

    // ---- ILU(0) of the near-field system matrix (preconditioner 2) ----------
    // CSR in node order: ptr, col (ascending), val, diag (position of the
    // diagonal).  Level sets: the rows of a level depend only on rows of
    // earlier levels (lower part for the factorisation and the forward
    // substitution, upper part for the backward one).

    // one row of the near field (or a constraint line) into the CSR: warp per node
    __global__ void ilu_fill_kernel(int64_t n, const int64_t *__restrict__ ptr,
                                    const int32_t *__restrict__ pos, const int32_t *__restrict__ row_leaf,
                                    const int64_t *__restrict__ nrow_ptr, const int64_t *__restrict__ ncol_ptr,
                                    const int64_t *__restrict__ nval_ptr, const int32_t *__restrict__ ncols,
                                    const double *__restrict__ S, const int32_t *__restrict__ con,
                                    int32_t *__restrict__ col, double *__restrict__ val)
    {
      const int64_t i    = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
      const int     lane = threadIdx.x & 31;
      if (i >= n)
        return;
      const int64_t o = ptr[i];
      if (con[i] != -2)
        {
          // a constrained row: 1 on the diagonal and +1 at the line's column
          // (bem_fma.cc:3190-3201 stores the constraint entries as they are)
          if (lane == 0)
            {
              const int c = con[i];
              if (c >= 0 && c != int(i))
                {
                  const bool lo = c < int(i);
                  col[o]        = lo ? c : int32_t(i);
                  col[o + 1]    = lo ? int32_t(i) : c;
                  val[o]        = 1.0;
                  val[o + 1]    = 1.0;
                }
              else
                {
                  col[o] = int32_t(i);
                  val[o] = 1.0;
                }
            }
          return;
        }
      const int     r  = pos[i];
      const int     lf = row_leaf[r];
      const int64_t c0 = ncol_ptr[lf], nc = ncol_ptr[lf + 1] - c0;
      const int64_t ld = (nc + 3) / 4 * 4;
      const double *v  = S + nval_ptr[lf] + (r - nrow_ptr[lf]) * ld;
      for (int64_t k = lane; k < nc; k += 32)
        {
          col[o + k] = ncols[c0 + k];
          val[o + k] = v[k];
        }
    }

    // IKJ ILU(0) of the rows of one level, a block per row with the row in
    // shared memory: for the row's columns k < i in ascending order,
    // a_ik /= a_kk, then a_ij -= a_ik a_kj for the columns j > k of row k that
    // row i holds (threads take row k's entries, a binary search finds j in
    // the row's sorted columns); row k is final (an earlier level)
    __global__ void ilu_factor_kernel(const int32_t *__restrict__ rows, const int64_t *__restrict__ ptr,
                                      const int32_t *__restrict__ col, double *__restrict__ val,
                                      const int64_t *__restrict__ diag)
    {
      extern __shared__ __align__(16) unsigned char ilu_smem[];
      const int     i  = rows[blockIdx.x];
      const int64_t a0 = ptr[i], n = ptr[i + 1] - a0, nd = diag[i] - a0;
      double       *sv = reinterpret_cast<double *>(ilu_smem);
      int32_t      *sc = reinterpret_cast<int32_t *>(sv + n);
      for (int64_t e = threadIdx.x; e < n; e += blockDim.x)
        {
          sv[e] = val[a0 + e];
          sc[e] = col[a0 + e];
        }
      __syncthreads();
      for (int64_t e = 0; e < nd; ++e)
        {
          const int     k   = sc[e];
          const int64_t dk  = diag[k], k1 = ptr[k + 1];
          const double  lik = sv[e] / val[dk];
          for (int64_t f = dk + 1 + threadIdx.x; f < k1; f += blockDim.x)
            {
              const int j  = col[f];
              int64_t   lo = e + 1, hi = n;
              while (lo < hi)
                {
                  const int64_t m = (lo + hi) >> 1;
                  if (sc[m] < j)
                    lo = m + 1;
                  else
                    hi = m;
                }
              if (lo < n && sc[lo] == j)
                sv[lo] -= lik * val[f];
            }
          __syncthreads();
          if (threadIdx.x == 0)
            sv[e] = lik;
        }
      __syncthreads();
      for (int64_t e = threadIdx.x; e < n; e += blockDim.x)
        val[a0 + e] = sv[e];
    }

    // z[r] = v[r] for the columns with sel[r] (v column stride ldv, z stride n)
    __global__ void copy_sel_kernel(int64_t n, int R, const double *__restrict__ v, int64_t ldv,
                                    double *__restrict__ z, const int *__restrict__ sel)
    {
      const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (idx >= n * R)
        return;
      const int64_t r = idx / n, t = idx - r * n;
      if (sel && !sel[r])
        return;
      z[idx] = v[r * ldv + t];
    }

    // forward (lower, unit diagonal) or backward (upper) substitution for the
    // rows of one level, in place on the selected columns of z (stride n):
    // warp per (row, column), lanes over the row's entries, fixed butterfly
    template <bool FWD>
    __global__ void ilu_solve_kernel(int nrows, const int32_t *__restrict__ rows, int R, int64_t n,
                                     const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                     const double *__restrict__ val, const int64_t *__restrict__ diag,
                                     double *__restrict__ z, const int *__restrict__ sel,
                                     const int *__restrict__ jvec)
    {
      const int w    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
      const int lane = threadIdx.x & 31;
      if (w >= nrows * R)
        return;
      const int r = w / nrows, i = rows[w - r * nrows];
      if ((sel && !sel[r]) || (jvec && jvec[r] < 0))
        return;
      double       *zr = z + int64_t(r) * n;
      const int64_t a0 = FWD ? ptr[i] : diag[i] + 1, a1 = FWD ? diag[i] : ptr[i + 1];
      double        s  = 0;
      for (int64_t e = a0 + lane; e < a1; e += 32)
        s += val[e] * zr[col[e]];
      for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0)
        zr[i] = FWD ? zr[i] - s : (zr[i] - s) / val[diag[i]];
    }

    template <typename T>
    __global__ void combine_p2m_kernel(int64_t n, int K4, const int32_t *__restrict__ prow_dof,
                                       const uint8_t *__restrict__ dir, const T *__restrict__ T1,
                                       const T *__restrict__ T2, T *__restrict__ Tc)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n)
        return;
      Tc[i] = dir[prow_dof[i / K4]] ? -T2[i] : T1[i];
    }

    inline unsigned nblocks(int64_t n, int t = 256) { return unsigned((n + t - 1) / t); }

    // Double-node constraint lines (deal.II ConstrainedOperator::vmult,
    // include/constrained_matrix.h:100-125): row rows[k] of y becomes
    // x[row] - x[cols[k]] (cols[k] < 0: x[row]).  One thread per (line, column).
    __global__ void constrain_rows_kernel(int n_con, int R, int64_t n, const int32_t *__restrict__ rows,
                                          const int32_t *__restrict__ cols,
                                          const double *__restrict__ x, double *__restrict__ y)
    {
      pdl_entry();
      const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= int64_t(n_con) * R)
        return;
      const int64_t r = t / n_con, k = t - r * n_con;
      const double *xr = x + r * n;
      const int32_t c  = cols[k];
      y[r * n + rows[k]] = xr[rows[k]] - (c >= 0 ? xr[c] : 0.0);
    }

    // Right-hand side of the constraint lines (bem_problem.cc:1405-1579), per
    // (line, column): kind 0 -> 0 (x_row = x_col); kind 1 -> tmp[p] (the
    // potential given at the set's Dirichlet node); kind 2 -> the normal
    // derivative of a Dirichlet-Dirichlet pair (p, q) from the nodal normals
    // nrm (3 per node) and the surface gradients sg of tmp (3 per node, column
    // after column): c = n_p.n_q, (s_q.n_p + (s_p.n_q) c) / (1 - c^2).  Then
    // b[row] = that value (ConstrainedOperator::distribute_rhs).
    __global__ void constraint_rhs_kernel(int n_con, int R, int64_t n, const int32_t *__restrict__ rows,
                                          const uint8_t *__restrict__ kind,
                                          const int32_t *__restrict__ p, const int32_t *__restrict__ q,
                                          const double *__restrict__ tmp,
                                          const double *__restrict__ nrm,
                                          const double *__restrict__ sg, double *__restrict__ b)
    {
      const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= int64_t(n_con) * R)
        return;
      const int64_t r = t / n_con, k = t - r * n_con;
      double        g = 0.0;
      if (kind[k] == 1)
        g = tmp[r * n + p[k]];
      else if (kind[k] == 2)
        {
          const double *np_ = nrm + 3 * int64_t(p[k]), *nq = nrm + 3 * int64_t(q[k]);
          const double *sp_ = sg + 3 * (r * n + p[k]), *sq = sg + 3 * (r * n + q[k]);
          const double  c   = np_[0] * nq[0] + np_[1] * nq[1] + np_[2] * nq[2];
          const double  sqnp = sq[0] * np_[0] + sq[1] * np_[1] + sq[2] * np_[2];
          const double  spnq = sp_[0] * nq[0] + sp_[1] * nq[1] + sp_[2] * nq[2];
          g = (1.0 / (1.0 - c * c)) * (sqnp + spnq * c);
        }
      b[r * n + rows[k]] = g;
    }

  } // namespace

  void launch_dots(int64_t n, int R, int ncols, int64_t ldv, int64_t ldr, const double *V,
                   const double *w, double *partial, int nblk, double *out, cudaStream_t s)
  {
    dim3 grid(nblk, R);
    dots_partial_kernel<<<grid, kDotBlock, 0, s>>>(n, ncols, ldv, ldr, V, w, nblk, partial);
    dots_final_kernel<<<nblocks(int64_t(R) * ncols * 32, 256), 256, 0, s>>>(R, ncols, nblk, partial, out);
    PIBEM_CUDA(cudaGetLastError());
    note_launch(2);
  }

  void launch_cgs_step(int mode, int64_t n, int R, int ncols, int64_t ldv, int64_t ldr,
                       const double *V, const double *hin, int ldh, double *w, int nblk,
                       double *partial, int *ticket, double *out, cudaStream_t s, const int *jvec,
                       int ldo)
  {
    dim3 grid(nblk, R);
    if (ldo <= 0)
      ldo = mode == 2 ? 1 : ncols;
    if (mode == 0)
      launch_pdl(cgs_step_kernel<0>, grid, kDotBlock, 0, s, n, ncols, ldv, ldr, V, hin, ldh, w, nblk, partial,
                                                     ticket, out, jvec, ldo);
    else if (mode == 1)
      launch_pdl(cgs_step_kernel<1>, grid, kDotBlock, 0, s, n, ncols, ldv, ldr, V, hin, ldh, w, nblk, partial,
                                                     ticket, out, jvec, ldo);
    else
      launch_pdl(cgs_step_kernel<2>, grid, kDotBlock, 0, s, n, ncols, ldv, ldr, V, hin, ldh, w, nblk, partial,
                                                     ticket, out, jvec, ldo);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_gemv_sub(int64_t n, int R, int ncols, int64_t ldv, int64_t ldr, const double *V,
                       const double *h, int ldh, double *w, double sign, cudaStream_t s,
                       const int *jvec, const int *sel)
  {
    gemv_sub_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, ncols, ldv, ldr, V, h, ldh, w, sign, jvec,
                                                   sel);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_normalize(int64_t n, int R, const double *w, const double *nrm2, double *out,
                        int64_t ldr, cudaStream_t s, const int *jvec, double *z, const int *sel)
  {
    launch_pdl(normalize_kernel, nblocks(n * R), 256, 0, s, n, R, w, nrm2, out, ldr, jvec, z, sel);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_gmres_cycle_init(int R, int m, const int *sel, const double *nrm2, double *g, int *kdone,
                               int *jvec, cudaStream_t s)
  {
    gmres_cycle_init_kernel<<<1, 256, 0, s>>>(R, m + 1, sel, nrm2, g, kdone, jvec);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_gmres_givens(int R, int m, const double *hb, double *H, double *cs, double *sn,
                           double *g, int *kdone, int *jvec, int *its, const int *maxit,
                           const double *bn, const double *tol, int *ctl,
                           cudaGraphConditionalHandle cond, bool use_cond, cudaStream_t s)
  {
    launch_pdl(gmres_givens_kernel, 1, 256, 0, s, R, m, hb, H, cs, sn, g, kdone, jvec, its, maxit, bn, tol,
                                          ctl, cond, use_cond ? 1 : 0);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_gmres_lsq(int R, int m, const int *sel, const double *H, const double *g,
                        const int *kdone, const int *jvec, double *y, cudaStream_t s)
  {
    gmres_lsq_kernel<<<1, 256, 0, s>>>(R, m, sel, H, g, kdone, jvec, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_gather_cols(int64_t n, int Rc, const int *cols, const double *src, int64_t lds,
                          double *dst, cudaStream_t s)
  {
    if (Rc == 0)
      return;
    launch_pdl(gather_cols_kernel, nblocks(n * Rc), 256, 0, s, n, Rc, cols, src, lds, dst);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_scatter_cols(int64_t n, int Rc, const int *cols, const double *src, double *dst,
                           int64_t ldd, cudaStream_t s)
  {
    if (Rc == 0)
      return;
    launch_pdl(scatter_cols_kernel, nblocks(n * Rc), 256, 0, s, n, Rc, cols, src, dst, ldd);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_gather_d2f(int64_t n, int Rc, const int *cols, const double *src, float *dst,
                         cudaStream_t s)
  {
    if (Rc == 0)
      return;
    launch_pdl(gather_d2f_kernel, nblocks(n * Rc), 256, 0, s, n, Rc, cols, src, dst);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_f2d_scatter(int64_t n, int Rc, const int *cols, const float *src, double *dst,
                          cudaStream_t s)
  {
    if (Rc == 0)
      return;
    launch_pdl(f2d_scatter_kernel, nblocks(n * Rc), 256, 0, s, n, Rc, cols, src, dst);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_axpby_sel(int64_t n, int R, const int *sel, double a, const double *x, double b,
                        double *y, cudaStream_t s)
  {
    axpby_sel_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, sel, a, x, b, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_axpby(int64_t n, double a, const double *x, double b, double *y, cudaStream_t s)
  {
    if (n == 0)
      return;
    axpby_kernel<<<nblocks(n), 256, 0, s>>>(n, a, x, b, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_convert_d2f(int64_t n, const double *a, float *b, cudaStream_t s)
  {
    if (n == 0)
      return;
    launch_pdl(d2f_kernel, nblocks(n), 256, 0, s, n, a, b);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
  void launch_convert_f2d(int64_t n, const float *a, double *b, cudaStream_t s)
  {
    if (n == 0)
      return;
    launch_pdl(f2d_kernel, nblocks(n), 256, 0, s, n, a, b);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_build_system_matrix(int64_t n_vals, int n_leaves, const int64_t *val_ptr,
                                  const int64_t *col_ptr, const int64_t *row_ptr,
                                  const int32_t *rows, const int32_t *cols, const uint8_t *dir,
                                  const double *alpha, const double *Nval, const double *Dval,
                                  double *S, float *S32, cudaStream_t s)
  {
    if (n_vals == 0)
      return;
    system_matrix_kernel<<<nblocks(n_vals), 256, 0, s>>>(n_vals, n_leaves, val_ptr, col_ptr,
                                                         row_ptr, rows, cols, dir, alpha, Nval,
                                                         Dval, S, S32);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_rhs_combine(int64_t n, int R, const double *tmp, const uint8_t *dir,
                          const double *alpha, const double *oN, const double *oD, double *rhs,
                          cudaStream_t s)
  {
    rhs_combine_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, tmp, dir, alpha, oN, oD, rhs);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_split_masks(int64_t n, int R, const double *tmp, const uint8_t *dir, double *a,
                          double *b, cudaStream_t s)
  {
    split_masks_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, tmp, dir, a, b);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_scatter(int64_t n, int R, const double *sol, const uint8_t *dir, double *phi,
                      double *dphi, cudaStream_t s)
  {
    scatter_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, sol, dir, phi, dphi);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_constrain_rows(int n_con, int R, int64_t n, const int32_t *rows, const int32_t *cols,
                             const double *x, double *y, cudaStream_t s)
  {
    if (n_con == 0 || R == 0)
      return;
    launch_pdl(constrain_rows_kernel, nblocks(int64_t(n_con) * R), 256, 0, s, n_con, R, n, rows, cols, x, y);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_constraint_rhs(int n_con, int R, int64_t n, const int32_t *rows, const uint8_t *kind,
                             const int32_t *p, const int32_t *q, const double *tmp,
                             const double *nrm, const double *sg, double *b, cudaStream_t s)
  {
    if (n_con == 0 || R == 0)
      return;
    constraint_rhs_kernel<<<nblocks(int64_t(n_con) * R), 256, 0, s>>>(n_con, R, n, rows, kind, p, q,
                                                                      tmp, nrm, sg, b);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_sub_norm(int64_t n, int R, const double *nrm2, double *x, cudaStream_t s)
  {
    sub_norm_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, nrm2, x);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_add_scalar(int64_t n, int R, const double *shift, double *x, cudaStream_t s)
  {
    add_scalar_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, shift, x);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  template <typename P>
  void launch_block_apply(int n_leaves, int max_rows, int R, int64_t n, const int64_t *row_ptr,
                          const int64_t *blk_ptr, const int32_t *rows, const P *Pinv,
                          const double *v, int64_t ldv, double *z, cudaStream_t s,
                          const double *nrm2, double *vout, int64_t ldo, const int *jvec,
                          const int *sel)
  {
    if (n_leaves == 0)
      return;
    const int    mr   = std::max(max_rows, 1);
    const size_t smem = size_t(8) * mr * sizeof(P);
    if (smem > 48 * 1024)
      raise_smem_limit(reinterpret_cast<const void *>(block_apply_kernel<P>), smem);
    launch_pdl(block_apply_kernel<P>, (n_leaves + 7) / 8, 256, smem, s, n_leaves, mr, R, n, ldv, row_ptr,
                                                                blk_ptr, rows, Pinv, v, z, nrm2,
                                                                vout, ldo, jvec, sel);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
  template void launch_block_apply<float>(int, int, int, int64_t, const int64_t *, const int64_t *,
                                          const int32_t *, const float *, const double *, int64_t,
                                          double *, cudaStream_t, const double *, double *, int64_t,
                                          const int *, const int *);
  template void launch_block_apply<double>(int, int, int, int64_t, const int64_t *, const int64_t *,
                                           const int32_t *, const double *, const double *, int64_t,
                                           double *, cudaStream_t, const double *, double *, int64_t,
                                           const int *, const int *);

  void launch_ilu_fill(int64_t n, const int64_t *ptr, const int32_t *pos, const int32_t *row_leaf,
                       const int64_t *nrow_ptr, const int64_t *ncol_ptr, const int64_t *nval_ptr,
                       const int32_t *ncols, const double *S, const int32_t *con, int32_t *col,
                       double *val, cudaStream_t s)
  {
    if (n == 0)
      return;
    ilu_fill_kernel<<<nblocks(n * 32), 256, 0, s>>>(n, ptr, pos, row_leaf, nrow_ptr, ncol_ptr, nval_ptr,
                                                    ncols, S, con, col, val);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_ilu_factor(const std::vector<int64_t> &lptr, const int32_t *rows, const int64_t *ptr,
                         const int32_t *col, double *val, const int64_t *diag, int64_t max_row,
                         cudaStream_t s)
  {
    const size_t smem = size_t(max_row) * (sizeof(double) + sizeof(int32_t));
    if (smem > 48 * 1024)
      PIBEM_CUDA(cudaFuncSetAttribute(ilu_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(smem)));
    for (size_t l = 0; l + 1 < lptr.size(); ++l)
      {
        const int64_t nr = lptr[l + 1] - lptr[l];
        if (nr == 0)
          continue;
        ilu_factor_kernel<<<unsigned(nr), 256, smem, s>>>(rows + lptr[l], ptr, col, val, diag);
        note_launch();
      }
    PIBEM_CUDA(cudaGetLastError());
  }

  void launch_copy_sel(int64_t n, int R, const double *v, int64_t ldv, double *z, const int *sel,
                       cudaStream_t s)
  {
    if (n * R == 0)
      return;
    copy_sel_kernel<<<nblocks(n * R), 256, 0, s>>>(n, R, v, ldv, z, sel);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }

  void launch_ilu_apply(const std::vector<int64_t> &lptr_lo, const int32_t *rows_lo,
                        const std::vector<int64_t> &lptr_up, const int32_t *rows_up, int R, int64_t n,
                        const int64_t *ptr, const int32_t *col, const double *val,
                        const int64_t *diag, double *z, const int *sel, const int *jvec,
                        cudaStream_t s)
  {
    for (size_t l = 0; l + 1 < lptr_lo.size(); ++l)
      {
        const int nr = int(lptr_lo[l + 1] - lptr_lo[l]);
        if (nr == 0)
          continue;
        ilu_solve_kernel<true><<<nblocks(int64_t(nr) * R * 32), 256, 0, s>>>(
          nr, rows_lo + lptr_lo[l], R, n, ptr, col, val, diag, z, sel, jvec);
        note_launch();
      }
    for (size_t l = 0; l + 1 < lptr_up.size(); ++l)
      {
        const int nr = int(lptr_up[l + 1] - lptr_up[l]);
        if (nr == 0)
          continue;
        ilu_solve_kernel<false><<<nblocks(int64_t(nr) * R * 32), 256, 0, s>>>(
          nr, rows_up + lptr_up[l], R, n, ptr, col, val, diag, z, sel, jvec);
        note_launch();
      }
    PIBEM_CUDA(cudaGetLastError());
  }

  template <typename T>
  void launch_combine_p2m(int64_t n_rows, int K4, const int32_t *prow_dof, const uint8_t *dir,
                          const T *T1, const T *T2, T *Tc, cudaStream_t s)
  {
    const int64_t n = n_rows * K4;
    if (n == 0)
      return;
    combine_p2m_kernel<T><<<nblocks(n), 256, 0, s>>>(n, K4, prow_dof, dir, T1, T2, Tc);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
  }
  template void launch_combine_p2m<float>(int64_t, int, const int32_t *, const uint8_t *,
                                          const float *, const float *, float *, cudaStream_t);
  template void launch_combine_p2m<double>(int64_t, int, const int32_t *, const uint8_t *,
                                           const double *, const double *, double *, cudaStream_t);
} // namespace pibem
