// Launchers of the vector kernels (krylov.cu).
#pragma once

#include <vector>

#include "kernels.h"

namespace pibem
{
  void launch_dots(int64_t n, int R, int ncols, int64_t ldv, int64_t ldr, const double *V,
                   const double *w, double *partial, int nblk, double *out, cudaStream_t s);
  // w -= sign * V h (ncols basis vectors; jvec non-null: column r takes
  // jvec[r]; sel non-null: the selected columns only)
  void launch_gemv_sub(int64_t n, int R, int ncols, int64_t ldv, int64_t ldr, const double *V,
                       const double *h, int ldh, double *w, double sign, cudaStream_t s,
                       const int *jvec = nullptr, const int *sel = nullptr);
  // one Arnoldi Gram-Schmidt pass in one launch (mode 0: dots; 1: subtract then
  // dots; 2: subtract then the squared norm); ticket: R ints, zero between
  // calls; out: ldo values per column (ldo <= 0: the pass's output count);
  // jvec non-null: column r takes ncols = jvec[r] + 1 (read on the device;
  // jvec[r] < 0: the column is skipped)
  void launch_cgs_step(int mode, int64_t n, int R, int ncols, int64_t ldv, int64_t ldr,
                       const double *V, const double *hin, int ldh, double *w, int nblk,
                       double *partial, int *ticket, double *out, cudaStream_t s,
                       const int *jvec = nullptr, int ldo = 0);
  // out[r] = w[r] / sqrt(nrm2[r]) (column stride ldr; jvec non-null: at basis
  // vector jvec[r] + 1 of out, columns with jvec[r] < 0 skipped; sel non-null:
  // selected columns only), also into z (stride n) when z is non-null
  void launch_normalize(int64_t n, int R, const double *w, const double *nrm2, double *out,
                        int64_t ldr, cudaStream_t s, const int *jvec = nullptr,
                        double *z = nullptr, const int *sel = nullptr);
  // device-driven GMRES cycles, one state per column (layout in krylov.cu)
  void launch_gmres_cycle_init(int R, int m, const int *sel, const double *nrm2, double *g, int *kdone,
                               int *jvec, cudaStream_t s);
  void launch_gmres_givens(int R, int m, const double *hb, double *H, double *cs, double *sn,
                           double *g, int *kdone, int *jvec, int *its, const int *maxit,
                           const double *bn, const double *tol, int *ctl,
                           cudaGraphConditionalHandle cond, bool use_cond, cudaStream_t s);
  void launch_gmres_lsq(int R, int m, const int *sel, const double *H, const double *g,
                        const int *kdone, const int *jvec, double *y, cudaStream_t s);
  // compaction of selected columns for the operator: dst[k] = src[cols[k]] and back
  void launch_gather_cols(int64_t n, int Rc, const int *cols, const double *src, int64_t lds,
                          double *dst, cudaStream_t s);
  // x32[k] = float(src[cols[k]]) / dst[cols[k]] = double(y32[k]) (column stride n)
  void launch_gather_d2f(int64_t n, int Rc, const int *cols, const double *src, float *dst,
                         cudaStream_t s);
  void launch_f2d_scatter(int64_t n, int Rc, const int *cols, const float *src, double *dst,
                          cudaStream_t s);
  void launch_scatter_cols(int64_t n, int Rc, const int *cols, const double *src, double *dst,
                           int64_t ldd, cudaStream_t s);
  // y[r] = a x[r] + b y[r] on the selected columns
  void launch_axpby_sel(int64_t n, int R, const int *sel, double a, const double *x, double b,
                        double *y, cudaStream_t s);
  // x[r] -= sqrt(nrm2[r])
  void launch_sub_norm(int64_t n, int R, const double *nrm2, double *x, cudaStream_t s);
  // ILU(0) of the near-field system matrix: the CSR rows (node order) from the
  // leaf blocks (con[i] != -2: a constraint line with column con[i]); the
  // factorisation level by level (lptr over rows, max_row the longest row);
  // and z = (L U)^-1 z in place on the columns r < R with sel[r] (if sel) and
  // jvec[r] >= 0 (if jvec)
  void launch_ilu_fill(int64_t n, const int64_t *ptr, const int32_t *pos, const int32_t *row_leaf,
                       const int64_t *nrow_ptr, const int64_t *ncol_ptr, const int64_t *nval_ptr,
                       const int32_t *ncols, const double *S, const int32_t *con, int32_t *col,
                       double *val, cudaStream_t s);
  void launch_ilu_factor(const std::vector<int64_t> &lptr, const int32_t *rows, const int64_t *ptr,
                         const int32_t *col, double *val, const int64_t *diag, int64_t max_row,
                         cudaStream_t s);
  void launch_ilu_apply(const std::vector<int64_t> &lptr_lo, const int32_t *rows_lo,
                        const std::vector<int64_t> &lptr_up, const int32_t *rows_up, int R, int64_t n,
                        const int64_t *ptr, const int32_t *col, const double *val,
                        const int64_t *diag, double *z, const int *sel, const int *jvec,
                        cudaStream_t s);
  // z[r] = v[r] (column strides ldv, n) for the columns r with sel[r] (all if !sel)
  void launch_copy_sel(int64_t n, int R, const double *v, int64_t ldv, double *z, const int *sel,
                       cudaStream_t s);
  void launch_axpby(int64_t n, double a, const double *x, double b, double *y, cudaStream_t s);
  void launch_rhs_combine(int64_t n, int R, const double *tmp, const uint8_t *dir,
                          const double *alpha, const double *oN, const double *oD, double *rhs,
                          cudaStream_t s);
  void launch_split_masks(int64_t n, int R, const double *tmp, const uint8_t *dir, double *a,
                          double *b, cudaStream_t s);
  void launch_scatter(int64_t n, int R, const double *sol, const uint8_t *dir, double *phi,
                      double *dphi, cudaStream_t s);
  void launch_add_scalar(int64_t n, int R, const double *shift, double *x, cudaStream_t s);
  // double-node constraint lines: operator rows and right-hand side
  void launch_constrain_rows(int n_con, int R, int64_t n, const int32_t *rows, const int32_t *cols,
                             const double *x, double *y, cudaStream_t s);
  void launch_constraint_rhs(int n_con, int R, int64_t n, const int32_t *rows, const uint8_t *kind,
                             const int32_t *p, const int32_t *q, const double *tmp,
                             const double *nrm, const double *sg, double *b, cudaStream_t s);
  // z = P^-1 v (leaf-block Jacobi); with nrm2: v is first normalised, column
  // r by sqrt(nrm2[r]), and written to vout (column stride ldo; jvec non-null:
  // at basis vector jvec[r] + 1 of vout, vectors n apart, columns with
  // jvec[r] < 0 skipped); sel non-null: the selected columns only
  template <typename P>
  void launch_block_apply(int n_leaves, int max_rows, int R, int64_t n, const int64_t *row_ptr,
                          const int64_t *blk_ptr, const int32_t *rows, const P *Pinv,
                          const double *v, int64_t ldv, double *z, cudaStream_t s,
                          const double *nrm2 = nullptr, double *vout = nullptr, int64_t ldo = 0,
                          const int *jvec = nullptr, const int *sel = nullptr);
} // namespace pibem
