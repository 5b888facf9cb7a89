// Launch interfaces of the device kernels (setup.cu, fmm.cu, krylov.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "pibem_internal.h"

namespace pibem
{
  // ---- setup (FP64) -------------------------------------------------------
  struct NearAssemblyArgs
  {
    int64_t          n_items = 0; // sum over leaves of rows * entries
    int              n_leaves = 0;
    const int64_t   *item_ptr = nullptr, *row_ptr = nullptr, *ent_ptr = nullptr,
                    *val_ptr = nullptr, *col_ptr = nullptr;
    const int64_t   *h_item_ptr = nullptr, *h_ent_ptr = nullptr, *h_val_ptr = nullptr;
    const int32_t   *rows = nullptr;
    const NearEntry *ents = nullptr;
    const double    *xyz = nullptr;
    const int32_t   *cells = nullptr, *dbl_off = nullptr, *dbl_ids = nullptr;
    int              nq = 0;
    const double    *qpts = nullptr, *qnrm = nullptr, *qjxw = nullptr, *qshape = nullptr;
    const int32_t   *gather_ptr = nullptr, *gather_ids = nullptr;
    double          *staging = nullptr;
    int64_t          staging_items = 0;
    int64_t         *sing_list = nullptr;     // staging_items entries: singular items of a batch
    unsigned long long *sing_count = nullptr; // their number
    double          *Nval = nullptr, *Dval = nullptr;
  };

  void set_telles_rules(const std::vector<double> pts[4], const std::vector<double> w[4], int n,
                        cudaStream_t s);
  void launch_quad_data(int64_t n_cells, int nq, const double *xyz, const int32_t *cells,
                        const double *gpts, const double *gw, double *qpts, double *qnrm,
                        double *qjxw, double *qshape, cudaStream_t s);
  void launch_near_assembly(const NearAssemblyArgs &a, cudaStream_t s);
  void launch_p2m_tables(int64_t n_rows, int K, int p, int n_leaves, const int64_t *row_ptr,
                         const int32_t *leaf_box, const int64_t *contrib_ptr,
                         const int32_t *contrib_q, const double *box_center,
                         const double *box_delta, const double *qpts, const double *qnrm,
                         const double *qjxw, const double *qshape, double *T1, double *T2,
                         cudaStream_t s);
  void launch_l2p_tables(int64_t n_pos, int K, int ldw, int n_leaves, const int64_t *pos_ptr,
                         const int32_t *leaf_box, const int32_t *nodes, const double *xyz,
                         const double *box_center, const double *box_delta, double *W,
                         cudaStream_t s);

  // ---- operator (T = double or float) -------------------------------------
  // Column modes of the multipole pass.
  enum : uint8_t
  {
    MODE_COMBINED = 0, // strengths (1-dir) Ker1 - dir Ker2 (system operator)
    MODE_KER1     = 1, // double layer only (N)
    MODE_KER2     = 2, // single layer only (D)
    MODE_SWAPPED  = 3  // strengths dir Ker1 - (1-dir) Ker2 (right-hand side: N phi_D - D dphi_N)
  };

  struct TreeDev
  {
    int            nb = 0, N = 0, L = 0;
    const int32_t *parent = nullptr, *child_first = nullptr, *nchild = nullptr,
                  *digit = nullptr, *nbeg = nullptr, *nend = nullptr, *node_sorted = nullptr;
    const double  *center = nullptr, *delta = nullptr;
    const double  *xyz = nullptr;
  };

  // resident blocks per SM of the one-column near SpMVs (their launch bounds)
  constexpr int NEAR_BLOCKS_PER_SM_F32  = 6;
  constexpr int NEAR_BLOCKS_PER_SM_WIDE = 5;

  template <typename T>
  struct OperatorDev
  {
    int p = 0, K = 0;
    // near field (leaf blocks)
    int            n_near_leaves = 0;
    int64_t        n_rows = 0;
    const int32_t *row_leaf = nullptr, *nrows = nullptr, *ncols = nullptr;
    const int64_t *nrow_ptr = nullptr, *ncol_ptr = nullptr, *nval_ptr = nullptr;
    // the leaves sorted by value bytes, 4 int64 per leaf: value offset, column
    // offset, row offset, rows | columns << 32 (one-column near SpMV)
    const int64_t *near_sched = nullptr;
    // p2m
    int            n_p2m_leaves = 0;
    const int64_t *prow_ptr = nullptr;
    const int32_t *pleaf_box = nullptr, *prow_dof = nullptr;
    const T       *T1 = nullptr, *T2 = nullptr;
    const float2  *Wff = nullptr; // L2P rows as (hi, lo) pairs (FP64-accurate operator)
    const T       *Tc = nullptr; // combined-strength table (set_bc): dir ? -T2 : T1
    // l2p (same row positions as the near field)
    const int32_t *lleaf_box = nullptr;
    const T       *W = nullptr;
    // batched translations: operator table [M2L offsets | 8 M2M | 8 L2L],
    // each K x K stored [in][out]; pair / chunk arrays of the plan
    const T       *ops = nullptr;
    // FP64 operator only: the table as (hi, lo) FP32 pairs; non-null selects
    // the float-float translation GEMM
    const float2  *ops_ff = nullptr;
    const int32_t *q_src = nullptr, *ch_start = nullptr, *ch_cnt = nullptr, *ch_op = nullptr;
    int            max_chunk_pairs = 0;
    int            n_boxes         = 0;
    int            m2l_chunk_end = 0;
    std::vector<int> up_chunk_ptr, down_chunk_ptr, up_box_ptr, down_box_ptr;
    const int32_t *up_box = nullptr, *down_box = nullptr, *up_q = nullptr, *down_q = nullptr;
    const int64_t *up_q_ptr = nullptr, *down_q_ptr = nullptr;
    // fused level passes (levels.cu): children of each up_box entry by octant,
    // L2L parent (-1: none) and octant of each down_box entry; the M2M
    // operators are ops[lv_op0 .. lv_op0 + 7], the L2L ones the next 8
    const int32_t *up_child8 = nullptr, *down_par = nullptr;
    const uint8_t *down_oct  = nullptr;
    int            lv_op0    = 0;
    const T       *lv_ops    = nullptr; // the 16 level operators, each padded to 16 bytes
    int           *dev_err   = nullptr; // set by a bounded device wait that timed out
    std::vector<char> down_l2l_level; // per level: its boxes receive L2L
    // target-major M2L products (fused passes): slot of each M2L pair, and the
    // slot range of each down_box entry
    const int32_t *m2l_yslot = nullptr, *down_m2l_beg = nullptr, *down_m2l_end = nullptr;
    int64_t        n_pairs = 0;
    int64_t        max_near_cols = 0;
    // tensor-core path of the FP32 translations (null: CUDA-core GEMM)
    const float   *tc_images = nullptr;
    int            tc_stages = 0; // pipeline stages of the tensor-core kernel (0: by fit)
    // FP64-accurate operator only: BF16 digit images of the operators and
    // their row exponents for the tensor-core FP64-accurate GEMM (ozaki_tc.cu)
    const uint16_t *oz_images = nullptr;
    const int16_t  *oz_ecol   = nullptr;
    int           *tc_err    = nullptr;
    // M2P per target CSR, evaluated per (pair, target node) item
    int            n_m2p_tgt = 0;
    int64_t        n_m2p_pairs = 0, n_m2p_items = 0, n_m2p_tnodes = 0;
    const int32_t *m2p_tgt = nullptr, *m2p_src = nullptr, *m2p_pair_tgt = nullptr;
    const int64_t *m2p_src_ptr = nullptr, *m2p_item_ptr = nullptr, *m2p_tnode_ptr = nullptr;
    const int32_t *m2p_item_pair = nullptr; // pair of each item
    const int32_t *m2p_tnodes = nullptr;    // collocation nodes of each target (m2p_tnode_ptr)
    T             *m2p_scratch = nullptr; // n_m2p_items * R
  };

  template <typename T>
  void launch_near_spmv(const OperatorDev<T> &op, int R, int N, const T *vals, const T *x, T *y,
                        bool accumulate, cudaStream_t s);
  template <typename T>
  void launch_p2m_apply(const OperatorDev<T> &op, int R, int N, const uint8_t *dir,
                        const uint8_t *modes, const T *x, T *M, bool combined, cudaStream_t s);
  // upward level l: M2M of the level-l children, gathered into the parents
  template <typename T>
  void launch_upward_level(const OperatorDev<T> &op, int R, int level, T *M, T *Y, cudaStream_t s);
  // M2L products of all levels into Y
  template <typename T>
  void launch_m2l_gemm(const OperatorDev<T> &op, int R, const T *M, T *Y, cudaStream_t s);
  // downward level l: L2L products, then L[b] = L2L + sum of M2L products
  // (fused passes: L[b] += L2L, the M2L sums being in place already)
  template <typename T>
  void launch_downward_level(const OperatorDev<T> &op, int R, int level, T *Lx, T *Y,
                             cudaStream_t s);
  template <typename T>
  void launch_m2p(const OperatorDev<T> &op, const TreeDev &td, int R, int N, const T *M, T *y,
                  cudaStream_t s);
  // FP64-accurate translation GEMM on the tensor cores (ozaki_tc.cu): digits of
  // the operators (host, once) and of the expansions (device, per product),
  // then Y = T E as (hi, lo) pairs; for K <= 96 (p <= 8)
  bool ozaki_ok(int K);
  void build_ozaki_images(const std::vector<double> &ops_out_in, int nops, int K,
                          std::vector<uint16_t> &img, std::vector<int16_t> &e_col);
  void launch_ozaki_slices(int64_t nrows, int K, const float2 *E, uint16_t *slices, int *e_row,
                           cudaStream_t s);
  void launch_ozaki_gemm(const OperatorDev<double> &op, int R, int c0, int c1,
                         const uint16_t *aslc, const int *e_row, int64_t a_rows, float2 *Y,
                         cudaStream_t s);
  // FP64-accurate tree passes on (hi, lo) float-float expansions (fmm.cu):
  // the translation GEMM, per-level passes with float-float sums, conversions
  template <typename IO>
  void launch_ff_gemm(const OperatorDev<double> &op, int R, int c0, int c1, const IO *E, IO *Y,
                      cudaStream_t s);
  void launch_upward_level_ff(const OperatorDev<double> &op, int R, int level, float2 *M, float2 *Y,
                              cudaStream_t s);
  void launch_m2l_ff(const OperatorDev<double> &op, int R, const float2 *M, float2 *Y,
                     cudaStream_t s);
  void launch_downward_level_ff(const OperatorDev<double> &op, int R, int level, float2 *Lx,
                                float2 *Y, cudaStream_t s);
  void launch_convert_d2ff(int64_t n, const double *a, float2 *b, cudaStream_t s);
  // FP64-accurate L2P from (hi, lo) locals (float-float), op.Wff rows
  void launch_l2p_ff(const OperatorDev<double> &op, int R, int N, const float2 *Lff, double *y,
                     cudaStream_t s);
  // FP64-accurate M2P from (hi, lo) multipoles (float-float evaluation)
  void launch_m2p_ff(const OperatorDev<double> &op, const TreeDev &td, int R, int N, const float2 *Mff,
                     double *y, cudaStream_t s);
  // whether the leaf blocks' x pairs (two buffers) fit in shared memory
  bool near_ff_fits(const OperatorDev<double> &op);
  // FP64-accurate near SpMV on (hi, lo) FP32 pairs, one launch per column:
  // y[r] (=|+=) vals x[r], x given as pairs, y in FP64
  void launch_near_spmv_ff(const OperatorDev<double> &op, int R, int N, const float2 *vals,
                           const float2 *xff, double *y, bool accumulate, cudaStream_t s);
  void launch_convert_ff2d(int64_t n, const float2 *a, double *b, cudaStream_t s);
  // M2L sums of all levels into Lx (the first step of the downward pass, before
  // the levels); does nothing unless the fused level passes apply
  template <typename T>
  void launch_m2l_sums(const OperatorDev<T> &op, int R, T *Lx, const T *Y, cudaStream_t s);
  // fused level passes of the FP32 operator (levels.cu), for every column
  // count (so that a column's result never depends on the batch it is in):
  // M2L sums of all levels in one launch, then one launch per level, no gathers
  bool          fused_levels_ok(int K, int R);
  size_t        fused_level_ops_floats(int K); // size of OperatorDev::lv_ops
  void launch_m2m_level_fused(const OperatorDev<float> &op, int R, int level, float *M,
                              cudaStream_t s);
  void launch_m2l_sums_fused(const OperatorDev<float> &op, int R, float *Lx, const float *Y,
                             cudaStream_t s);
  void launch_l2l_level_fused(const OperatorDev<float> &op, int R, int level, float *Lx,
                              cudaStream_t s);
  void ensure_fmm_tables(int device, cudaStream_t s);
  template <typename T>
  void launch_l2p(const OperatorDev<T> &op, int R, int N, const T *Lx, T *y, cudaStream_t s);

  // ---- tensor-core translations (m2l_tc.cu) ----------------------------------
  struct TcGeometry
  {
    int    K = 0, Kp = 0, Np = 0, stages = 3;
    size_t smem = 0;
    bool   ok   = false;
  };
  TcGeometry tc_geometry(int K);
  // hi/lo TF32 images of row-major [out][in] operators in the MMA B layout
  void build_tc_images(const std::vector<double> &ops_out_in, int nops, int K,
                       std::vector<float> &img);
  // Y row of (pair q, rhs r): (yslot ? yslot[q] : q) * R + r, rows of ldy
  // values (ldy a multiple of 4 when yslot is given)
  void launch_tc_gemm(const OperatorDev<float> &op, int R, int c0, int c1, const float *E, float *Y,
                      const int32_t *yslot, int ldy, int *err, cudaStream_t s);

  // ---- L2 projections onto the Q1 space (projection.cu) ------------------------
  struct ProjectionArgs
  {
    int            mode = 0; // 0 normals, 1 surface gradient of u, 2 gradient (u = phi, dudn)
    int64_t        n_nodes = 0, n_cells = 0;
    int            nq = 0, R = 1;
    const int32_t *cells = nullptr, *elem_off = nullptr, *elem_ids = nullptr;
    const double  *xyz = nullptr, *gpts = nullptr, *qshape = nullptr, *qjxw = nullptr,
                  *qnrm = nullptr, *u = nullptr, *dudn = nullptr;
    double        *work = nullptr; // l2_projection_work() doubles
    double        *out  = nullptr; // R x N x 3, node-major
    int            max_iterations = 1000;
    double         tolerance      = 1e-13;
    int           *iterations     = nullptr;
  };
  void   l2_projection(const ProjectionArgs &a, cudaStream_t s);
  size_t l2_projection_work(int64_t n_nodes, int64_t n_cells, int R);

  // ---- vector kernels (krylov.cu) -------------------------------------------
  void launch_convert_d2f(int64_t n, const double *a, float *b, cudaStream_t s);
  void launch_convert_f2d(int64_t n, const float *a, double *b, cudaStream_t s);
  // Tc[row] = dir[dof(row)] ? -T2[row] : T1[row] for the rows of the P2M tables
  template <typename T>
  void launch_combine_p2m(int64_t n_rows, int K4, const int32_t *prow_dof, const uint8_t *dir,
                          const T *T1, const T *T2, T *Tc, cudaStream_t s);
  void launch_build_system_matrix(int64_t n_vals, int n_leaves, const int64_t *val_ptr,
                                  const int64_t *col_ptr, const int64_t *row_ptr,
                                  const int32_t *rows, const int32_t *cols, const uint8_t *dir,
                                  const double *alpha, const double *Nval, const double *Dval,
                                  double *S, float *S32, cudaStream_t s);
} // namespace pibem
