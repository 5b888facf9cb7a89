// Handle and C ABI (include/pibem_gpu.h): mesh set-up, boundary conditions,
// FMM operator applications and the GMRES solve, all on one GPU.
//
//   pibem_set_mesh       BEMFMA::init_fma + generate_octree_blocking +
//                        direct_integrals + multipole_integrals (bem_fma.cc:42,3615,108,1609)
//   pibem_fmm_matvec     generate_multipole_expansions + multipole_matr_vect_products
//   pibem_compute_alpha  BEMProblem::compute_alpha   (bem_problem.cc:1139)
//   pibem_system_matvec  BEMProblem::vmult           (bem_problem.cc:1165)
//   pibem_compute_rhs    BEMProblem::compute_rhs     (bem_problem.cc:1220)
//   pibem_solve          BEMProblem::solve_system    (bem_problem.cc:1267)
#include <omp.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <functional>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "kernels.h"
#include "krylov.h"
#include "pdl.cuh"
#include "pibem_internal.h"

using namespace pibem;

static std::atomic<int64_t> g_launches{0};
static std::mutex          g_near_assembly_mu; // see set_mesh_impl

namespace pibem
{
  // launches made by this host thread (stream capture counts its own kernels)
  static thread_local int64_t t_launches = 0;
  void    note_launch(int64_t n)
  {
    g_launches.fetch_add(n, std::memory_order_relaxed);
    t_launches += n;
  }
  int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

  void raise_smem_limit(const void *fn, size_t bytes)
  {
    static std::mutex                                   mu;
    static std::map<std::pair<int, const void *>, size_t> set;
    int dev = 0;
    PIBEM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = set[{dev, fn}];
    if (bytes <= cur)
      return;
    PIBEM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
    cur = bytes;
  }
} // namespace pibem

namespace
{
  __global__ void diag_block_gather_kernel(int64_t n_rows, const int32_t *__restrict__ row_leaf,
                                           const int64_t *__restrict__ row_ptr,
                                           const int64_t *__restrict__ col_ptr,
                                           const int64_t *__restrict__ val_ptr,
                                           const int64_t *__restrict__ blk_ptr,
                                           const int32_t *__restrict__ diag_col,
                                           const double *__restrict__ S, double *__restrict__ B)
  {
    int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (row >= n_rows)
      return;
    int     leaf = row_leaf[row];
    int64_t r0 = row_ptr[leaf], nr = row_ptr[leaf + 1] - r0, r = row - r0;
    int64_t ld = (col_ptr[leaf + 1] - col_ptr[leaf] + 3) / 4 * 4;
    for (int64_t c = 0; c < nr; ++c)
      B[blk_ptr[leaf] + r * nr + c] = S[val_ptr[leaf] + r * ld + diag_col[r0 + c]];
  }

  // Gauss-Jordan inverse with partial pivoting (host, small dense blocks).
  bool invert(int n, double *a, double *inv)
  {
    std::vector<double> m(a, a + size_t(n) * n);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        inv[size_t(i) * n + j] = i == j ? 1.0 : 0.0;
    for (int c = 0; c < n; ++c)
      {
        int    piv = c;
        double best = std::fabs(m[size_t(c) * n + c]);
        for (int r = c + 1; r < n; ++r)
          if (std::fabs(m[size_t(r) * n + c]) > best)
            {
              best = std::fabs(m[size_t(r) * n + c]);
              piv  = r;
            }
        if (!(best > 0))
          return false;
        if (piv != c)
          for (int j = 0; j < n; ++j)
            {
              std::swap(m[size_t(c) * n + j], m[size_t(piv) * n + j]);
              std::swap(inv[size_t(c) * n + j], inv[size_t(piv) * n + j]);
            }
        double d = 1.0 / m[size_t(c) * n + c];
        for (int j = 0; j < n; ++j)
          {
            m[size_t(c) * n + j] *= d;
            inv[size_t(c) * n + j] *= d;
          }
        for (int r = 0; r < n; ++r)
          if (r != c)
            {
              double f = m[size_t(r) * n + c];
              if (f != 0)
                for (int j = 0; j < n; ++j)
                  {
                    m[size_t(r) * n + j] -= f * m[size_t(c) * n + j];
                    inv[size_t(r) * n + j] -= f * inv[size_t(c) * n + j];
                  }
            }
      }
    return true;
  }

  template <typename T>
  void transpose_ops(const std::vector<double> &src, int nops, int K, std::vector<T> &dst)
  {
    dst.resize(size_t(nops) * K * K);
    for (int o = 0; o < nops; ++o)
      for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j)
          dst[size_t(o) * K * K + size_t(j) * K + i] = T(src[size_t(o) * K * K + size_t(i) * K + j]);
  }
} // namespace

namespace pibem
{
  // stage of one column (right-hand side) in the solve engine (capi.cu)
  enum ColStage : uint8_t
  {
    ST_FREE,      // slot unused
    ST_RHS,       // needs its right-hand side b = rhs(tmp)
    ST_ASSESS,    // mixed: the refinement decision on |r|
    ST_TRUERES,   // mixed: needs r = b - A64 x
    ST_R32,       // mixed: needs r <- r - A32 d
    ST_INNER,     // mixed: a restart of the correction's GMRES (w = r - A32 d)
    ST_RES,       // plain: a restart of GMRES (w = b - A64 x)
    ST_ARNOLDI,   // in a GMRES cycle on the device
    ST_CYCLE_END, // its cycle ended: x (plain) or d (mixed) += P^-1 V y
    ST_XUPD,      // mixed: x += d after a correction
    ST_DONE       // solved; waiting to be collected
  };

  struct ColHost
  {
    ColStage st         = ST_FREE;
    int64_t  rid        = -1;
    bool     final_pass = false; // mixed: the exact residual after the refinement loop
    bool     r_exact    = true;  // mixed: r is b - A64 x (not the A32-updated estimate)
    bool     refine_inc = false; // mixed: the pending residual ends a refinement step
    bool     ok         = false;
    int      refine = 0, iters = 0, its_inner = 0, inner_maxit = 0;
    int      c32 = 0, c64 = 0; // operator applications of this column
    double   bn_outer = 1, bn_inner = 1, rel = 1, itol = 0;
    std::chrono::steady_clock::time_point t0;
    double   seconds = 0;
  };

  // One GMRES cycle graph (per active-column count and buffer set)
  struct CycleGraph
  {
    std::array<uintptr_t, 48> key{};
    cudaGraphExec_t           exec    = nullptr;
    int64_t                   kernels = 0;
    int                       c32 = 0, c64 = 0;
  };

  // Device state of the solve engine: S column slots, Krylov dimension m;
  // vectors slot-strided (column k at k N), Krylov bases (m + 1) N apart
  struct Engine
  {
    int                  S = 0, m = 0;
    bool                 mixed = false, prec = false;
    std::vector<ColHost> col;
    DBuf<double>         V, z, w, u, b, x, r, d, tmp, cz, cw, hb, partial, H, cs, sn, g, y, bn, tol, nrm;
    DBuf<int>            ticket, kdone, jvec, its, maxit, sel, act, ctl;
    PinnedBuf<int>       ipin;
    std::vector<double>  h_bn, h_tol;
    std::vector<int>     h_its, h_maxit, h_jvec, h_ctl;
  };
} // namespace pibem

struct pibem_handle
{
  pibem_params prm;
  std::string  err;
  cudaStream_t stream = nullptr, own = nullptr;
  // the two branches of the operator: the tree passes (the critical path) on a
  // stream of the highest priority, the near field and M2P on one of the lowest
  cudaStream_t main_hp = nullptr, side = nullptr;
  cudaEvent_t  ev_fork = nullptr, ev_up = nullptr, ev_side = nullptr, ev_main = nullptr;
  bool         mesh_ok = false, bc_ok = false;
  MeshHost     mesh;
  int          nq = 0, n_tel = 0;
  std::vector<double> gpts, gw, tpts[4], tw[4];
  Tree         tree;
  Plan         plan;
  double       setup_seconds = 0;
  bool         tree_on_host  = false; // the octree came from the host builder (capacity)
  // wall time of the set-up phases of the last pibem_set_mesh (pibem_setup_phases)
  double       setup_phase[PIBEM_SETUP_PHASES] = {};
  size_t       bytes_resident = 0;
  // mesh
  DBuf<double>  d_xyz, d_qpts, d_qnrm, d_qjxw, d_qshape, d_gpts, d_gw;
  DBuf<int32_t> d_cells, d_dbl_off, d_dbl_ids, d_elem_off, d_elem_ids;
  DBuf<double>  d_proj; // L2-projection work (grow-only)
  // tree
  DBuf<int32_t> d_parent, d_child_first, d_nchild, d_digit, d_nbeg, d_nend, d_node_sorted;
  DBuf<double>  d_center, d_delta;
  // plan
  DBuf<int64_t> d_nrow_ptr, d_ncol_ptr, d_nval_ptr, d_nent_ptr, d_prow_ptr, d_pcontrib_ptr,
    d_m2l_src_ptr, d_m2p_src_ptr, d_item_ptr, d_blk_ptr, d_m2p_item_ptr, d_m2p_tnode_ptr,
    d_up_q_ptr, d_down_q_ptr, d_near_sched;
  DBuf<int32_t> d_row_leaf, d_nrows, d_ncols, d_pleaf_box, d_prow_dof, d_pcontrib_q, d_lleaf_box,
    d_gather_ptr, d_gather_ids, d_m2l_tgt, d_m2l_src, d_m2l_off, d_m2p_tgt, d_m2p_src, d_l2l_box,
    d_parents, d_diag_col, d_m2p_pair_tgt, d_q_src, d_ch_start, d_ch_cnt, d_ch_op, d_up_box,
    d_down_box, d_up_q, d_down_q, d_up_child8, d_down_par, d_m2p_item_pair, d_m2l_yslot,
    d_down_m2l_beg, d_down_m2l_end, d_m2p_tnodes;
  DBuf<uint8_t> d_down_oct;
  DBuf<NearEntry> d_entries;
  DBuf<double>  d_N, d_D, d_S, d_T1, d_T2, d_W, d_ops, d_Tc;
  // leaf-block Jacobi inverses, column-major: FP32 for the mixed path, FP64
  // for the plain FP64 path
  DBuf<float>   d_Pinv;
  DBuf<double>  d_Pinv64;
  DBuf<float>   d_S32, d_T1f, d_T2f, d_Wf, d_opsf, d_tcimg, d_Tcf, d_lvopsf;
  DBuf<float2>  d_opsff; // the FP64 operator table as (hi, lo) FP32 pairs
  // FP64-accurate near field as (hi, lo) FP32 pairs (modes other than FP64):
  // the system matrix S and the right-hand side's matrix (S of the
  // complementary mask), and the pair copy of x
  DBuf<float2>  d_Sff, d_Srff, d_xff;
  DBuf<float2>  d_Wff;  // L2P rows as pairs (modes other than FP64)
  DBuf<double>  d_Tcr;  // P2M strengths of the right-hand side: dir ? T1 : -T2
  DBuf<int>     d_err;
  // ILU(0) of the near-field system matrix (preconditioner 2): CSR in node
  // order (values: L below the diagonal, unit diagonal implied; U from it),
  // the position of each row's diagonal, and the rows by level of the lower
  // and of the upper triangle (the rows of a level depend on earlier levels
  // only); level bounds on the host
  DBuf<int64_t> d_ilu_ptr, d_ilu_diag;
  DBuf<int32_t> d_ilu_col, d_ilu_rows_lo, d_ilu_rows_up;
  DBuf<double>  d_ilu_val;
  std::vector<int64_t> ilu_lptr_lo, ilu_lptr_up;
  bool          ilu_on = false;
  bool          use_tc = true;
  std::vector<int64_t> blk_ptr;
  int                  max_leaf_rows = 0;
  OperatorDev<double> op64;
  OperatorDev<float>  op32;
  TreeDev             td;
  // boundary conditions
  std::vector<uint8_t> dir;
  DBuf<uint8_t>        d_dir, d_modes, d_modes32;
  int                  modes32_R = 0; // d_modes32 holds MODE_COMBINED for this many columns
  DBuf<double>         d_alpha;
  bool                 have_dirichlet = true;
  // double-node constraint lines of the solve (made by set_bc): row, entry
  // column (-1: none), kind (0: x_row = x_col; 1: x_row = tmp_rhs[p]; 2: the
  // Dirichlet-Dirichlet normal derivative of the pair (p, q))
  std::vector<int32_t> con_row, con_col, con_p, con_q;
  std::vector<uint8_t> con_kind;
  bool                 con_proj = false; // some line needs normals and surface gradients
  DBuf<int32_t>        d_con_row, d_con_col, d_con_p, d_con_q;
  DBuf<uint8_t>        d_con_kind;
  DBuf<double>         d_con_nrm, d_con_sg; // nodal normals (kept per mesh), surface gradients
  // work
  DBuf<double> d_M64, d_L64, d_x64, d_y64, d_t1, d_t2, d_t3, d_t4, d_m2p64, d_Y64;
  DBuf<float>  d_M32, d_L32, d_x32, d_y32, d_m2p32, d_Y32;
  DBuf<float2> d_Mff, d_Lff; // (hi, lo) expansions of the float-float tree passes
  // tensor-core FP64-accurate M2L: operator digit images and row exponents,
  // expansion digits and row exponents (work)
  DBuf<uint16_t> d_ozimg, d_ozslc;
  DBuf<int16_t>  d_ozecol;
  DBuf<int>      d_ozerow;
  PinnedBuf<double> g_small; // small reads the host waits for (norms)
  DBuf<double> sh_part, sh_nrm; // pure-Neumann shift of the operator input / output
  // solve temporaries and host-pointer staging (grow-only: no cudaMalloc / cudaFree,
  // and so no device-wide synchronisation, once a handle has solved its largest batch)
  DBuf<double> sv_b, sv_x, sv_r, sv_d, sv_w, sv_part, sv_nrm;
  DBuf<double> io_buf[4];
  // the FP32 operator (near SpMV + far field on d_x32 -> d_y32) as one CUDA
  // graph, captured for the buffers and column count in g32_key
  cudaGraphExec_t g32_exec = nullptr;
  uintptr_t       g32_key[8] = {};
  int64_t         g32_kernels = 0;
  // the solve engine and its GMRES cycle graphs (a conditional while node
  // around one Arnoldi step of the active columns)
  Engine                  eng;
  std::vector<CycleGraph> cycle_graphs;
  bool                    slots_open = false; // pibem_slots_open
  // d_modes holds this mode for modes_R columns (-1: other contents)
  int             modes_R = -1;
  uint8_t         modes_val = 0;
  // timing (timing_hold_ns: the stream is held this long before the first
  // phase event of each application, pibem_set_profiling(h, 2))
  bool        timing = false;
  int64_t     timing_hold_ns = 0;
  cudaEvent_t ev[8] = {};
  double      phase_ms[7] = {0, 0, 0, 0, 0, 0, 0};
  double      phase_tot[2][7] = {};
  int64_t     phase_cnt[2] = {0, 0};
  int         cnt64 = 0, cnt32 = 0;
  int64_t     m2p_items = 0, m2p_tnodes = 0;

  // unknowns per column: the collocation nodes (the mesh's own nodes; a
  // double body's reflected nodes carry no unknowns)
  int64_t N() const { return mesh.n_dofs; }

  // Device memory held by the handle (every buffer above, at its capacity).
  size_t device_bytes() const
  {
    size_t t = 0;
    auto   add = [&t](const auto &...b) { ((t += b.bytes()), ...); };
    add(d_xyz, d_qpts, d_qnrm, d_qjxw, d_qshape, d_gpts, d_gw, d_cells, d_dbl_off, d_dbl_ids,
        d_elem_off, d_elem_ids, d_proj);
    add(d_parent, d_child_first, d_nchild, d_digit, d_nbeg, d_nend, d_node_sorted, d_center,
        d_delta);
    add(d_nrow_ptr, d_ncol_ptr, d_nval_ptr, d_nent_ptr, d_prow_ptr, d_pcontrib_ptr, d_m2l_src_ptr,
        d_m2p_src_ptr, d_item_ptr, d_blk_ptr, d_m2p_item_ptr, d_m2p_tnode_ptr, d_up_q_ptr,
        d_down_q_ptr, d_near_sched);
    add(d_row_leaf, d_nrows, d_ncols, d_pleaf_box, d_prow_dof, d_pcontrib_q, d_lleaf_box,
        d_gather_ptr, d_gather_ids, d_m2l_tgt, d_m2l_src, d_m2l_off, d_m2p_tgt, d_m2p_src,
        d_l2l_box, d_parents, d_diag_col, d_m2p_pair_tgt, d_q_src, d_ch_start, d_ch_cnt, d_ch_op,
        d_up_box, d_down_box, d_up_q, d_down_q, d_up_child8, d_down_par, d_down_oct,
        d_m2p_item_pair, d_m2l_yslot, d_down_m2l_beg, d_down_m2l_end, d_m2p_tnodes);
    add(d_con_row, d_con_col, d_con_p, d_con_q, d_con_kind, d_con_nrm, d_con_sg);
    add(d_ilu_ptr, d_ilu_diag, d_ilu_col, d_ilu_rows_lo, d_ilu_rows_up, d_ilu_val);
    add(d_Sff, d_Srff, d_xff, d_Wff, d_Tcr);
    add(d_entries, d_N, d_D, d_S, d_T1, d_T2, d_W, d_ops, d_Pinv, d_Pinv64, d_Tc, d_Tcf, d_S32, d_T1f, d_T2f, d_Wf,
        d_opsf, d_opsff, d_tcimg, d_lvopsf, d_err, d_dir, d_modes, d_modes32, d_alpha);
    add(d_M64, d_L64, d_x64, d_y64, d_t1, d_t2, d_t3, d_t4, d_m2p64, d_Y64, d_M32, d_L32, d_x32,
        d_y32, d_m2p32, d_Y32, d_Mff, d_Lff, d_ozimg, d_ozslc, d_ozecol, d_ozerow);
    add(sv_b, sv_x, sv_r, sv_d, sv_w, sv_part, sv_nrm, sh_part, sh_nrm);
    add(eng.V, eng.z, eng.w, eng.u, eng.b, eng.x, eng.r, eng.d, eng.tmp, eng.cz, eng.cw, eng.hb,
        eng.partial, eng.H, eng.cs, eng.sn, eng.g, eng.y, eng.bn, eng.tol, eng.nrm);
    add(eng.ticket, eng.kdone, eng.jvec, eng.its, eng.maxit, eng.sel, eng.act, eng.ctl);
    for (const auto &b : io_buf)
      t += b.bytes();
    return t;
  }
};

namespace
{
  int fail(pibem_handle *h, const Error &e)
  {
    if (h)
      h->err = e.what();
    return e.code;
  }

  template <typename F>
  int guarded(pibem_handle *h, F &&f)
  {
    if (!h)
      return PIBEM_EINVAL;
    try
      {
        PIBEM_CUDA(cudaSetDevice(h->prm.device));
        f();
        return PIBEM_OK;
      }
    catch (const Error &e)
      {
        return fail(h, e);
      }
    catch (const std::bad_alloc &)
      {
        h->err = "host allocation failed";
        return PIBEM_ENOMEM_HBM;
      }
    catch (const std::exception &e)
      {
        h->err = e.what();
        return PIBEM_EINVAL;
      }
  }

  // Holds one thread for about ns nanoseconds (the global timer, at most
  // 200,000 sleeps of 1 us), so that the host can enqueue an operator
  // application behind it before the GPU reaches its first phase event.
  __global__ void hold_stream_kernel(int64_t ns)
  {
    uint64_t t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (int i = 0; i < 200000; ++i)
      {
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (int64_t(t - t0) >= ns)
          break;
        __nanosleep(1000);
      }
  }

  // Phase event i.  With a hold set, the first event of an application comes
  // after a short kernel that keeps the stream busy while the host enqueues
  // the application, so that the phase times are GPU execution times and not
  // host launch latency (the GPU would otherwise wait idle between events).
  void record(pibem_handle *h, int i)
  {
    if (!h->timing)
      return;
    if (i == 0 && h->timing_hold_ns > 0)
      {
        hold_stream_kernel<<<1, 1, 0, h->stream>>>(h->timing_hold_ns);
        PIBEM_CUDA(cudaGetLastError());
      }
    PIBEM_CUDA(cudaEventRecord(h->ev[i], h->stream));
  }

  // ---------------------------------------------------------------------
  // Far field (P2M ... L2P) added to y for R columns, in stages.
  // ---------------------------------------------------------------------
  template <typename T>
  void far_alloc(pibem_handle *h, OperatorDev<T> &op, DBuf<T> &M, DBuf<T> &Lx, DBuf<T> &scr,
                 DBuf<T> &Y, int R)
  {
    // rows of K values; the target-major M2L products of the fused level
    // passes use rows of K rounded up to 4 (16-byte aligned rows)
    Y.alloc(std::max<size_t>(1, size_t(op.n_pairs) * R * ((op.K + 3) / 4 * 4)));
    const size_t need = size_t(h->tree.nb) * R * op.K;
    if (M.n < need)
      {
        M.alloc(need);
        Lx.alloc(need);
      }
    scr.alloc(std::max<size_t>(1, size_t(op.n_m2p_items) * R));
    op.m2p_scratch = scr.p;
    if constexpr (std::is_same<T, double>::value)
      if (op.ops_ff)
        {
          h->d_Mff.alloc(need);
          h->d_Lff.alloc(need);
        }
  }

  // P2M and the upward pass: M of every box
  template <typename T>
  void far_up(pibem_handle *h, OperatorDev<T> &op, DBuf<T> &M, DBuf<T> &Y, int R,
              const uint8_t *modes, const T *x, bool combined, cudaStream_t s)
  {
    const size_t need = size_t(h->tree.nb) * R * op.K;
    PIBEM_CUDA(cudaMemsetAsync(M.p, 0, need * sizeof(T), s));
    launch_p2m_apply<T>(op, R, int(h->N()), h->d_dir.p, modes, x, M.p, combined, s);
    record(h, 2);
    if constexpr (std::is_same<T, double>::value)
      if (op.ops_ff)
        {
          // float-float passes on (hi, lo) expansions (M2P reads them too)
          float2 *Mff = h->d_Mff.p, *Yff = reinterpret_cast<float2 *>(Y.p);
          launch_convert_d2ff(int64_t(need), M.p, Mff, s);
          for (int l = h->tree.L; l >= 1; --l)
            launch_upward_level_ff(op, R, l, Mff, Yff, s);
          record(h, 3);
          return;
        }
    for (int l = h->tree.L; l >= 1; --l)
      launch_upward_level<T>(op, R, l, M.p, Y.p, s);
    record(h, 3);
  }

  // M2L and the downward pass: L of every box with nodes
  template <typename T>
  void far_down(pibem_handle *h, OperatorDev<T> &op, DBuf<T> &M, DBuf<T> &Lx, DBuf<T> &Y, int R,
                cudaStream_t s)
  {
    if constexpr (std::is_same<T, double>::value)
      if (op.ops_ff)
        {
          // float-float passes on (hi, lo) expansions; L back in FP64 for L2P
          const size_t need = size_t(h->tree.nb) * R * op.K;
          float2      *Mff = h->d_Mff.p, *Lff = h->d_Lff.p, *Yff = reinterpret_cast<float2 *>(Y.p);
          if (op.oz_images && op.dev_err)
            {
              // tensor-core FP64-accurate M2L from the digits of the multipoles
              const int64_t rows = int64_t(h->tree.nb) * R;
              h->d_ozslc.alloc(size_t(6) * rows * 128);
              h->d_ozerow.alloc(size_t(rows));
              launch_ozaki_slices(rows, op.K, Mff, h->d_ozslc.p, h->d_ozerow.p, s);
              launch_ozaki_gemm(op, R, 0, op.m2l_chunk_end, h->d_ozslc.p, h->d_ozerow.p, rows, Yff,
                                s);
            }
          else
            launch_m2l_ff(op, R, Mff, Yff, s);
          record(h, 4);
          for (int l = 1; l <= h->tree.L; ++l)
            launch_downward_level_ff(op, R, l, Lff, Yff, s);
          if (!op.Wff) // L2P reads the pairs when it has pair rows
            launch_convert_ff2d(int64_t(need), Lff, Lx.p, s);
          record(h, 5);
          return;
        }
    launch_m2l_gemm<T>(op, R, M.p, Y.p, s);
    record(h, 4);
    launch_m2l_sums<T>(op, R, Lx.p, Y.p, s);
    for (int l = 1; l <= h->tree.L; ++l)
      launch_downward_level<T>(op, R, l, Lx.p, Y.p, s);
    record(h, 5);
  }

  // L2P into y: the FP64-accurate operator reads the (hi, lo) locals
  template <typename T>
  void l2p_apply(pibem_handle *h, const OperatorDev<T> &op, int R, const T *Lx, T *y, cudaStream_t st)
  {
    if constexpr (std::is_same<T, double>::value)
      if (op.ops_ff && op.Wff)
        {
          launch_l2p_ff(op, R, int(h->N()), h->d_Lff.p, y, st);
          return;
        }
    launch_l2p<T>(op, R, int(h->N()), Lx, y, st);
  }

  // M2P into y: the FP64-accurate operator evaluates from the (hi, lo)
  // multipoles in float-float
  template <typename T>
  void m2p_apply(pibem_handle *h, const OperatorDev<T> &op, int R, const T *M, T *y, cudaStream_t st)
  {
    if constexpr (std::is_same<T, double>::value)
      if (op.ops_ff)
        {
          launch_m2p_ff(op, h->td, R, int(h->N()), h->d_Mff.p, y, st);
          return;
        }
    launch_m2p<T>(op, h->td, R, int(h->N()), M, y, st);
  }

  template <typename T>
  void far_field(pibem_handle *h, OperatorDev<T> &op, DBuf<T> &M, DBuf<T> &Lx, DBuf<T> &scr,
                 DBuf<T> &Y, int R, const uint8_t *modes, const T *x, T *y, bool combined = false)
  {
    const int    N = int(h->N());
    cudaStream_t s = h->stream;
    far_alloc<T>(h, op, M, Lx, scr, Y, R);
    far_up<T>(h, op, M, Y, R, modes, x, combined, s);
    far_down<T>(h, op, M, Lx, Y, R, s);
    m2p_apply<T>(h, op, R, M.p, y, s);
    record(h, 6);
    l2p_apply<T>(h, op, R, Lx.p, y, s);
    record(h, 7);
  }

  // The system operator y = S x (near field + combined far field).  Without
  // phase timing the independent branches run on two streams: the near SpMV
  // (HBM-bound) and then M2P on the handle's low-priority side stream, beside
  // P2M, the upward pass, M2L and the downward pass (latency-bound, the
  // critical path) on its high-priority stream; L2P joins them, and the
  // caller's stream waits for the result.  y is written by the near SpMV and then added
  // to by M2P and L2P in that order, as in the one-stream sequence, so the
  // result is the same bit for bit.
  // y = near x: with vals_ff (FP64-accurate operator) on (hi, lo) FP32 pairs
  template <typename T>
  void near_apply(pibem_handle *h, const OperatorDev<T> &op, int R, const T *vals,
                  const float2 *vals_ff, const T *x, T *y, cudaStream_t st)
  {
    const int N = int(h->N());
    if constexpr (std::is_same<T, double>::value)
      if (vals_ff && near_ff_fits(op))
        {
          h->d_xff.alloc(size_t(R) * N);
          launch_convert_d2ff(int64_t(R) * N, x, h->d_xff.p, st);
          launch_near_spmv_ff(op, R, N, vals_ff, h->d_xff.p, y, false, st);
          return;
        }
    launch_near_spmv<T>(op, R, N, vals, x, y, false, st);
  }

  template <typename T>
  void system_operator(pibem_handle *h, OperatorDev<T> &op, const T *vals, DBuf<T> &M,
                       DBuf<T> &Lx, DBuf<T> &scr, DBuf<T> &Y, int R, const uint8_t *modes,
                       const T *x, T *y, const float2 *vals_ff = nullptr)
  {
    const int    N = int(h->N());
    cudaStream_t s = h->stream;
    PdlScope     pdl_scope(R == 1);
    if (h->timing || !h->side)
      {
        record(h, 0);
        near_apply<T>(h, op, R, vals, vals_ff, x, y, s);
        record(h, 1);
        far_field<T>(h, op, M, Lx, scr, Y, R, modes, x, y, true);
        return;
      }
    cudaStream_t side = h->side, main = h->main_hp;
    far_alloc<T>(h, op, M, Lx, scr, Y, R);
    PIBEM_CUDA(cudaEventRecord(h->ev_fork, s));
    PIBEM_CUDA(cudaStreamWaitEvent(side, h->ev_fork, 0));
    PIBEM_CUDA(cudaStreamWaitEvent(main, h->ev_fork, 0));
    near_apply<T>(h, op, R, vals, vals_ff, x, y, side);
    far_up<T>(h, op, M, Y, R, modes, x, true, main);
    PIBEM_CUDA(cudaEventRecord(h->ev_up, main));
    PIBEM_CUDA(cudaStreamWaitEvent(side, h->ev_up, 0));
    m2p_apply<T>(h, op, R, M.p, y, side);
    PIBEM_CUDA(cudaEventRecord(h->ev_side, side));
    far_down<T>(h, op, M, Lx, Y, R, main);
    PIBEM_CUDA(cudaStreamWaitEvent(main, h->ev_side, 0));
    l2p_apply<T>(h, op, R, Lx.p, y, main);
    PIBEM_CUDA(cudaEventRecord(h->ev_main, main));
    PIBEM_CUDA(cudaStreamWaitEvent(s, h->ev_main, 0));
  }

  // prec: 0 FP64 operator, 1 FP32 operator
  void finish_timing(pibem_handle *h, int prec = 0)
  {
    if (!h->timing)
      return;
    PIBEM_CUDA(cudaEventSynchronize(h->ev[7]));
    for (int i = 0; i < 7; ++i)
      {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev[i], h->ev[i + 1]);
        h->phase_ms[i] = ms;
        h->phase_tot[prec][i] += ms;
      }
    h->phase_cnt[prec] += 1;
  }

  // [phi_0..phi_{R-1}, dphi_0..dphi_{R-1}] -> [outN..., outD...]  (FP64)
  void fmm_apply64(pibem_handle *h, int R, const double *phi, const double *dphi, double *oN,
                   double *oD)
  {
    const int64_t N = h->N();
    cudaStream_t  s = h->stream;
    h->d_x64.alloc(size_t(2 * R) * N);
    h->d_y64.alloc(size_t(2 * R) * N);
    PIBEM_CUDA(cudaMemcpyAsync(h->d_x64.p, phi, sizeof(double) * R * N, cudaMemcpyDeviceToDevice, s));
    PIBEM_CUDA(cudaMemcpyAsync(h->d_x64.p + R * N, dphi, sizeof(double) * R * N,
                               cudaMemcpyDeviceToDevice, s));
    std::vector<uint8_t> modes(2 * R);
    for (int r = 0; r < R; ++r)
      {
        modes[r]     = MODE_KER1;
        modes[R + r] = MODE_KER2;
      }
    h->d_modes.upload(modes, s);
    h->modes_R = -1;
    record(h, 0);
    launch_near_spmv<double>(h->op64, R, int(N), h->d_N.p, h->d_x64.p, h->d_y64.p, false, s);
    launch_near_spmv<double>(h->op64, R, int(N), h->d_D.p, h->d_x64.p + R * N,
                             h->d_y64.p + R * N, false, s);
    record(h, 1);
    far_field<double>(h, h->op64, h->d_M64, h->d_L64, h->d_m2p64, h->d_Y64, 2 * R, h->d_modes.p,
                      h->d_x64.p, h->d_y64.p);
    finish_timing(h, 0);
    PIBEM_CUDA(cudaMemcpyAsync(oN, h->d_y64.p, sizeof(double) * R * N, cudaMemcpyDeviceToDevice, s));
    PIBEM_CUDA(cudaMemcpyAsync(oD, h->d_y64.p + R * N, sizeof(double) * R * N,
                               cudaMemcpyDeviceToDevice, s));
    h->cnt64 += R;
  }

  // Near-field N only with the double-layer far field (alpha needs N*1 only).
  void ker1_apply64(pibem_handle *h, const double *x, double *y)
  {
    const int64_t        N = h->N();
    std::vector<uint8_t> modes(1, MODE_KER1);
    h->d_modes.upload(modes, h->stream);
    h->modes_R = -1;
    record(h, 0);
    launch_near_spmv<double>(h->op64, 1, int(N), h->d_N.p, x, y, false, h->stream);
    record(h, 1);
    far_field<double>(h, h->op64, h->d_M64, h->d_L64, h->d_m2p64, h->d_Y64, 1, h->d_modes.p, x, y);
    finish_timing(h, 0);
  }

  // d_modes = mode for R columns (uploaded only when it changes, so that the
  // operator can be captured into a graph)
  void set_modes(pibem_handle *h, int R, uint8_t mode)
  {
    if (h->modes_R == R && h->modes_val == mode)
      return;
    std::vector<uint8_t> modes(R, mode);
    h->d_modes.upload(modes, h->stream);
    h->modes_R   = R;
    h->modes_val = mode;
  }

  // Pure-Neumann shift of bem_problem.cc:1169-1172 / 1214-1215: v -= ||v||_2.
  // (on the device, without a host round trip, so that it can be captured)
  void shift_by_norm(pibem_handle *h, int R, double *v)
  {
    const int64_t N    = h->N();
    const int     nblk = 64;
    h->sh_part.alloc(size_t(R) * nblk);
    h->sh_nrm.alloc(R);
    launch_dots(N, R, 1, N, N, v, v, h->sh_part.p, nblk, h->sh_nrm.p, h->stream);
    launch_sub_norm(N, R, h->sh_nrm.p, v, h->stream);
  }

  // ConstrainedOperator::vmult (include/constrained_matrix.h:100-125): every
  // constrained row of y replaced by its line x[row] - x[col].
  void constrain_rows(pibem_handle *h, int R, const double *x, double *y)
  {
    launch_constrain_rows(int(h->con_row.size()), R, h->N(), h->d_con_row.p, h->d_con_col.p, x, y,
                          h->stream);
  }

  // BEMProblem::vmult for R columns, FP64 (device in/out); constrained: the
  // solve's operator (the constraint lines of its double nodes).
  void system_apply64(pibem_handle *h, int R, const double *x, double *y, bool constrained = false)
  {
    const int64_t N = h->N();
    cudaStream_t  s = h->stream;
    const double *xin = x;
    if (!h->have_dirichlet)
      {
        h->d_t4.alloc(size_t(R) * N);
        PIBEM_CUDA(cudaMemcpyAsync(h->d_t4.p, x, sizeof(double) * R * N, cudaMemcpyDeviceToDevice, s));
        shift_by_norm(h, R, h->d_t4.p);
        xin = h->d_t4.p;
      }
    set_modes(h, R, MODE_COMBINED);
    system_operator<double>(h, h->op64, h->d_S.p, h->d_M64, h->d_L64, h->d_m2p64, h->d_Y64, R,
                            h->d_modes.p, xin, y, h->op64.ops_ff ? h->d_Sff.p : nullptr);
    finish_timing(h, 0);
    if (!h->have_dirichlet)
      shift_by_norm(h, R, y);
    if (constrained)
      constrain_rows(h, R, x, y);
    h->cnt64 += R;
  }

  // Near SpMV + far field of the FP32 system operator, d_x32 -> d_y32.
  void operator32_body(pibem_handle *h, int R)
  {
    system_operator<float>(h, h->op32, h->d_S32.p, h->d_M32, h->d_L32, h->d_m2p32, h->d_Y32, R,
                           h->d_modes32.p, h->d_x32.p, h->d_y32.p);
  }

  void drop_graph(pibem_handle *h)
  {
    if (h->g32_exec)
      cudaGraphExecDestroy(h->g32_exec);
    h->g32_exec = nullptr;
    for (auto &c : h->cycle_graphs)
      if (c.exec)
        cudaGraphExecDestroy(c.exec);
    h->cycle_graphs.clear();
  }

  // The FP32 operator is applied once per GMRES iteration with the same buffers,
  // so it is captured once as a CUDA graph (about 45 kernels) and replayed: one
  // launch instead of ~45, and no launch gaps between its small kernels.  Not
  // used while phase timing is on (its events are host-recorded) or when the
  // caller's stream is itself being captured.
  void operator32(pibem_handle *h, int R)
  {
    cudaStream_t s = h->stream;
    if (h->modes32_R != R)
      {
        std::vector<uint8_t> modes(R, MODE_COMBINED);
        h->d_modes32.upload(modes, s);
        h->modes32_R = R;
      }
    bool graph = !h->timing;
    if (graph)
      {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        PIBEM_CUDA(cudaStreamIsCapturing(s, &cs));
        graph = cs == cudaStreamCaptureStatusNone;
      }
    if (!graph)
      {
        operator32_body(h, R);
        return;
      }
    auto key_of = [&](uintptr_t k[8]) {
      k[0] = uintptr_t(R);
      k[1] = uintptr_t(h->d_x32.p);
      k[2] = uintptr_t(h->d_y32.p);
      k[3] = uintptr_t(h->d_M32.p);
      k[4] = uintptr_t(h->d_L32.p);
      k[5] = uintptr_t(h->d_Y32.p);
      k[6] = uintptr_t(h->d_m2p32.p);
      k[7] = uintptr_t(h->d_modes32.p) ^ uintptr_t(s);
    };
    uintptr_t key[8];
    key_of(key);
    if (h->g32_exec && std::equal(key, key + 8, h->g32_key))
      {
        PIBEM_CUDA(cudaGraphLaunch(h->g32_exec, s));
        note_launch(h->g32_kernels);
        return;
      }
    // New buffers or column count: apply once directly (this also grows the
    // work buffers to their final size), then capture the same sequence.
    drop_graph(h);
    operator32_body(h, R);
    key_of(key);
    const int64_t l0 = t_launches;
    cudaGraph_t   g  = nullptr;
    PIBEM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    try
      {
        operator32_body(h, R);
      }
    catch (...)
      {
        cudaStreamEndCapture(s, &g);
        if (g)
          cudaGraphDestroy(g);
        throw;
      }
    PIBEM_CUDA(cudaStreamEndCapture(s, &g));
    // kernel nodes keep the priority of the stream they were captured from
    const cudaError_t e =
      cudaGraphInstantiateWithFlags(&h->g32_exec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
      {
        h->g32_exec = nullptr;
        throw Error(PIBEM_ECUDA, std::string("graph instantiation: ") + cudaGetErrorString(e));
      }
    // the captured kernels did not run: count them at each replay instead
    h->g32_kernels = t_launches - l0;
    g_launches.fetch_sub(h->g32_kernels, std::memory_order_relaxed);
    t_launches = l0;
    std::copy(key, key + 8, h->g32_key);
  }

  // Same operator in FP32 (input and output FP64).
  void system_apply32(pibem_handle *h, int R, const double *x, double *y, bool constrained = false)
  {
    const int64_t N = h->N();
    cudaStream_t  s = h->stream;
    const double *xin = x;
    if (!h->have_dirichlet)
      {
        h->d_t4.alloc(size_t(R) * N);
        PIBEM_CUDA(cudaMemcpyAsync(h->d_t4.p, x, sizeof(double) * R * N, cudaMemcpyDeviceToDevice, s));
        shift_by_norm(h, R, h->d_t4.p);
        xin = h->d_t4.p;
      }
    h->d_x32.alloc(size_t(R) * N);
    h->d_y32.alloc(size_t(R) * N);
    launch_convert_d2f(int64_t(R) * N, xin, h->d_x32.p, s);
    operator32(h, R);
    finish_timing(h, 1);
    launch_convert_f2d(int64_t(R) * N, h->d_y32.p, y, s);
    if (!h->have_dirichlet)
      shift_by_norm(h, R, y);
    if (constrained)
      constrain_rows(h, R, x, y);
    h->cnt32 += R;
  }

  void compute_rhs_dev(pibem_handle *h, int R, const double *tmp, double *rhs);
  void constrain_rhs(pibem_handle *h, int R, const double *tmp, double *b);

  // ---------------------------------------------------------------------
  // The solve engine.  Every right-hand side ("column") of a solve -- the
  // batch of pibem_solve, or the request slots of the pibem_slots_* entry
  // points -- runs its own state machine:
  //   plain FP64 path (BEMProblem::solve_system, bem_problem.cc:1267-1347):
  //     b = rhs(tmp), x0 = b, restarted GMRES(m) on the FP64 operator with
  //     right leaf-block Jacobi preconditioning, stopping at the relative true
  //     residual ||b - A x|| / ||b|| <= tol, checked at every restart;
  //   mixed path: FP64 iterative refinement from x0 = 0 around GMRES(m) on the
  //     FP32 operator: each correction d solves A32 d = r to an inner tolerance;
  //     the first residual after a correction is b - A64 x, later ones are
  //     updated as r <- r - A32 d (|d| shrinks by the inner tolerance at each
  //     step, so the update's rounding stays far below the target); an
  //     estimate that meets the tolerance is confirmed with b - A64 x before the
  //     column stops (A64: the FP64-accurate operator).
  // The host advances the columns from event to event.  Each operator
  // application is shared by the columns that need it at that moment (they are
  // gathered into one contiguous batch), and the Arnoldi steps of every column
  // inside a GMRES cycle run on the device -- CGS2 in FP64, the Hessenberg
  // column's Givens rotation and the stopping test (gmres_givens_kernel) -- as
  // one CUDA graph, a conditional while node around one step, until some column
  // ends its cycle (it met its tolerance, took m steps or reached its iteration
  // limit).  While phase timing is on, or the caller's stream is itself being
  // captured, the same launches are issued step by step.  A column's arithmetic
  // never depends on the other columns, so its result is the same alone, in a
  // batch, or admitted while other columns are in the middle of their solves.
  // ---------------------------------------------------------------------

  // R columns of n doubles from src (column stride lds) to dst (column stride ldd)
  void copy_cols(double *dst, int64_t ldd, const double *src, int64_t lds, int64_t n, int R,
                 cudaStream_t s)
  {
    PIBEM_CUDA(cudaMemcpy2DAsync(dst, size_t(ldd) * sizeof(double), src, size_t(lds) * sizeof(double),
                                 size_t(n) * sizeof(double), size_t(R), cudaMemcpyDeviceToDevice, s));
  }

  // z = P^-1 v for R columns (v column stride ldv).  Leaf-block Jacobi: the
  // FP64 inverses where the handle keeps them (GMRES on an FP64-accurate
  // operator), else the FP32 ones.  ILU(0): z = v, then the level-scheduled
  // forward and backward substitutions in place (FP64).  With nrm2, v / |v|
  // is also written to vout (column stride ldo, at column jvec[r] + 1).
  void apply_prec(pibem_handle *h, int R, const double *v, int64_t ldv, double *z, cudaStream_t s,
                  const double *nrm2 = nullptr, double *vout = nullptr, int64_t ldo = 0,
                  const int *jvec = nullptr, const int *sel = nullptr)
  {
    const int64_t N = h->N();
    if (h->ilu_on)
      {
        if (nrm2)
          launch_normalize(N, R, v, nrm2, vout, ldo, s, jvec, z, sel);
        else
          launch_copy_sel(N, R, v, ldv, z, sel, s);
        launch_ilu_apply(h->ilu_lptr_lo, h->d_ilu_rows_lo.p, h->ilu_lptr_up, h->d_ilu_rows_up.p, R, N,
                         h->d_ilu_ptr.p, h->d_ilu_col.p, h->d_ilu_val.p, h->d_ilu_diag.p, z, sel,
                         jvec, s);
        return;
      }
    const int nl = int(h->blk_ptr.size()) - 1;
    if (h->d_Pinv64.p)
      launch_block_apply(nl, h->max_leaf_rows, R, N, h->d_nrow_ptr.p, h->d_blk_ptr.p, h->d_nrows.p,
                         h->d_Pinv64.p, v, ldv, z, s, nrm2, vout, ldo, jvec, sel);
    else
      launch_block_apply(nl, h->max_leaf_rows, R, N, h->d_nrow_ptr.p, h->d_blk_ptr.p, h->d_nrows.p,
                         h->d_Pinv.p, v, ldv, z, s, nrm2, vout, ldo, jvec, sel);
  }

  // n values from the device into out, through the handle's page-locked buffer
  // (stream-ordered, then synchronised)
  void read_small(pibem_handle *h, double *out, const double *dev, size_t n, cudaStream_t s)
  {
    h->g_small.alloc(std::max<size_t>(n, 64));
    PIBEM_CUDA(cudaMemcpyAsync(h->g_small.p, dev, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    PIBEM_CUDA(cudaStreamSynchronize(s));
    std::copy(h->g_small.p, h->g_small.p + n, out);
  }

  constexpr int ENG_NBLK = 2 * 152; // partial-sum blocks of the GMRES norms and Gram-Schmidt passes
  constexpr int ENG_NBLK_REFINE = 64; // of the refinement residual norms

  // (re)size the engine for S columns and Krylov dimension m; keeps nothing
  void engine_open(pibem_handle *h, int S, int m)
  {
    Engine       &E = h->eng;
    const int64_t N = h->N();
    if (S < 1 || S > 1024)
      throw Error(PIBEM_EINVAL, "between 1 and 1024 columns per solve / slots per handle");
    if (m < 1)
      throw Error(PIBEM_EINVAL, "GMRES restart length must be at least 1");
    const int L = m + 1;
    E.S         = S;
    E.m         = m;
    E.mixed     = h->prm.precision_mode == PIBEM_PRECISION_MIXED;
    E.prec      = h->prm.preconditioner != 0;
    E.col.assign(S, ColHost());
    E.V.alloc(size_t(S) * L * N);
    for (DBuf<double> *v : {&E.b, &E.x, &E.r, &E.d, &E.tmp, &E.u})
      v->alloc(size_t(S) * N);
    // z, w and the contiguous batch also hold the idle padding columns of the
    // cycle graphs (S .. bucket(S) - 1, at most S of them); their z is zero
    for (DBuf<double> *v : {&E.z, &E.w, &E.cz, &E.cw})
      v->alloc(size_t(2 * S) * N);
    PIBEM_CUDA(cudaMemsetAsync(E.z.p + size_t(S) * N, 0, sizeof(double) * size_t(S) * N, h->stream));
    E.hb.alloc(size_t(S) * (2 * L + 1));
    E.partial.alloc(size_t(S) * ENG_NBLK * L);
    E.H.alloc(size_t(S) * L * m);
    E.cs.alloc(size_t(S) * m);
    E.sn.alloc(size_t(S) * m);
    E.g.alloc(size_t(S) * L);
    E.y.alloc(size_t(S) * L);
    E.bn.alloc(S);
    E.tol.alloc(S);
    E.nrm.alloc(S);
    E.ticket.alloc(S);
    E.ticket.zero(h->stream);
    for (DBuf<int> *v : {&E.kdone, &E.jvec, &E.its, &E.maxit, &E.sel})
      v->alloc(S);
    E.act.alloc(2 * S);
    std::vector<int> minus(S, -1);
    E.jvec.upload(minus, h->stream);
    E.ctl.alloc(4);
    E.ipin.alloc(size_t(3) * S + 4);
    E.h_bn.assign(S, 1.0);
    E.h_tol.assign(S, 0.0);
    E.h_its.assign(S, 0);
    E.h_maxit.assign(S, 0);
    E.h_jvec.assign(S, -1);
  }

  std::vector<int> cols_in(const Engine &E, ColStage st)
  {
    std::vector<int> c;
    for (int k = 0; k < E.S; ++k)
      if (E.col[k].st == st)
        c.push_back(k);
    return c;
  }

  void upload_sel(pibem_handle *h, const std::vector<int> &cols)
  {
    Engine          &E = h->eng;
    std::vector<int> sel(E.S, 0);
    for (int c : cols)
      sel[c] = 1;
    E.sel.upload(sel, h->stream);
  }

  // squared 2-norms of the S slot columns of v (nblk partial blocks), into out
  void eng_norms(pibem_handle *h, const double *v, int nblk, std::vector<double> &out)
  {
    Engine       &E = h->eng;
    const int64_t N = h->N();
    launch_dots(N, E.S, 1, N, N, v, v, E.partial.p, nblk, E.nrm.p, h->stream);
    out.resize(E.S);
    read_small(h, out.data(), E.nrm.p, E.S, h->stream);
  }

  enum EngOp
  {
    OP_A32,
    OP_A64,
    OP_RHS
  };

  // the operator (or the right-hand side) on the listed columns: in and out
  // slot-strided (column k at k N), through the contiguous batch cz -> cw
  void eng_apply(pibem_handle *h, EngOp op, const std::vector<int> &cols, const double *in,
                 double *out)
  {
    Engine       &E = h->eng;
    const int64_t N = h->N();
    cudaStream_t  s = h->stream;
    const int     R = int(cols.size());
    if (R == 0)
      return;
    E.act.upload(cols, s);
    launch_gather_cols(N, R, E.act.p, in, N, E.cz.p, s);
    if (op == OP_A32)
      system_apply32(h, R, E.cz.p, E.cw.p, true);
    else if (op == OP_A64)
      system_apply64(h, R, E.cz.p, E.cw.p, true);
    else
      {
        compute_rhs_dev(h, R, E.cz.p, E.cw.p);
        constrain_rhs(h, R, E.cz.p, E.cw.p);
      }
    launch_scatter_cols(N, R, E.act.p, E.cw.p, out, N, s);
    for (int c : cols)
      {
        if (op == OP_A32)
          E.col[c].c32++;
        else
          E.col[c].c64++;
      }
  }

  void eng_copy(pibem_handle *h, double *dst, const double *src, const std::vector<int> &cols)
  {
    const int64_t N = h->N();
    for (int c : cols)
      PIBEM_CUDA(cudaMemcpyAsync(dst + int64_t(c) * N, src + int64_t(c) * N, sizeof(double) * N,
                                 cudaMemcpyDeviceToDevice, h->stream));
  }
  void eng_zero(pibem_handle *h, double *v, const std::vector<int> &cols)
  {
    const int64_t N = h->N();
    for (int c : cols)
      PIBEM_CUDA(cudaMemsetAsync(v + int64_t(c) * N, 0, sizeof(double) * N, h->stream));
  }

  // Operator batch sizes of the cycle graphs (one graph each): the active
  // column count rounded up to 1, 2, 3, 4, 6, 8, 12, 16, ... (at most half
  // again), so that a changing count reuses a few graphs
  int eng_bucket(int n)
  {
    int b = 1;
    while (b < n)
      b = (b & (b - 1)) == 0 && b >= 2 ? b + b / 2 : (b == 1 ? 2 : (b / 3) * 4);
    return b;
  }

  // One Arnoldi step of every column in a cycle (E.act holds them, R' of them):
  // w = A z (through the contiguous batch), CGS2 into hb, V_{j+1} = w / |w| and
  // the next z, then the Givens step.
  void eng_step(pibem_handle *h, int Ra, const std::function<void(const double *, double *, int)> &A,
                cudaGraphConditionalHandle cond, bool use_cond)
  {
    Engine       &E   = h->eng;
    const int64_t N   = h->N();
    cudaStream_t  s   = h->stream;
    const int     L   = E.m + 1;
    const int64_t ldr = int64_t(L) * N;
    double *h1 = E.hb.p, *h2 = h1 + size_t(E.S) * L, *nr = h2 + size_t(E.S) * L;
    if (E.mixed && h->have_dirichlet && h->con_row.empty())
      {
        // the FP32 operator straight on the gathered columns: gather + FP32
        // conversion and FP64 conversion + scatter fused (as system_apply32)
        h->d_x32.alloc(size_t(Ra) * N);
        h->d_y32.alloc(size_t(Ra) * N);
        launch_gather_d2f(N, Ra, E.act.p, E.z.p, h->d_x32.p, s);
        operator32(h, Ra);
        finish_timing(h, 1);
        launch_f2d_scatter(N, Ra, E.act.p, h->d_y32.p, E.w.p, s);
        h->cnt32 += Ra;
      }
    else
      {
        launch_gather_cols(N, Ra, E.act.p, E.z.p, N, E.cz.p, s);
        A(E.cz.p, E.cw.p, Ra);
        launch_scatter_cols(N, Ra, E.act.p, E.cw.p, E.w.p, N, s);
      }
    launch_cgs_step(0, N, E.S, 0, N, ldr, E.V.p, nullptr, 0, E.w.p, ENG_NBLK, E.partial.p,
                    E.ticket.p, h1, s, E.jvec.p, L);
    launch_cgs_step(1, N, E.S, 0, N, ldr, E.V.p, h1, L, E.w.p, ENG_NBLK, E.partial.p, E.ticket.p, h2,
                    s, E.jvec.p, L);
    launch_cgs_step(2, N, E.S, 0, N, ldr, E.V.p, h2, L, E.w.p, ENG_NBLK, E.partial.p, E.ticket.p, nr,
                    s, E.jvec.p, 1);
    if (E.prec) // V_{j+1} = w / |w| and the next step's z = P^-1 V_{j+1} in one pass
      apply_prec(h, E.S, E.w.p, N, E.z.p, s, nr, E.V.p, ldr, E.jvec.p);
    else
      launch_normalize(N, E.S, E.w.p, nr, E.V.p, ldr, s, E.jvec.p, E.z.p);
    launch_gmres_givens(E.S, E.m, h1, E.H.p, E.cs.p, E.sn.p, E.g.p, E.kdone.p, E.jvec.p, E.its.p,
                        E.maxit.p, E.bn.p, E.tol.p, E.ctl.p, cond, use_cond, s);
  }

  // Runs the Arnoldi steps of the columns in a cycle until one of them ends its
  // cycle or quantum steps have run; returns the steps run.
  int eng_cycle(pibem_handle *h, const std::vector<int> &act, int quantum)
  {
    Engine      &E  = h->eng;
    cudaStream_t s  = h->stream;
    const int    Ra = eng_bucket(int(act.size())); // operator batch of the graph
    auto A = [h](const double *in, double *out, int R) {
      if (h->eng.mixed)
        system_apply32(h, R, in, out, true);
      else
        system_apply64(h, R, in, out, true);
    };
    // the active columns, padded to a bucket of the graph cache with idle
    // columns beyond S (zero input, output not used)
    const int Rb = eng_bucket(int(act.size()));
    std::vector<int> actp(act);
    for (int k = 0; int(actp.size()) < Rb; ++k)
      actp.push_back(E.S + k);
    E.act.upload(actp, s);
    // the steps go on until every column ended its cycle (a column that ended
    // waits, frozen, and the columns' next operator applications stay
    // batched) or for at most a quantum of steps (serving: new submissions
    // join, and finished columns leave, at the next call)
    E.h_ctl = {0, 0, quantum > 0 ? quantum : std::numeric_limits<int>::max(), 0};
    E.ctl.upload(E.h_ctl, s);
    bool graph = !h->timing;
    if (graph)
      {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        PIBEM_CUDA(cudaStreamIsCapturing(s, &cs));
        graph = cs == cudaStreamCaptureStatusNone;
      }
    if (!graph)
      {
        int steps = 0;
        while (true)
          {
            eng_step(h, Ra, A, 0, false);
            ++steps;
            PIBEM_CUDA(cudaMemcpyAsync(E.ipin.p, E.ctl.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            PIBEM_CUDA(cudaStreamSynchronize(s));
            if (!E.ipin.p[0])
              break;
          }
        return steps;
      }
    // the operator reads d_modes: COMBINED for the Ra columns (other calls
    // may have left other modes there)
    if (!E.mixed)
      set_modes(h, Ra, MODE_COMBINED);
    // every buffer a step touches (a reallocation changes an address)
    auto bufs_now = [&](int i) -> const void * {
      const void *b[] = {E.V.p,    E.z.p,     E.w.p,      E.hb.p,    E.partial.p, E.ticket.p,
                         E.H.p,    E.cs.p,    E.sn.p,     E.g.p,     E.kdone.p,   E.jvec.p,
                         E.its.p,  E.maxit.p, E.bn.p,     E.tol.p,   E.ctl.p,     E.act.p,
                         E.cz.p,   E.cw.p,    h->d_x32.p, h->d_y32.p, h->d_M32.p, h->d_L32.p,
                         h->d_Y32.p, h->d_m2p32.p, h->d_M64.p, h->d_L64.p, h->d_Y64.p,
                         h->d_m2p64.p, h->d_t4.p, h->d_Mff.p, h->d_Lff.p, h->d_xff.p,
                         h->d_ozslc.p, h->d_modes.p, h->d_modes32.p, h->sh_part.p,
                         h->d_ilu_val.p, h->d_ilu_col.p, h->d_ilu_ptr.p, h->d_ilu_diag.p,
                         h->d_ilu_rows_lo.p, h->d_ilu_rows_up.p};
      return b[i];
    };
    constexpr int             nb = 44;
    std::array<uintptr_t, 48> key{};
    key[0] = uintptr_t(Ra) | (uintptr_t(E.S) << 16) | (uintptr_t(E.m) << 32) |
             (uintptr_t(E.prec) << 48) | (uintptr_t(E.mixed) << 49) | (uintptr_t(h->ilu_on) << 50);
    key[1] = uintptr_t(s);
    for (int i = 0; i < nb; ++i)
      key[2 + i] = uintptr_t(bufs_now(i));
    CycleGraph *cg = nullptr;
    for (auto &c : h->cycle_graphs)
      if (c.exec && c.key == key)
        cg = &c;
    if (!cg)
      {
        // one uncaptured operator application on Ra columns first (its result
        // is not used): it sizes the operator's work buffers for Ra columns, so
        // nothing is allocated during the capture
        {
          PIBEM_CUDA(cudaMemsetAsync(E.cz.p, 0, sizeof(double) * Ra * h->N(), s));
          const int64_t l0 = t_launches;
          const int     c32 = h->cnt32, c64 = h->cnt64;
          A(E.cz.p, E.cw.p, Ra);
          const int64_t extra = t_launches - l0;
          g_launches.fetch_sub(extra, std::memory_order_relaxed);
          t_launches = l0;
          h->cnt32   = c32;
          h->cnt64   = c64;
        }
        for (int i = 0; i < nb; ++i)
          key[2 + i] = uintptr_t(bufs_now(i));
        // a graph per active-column count; the oldest goes when there are eight
        if (h->cycle_graphs.size() >= 8)
          {
            cudaGraphExecDestroy(h->cycle_graphs.front().exec);
            h->cycle_graphs.erase(h->cycle_graphs.begin());
          }
        cudaGraph_t                g = nullptr;
        cudaGraphConditionalHandle cond{};
        PIBEM_CUDA(cudaGraphCreate(&g, 0));
        struct GraphGuard
        {
          cudaGraph_t &g;
          ~GraphGuard()
          {
            if (g)
              cudaGraphDestroy(g);
          }
        } guard{g};
        PIBEM_CUDA(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np = {};
        np.type                = cudaGraphNodeTypeConditional;
        np.conditional.handle  = cond;
        np.conditional.type    = cudaGraphCondTypeWhile;
        np.conditional.size    = 1;
        cudaGraphNode_t node   = nullptr;
        PIBEM_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
        cudaGraph_t   body = np.conditional.phGraph_out[0];
        const int64_t l0   = t_launches;
        const int     c32 = h->cnt32, c64 = h->cnt64;
        PIBEM_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeRelaxed));
        try
          {
            eng_step(h, Ra, A, cond, true);
          }
        catch (...)
          {
            cudaGraph_t tmp = nullptr;
            cudaStreamEndCapture(s, &tmp);
            throw;
          }
        PIBEM_CUDA(cudaStreamEndCapture(s, &body));
        CycleGraph c;
        c.key = key;
        // the captured kernels did not run: they are counted per executed step
        c.kernels = t_launches - l0;
        g_launches.fetch_sub(c.kernels, std::memory_order_relaxed);
        t_launches = l0;
        c.c32      = h->cnt32 - c32;
        c.c64      = h->cnt64 - c64;
        h->cnt32   = c32;
        h->cnt64   = c64;
        const cudaError_t e =
          cudaGraphInstantiateWithFlags(&c.exec, g, cudaGraphInstantiateFlagUseNodePriority);
        if (e != cudaSuccess)
          throw Error(PIBEM_ECUDA, std::string("GMRES cycle graph instantiation: ") +
                                     cudaGetErrorString(e));
        h->cycle_graphs.push_back(c);
        cg = &h->cycle_graphs.back();
      }
    PIBEM_CUDA(cudaGraphLaunch(cg->exec, s));
    PIBEM_CUDA(cudaMemcpyAsync(E.ipin.p, E.ctl.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    PIBEM_CUDA(cudaStreamSynchronize(s));
    const int steps = E.ipin.p[1];
    note_launch(cg->kernels * steps);
    h->cnt32 += cg->c32 * steps;
    h->cnt64 += cg->c64 * steps;
    return steps;
  }

  // Advances every column from event to event until each has finished or waits
  // in a GMRES cycle, then runs the cycle graph once (until some column ends
  // its cycle, or for at most quantum steps when quantum > 0).  Returns the
  // number of columns that finished.
  int engine_advance(pibem_handle *h, int quantum = 0)
  {
    Engine             &E    = h->eng;
    const int64_t       N    = h->N();
    cudaStream_t        s    = h->stream;
    const pibem_params &P    = h->prm;
    const int           L    = E.m + 1;
    const int64_t       ldr  = int64_t(L) * N;
    const int           max_refine = 12;
    int                 finished   = 0;
    std::vector<double> nv;
    auto finish = [&](int c) {
      ColHost &C = E.col[c];
      C.st       = ST_DONE;
      C.seconds  = std::chrono::duration<double>(std::chrono::steady_clock::now() - C.t0).count();
      ++finished;
    };
    bool progress = true;
    while (progress)
      {
        progress = false;
        // right-hand sides of newly admitted columns
        std::vector<int> cols = cols_in(E, ST_RHS);
        if (!cols.empty())
          {
            progress = true;
            eng_apply(h, OP_RHS, cols, E.tmp.p, E.b.p);
            if (E.mixed)
              {
                eng_norms(h, E.b.p, ENG_NBLK_REFINE, nv);
                eng_zero(h, E.x.p, cols);
                eng_copy(h, E.r.p, E.b.p, cols);
                for (int c : cols)
                  {
                    ColHost &C = E.col[c];
                    C.bn_outer = nv[c] > 0 ? std::sqrt(nv[c]) : 1.0; // norms of b: sqrt, 0 -> 1
                    C.r_exact  = true;
                    C.refine   = 0;
                    C.iters    = 0;
                    C.st       = ST_ASSESS;
                  }
              }
            else
              {
                eng_norms(h, E.b.p, ENG_NBLK, nv);
                eng_copy(h, E.x.p, E.b.p, cols); // initial guess = rhs (bem_problem.cc:1295)
                for (int c : cols)
                  {
                    ColHost &C = E.col[c];
                    C.bn_inner = nv[c] > 0 ? std::sqrt(nv[c]) : 1.0;
                    C.its_inner   = 0;
                    C.inner_maxit = P.solver_max_steps;
                    C.itol        = P.solver_tolerance;
                    C.st          = ST_RES;
                  }
              }
          }
        // end of a GMRES cycle: x (plain) or d (mixed) += P^-1 V y
        cols = cols_in(E, ST_CYCLE_END);
        if (!cols.empty())
          {
            progress = true;
            upload_sel(h, cols);
            launch_gmres_lsq(E.S, E.m, E.sel.p, E.H.p, E.g.p, E.kdone.p, E.jvec.p, E.y.p, s);
            eng_zero(h, E.u.p, cols);
            launch_gemv_sub(N, E.S, 0, N, ldr, E.V.p, E.y.p, L, E.u.p, -1.0, s, E.jvec.p, E.sel.p);
            double *tgt = E.mixed ? E.d.p : E.x.p;
            if (E.prec)
              {
                apply_prec(h, E.S, E.u.p, N, E.z.p, s, nullptr, nullptr, 0, nullptr, E.sel.p);
                launch_axpby_sel(N, E.S, E.sel.p, 1.0, E.z.p, 1.0, tgt, s);
              }
            else
              launch_axpby_sel(N, E.S, E.sel.p, 1.0, E.u.p, 1.0, tgt, s);
            for (int c : cols)
              {
                E.h_jvec[c] = -1;
                E.col[c].st = E.mixed ? ST_INNER : ST_RES;
              }
            E.jvec.upload(E.h_jvec, s);
          }
        // mixed: r = b - A64 x
        cols = cols_in(E, ST_TRUERES);
        if (!cols.empty())
          {
            progress = true;
            eng_apply(h, OP_A64, cols, E.x.p, E.w.p);
            eng_copy(h, E.r.p, E.b.p, cols);
            upload_sel(h, cols);
            launch_axpby_sel(N, E.S, E.sel.p, -1.0, E.w.p, 1.0, E.r.p, s);
            for (int c : cols)
              {
                ColHost &C = E.col[c];
                C.r_exact  = true;
                if (C.refine_inc)
                  {
                    C.refine++;
                    C.refine_inc = false;
                  }
                C.st = ST_ASSESS;
              }
          }
        // mixed: r <- r - A32 d
        cols = cols_in(E, ST_R32);
        if (!cols.empty())
          {
            progress = true;
            eng_apply(h, OP_A32, cols, E.d.p, E.w.p);
            upload_sel(h, cols);
            launch_axpby_sel(N, E.S, E.sel.p, -1.0, E.w.p, 1.0, E.r.p, s);
            for (int c : cols)
              {
                ColHost &C = E.col[c];
                C.r_exact  = false;
                C.refine++;
                C.st = ST_ASSESS;
              }
          }
        // mixed: the refinement decision on |r|
        cols = cols_in(E, ST_ASSESS);
        if (!cols.empty())
          {
            progress = true;
            eng_norms(h, E.r.p, ENG_NBLK_REFINE, nv);
            std::vector<int> start;
            for (int c : cols)
              {
                ColHost &C = E.col[c];
                C.rel      = std::sqrt(nv[c]) / C.bn_outer;
                C.ok       = C.rel <= P.solver_tolerance;
                C.itol     = C.ok ? std::numeric_limits<double>::infinity()
                                  : std::max(P.inner_tolerance, 0.5 * P.solver_tolerance / C.rel);
                if (C.final_pass)
                  finish(c);
                else if (C.ok && !C.r_exact)
                  C.st = ST_TRUERES; // confirm the estimate with the FP64-accurate operator
                else if (C.ok || C.refine == max_refine || C.iters >= P.solver_max_steps)
                  {
                    if (!C.r_exact)
                      {
                        C.final_pass = true; // a stop on the step limits: the exact residual
                        C.st         = ST_TRUERES;
                      }
                    else
                      finish(c);
                  }
                else
                  start.push_back(c);
              }
            if (!start.empty())
              {
                // a new correction: d = 0, the inner right-hand side is r
                eng_zero(h, E.d.p, start);
                eng_norms(h, E.r.p, ENG_NBLK, nv);
                for (int c : start)
                  {
                    ColHost &C    = E.col[c];
                    C.bn_inner    = nv[c] > 0 ? std::sqrt(nv[c]) : 1.0;
                    C.its_inner   = 0;
                    C.inner_maxit = P.solver_max_steps - C.iters;
                    C.st          = ST_INNER;
                  }
              }
          }
        // a GMRES restart: w = rhs - A x, and the cycle start or the stop
        const ColStage rst = E.mixed ? ST_INNER : ST_RES;
        cols               = cols_in(E, rst);
        if (!cols.empty())
          {
            progress = true;
            // mixed: A32 on d against r; plain: A64 on x against b
            eng_apply(h, E.mixed ? OP_A32 : OP_A64, cols, E.mixed ? E.d.p : E.x.p, E.w.p);
            upload_sel(h, cols);
            launch_axpby_sel(N, E.S, E.sel.p, 1.0, E.mixed ? E.r.p : E.b.p, -1.0, E.w.p, s);
            eng_norms(h, E.w.p, ENG_NBLK, nv);
            std::vector<int> cyc;
            for (int c : cols)
              {
                ColHost     &C   = E.col[c];
                const double rel = std::sqrt(nv[c]) / C.bn_inner;
                if (rel <= C.itol || C.its_inner >= C.inner_maxit)
                  {
                    if (!E.mixed)
                      {
                        C.rel   = rel;
                        C.iters = C.its_inner;
                        finish(c);
                        continue;
                      }
                    // the correction is done: x += d, then the new residual
                    C.iters += C.its_inner;
                    C.st = ST_XUPD;
                    continue;
                  }
                cyc.push_back(c);
              }
            if (!cyc.empty())
              {
                upload_sel(h, cyc);
                // V[c][0] = w / |w| (and z = V_0 without preconditioner)
                launch_normalize(N, E.S, E.w.p, E.nrm.p, E.V.p, ldr, s, nullptr,
                                 E.prec ? nullptr : E.z.p, E.sel.p);
                if (E.prec)
                  apply_prec(h, E.S, E.V.p, ldr, E.z.p, s, nullptr, nullptr, 0, nullptr, E.sel.p);
                launch_gmres_cycle_init(E.S, E.m, E.sel.p, E.nrm.p, E.g.p, E.kdone.p, E.jvec.p, s);
                for (int c : cyc)
                  {
                    ColHost &C   = E.col[c];
                    E.h_bn[c]    = C.bn_inner;
                    E.h_tol[c]   = C.itol;
                    E.h_its[c]   = C.its_inner;
                    E.h_maxit[c] = C.inner_maxit;
                    E.h_jvec[c]  = 0;
                    C.st         = ST_ARNOLDI;
                  }
                E.bn.upload(E.h_bn, s);
                E.tol.upload(E.h_tol, s);
                E.its.upload(E.h_its, s);
                E.maxit.upload(E.h_maxit, s);
              }
          }
        // mixed: x += d after a correction
        cols = cols_in(E, ST_XUPD);
        if (!cols.empty())
          {
            progress = true;
            upload_sel(h, cols);
            launch_axpby_sel(N, E.S, E.sel.p, 1.0, E.d.p, 1.0, E.x.p, s);
            for (int c : cols)
              {
                ColHost &C = E.col[c];
                if (C.refine == 0)
                  {
                    C.refine_inc = true;
                    C.st         = ST_TRUERES;
                  }
                else
                  C.st = ST_R32;
              }
          }
      }
    // the Arnoldi steps of the columns in a cycle
    std::vector<int> act = cols_in(E, ST_ARNOLDI);
    if (!act.empty())
      {
        eng_cycle(h, act, quantum);
        const int S = E.S;
        PIBEM_CUDA(cudaMemcpyAsync(E.ipin.p, E.jvec.p, sizeof(int) * S, cudaMemcpyDeviceToHost, s));
        PIBEM_CUDA(cudaMemcpyAsync(E.ipin.p + S, E.kdone.p, sizeof(int) * S, cudaMemcpyDeviceToHost, s));
        PIBEM_CUDA(cudaMemcpyAsync(E.ipin.p + 2 * S, E.its.p, sizeof(int) * S, cudaMemcpyDeviceToHost, s));
        PIBEM_CUDA(cudaStreamSynchronize(s));
        bool ended = false;
        for (int c : act)
          {
            ColHost  &C   = E.col[c];
            const int jv  = E.ipin.p[c], it = E.ipin.p[2 * S + c];
            const int now = it - C.its_inner; // steps this column took
            if (E.mixed)
              C.c32 += now;
            else
              C.c64 += now;
            C.its_inner = it;
            E.h_its[c]  = it;
            if (jv <= -2)
              {
                // ended its cycle after -2 - jv steps (the count lsq takes)
                E.h_jvec[c] = -2 - jv;
                C.st        = ST_CYCLE_END;
                ended       = true;
              }
            else
              E.h_jvec[c] = jv;
          }
        if (ended)
          E.jvec.upload(E.h_jvec, s);
      }
    return finished;
  }

  // The double-node constraint lines of BEMProblem::compute_constraints
  // (bem_problem.cc:1405-1579) for the current Dirichlet mask.  Per set, with
  // i its first Dirichlet node in ascending order (else its smallest id), made
  // once, when the loop reaches i:
  //   i Neumann:               x_d - x_i = 0 for the other nodes d;
  //   i Dirichlet, d Neumann:  x_d = tmp_rhs[i];
  //   i, d Dirichlet:          with continuous_gradient, x_i and x_d are the
  //     normal derivatives from the normals and surface gradients (the
  //     reference's flat-edge branch, normal_distance / normal_distance < 1e-4,
  //     is never taken); a line made again keeps its place and takes the new
  //     value, so with several Dirichlet doubles x_i follows the last one.
  // Hanging-node lines do not arise on the conforming meshes taken here.
  void build_constraints(pibem_handle *h)
  {
    const MeshHost &m = h->mesh;
    const int64_t   N = h->N();
    h->con_row.clear();
    h->con_col.clear();
    h->con_p.clear();
    h->con_q.clear();
    h->con_kind.clear();
    std::unordered_map<int32_t, size_t> at;
    auto line = [&](int32_t row) {
      auto it = at.find(row);
      if (it != at.end())
        return it->second;
      at[row] = h->con_row.size();
      h->con_row.push_back(row);
      h->con_col.push_back(-1);
      h->con_p.push_back(-1);
      h->con_q.push_back(-1);
      h->con_kind.push_back(0);
      return h->con_row.size() - 1;
    };
    for (int32_t i = 0; i < int32_t(N); ++i)
      {
        const int32_t *b = m.dbl_ids.data() + m.dbl_off[i], *e = m.dbl_ids.data() + m.dbl_off[i + 1];
        if (e - b < 2)
          continue;
        int32_t first = *b;
        for (const int32_t *d = b; d != e; ++d)
          if (h->dir[*d])
            {
              first = *d;
              break;
            }
        if (i != first)
          continue;
        for (const int32_t *d = b; d != e; ++d)
          {
            if (*d == i)
              continue;
            if (h->dir[i] && h->dir[*d])
              {
                if (!h->prm.continuous_gradient)
                  continue;
                const size_t kd = line(*d), ki = line(i);
                h->con_kind[ki] = 2;
                h->con_p[ki]    = i;
                h->con_q[ki]    = *d;
                h->con_kind[kd] = 2;
                h->con_p[kd]    = *d;
                h->con_q[kd]    = i;
              }
            else if (h->dir[i])
              {
                const size_t kd = line(*d);
                h->con_kind[kd] = 1;
                h->con_p[kd]    = i;
              }
            else
              h->con_col[line(*d)] = i;
          }
      }
    h->con_proj = std::find(h->con_kind.begin(), h->con_kind.end(), uint8_t(2)) != h->con_kind.end();
    cudaStream_t s = h->stream;
    h->d_con_row.upload(h->con_row, s);
    h->d_con_col.upload(h->con_col, s);
    h->d_con_p.upload(h->con_p, s);
    h->d_con_q.upload(h->con_q, s);
    h->d_con_kind.upload(h->con_kind, s);
  }

  void build_preconditioner(pibem_handle *h)
  {
    const Plan   &pl = h->plan;
    const int     nl = int(pl.nleaf_box.size());
    cudaStream_t  s  = h->stream;
    h->blk_ptr.assign(nl + 1, 0);
    h->max_leaf_rows = 0;
    for (int k = 0; k < nl; ++k)
      {
        int64_t nr       = pl.nrow_ptr[k + 1] - pl.nrow_ptr[k];
        h->blk_ptr[k + 1] = h->blk_ptr[k] + nr * nr;
        h->max_leaf_rows  = std::max(h->max_leaf_rows, int(nr));
      }
    h->d_blk_ptr.upload(h->blk_ptr, s);
    DBuf<double> blocks;
    blocks.alloc(h->blk_ptr[nl]);
    int64_t nrows = int64_t(pl.nrows.size());
    if (nrows)
      diag_block_gather_kernel<<<unsigned((nrows + 127) / 128), 128, 0, s>>>(
        nrows, h->d_row_leaf.p, h->d_nrow_ptr.p, h->d_ncol_ptr.p, h->d_nval_ptr.p, h->d_blk_ptr.p,
        h->d_diag_col.p, h->d_S.p, blocks.p);
    PIBEM_CUDA(cudaGetLastError());
    note_launch();
    std::vector<double> hb(h->blk_ptr[nl]), inv(h->blk_ptr[nl]);
    blocks.download(hb.data(), hb.size(), s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    // a constrained row of the solve's operator is its constraint line: the
    // same line in the row's block (its entry where the column is in the block)
    if (!h->con_row.empty())
      {
        std::vector<int64_t> pos(h->N(), -1); // node -> near row position
        for (size_t r = 0; r < pl.nrows.size(); ++r)
          pos[pl.nrows[r]] = int64_t(r);
        for (size_t k = 0; k < h->con_row.size(); ++k)
          {
            const int64_t r = pos[h->con_row[k]];
            const int     lf = pl.row_leaf[r];
            const int64_t r0 = pl.nrow_ptr[lf], n = pl.nrow_ptr[lf + 1] - r0;
            double       *row = &hb[h->blk_ptr[lf] + (r - r0) * n];
            std::fill(row, row + n, 0.0);
            row[r - r0] = 1.0;
            if (h->con_col[k] >= 0)
              {
                const int64_t c = pos[h->con_col[k]];
                if (c >= r0 && c < r0 + n)
                  row[c - r0] = -1.0;
              }
          }
      }
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < nl; ++k)
      {
        int n = int(pl.nrow_ptr[k + 1] - pl.nrow_ptr[k]);
        double *b = &inv[h->blk_ptr[k]];
        if (!invert(n, &hb[h->blk_ptr[k]], b))
          for (int i = 0; i < n; ++i)
            for (int j2 = 0; j2 < n; ++j2)
              b[size_t(i) * n + j2] = i == j2 ? 1.0 : 0.0;
        // stored column by column: the apply reads a column across the rows
        for (int i = 0; i < n; ++i)
          for (int j2 = i + 1; j2 < n; ++j2)
            std::swap(b[size_t(i) * n + j2], b[size_t(j2) * n + i]);
      }
    std::vector<float> inv32(inv.begin(), inv.end());
    h->d_Pinv.upload(inv32, s);
    h->d_Pinv64.release();
    if (h->prm.precision_mode != PIBEM_PRECISION_MIXED) // solves on an FP64-accurate operator
      h->d_Pinv64.upload(inv, s);
  }

  // ILU(0) of the near-field system matrix, the preconditioner the reference
  // builds in BEMFMA::FMA_preconditioner (bem_fma.cc:3080-3411) and factors
  // with Trilinos' PreconditionILU at its defaults (no fill, no diagonal
  // shift; bem_problem.cc:1302): the pattern is each row's near field (the
  // row's leaf columns), the values S = N (Neumann columns) or -D (Dirichlet
  // columns) with alpha on the diagonal of unconstrained Neumann rows, and a
  // constrained row is its constraint line {i: 1, c: +1} as the constraint
  // matrix stores it (:3190-3201).  The factorisation and the triangular
  // substitutions run level by level on the device.
  void build_ilu(pibem_handle *h)
  {
    const Plan   &pl = h->plan;
    const int64_t n  = h->N();
    cudaStream_t  s  = h->stream;
    std::vector<int32_t> pos(n, -1), con(n, -2);
    for (size_t r = 0; r < pl.nrows.size(); ++r)
      pos[pl.nrows[r]] = int32_t(r);
    for (size_t k = 0; k < h->con_row.size(); ++k)
      con[h->con_row[k]] = h->con_col[k];
    // the sorted columns of row i: a view of its leaf's columns, or the line
    auto cols_of = [&](int64_t i, int32_t *pair, const int32_t *&c, int64_t &nc) {
      if (con[i] != -2)
        {
          const int32_t j = con[i];
          nc              = (j >= 0 && j != i) ? 2 : 1;
          pair[0]         = nc == 2 ? std::min<int32_t>(j, int32_t(i)) : int32_t(i);
          pair[1]         = nc == 2 ? std::max<int32_t>(j, int32_t(i)) : int32_t(i);
          c               = pair;
          return;
        }
      if (pos[i] < 0)
        throw Error(PIBEM_EINVAL, "ILU: a node without a near-field row");
      const int lf = pl.row_leaf[pos[i]];
      c            = pl.ncols.data() + pl.ncol_ptr[lf];
      nc           = pl.ncol_ptr[lf + 1] - pl.ncol_ptr[lf];
    };
    std::vector<int64_t> ptr(n + 1, 0), diag(n);
    std::vector<int32_t> lev_lo(n, 0), lev_up(n, 0);
    int64_t              max_row = 0;
    int32_t              pair[2];
    for (int64_t i = 0; i < n; ++i)
      {
        const int32_t *c;
        int64_t        nc;
        cols_of(i, pair, c, nc);
        const int64_t d = std::lower_bound(c, c + nc, int32_t(i)) - c;
        if (d == nc || c[d] != i)
          throw Error(PIBEM_EINVAL, "ILU: a near-field row without its diagonal");
        ptr[i + 1] = ptr[i] + nc;
        diag[i]    = ptr[i] + d;
        max_row    = std::max(max_row, nc);
        int32_t l  = 0;
        for (int64_t k = 0; k < d; ++k)
          l = std::max(l, lev_lo[c[k]] + 1);
        lev_lo[i] = l;
      }
    for (int64_t i = n - 1; i >= 0; --i)
      {
        const int32_t *c;
        int64_t        nc;
        cols_of(i, pair, c, nc);
        int32_t l = 0;
        for (int64_t k = diag[i] - ptr[i] + 1; k < nc; ++k)
          l = std::max(l, lev_up[c[k]] + 1);
        lev_up[i] = l;
      }
    if (max_row * int64_t(sizeof(double) + sizeof(int32_t)) > 200 * 1024)
      throw Error(PIBEM_EINVAL, "ILU: a near-field row longer than the factorisation's shared memory");
    // rows grouped by level (ascending row order within a level)
    auto group = [n](const std::vector<int32_t> &lev, std::vector<int64_t> &lptr,
                     std::vector<int32_t> &rows) {
      const int32_t nlev = n ? *std::max_element(lev.begin(), lev.end()) + 1 : 0;
      lptr.assign(size_t(nlev) + 1, 0);
      for (int64_t i = 0; i < n; ++i)
        ++lptr[lev[i] + 1];
      for (int32_t l = 0; l < nlev; ++l)
        lptr[l + 1] += lptr[l];
      rows.resize(n);
      std::vector<int64_t> at(lptr.begin(), lptr.end() - 1);
      for (int64_t i = 0; i < n; ++i)
        rows[at[lev[i]]++] = int32_t(i);
    };
    std::vector<int32_t> rows_lo, rows_up;
    group(lev_lo, h->ilu_lptr_lo, rows_lo);
    group(lev_up, h->ilu_lptr_up, rows_up);
    h->d_ilu_ptr.upload(ptr, s);
    h->d_ilu_diag.upload(diag, s);
    h->d_ilu_rows_lo.upload(rows_lo, s);
    h->d_ilu_rows_up.upload(rows_up, s);
    h->d_ilu_col.alloc(std::max<int64_t>(1, ptr[n]));
    h->d_ilu_val.alloc(std::max<int64_t>(1, ptr[n]));
    DBuf<int32_t> d_pos, d_con;
    d_pos.upload(pos, s);
    d_con.upload(con, s);
    launch_ilu_fill(n, h->d_ilu_ptr.p, d_pos.p, h->d_row_leaf.p, h->d_nrow_ptr.p, h->d_ncol_ptr.p,
                    h->d_nval_ptr.p, h->d_ncols.p, h->d_S.p, d_con.p, h->d_ilu_col.p, h->d_ilu_val.p,
                    s);
    launch_ilu_factor(h->ilu_lptr_lo, h->d_ilu_rows_lo.p, h->d_ilu_ptr.p, h->d_ilu_col.p,
                      h->d_ilu_val.p, h->d_ilu_diag.p, max_row, s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    h->ilu_on = true;
  }

  void fill_operator_views(pibem_handle *h)
  {
    const Plan &pl = h->plan;
    auto        fill = [&](auto &op) {
      op.p             = pl.p;
      op.K             = pl.K;
      op.n_near_leaves = int(pl.nleaf_box.size());
      op.n_rows        = int64_t(pl.nrows.size());
      op.row_leaf      = h->d_row_leaf.p;
      op.nrows         = h->d_nrows.p;
      op.ncols         = h->d_ncols.p;
      op.nrow_ptr      = h->d_nrow_ptr.p;
      op.ncol_ptr      = h->d_ncol_ptr.p;
      op.nval_ptr      = h->d_nval_ptr.p;
      op.near_sched    = h->d_near_sched.p;
      op.n_p2m_leaves  = int(pl.pleaf_box.size());
      op.prow_ptr      = h->d_prow_ptr.p;
      op.pleaf_box     = h->d_pleaf_box.p;
      op.prow_dof      = h->d_prow_dof.p;
      op.lleaf_box     = h->d_lleaf_box.p;
      op.q_src         = h->d_q_src.p;
      op.ch_start      = h->d_ch_start.p;
      op.ch_cnt        = h->d_ch_cnt.p;
      op.ch_op         = h->d_ch_op.p;
      op.m2l_chunk_end = pl.m2l_chunk_end;
      op.max_chunk_pairs = pl.ch_cnt.empty() ? 0 : *std::max_element(pl.ch_cnt.begin(), pl.ch_cnt.end());
      op.n_boxes         = h->tree.nb;
      op.up_chunk_ptr  = pl.up_chunk_ptr;
      op.down_chunk_ptr = pl.down_chunk_ptr;
      op.up_box_ptr    = pl.up_box_ptr;
      op.down_box_ptr  = pl.down_box_ptr;
      op.up_box        = h->d_up_box.p;
      op.down_box      = h->d_down_box.p;
      op.up_q          = h->d_up_q.p;
      op.down_q        = h->d_down_q.p;
      op.up_q_ptr      = h->d_up_q_ptr.p;
      op.down_q_ptr    = h->d_down_q_ptr.p;
      op.up_child8     = h->d_up_child8.p;
      op.down_par      = h->d_down_par.p;
      op.down_oct      = h->d_down_oct.p;
      op.m2l_yslot     = h->d_m2l_yslot.p;
      op.down_m2l_beg  = h->d_down_m2l_beg.p;
      op.down_m2l_end  = h->d_down_m2l_end.p;
      op.lv_op0        = int(pl.offsets.size() / 3);
      op.down_l2l_level.assign(pl.down_box_ptr.size(), 0);
      for (size_t l = 0; l + 1 < pl.down_box_ptr.size(); ++l)
        for (int i = pl.down_box_ptr[l]; i < pl.down_box_ptr[l + 1]; ++i)
          if (pl.down_par[i] >= 0)
            op.down_l2l_level[l] = 1;
      op.n_pairs       = int64_t(pl.q_src.size());
      op.Tc            = nullptr; // made by set_bc
      op.max_near_cols = 0;
      for (size_t k2 = 0; k2 + 1 < pl.ncol_ptr.size(); ++k2)
        op.max_near_cols = std::max<int64_t>(op.max_near_cols, pl.ncol_ptr[k2 + 1] - pl.ncol_ptr[k2]);
      op.n_m2p_tgt     = int(pl.m2p_tgt.size());
      op.n_m2p_pairs   = int64_t(pl.m2p_src.size());
      op.n_m2p_items   = h->m2p_items;
      op.n_m2p_tnodes  = h->m2p_tnodes;
      op.m2p_tgt       = h->d_m2p_tgt.p;
      op.m2p_src       = h->d_m2p_src.p;
      op.m2p_src_ptr   = h->d_m2p_src_ptr.p;
      op.m2p_pair_tgt  = h->d_m2p_pair_tgt.p;
      op.m2p_item_ptr  = h->d_m2p_item_ptr.p;
      op.m2p_item_pair = h->d_m2p_item_pair.p;
      op.m2p_tnode_ptr = h->d_m2p_tnode_ptr.p;
      op.m2p_tnodes    = h->d_m2p_tnodes.p;
    };
    fill(h->op64);
    fill(h->op32);
    h->op64.T1      = h->d_T1.p;
    h->op64.T2      = h->d_T2.p;
    h->op64.W       = h->d_W.p;
    h->op64.Wff     = h->d_Wff.n ? h->d_Wff.p : nullptr;
    h->op64.ops     = h->d_ops.p;
    h->op64.oz_images = h->d_ozimg.n ? h->d_ozimg.p : nullptr;
    h->op64.oz_ecol   = h->d_ozecol.n ? h->d_ozecol.p : nullptr;
    h->op64.dev_err   = h->d_err.p;
    h->op64.ops_ff  = h->prm.precision_mode == PIBEM_PRECISION_FLOAT_FLOAT ? h->d_opsff.p : nullptr;
    h->op32.T1      = h->d_T1f.p;
    h->op32.T2      = h->d_T2f.p;
    h->op32.W       = h->d_Wf.p;
    h->op32.ops     = h->d_opsf.p;
    h->op32.lv_ops  = h->d_lvopsf.p;
    h->op32.dev_err = h->d_err.p;
    h->op32.tc_images = h->d_tcimg.n ? h->d_tcimg.p : nullptr;
    h->op32.tc_stages = h->prm.m2l_stages;
    h->op32.tc_err    = h->d_err.p;
    TreeDev &td               = h->td;
    td.nb                     = h->tree.nb;
    td.N                      = int(h->N());
    td.L                      = h->tree.L;
    td.parent                 = h->d_parent.p;
    td.child_first            = h->d_child_first.p;
    td.nchild                 = h->d_nchild.p;
    td.digit                  = h->d_digit.p;
    td.nbeg                   = h->d_nbeg.p;
    td.nend                   = h->d_nend.p;
    td.node_sorted            = h->d_node_sorted.p;
    td.center                 = h->d_center.p;
    td.delta                  = h->d_delta.p;
    td.xyz                    = h->d_xyz.p;
  }

  // Every index a kernel will dereference is checked here, on the host, so that
  // an inconsistent plan becomes PIBEM_EINVAL instead of a device fault.
  void validate_plan(const MeshHost &m, const Tree &t, const Plan &pl, int nq)
  {
    auto need = [](bool ok, const char *what) {
      if (!ok)
        throw Error(PIBEM_EINVAL, std::string("internal plan check failed: ") + what);
    };
    const int64_t N = m.n_dofs, Q = m.n_cells * nq;
    const int     nl = int(pl.nleaf_box.size());
    need(pl.nrow_ptr.size() == size_t(nl + 1) && pl.ncol_ptr.size() == size_t(nl + 1) &&
           pl.nent_ptr.size() == size_t(nl + 1) && pl.nval_ptr.size() == size_t(nl + 1),
         "near pointer sizes");
    need(int64_t(pl.gather_ptr.size()) == pl.ncol_ptr[nl] + 1, "gather_ptr size");
    for (int k = 0; k < nl; ++k)
      {
        int64_t nr = pl.nrow_ptr[k + 1] - pl.nrow_ptr[k], nc = pl.ncol_ptr[k + 1] - pl.ncol_ptr[k],
                ne = pl.nent_ptr[k + 1] - pl.nent_ptr[k];
        need(nr > 0 && nc > 0 && ne > 0, "empty near leaf");
        need(pl.nval_ptr[k + 1] - pl.nval_ptr[k] == nr * ((nc + 3) / 4 * 4), "near value block size");
        need(pl.nval_ptr[k] % 4 == 0, "near value block alignment");
        need(pl.nleaf_box[k] >= 0 && pl.nleaf_box[k] < t.nb, "near leaf box");
        for (int64_t e = pl.nent_ptr[k]; e < pl.nent_ptr[k + 1]; ++e)
          {
            const NearEntry &E = pl.entries[e];
            need(E.cell >= 0 && E.cell < m.n_cells, "entry cell");
            need(E.qmask != 0 && (nq == 64 || (E.qmask >> nq) == 0), "entry quad mask");
            for (int j = 0; j < 4; ++j)
              need(E.lcol[j] >= 0 && E.lcol[j] < nc, "entry column");
          }
        for (int64_t c = pl.ncol_ptr[k]; c < pl.ncol_ptr[k + 1]; ++c)
          {
            need(pl.gather_ptr[c] <= pl.gather_ptr[c + 1], "gather order");
            for (int g = pl.gather_ptr[c]; g < pl.gather_ptr[c + 1]; ++g)
              need(pl.gather_ids[g] >= 0 && pl.gather_ids[g] < 4 * ne, "gather id");
          }
      }
    for (int32_t v : pl.nrows)
      need(v >= 0 && v < N, "near row node");
    for (int32_t v : pl.ncols)
      need(v >= 0 && v < N, "near column node");
    for (size_t r = 0; r < pl.row_leaf.size(); ++r)
      need(pl.row_leaf[r] >= 0 && pl.row_leaf[r] < nl && pl.nrow_ptr[pl.row_leaf[r]] <= int64_t(r) &&
             int64_t(r) < pl.nrow_ptr[pl.row_leaf[r] + 1],
           "row leaf");
    const int np = int(pl.pleaf_box.size());
    need(pl.prow_ptr.size() == size_t(np + 1), "p2m row ptr");
    need(pl.pcontrib_ptr.size() == pl.prow_dof.size() + 1, "p2m contrib ptr");
    for (int k = 0; k < np; ++k)
      need(pl.prow_ptr[k + 1] > pl.prow_ptr[k] && pl.pleaf_box[k] >= 0 && pl.pleaf_box[k] < t.nb,
           "p2m leaf");
    for (int32_t v : pl.prow_dof)
      need(v >= 0 && v < N, "p2m row dof");
    for (int32_t v : pl.pcontrib_q)
      need(v >= 0 && int64_t(v) < 4 * Q, "p2m contribution");
    const int noff = int(pl.offsets.size() / 3);
    const int64_t nq_pairs = int64_t(pl.q_src.size());
    need(pl.q_op.size() == size_t(nq_pairs), "pair arrays");
    for (size_t i = 0; i < pl.q_src.size(); ++i)
      need(pl.q_src[i] >= 0 && pl.q_src[i] < t.nb && pl.q_op[i] >= 0 && pl.q_op[i] < noff + 16,
           "translation pair");
    for (size_t ch = 0; ch < pl.ch_start.size(); ++ch)
      {
        need(pl.ch_cnt[ch] > 0 && pl.ch_cnt[ch] <= 128 && pl.ch_start[ch] >= 0 &&
               int64_t(pl.ch_start[ch]) + pl.ch_cnt[ch] <= nq_pairs,
             "translation chunk");
        for (int i = 0; i < pl.ch_cnt[ch]; ++i)
          need(pl.q_op[pl.ch_start[ch] + i] == pl.ch_op[ch], "chunk operator");
      }
    need(pl.up_q_ptr.size() == pl.up_box.size() + 1 && pl.down_q_ptr.size() == pl.down_box.size() + 1,
         "gather sizes");
    for (int32_t v : pl.up_box)
      need(v >= 0 && v < t.nb, "up box");
    for (int32_t v : pl.down_box)
      need(v >= 0 && v < t.nb, "down box");
    for (int32_t v : pl.up_q)
      need(v >= 0 && v < nq_pairs, "up pair");
    need(pl.up_chunk_ptr.size() == size_t(t.L + 2) && pl.down_chunk_ptr.size() == size_t(t.L + 2) &&
           pl.up_box_ptr.size() == size_t(t.L + 2) && pl.down_box_ptr.size() == size_t(t.L + 2) &&
           pl.up_box_ptr[t.L + 1] == int(pl.up_box.size()) &&
           pl.down_box_ptr[t.L + 1] == int(pl.down_box.size()) &&
           pl.up_chunk_ptr[t.L + 1] <= int(pl.ch_start.size()) &&
           pl.down_chunk_ptr[t.L + 1] <= int(pl.ch_start.size()),
         "level range sizes");
    for (int l = 1; l <= t.L; ++l)
      need(pl.up_chunk_ptr[l] <= pl.up_chunk_ptr[l + 1] && pl.down_chunk_ptr[l] <= pl.down_chunk_ptr[l + 1] &&
             pl.up_box_ptr[l] <= pl.up_box_ptr[l + 1] && pl.down_box_ptr[l] <= pl.down_box_ptr[l + 1] &&
             pl.up_chunk_ptr[l] >= 0 && pl.down_chunk_ptr[l] >= 0 && pl.up_box_ptr[l] >= 0 &&
             pl.down_box_ptr[l] >= 0,
           "level ranges");
    for (int32_t v : pl.down_q)
      need(v >= 0 && v < nq_pairs, "down pair");
    need(pl.up_child8.size() == 8 * pl.up_box.size() && pl.down_par.size() == pl.down_box.size() &&
           pl.down_oct.size() == pl.down_box.size(),
         "level tables");
    for (int32_t v : pl.up_child8)
      need(v >= -1 && v < t.nb, "up child");
    need(pl.m2l_yslot.size() == size_t(pl.n_m2l) && pl.down_m2l_beg.size() == pl.down_box.size() &&
           pl.down_m2l_end.size() == pl.down_box.size(),
         "target-major M2L tables");
    {
      std::vector<char> seen(pl.m2l_yslot.size(), 0);
      for (int32_t v : pl.m2l_yslot)
        {
          need(v >= 0 && v < int64_t(seen.size()) && !seen[v], "M2L slot");
          seen[v] = 1;
        }
      for (size_t i = 0; i < pl.down_box.size(); ++i)
        need(pl.down_m2l_beg[i] >= 0 && pl.down_m2l_beg[i] <= pl.down_m2l_end[i] &&
               pl.down_m2l_end[i] <= int64_t(pl.m2l_yslot.size()),
             "M2L slot range");
    }
    for (size_t i = 0; i < pl.down_box.size(); ++i)
      need(pl.down_par[i] >= -1 && pl.down_par[i] < t.nb && pl.down_oct[i] < 8 &&
             (pl.down_par[i] < 0 || pl.down_q_ptr[i + 1] > pl.down_q_ptr[i]),
           "down box table");
    need(pl.m2l_src_ptr.size() == pl.m2l_tgt.size() + 1, "m2l ptr");
    for (size_t i = 0; i < pl.m2l_src.size(); ++i)
      need(pl.m2l_src[i] >= 0 && pl.m2l_src[i] < t.nb && pl.m2l_off[i] >= 0 && pl.m2l_off[i] < noff,
           "m2l pair");
    for (int32_t v : pl.m2l_tgt)
      need(v >= 0 && v < t.nb, "m2l target");
    need(pl.m2p_src_ptr.size() == pl.m2p_tgt.size() + 1, "m2p ptr");
    for (int32_t v : pl.m2p_tgt)
      need(v >= 0 && v < t.nb && t.nend[v] > t.nbeg[v], "m2p target");
    for (int32_t v : pl.m2p_src)
      need(v >= 0 && v < t.nb, "m2p source");
    for (int b = 1; b < t.nb; ++b)
      need(t.parent[b] >= 0 && t.parent[b] < b && t.digit[b] >= 0 && t.digit[b] < 8, "box parent");
    for (int b = 0; b < t.nb; ++b)
      need(t.nchild[b] == 0 || (t.child_first[b] > b && t.child_first[b] + t.nchild[b] <= t.nb),
           "box children");
  }

  void set_mesh_impl(pibem_handle *h, int64_t n_nodes, const double *xyz, int64_t n_cells,
                     const int32_t *cells, const int32_t *doff, const int32_t *dids)
  {
    auto t0 = std::chrono::steady_clock::now();
    auto tp = t0;
    auto phase = [&](int i) {
      const auto now     = std::chrono::steady_clock::now();
      h->setup_phase[i]  = std::chrono::duration<double>(now - tp).count();
      tp                 = now;
    };
    std::fill(h->setup_phase, h->setup_phase + PIBEM_SETUP_PHASES, 0.0);
    drop_graph(h); // its kernels carry the previous mesh's sizes
    h->d_con_nrm.release();
    if (n_nodes <= 0 || n_cells <= 0 || !xyz || !cells)
      throw Error(PIBEM_EINVAL, "empty mesh");
    if ((doff == nullptr) != (dids == nullptr))
      throw Error(PIBEM_EINVAL, "double_offsets and double_ids must both be given or both NULL");
    if (n_nodes > INT32_MAX / 8 || n_cells * 64 > INT32_MAX)
      throw Error(PIBEM_EINVAL, "mesh too large for 32-bit node / quadrature ids");
    const pibem_params &P = h->prm;
    cudaStream_t        s = h->stream;
    h->mesh_ok = h->bc_ok = false;
    for (int64_t i = 0; i < 4 * n_cells; ++i)
      if (cells[i] < 0 || cells[i] >= n_nodes)
        throw Error(PIBEM_EINVAL, "cell node id out of range");
    for (int64_t i = 0; i < 3 * n_nodes; ++i)
      if (!std::isfinite(xyz[i]))
        throw Error(PIBEM_EINVAL, "non-finite node coordinate");
    std::vector<std::vector<int32_t>> sets(static_cast<size_t>(n_nodes));
    for (int64_t i = 0; i < n_nodes; ++i)
      {
        std::vector<int32_t> &set = sets[size_t(i)];
        set.push_back(int32_t(i));
        if (doff)
          for (int32_t k = doff[i]; k < doff[i + 1]; ++k)
            {
              if (dids[k] < 0 || dids[k] >= n_nodes)
                throw Error(PIBEM_EINVAL, "double node id out of range");
              set.push_back(dids[k]);
            }
        std::sort(set.begin(), set.end());
        set.erase(std::unique(set.begin(), set.end()), set.end());
      }
    MeshHost &m = h->mesh;
    mirror_mesh(n_nodes, xyz, n_cells, cells, sets, P.double_body != 0, P.symmetry_plane_z_level, m);
    n_nodes = m.n_nodes;
    n_cells = m.n_cells;
    m.elem_off.assign(n_nodes + 1, 0);
    for (int64_t i = 0; i < 4 * n_cells; ++i)
      m.elem_off[m.cells[i] + 1]++;
    for (int64_t i = 0; i < n_nodes; ++i)
      m.elem_off[i + 1] += m.elem_off[i];
    m.elem_ids.assign(m.elem_off[n_nodes], 0);
    {
      std::vector<int32_t> fillp(m.elem_off.begin(), m.elem_off.end() - 1);
      for (int64_t c = 0; c < n_cells; ++c)
        for (int j = 0; j < 4; ++j)
          m.elem_ids[fillp[m.cells[4 * c + j]]++] = int32_t(c);
    }
    // quadrature rules
    gauss_rule_2d(P.quadrature_order, h->gpts, h->gw);
    h->nq    = int(h->gw.size());
    for (int v = 0; v < 4; ++v)
      telles_rule_2d(P.singular_quadrature_order, v, h->tpts[v], h->tw[v]);
    h->n_tel = int(h->tw[0].size());
    // device mesh and quadrature data
    h->d_xyz.upload(m.xyz, s);
    h->d_cells.upload(m.cells, s);
    h->d_dbl_off.upload(m.dbl_off, s);
    h->d_dbl_ids.upload(m.dbl_ids, s);
    h->d_gpts.upload(h->gpts, s);
    h->d_elem_off.upload(m.elem_off, s);
    h->d_elem_ids.upload(m.elem_ids, s);
    h->d_gw.upload(h->gw, s);
    const int64_t Q = n_cells * h->nq;
    h->d_qpts.alloc(3 * Q);
    h->d_qnrm.alloc(3 * Q);
    h->d_qjxw.alloc(Q);
    h->d_qshape.alloc(4 * Q);
    launch_quad_data(n_cells, h->nq, h->d_xyz.p, h->d_cells.p, h->d_gpts.p, h->d_gw.p,
                     h->d_qpts.p, h->d_qnrm.p, h->d_qjxw.p, h->d_qshape.p, s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    phase(0);
    // octree and lists on the device; on the host when a list exceeds the
    // device builder's capacity (the same tree either way)
    if (!build_tree_device(m, h->d_xyz.p, h->d_qpts.p, h->nq, P.num_octree_levels,
                           P.max_nodes_per_childless_block, h->d_dbl_off.p, h->d_dbl_ids.p,
                           h->d_elem_off.p, h->d_elem_ids.p, h->tree, s))
      {
        std::vector<double> qpts(3 * Q);
        h->d_qpts.download(qpts.data(), qpts.size(), s);
        PIBEM_CUDA(cudaStreamSynchronize(s));
        build_tree(m, qpts, h->nq, P.num_octree_levels, P.max_nodes_per_childless_block, h->tree);
        h->tree_on_host = true;
      }
    else
      h->tree_on_host = false;
    phase(1);
    build_plan(m, h->tree, h->nq, P.fma_truncation_order, h->plan,
               P.m2l_chunk_pairs > 0 ? P.m2l_chunk_pairs : 128);
    phase(2);
    const Tree &t  = h->tree;
    const Plan &pl = h->plan;
    const int   K  = pl.K;
    validate_plan(m, t, pl, h->nq);
    // tree arrays
    std::vector<double> center(3 * size_t(t.nb));
    for (int b = 0; b < t.nb; ++b)
      t.center(b, &center[3 * size_t(b)]);
    h->d_parent.upload(t.parent, s);
    h->d_child_first.upload(t.child_first, s);
    h->d_nchild.upload(t.nchild, s);
    h->d_digit.upload(t.digit, s);
    h->d_nbeg.upload(t.nbeg, s);
    h->d_nend.upload(t.nend, s);
    h->d_node_sorted.upload(t.node_sorted, s);
    h->d_center.upload(center, s);
    h->d_delta.upload(t.delta, s);
    // plan arrays
    h->d_nrow_ptr.upload(pl.nrow_ptr, s);
    h->d_ncol_ptr.upload(pl.ncol_ptr, s);
    h->d_nval_ptr.upload(pl.nval_ptr, s);
    {
      // one-column near SpMV schedule: the leaves by value bytes, largest first
      const int        nl = int(pl.nleaf_box.size());
      std::vector<int> order(nl);
      for (int k = 0; k < nl; ++k)
        order[k] = k;
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return pl.nval_ptr[a + 1] - pl.nval_ptr[a] > pl.nval_ptr[b + 1] - pl.nval_ptr[b];
      });
      std::vector<int64_t> sched(4 * size_t(nl));
      for (int i = 0; i < nl; ++i)
        {
          const int     k  = order[i];
          const int64_t nr = pl.nrow_ptr[k + 1] - pl.nrow_ptr[k], nc = pl.ncol_ptr[k + 1] - pl.ncol_ptr[k];
          sched[4 * size_t(i) + 0] = pl.nval_ptr[k];
          sched[4 * size_t(i) + 1] = pl.ncol_ptr[k];
          sched[4 * size_t(i) + 2] = pl.nrow_ptr[k];
          sched[4 * size_t(i) + 3] = int64_t(uint64_t(nr) | (uint64_t(nc) << 32));
        }
      h->d_near_sched.upload(sched, s);
    }
    h->d_nent_ptr.upload(pl.nent_ptr, s);
    h->d_row_leaf.upload(pl.row_leaf, s);
    h->d_nrows.upload(pl.nrows, s);
    h->d_ncols.upload(pl.ncols, s);
    h->d_entries.upload(pl.entries, s);
    h->d_gather_ptr.upload(pl.gather_ptr, s);
    h->d_gather_ids.upload(pl.gather_ids, s);
    h->d_pleaf_box.upload(pl.pleaf_box, s);
    h->d_prow_ptr.upload(pl.prow_ptr, s);
    h->d_prow_dof.upload(pl.prow_dof, s);
    h->d_pcontrib_ptr.upload(pl.pcontrib_ptr, s);
    h->d_pcontrib_q.upload(pl.pcontrib_q, s);
    h->d_lleaf_box.upload(pl.lleaf_box, s);
    h->d_m2l_tgt.upload(pl.m2l_tgt, s);
    h->d_m2l_src_ptr.upload(pl.m2l_src_ptr, s);
    h->d_m2l_src.upload(pl.m2l_src, s);
    h->d_m2l_off.upload(pl.m2l_off, s);
    h->d_m2p_tgt.upload(pl.m2p_tgt, s);
    h->d_m2p_src_ptr.upload(pl.m2p_src_ptr, s);
    h->d_m2p_src.upload(pl.m2p_src, s);
    h->d_q_src.upload(pl.q_src, s);

    h->d_ch_start.upload(pl.ch_start, s);
    h->d_ch_cnt.upload(pl.ch_cnt, s);
    h->d_ch_op.upload(pl.ch_op, s);
    h->d_up_box.upload(pl.up_box, s);
    h->d_down_box.upload(pl.down_box, s);
    h->d_up_q.upload(pl.up_q, s);
    h->d_down_q.upload(pl.down_q, s);
    h->d_up_q_ptr.upload(pl.up_q_ptr, s);
    h->d_down_q_ptr.upload(pl.down_q_ptr, s);
    h->d_up_child8.upload(pl.up_child8, s);
    h->d_down_par.upload(pl.down_par, s);
    h->d_down_oct.upload(pl.down_oct, s);
    h->d_m2l_yslot.upload(pl.m2l_yslot, s);
    h->d_down_m2l_beg.upload(pl.down_m2l_beg, s);
    h->d_down_m2l_end.upload(pl.down_m2l_end, s);
    // M2P work items: one per (pair, node of the pair's target box)
    {
      const size_t         nt = pl.m2p_tgt.size();
      std::vector<int32_t> pair_tgt(pl.m2p_src.size()), tnodes;
      std::vector<int64_t> item_ptr(pl.m2p_src.size() + 1, 0), tnode_ptr(nt + 1, 0);
      for (size_t ti = 0; ti < nt; ++ti)
        {
          const int b = pl.m2p_tgt[ti];
          for (int k = t.nbeg[b]; k < t.nend[b]; ++k)
            if (t.node_sorted[k] < m.n_dofs)
              tnodes.push_back(t.node_sorted[k]);
          tnode_ptr[ti + 1] = int64_t(tnodes.size());
          const int64_t nn  = tnode_ptr[ti + 1] - tnode_ptr[ti];
          if (nn == 0)
            throw Error(PIBEM_EINVAL, "internal plan check failed: M2P target without collocation nodes");
          for (int64_t e = pl.m2p_src_ptr[ti]; e < pl.m2p_src_ptr[ti + 1]; ++e)
            {
              pair_tgt[e]     = int32_t(ti);
              item_ptr[e + 1] = item_ptr[e] + nn;
            }
        }
      h->m2p_items  = item_ptr.back();
      h->m2p_tnodes = tnode_ptr.back();
      std::vector<int32_t> item_pair(size_t(h->m2p_items));
      for (size_t e = 0; e + 1 < item_ptr.size(); ++e)
        std::fill(item_pair.begin() + item_ptr[e], item_pair.begin() + item_ptr[e + 1], int32_t(e));
      h->d_m2p_item_pair.upload(item_pair, s);
      h->d_m2p_pair_tgt.upload(pair_tgt, s);
      h->d_m2p_item_ptr.upload(item_ptr, s);
      h->d_m2p_tnode_ptr.upload(tnode_ptr, s);
      h->d_m2p_tnodes.upload(tnodes, s);
    }
    ensure_fmm_tables(P.device, s);
    phase(3);
    // diagonal column of every row inside its leaf (block-Jacobi)
    {
      std::vector<int32_t> dc(pl.nrows.size());
      for (size_t k = 0; k + 1 < pl.nrow_ptr.size(); ++k)
        for (int64_t r = pl.nrow_ptr[k]; r < pl.nrow_ptr[k + 1]; ++r)
          {
            auto b = pl.ncols.begin() + pl.ncol_ptr[k], e = pl.ncols.begin() + pl.ncol_ptr[k + 1];
            auto it = std::lower_bound(b, e, pl.nrows[r]);
            if (it == e || *it != pl.nrows[r])
              throw Error(PIBEM_EINVAL, "collocation node missing from its own near field");
            dc[r] = int32_t(it - b);
          }
      h->d_diag_col.upload(dc, s);
    }
    // near-field integrals
    {
      const int            nl = int(pl.nleaf_box.size());
      std::vector<int64_t> item_ptr(nl + 1, 0);
      for (int k = 0; k < nl; ++k)
        item_ptr[k + 1] = item_ptr[k] + (pl.nrow_ptr[k + 1] - pl.nrow_ptr[k]) *
                                          (pl.nent_ptr[k + 1] - pl.nent_ptr[k]);
      h->d_item_ptr.upload(item_ptr, s);
      const int64_t nval = pl.nval_ptr[nl];
      h->d_N.alloc(nval);
      h->d_D.alloc(nval);
      h->d_N.zero(s);
      h->d_D.zero(s);
      DBuf<double> staging;
      int64_t      st_items = std::min<int64_t>(item_ptr[nl], int64_t(1) << 24);
      int64_t      maxrow   = 0;
      for (int k = 0; k < nl; ++k)
        maxrow = std::max<int64_t>(maxrow, pl.nent_ptr[k + 1] - pl.nent_ptr[k]);
      st_items = std::max(st_items, maxrow);
      staging.alloc(8 * std::max<int64_t>(st_items, 1));
      DBuf<int64_t>            sing_list;
      DBuf<unsigned long long> sing_count;
      sing_list.alloc(std::max<int64_t>(st_items, 1));
      sing_count.alloc(1);
      NearAssemblyArgs a;
      a.n_items       = item_ptr[nl];
      a.n_leaves      = nl;
      a.item_ptr      = h->d_item_ptr.p;
      a.row_ptr       = h->d_nrow_ptr.p;
      a.ent_ptr       = h->d_nent_ptr.p;
      a.val_ptr       = h->d_nval_ptr.p;
      a.col_ptr       = h->d_ncol_ptr.p;
      a.h_item_ptr    = item_ptr.data();
      a.h_ent_ptr     = pl.nent_ptr.data();
      a.h_val_ptr     = pl.nval_ptr.data();
      a.rows          = h->d_nrows.p;
      a.ents          = h->d_entries.p;
      a.xyz           = h->d_xyz.p;
      a.cells         = h->d_cells.p;
      a.dbl_off       = h->d_dbl_off.p;
      a.dbl_ids       = h->d_dbl_ids.p;
      a.nq            = h->nq;
      a.qpts          = h->d_qpts.p;
      a.qnrm          = h->d_qnrm.p;
      a.qjxw          = h->d_qjxw.p;
      a.qshape        = h->d_qshape.p;
      a.gather_ptr    = h->d_gather_ptr.p;
      a.gather_ids    = h->d_gather_ids.p;
      a.staging       = staging.p;
      a.staging_items = st_items;
      a.sing_list     = sing_list.p;
      a.sing_count    = sing_count.p;
      a.Nval          = h->d_N.p;
      a.Dval          = h->d_D.p;
      if (nl > 0)
        {
          // the singular rules live in constant memory shared by every handle of
          // the process: one near-field assembly at a time
          std::lock_guard<std::mutex> lock(g_near_assembly_mu);
          set_telles_rules(h->tpts, h->tw, h->n_tel, s);
          launch_near_assembly(a, s);
          PIBEM_CUDA(cudaStreamSynchronize(s));
        }
      PIBEM_CUDA(cudaStreamSynchronize(s));
      h->d_S.alloc(nval);
      h->d_S32.alloc(nval);
    }
    phase(4);
    // P2M and L2P tables
    {
      const int64_t nrows_p = int64_t(pl.prow_dof.size());
      const int64_t K4      = (K + 3) / 4 * 4;
      h->d_T1.alloc(nrows_p * K4);
      h->d_T2.alloc(nrows_p * K4);
      h->d_T1.zero(s);
      h->d_T2.zero(s);
      launch_p2m_tables(nrows_p, K, pl.p, int(pl.pleaf_box.size()), h->d_prow_ptr.p,
                        h->d_pleaf_box.p, h->d_pcontrib_ptr.p, h->d_pcontrib_q.p, h->d_center.p,
                        h->d_delta.p, h->d_qpts.p, h->d_qnrm.p, h->d_qjxw.p, h->d_qshape.p,
                        h->d_T1.p, h->d_T2.p, s);
      h->d_T1f.alloc(nrows_p * K4);
      h->d_T2f.alloc(nrows_p * K4);
      launch_convert_d2f(nrows_p * K4, h->d_T1.p, h->d_T1f.p, s);
      launch_convert_d2f(nrows_p * K4, h->d_T2.p, h->d_T2f.p, s);
      const int64_t npos = int64_t(pl.lnode_ids.size());
      // rows padded to K4 values (zero beyond K): 16-byte aligned rows for L2P
      h->d_W.alloc(npos * K4);
      h->d_W.zero(s);
      launch_l2p_tables(npos, K, int(K4), int(pl.lleaf_box.size()), h->d_nrow_ptr.p,
                        h->d_lleaf_box.p, h->d_nrows.p, h->d_xyz.p, h->d_center.p, h->d_delta.p,
                        h->d_W.p, s);
      h->d_Wf.alloc(npos * K4);
      launch_convert_d2f(npos * K4, h->d_W.p, h->d_Wf.p, s);
      h->d_Wff.release();
      if (P.precision_mode != PIBEM_PRECISION_FP64 && npos > 0)
        {
          h->d_Wff.alloc(npos * K4);
          launch_convert_d2ff(npos * K4, h->d_W.p, h->d_Wff.p, s);
        }
    }
    PIBEM_CUDA(cudaStreamSynchronize(s));
    phase(5);
    // translation operators
    {
      std::vector<double> m2m, l2l, m2l;
      build_m2m_ops(pl.p, m2m);
      build_l2l_ops(pl.p, l2l);
      const int nof = int(pl.offsets.size() / 3);
      m2l.assign(size_t(std::max(nof, 1)) * K * K, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
      for (int o = 0; o < nof; ++o)
        build_m2l_op(pl.p, pl.offsets[3 * o], pl.offsets[3 * o + 1], pl.offsets[3 * o + 2],
                     &m2l[size_t(o) * K * K]);
      // concatenated table [M2L offsets | 8 M2M | 8 L2L], [in][out] per operator
      const int nops = nof + 16;
      std::vector<double> all(size_t(nops) * K * K);
      std::copy(m2l.begin(), m2l.begin() + size_t(nof) * K * K, all.begin());
      std::copy(m2m.begin(), m2m.end(), all.begin() + size_t(nof) * K * K);
      std::copy(l2l.begin(), l2l.end(), all.begin() + size_t(nof + 8) * K * K);
      std::vector<double> td;
      std::vector<float>  tf;
      transpose_ops(all, nops, K, td);
      h->d_ops.upload(td, s);
      transpose_ops(all, nops, K, tf);
      h->d_opsf.upload(tf, s);
      {
        // the 16 level operators (8 M2M, 8 L2L), each padded to 16 bytes
        const size_t        kk = fused_level_ops_floats(K) / 16;
        std::vector<float> lv(16 * kk, 0.0f);
        for (int o = 0; o < 16; ++o)
          std::copy(tf.begin() + size_t(nof + o) * K * K, tf.begin() + size_t(nof + o + 1) * K * K,
                    lv.begin() + o * kk);
        h->d_lvopsf.upload(lv, s);
      }
      {
        std::vector<float2> ff(td.size());
        for (size_t i = 0; i < td.size(); ++i)
          {
            const float hi = float(td[i]);
            ff[i]          = make_float2(hi, float(td[i] - double(hi)));
          }
        h->d_opsff.upload(ff, s);
      }
      h->d_tcimg.release();
      if (h->use_tc && tc_geometry(K).ok)
        {
          std::vector<float> img;
          build_tc_images(all, nops, K, img);
          h->d_tcimg.upload(img, s);
        }
      h->d_ozimg.release();
      h->d_ozecol.release();
      if (h->use_tc && h->prm.precision_mode != PIBEM_PRECISION_FP64 && ozaki_ok(K))
        {
          std::vector<uint16_t> oimg;
          std::vector<int16_t>  ecol;
          build_ozaki_images(all, nops, K, oimg, ecol);
          h->d_ozimg.upload(oimg, s);
          h->d_ozecol.upload(ecol, s);
        }
      h->d_err.alloc(1);
      h->d_err.zero(s);
      PIBEM_CUDA(cudaStreamSynchronize(s));
    }
    phase(6);
    fill_operator_views(h);
    // free setup-only buffers
    h->d_entries.release();
    h->d_gather_ptr.release();
    h->d_gather_ids.release();
    h->d_item_ptr.release();
    h->d_pcontrib_ptr.release();
    h->d_pcontrib_q.release();
    PIBEM_CUDA(cudaStreamSynchronize(s));
    h->bytes_resident = h->d_N.bytes() * 3 + h->d_S32.bytes() + h->d_T1.bytes() * 2 +
                        h->d_T1f.bytes() * 2 + h->d_W.bytes() + h->d_Wf.bytes() +
                        h->d_ops.bytes() + h->d_opsf.bytes() + h->d_qpts.bytes() * 2 +
                        h->d_qshape.bytes() + h->d_qjxw.bytes() +
                        (P.precision_mode != PIBEM_PRECISION_FP64
                           ? 2 * h->d_N.bytes() + h->d_T1.bytes() + h->d_W.bytes()
                           : 0);
    if (P.hbm_budget_gb > 0 && double(h->bytes_resident) > P.hbm_budget_gb * 1e9)
      throw Error(PIBEM_ENOMEM_HBM, "resident operator exceeds the HBM budget");
    phase(7);
    h->mesh_ok       = true;
    h->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  void set_bc_impl(pibem_handle *h, const uint8_t *mask)
  {
    drop_graph(h);
    if (!h->mesh_ok)
      throw Error(PIBEM_EINVAL, "pibem_set_bc before pibem_set_mesh");
    if (!mask)
      throw Error(PIBEM_EINVAL, "null mask");
    const int64_t N = h->N();
    cudaStream_t  s = h->stream;
    h->dir.assign(mask, mask + N);
    h->have_dirichlet = false;
    for (auto &v : h->dir)
      {
        v = v ? 1 : 0;
        h->have_dirichlet |= v != 0;
      }
    h->d_dir.upload(h->dir, s);
    // alpha = -N 1 (interior), -1 - N 1 (exterior)
    h->d_alpha.alloc(N);
    h->d_t1.alloc(N);
    std::vector<double> ones(N, -1.0);
    h->d_t1.upload(ones, s);
    ker1_apply64(h, h->d_t1.p, h->d_alpha.p);
    if (h->prm.is_external_flow)
      {
        std::vector<double> m1(N, 1.0);
        h->d_t2.upload(m1, s);
        launch_axpby(N, -1.0, h->d_t2.p, 1.0, h->d_alpha.p, s);
      }
    const Plan &pl = h->plan;
    launch_build_system_matrix(pl.nval_ptr.back(), int(pl.nleaf_box.size()), h->d_nval_ptr.p,
                               h->d_ncol_ptr.p, h->d_nrow_ptr.p, h->d_nrows.p, h->d_ncols.p,
                               h->d_dir.p, h->d_alpha.p, h->d_N.p, h->d_D.p, h->d_S.p, h->d_S32.p,
                               s);
    // FP64-accurate near field as FP32 pairs: S, and S of the complementary mask
    // for the right-hand side (not needed by the plain FP64 path)
    h->d_Sff.release();
    h->d_Srff.release();
    h->d_Tcr.release();
    if (h->prm.precision_mode != PIBEM_PRECISION_FP64 && pl.nval_ptr.back() > 0)
      {
        const int64_t nval = pl.nval_ptr.back();
        h->d_Sff.alloc(nval);
        launch_convert_d2ff(nval, h->d_S.p, h->d_Sff.p, s);
        std::vector<uint8_t> dirc(h->dir.size());
        for (size_t i = 0; i < dirc.size(); ++i)
          dirc[i] = h->dir[i] ? 0 : 1;
        DBuf<uint8_t> d_dirc;
        d_dirc.upload(dirc, s);
        DBuf<double> Sr;
        Sr.alloc(nval);
        launch_build_system_matrix(nval, int(pl.nleaf_box.size()), h->d_nval_ptr.p, h->d_ncol_ptr.p,
                                   h->d_nrow_ptr.p, h->d_nrows.p, h->d_ncols.p, d_dirc.p,
                                   h->d_alpha.p, h->d_N.p, h->d_D.p, Sr.p, nullptr, s);
        h->d_Srff.alloc(nval);
        launch_convert_d2ff(nval, Sr.p, h->d_Srff.p, s);
        // P2M strengths of the right-hand side, one table row per row:
        // N on Dirichlet, -D on Neumann DoFs (the combined table of the
        // complementary mask)
        const int64_t nr = int64_t(pl.prow_dof.size());
        const int     K4 = (pl.K + 3) / 4 * 4;
        h->d_Tcr.alloc(std::max<int64_t>(1, nr * K4));
        launch_combine_p2m<double>(nr, K4, h->d_prow_dof.p, d_dirc.p, h->d_T1.p, h->d_T2.p,
                                   h->d_Tcr.p, s);
        PIBEM_CUDA(cudaStreamSynchronize(s));
      }
    // combined-strength P2M tables of the system operator (one row read per row)
    {
      const int64_t nr = int64_t(pl.prow_dof.size());
      const int     K4 = (pl.K + 3) / 4 * 4;
      h->d_Tc.alloc(std::max<int64_t>(1, nr * K4));
      h->d_Tcf.alloc(std::max<int64_t>(1, nr * K4));
      launch_combine_p2m<double>(nr, K4, h->d_prow_dof.p, h->d_dir.p, h->d_T1.p, h->d_T2.p,
                                 h->d_Tc.p, s);
      launch_combine_p2m<float>(nr, K4, h->d_prow_dof.p, h->d_dir.p, h->d_T1f.p, h->d_T2f.p,
                                h->d_Tcf.p, s);
      h->op64.Tc = h->d_Tc.p;
      h->op32.Tc = h->d_Tcf.p;
    }
    build_constraints(h);
    h->ilu_on = false;
    if (h->prm.preconditioner == 1)
      build_preconditioner(h);
    else if (h->prm.preconditioner == 2)
      build_ilu(h);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    h->bc_ok = true;
  }

  // A bounded device wait that gave up (tensor-core translations) is reported
  // as PIBEM_ETIMEDOUT; the flag is cleared for the next call.
  void check_device_error(pibem_handle *h)
  {
    if (!h->d_err.n)
      return;
    int e = 0;
    h->d_err.download(&e, 1, h->stream);
    PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    if (e)
      {
        h->d_err.zero(h->stream);
        throw Error(PIBEM_ETIMEDOUT, "a bounded device wait timed out in the translations");
      }
  }

  // BEMProblem::compute_rhs (bem_problem.cc:1220-1260): rhs = -(alpha + N) phi_D + D dphi_N
  // with phi_D = tmp on Dirichlet nodes, dphi_N = tmp on Neumann nodes.  The
  // near field applies N and D to the masked columns; the far field takes
  // both layers in one expansion per column, with strengths N on Dirichlet and
  // -D on Neumann DoFs (MODE_SWAPPED): R columns of far field instead of 2R.
  void compute_rhs_dev(pibem_handle *h, int R, const double *tmp, double *rhs)
  {
    const int64_t N = h->N();
    cudaStream_t  s = h->stream;
    h->d_t1.alloc(size_t(R) * N);
    h->d_t2.alloc(size_t(R) * N);
    h->d_t3.alloc(size_t(2 * R) * N);
    launch_split_masks(N, R, tmp, h->d_dir.p, h->d_t1.p, h->d_t2.p, s);
    set_modes(h, R, MODE_SWAPPED);
    if (h->op64.ops_ff && h->d_Srff.p && near_ff_fits(h->op64))
      {
        // FP64-accurate operator: the near part is one SpMV with the matrix of
        // the complementary mask (N on Dirichlet, -D on Neumann columns, alpha
        // on Dirichlet rows) on float-float pairs; rhs = -(near + far)
        record(h, 0);
        near_apply<double>(h, h->op64, R, nullptr, h->d_Srff.p, tmp, rhs, s);
        record(h, 1);
        {
          // P2M from the right-hand side's combined table (one row read per row)
          struct TcSwap
          {
            OperatorDev<double> &op;
            const double        *saved;
            ~TcSwap() { op.Tc = saved; }
          } swap{h->op64, h->op64.Tc};
          h->op64.Tc = h->d_Tcr.p;
          far_field<double>(h, h->op64, h->d_M64, h->d_L64, h->d_m2p64, h->d_Y64, R, h->d_modes.p,
                            tmp, rhs, true);
        }
        finish_timing(h, 0);
        h->cnt64 += R;
        launch_axpby(int64_t(R) * N, 0.0, rhs, -1.0, rhs, s);
        return;
      }
    double *yN = h->d_t3.p, *yD = h->d_t3.p + int64_t(R) * N;
    record(h, 0);
    launch_near_spmv<double>(h->op64, R, int(N), h->d_N.p, h->d_t1.p, yN, false, s);
    launch_near_spmv<double>(h->op64, R, int(N), h->d_D.p, h->d_t2.p, yD, false, s);
    record(h, 1);
    far_field<double>(h, h->op64, h->d_M64, h->d_L64, h->d_m2p64, h->d_Y64, R, h->d_modes.p, tmp, yN);
    finish_timing(h, 0);
    h->cnt64 += R;
    // yN = N phi_D + far (N phi_D - D dphi_N), yD = near D dphi_N
    launch_rhs_combine(N, R, tmp, h->d_dir.p, h->d_alpha.p, yN, yD, rhs, s);
  }

  // L2 projection of R columns onto the Q1 space of the mesh (device in/out):
  // mode 0 normals, 1 surface gradients of u, 2 gradients of (u, dudn).
  void projection_dev(pibem_handle *h, int mode, int R, const double *du, const double *dd,
                      double *dout)
  {
    const int64_t N = h->N();
    h->d_proj.alloc(l2_projection_work(N, h->mesh.n_cells_body, R));
    ProjectionArgs a;
    a.mode     = mode;
    a.n_nodes  = N;
    a.n_cells  = h->mesh.n_cells_body; // a double body's reflected cells come after these
    a.nq       = h->nq;
    a.R        = R;
    a.cells    = h->d_cells.p;
    a.elem_off = h->d_elem_off.p;
    a.elem_ids = h->d_elem_ids.p;
    a.xyz      = h->d_xyz.p;
    a.gpts     = h->d_gpts.p;
    a.qshape   = h->d_qshape.p;
    a.qjxw     = h->d_qjxw.p;
    a.qnrm     = h->d_qnrm.p;
    a.u        = du;
    a.dudn     = dd;
    a.work     = h->d_proj.p;
    a.out      = dout;
    l2_projection(a, h->stream);
  }

  // ConstrainedOperator::distribute_rhs (include/constrained_matrix.h:172-181):
  // the constrained rows of b take their lines' values.
  void constrain_rhs(pibem_handle *h, int R, const double *tmp, double *b)
  {
    const int nc = int(h->con_row.size());
    if (nc == 0)
      return;
    const int64_t N = h->N();
    if (h->con_proj)
      {
        if (!h->d_con_nrm.p)
          {
            h->d_con_nrm.alloc(3 * N);
            projection_dev(h, 0, 1, nullptr, nullptr, h->d_con_nrm.p);
          }
        h->d_con_sg.alloc(size_t(3) * R * N);
        projection_dev(h, 1, R, tmp, nullptr, h->d_con_sg.p);
      }
    launch_constraint_rhs(nc, R, N, h->d_con_row.p, h->d_con_kind.p, h->d_con_p.p, h->d_con_q.p, tmp,
                          h->con_proj ? h->d_con_nrm.p : nullptr,
                          h->con_proj ? h->d_con_sg.p : nullptr, b, h->stream);
  }

  // The mixed path forms its right-hand sides and FP64 residuals with the
  // FP64-accurate float-float translations (FP64 near field and expansions):
  // the handle's FP64 operator view takes them for the scope of this guard.
  struct FfGuard
  {
    OperatorDev<double> &op;
    const float2        *prev;
    FfGuard(pibem_handle *h) : op(h->op64), prev(h->op64.ops_ff)
    {
      if (h->prm.precision_mode == PIBEM_PRECISION_MIXED)
        op.ops_ff = h->d_opsff.p;
    }
    ~FfGuard() { op.ops_ff = prev; }
  };

  void solve_dev(pibem_handle *h, int R, double *phi, double *dphi, const double *tmp,
                 pibem_solve_stats *st)
  {
    if (!h->bc_ok)
      throw Error(PIBEM_EINVAL, "pibem_solve before pibem_set_bc");
    if (h->slots_open)
      throw Error(PIBEM_EINVAL, "pibem_solve while request slots are open (pibem_slots_close first)");
    auto          t0 = std::chrono::steady_clock::now();
    const int64_t N  = h->N();
    cudaStream_t  s  = h->stream;
    const pibem_params &P = h->prm;
    h->cnt64 = h->cnt32 = 0;
    FfGuard ff(h);
    engine_open(h, R, P.gmres_restart);
    Engine &E = h->eng;
    PIBEM_CUDA(cudaMemcpyAsync(E.tmp.p, tmp, sizeof(double) * R * N, cudaMemcpyDeviceToDevice, s));
    for (int c = 0; c < R; ++c)
      {
        E.col[c].st = ST_RHS;
        E.col[c].t0 = t0;
      }
    for (int64_t rounds = 0;; ++rounds)
      {
        bool all = true;
        for (int c = 0; c < R; ++c)
          all = all && E.col[c].st == ST_DONE;
        if (all)
          break;
        // every round finishes a column, moves one on or runs at least one
        // Arnoldi step, and each column takes at most about 13 (max_steps + 4)
        // rounds; this bound only guards against an internal error
        if (rounds > 64 * (int64_t(P.solver_max_steps) + 16) * R)
          throw Error(PIBEM_ECUDA, "internal error: the solve engine does not advance");
        engine_advance(h);
      }
    launch_scatter(N, R, E.x.p, h->d_dir.p, phi, dphi, s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    check_device_error(h);
    double worst = 0;
    int    iters = 0, refine = 0;
    for (int c = 0; c < R; ++c)
      {
        worst  = std::max(worst, E.col[c].rel);
        iters  = std::max(iters, E.col[c].iters);
        refine = std::max(refine, E.col[c].refine);
      }
    if (st)
      {
        st->iterations        = iters;
        st->refinement_steps  = E.mixed ? refine : 0;
        st->fp64_matvecs      = h->cnt64;
        st->fp32_matvecs      = h->cnt32;
        st->relative_residual = worst;
        st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      }
    if (!(worst <= P.solver_tolerance))
      throw Error(PIBEM_ENOCONV, "GMRES did not reach the tolerance (relative residual " +
                                   std::to_string(worst) + ")");
  }

  // host <-> device staging of the host-pointer entry points, in the handle's
  // grow-only slots
  struct HostIO
  {
    pibem_handle *h;
    int           next = 0;
    double *in(const double *hp, size_t n)
    {
      DBuf<double> &b = h->io_buf[next++];
      b.upload(hp, n, h->stream);
      return b.p;
    }
    double *scratch(size_t n)
    {
      DBuf<double> &b = h->io_buf[next++];
      b.alloc(n);
      return b.p;
    }
  };
} // namespace

extern "C"
{
  int pibem_create(const pibem_params *params, pibem_handle **out)
  {
    if (!params || !out)
      return PIBEM_EINVAL;
    *out = nullptr;
    const pibem_params &P = *params;
    if (P.fma_truncation_order < 1 || P.fma_truncation_order > 10 || P.num_octree_levels < 1 ||
        P.num_octree_levels > 20 || P.max_nodes_per_childless_block < 1 ||
        P.quadrature_order < 1 || P.quadrature_order > 8 || P.singular_quadrature_order < 1 ||
        P.singular_quadrature_order > 12 || P.gmres_restart < 1 || P.solver_max_steps < 1 ||
        !(P.solver_tolerance > 0) || P.precision_mode < PIBEM_PRECISION_FP64 ||
        P.precision_mode > PIBEM_PRECISION_FLOAT_FLOAT || P.m2l_engine < PIBEM_M2L_TENSOR_CORE ||
        P.m2l_engine > PIBEM_M2L_CUDA_CORE ||
        (P.m2l_chunk_pairs != 0 && (P.m2l_chunk_pairs < 16 || P.m2l_chunk_pairs > 128)) ||
        (P.m2l_stages != 0 && P.m2l_stages != 2 && P.m2l_stages != 3) || P.preconditioner < 0 ||
        P.preconditioner > 2)
      return PIBEM_EINVAL;
    pibem_handle *h = new (std::nothrow) pibem_handle();
    if (!h)
      return PIBEM_ENOMEM_HBM;
    h->prm = P;
    try
      {
        PIBEM_CUDA(cudaSetDevice(P.device));
        PIBEM_CUDA(cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking));
        int prio_lo = 0, prio_hi = 0; // least, greatest
        PIBEM_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
        PIBEM_CUDA(cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio_lo));
        PIBEM_CUDA(cudaStreamCreateWithPriority(&h->main_hp, cudaStreamNonBlocking, prio_hi));
        for (cudaEvent_t *e : {&h->ev_fork, &h->ev_up, &h->ev_side, &h->ev_main})
          PIBEM_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        h->stream = h->own;
        const char *env = std::getenv("PIBEM_PHASE_TIMING");
        h->timing       = env && env[0] == '1';
        h->use_tc       = P.m2l_engine != PIBEM_M2L_CUDA_CORE;
        for (auto &e : h->ev)
          PIBEM_CUDA(cudaEventCreate(&e));
      }
    catch (const Error &e)
      {
        int c = e.code;
        delete h;
        return c;
      }
    *out = h;
    return PIBEM_OK;
  }

  int pibem_destroy(pibem_handle *h)
  {
    if (!h)
      return PIBEM_EINVAL;
    cudaSetDevice(h->prm.device);
    if (h->stream)
      cudaStreamSynchronize(h->stream);
    for (auto &e : h->ev)
      if (e)
        cudaEventDestroy(e);
    for (cudaEvent_t e : {h->ev_fork, h->ev_up, h->ev_side, h->ev_main})
      if (e)
        cudaEventDestroy(e);
    for (cudaStream_t st : {h->side, h->main_hp})
      if (st)
        {
          cudaStreamSynchronize(st);
          cudaStreamDestroy(st);
        }
    cudaStream_t own = h->own;
    drop_graph(h);
    delete h;
    if (own)
      cudaStreamDestroy(own);
    return PIBEM_OK;
  }

  const char *pibem_last_error(const pibem_handle *h) { return h ? h->err.c_str() : "null handle"; }

  int pibem_set_stream(pibem_handle *h, void *stream)
  {
    return guarded(h, [&] { h->stream = stream ? (cudaStream_t)stream : h->own; });
  }

  int pibem_set_mesh(pibem_handle *h, int64_t n_nodes, const double *xyz, int64_t n_cells,
                     const int32_t *cell_nodes, const int32_t *doff, const int32_t *dids)
  {
    return guarded(h, [&] { set_mesh_impl(h, n_nodes, xyz, n_cells, cell_nodes, doff, dids); });
  }

  int pibem_set_bc(pibem_handle *h, const uint8_t *mask)
  {
    return guarded(h, [&] { set_bc_impl(h, mask); });
  }

  int pibem_fmm_matvec(pibem_handle *h, int32_t R, const double *phi, const double *dphi,
                       double *oN, double *oD)
  {
    return guarded(h, [&] {
      if (!h->mesh_ok)
        throw Error(PIBEM_EINVAL, "pibem_fmm_matvec before pibem_set_mesh");
      if (R < 1 || !phi || !dphi || !oN || !oD)
        throw Error(PIBEM_EINVAL, "bad arguments");
      const size_t n = size_t(R) * h->N();
      HostIO       io{h};
      double      *dp = io.in(phi, n), *dd = io.in(dphi, n);
      double      *on = io.scratch(n), *od = io.scratch(n);
      if (h->d_dir.n == 0)
        {
          std::vector<uint8_t> z(h->N(), 0);
          h->d_dir.upload(z, h->stream);
        }
      fmm_apply64(h, R, dp, dd, on, od);
      PIBEM_CUDA(cudaMemcpyAsync(oN, on, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaMemcpyAsync(oD, od, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int pibem_compute_alpha(pibem_handle *h, double *alpha)
  {
    return guarded(h, [&] {
      if (!h->bc_ok)
        throw Error(PIBEM_EINVAL, "pibem_compute_alpha before pibem_set_bc");
      h->d_alpha.download(alpha, h->N(), h->stream);
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int pibem_apply_preconditioner(pibem_handle *h, int32_t R, const double *v, double *z)
  {
    return guarded(h, [&] {
      if (!h->bc_ok)
        throw Error(PIBEM_EINVAL, "pibem_apply_preconditioner before pibem_set_bc");
      if (R < 1 || !v || !z)
        throw Error(PIBEM_EINVAL, "bad arguments");
      const int64_t N  = h->N();
      const size_t  n  = size_t(R) * N;
      HostIO        io{h};
      double       *dv = io.in(v, n), *dz = io.scratch(n);
      if (h->prm.preconditioner == 0)
        PIBEM_CUDA(cudaMemcpyAsync(dz, dv, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      else
        apply_prec(h, R, dv, N, dz, h->stream);
      PIBEM_CUDA(cudaMemcpyAsync(z, dz, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int pibem_system_matvec(pibem_handle *h, int32_t R, const double *x, double *y)
  {
    return guarded(h, [&] {
      if (!h->bc_ok)
        throw Error(PIBEM_EINVAL, "pibem_system_matvec before pibem_set_bc");
      if (R < 1 || !x || !y)
        throw Error(PIBEM_EINVAL, "bad arguments");
      const size_t n  = size_t(R) * h->N();
      HostIO       io{h};
      double      *dx = io.in(x, n), *dy = io.scratch(n);
      if (h->prm.precision_mode == PIBEM_PRECISION_MIXED && std::getenv("PIBEM_MATVEC_FP32"))
        system_apply32(h, R, dx, dy);
      else
        system_apply64(h, R, dx, dy);
      check_device_error(h);
      PIBEM_CUDA(cudaMemcpyAsync(y, dy, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int pibem_compute_rhs(pibem_handle *h, int32_t R, const double *tmp, double *rhs)
  {
    return guarded(h, [&] {
      if (!h->bc_ok)
        throw Error(PIBEM_EINVAL, "pibem_compute_rhs before pibem_set_bc");
      const size_t n  = size_t(R) * h->N();
      HostIO       io{h};
      double      *dt = io.in(tmp, n), *db = io.scratch(n);
      compute_rhs_dev(h, R, dt, db);
      PIBEM_CUDA(cudaMemcpyAsync(rhs, db, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int pibem_solve(pibem_handle *h, int32_t R, double *phi, double *dphi, const double *tmp,
                  pibem_solve_stats *st)
  {
    int rc = guarded(h, [&] {
      if (R < 1 || !phi || !dphi || !tmp)
        throw Error(PIBEM_EINVAL, "bad arguments");
      const size_t n  = size_t(R) * h->N();
      HostIO       io{h};
      double      *dp = io.in(phi, n), *dd = io.in(dphi, n), *dt = io.in(tmp, n);
      int          code = PIBEM_OK;
      std::string  msg;
      try
        {
          solve_dev(h, R, dp, dd, dt, st);
        }
      catch (const Error &e)
        {
          if (e.code != PIBEM_ENOCONV)
            throw;
          code = e.code;
          msg  = e.what();
        }
      PIBEM_CUDA(cudaMemcpyAsync(phi, dp, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaMemcpyAsync(dphi, dd, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
      if (code != PIBEM_OK)
        throw Error(code, msg);
    });
    return rc;
  }

  int pibem_solve_device(pibem_handle *h, int32_t R, double *phi, double *dphi, const double *tmp,
                         pibem_solve_stats *st)
  {
    return guarded(h, [&] {
      if (R < 1 || !phi || !dphi || !tmp)
        throw Error(PIBEM_EINVAL, "bad arguments");
      solve_dev(h, R, phi, dphi, tmp, st);
    });
  }

  // L2 projections (BEMProblem::compute_normals / compute_surface_gradients /
  // compute_gradients, source/bem_problem.cc:1747-2070)
  // ---- request slots: continuous batching of solves on one mesh ----------
  int pibem_slots_open(pibem_handle *h, int32_t max_slots)
  {
    return guarded(h, [&] {
      if (!h->bc_ok)
        throw Error(PIBEM_EINVAL, "pibem_slots_open before pibem_set_bc");
      engine_open(h, max_slots, h->prm.gmres_restart);
      h->slots_open = true;
    });
  }

  int pibem_slots_close(pibem_handle *h)
  {
    return guarded(h, [&] {
      h->slots_open = false;
      h->eng.col.assign(h->eng.S, ColHost());
    });
  }

  int pibem_slots_submit(pibem_handle *h, int64_t request_id, const double *tmp_rhs, int32_t *slot)
  {
    return guarded(h, [&] {
      if (!h->slots_open)
        throw Error(PIBEM_EINVAL, "pibem_slots_submit before pibem_slots_open");
      if (!tmp_rhs)
        throw Error(PIBEM_EINVAL, "null tmp_rhs");
      Engine &E = h->eng;
      int     c = 0;
      while (c < E.S && E.col[c].st != ST_FREE)
        ++c;
      if (c == E.S)
        throw Error(PIBEM_EAGAIN, "no free slot");
      const int64_t N = h->N();
      PIBEM_CUDA(cudaMemcpyAsync(E.tmp.p + int64_t(c) * N, tmp_rhs, sizeof(double) * N,
                                 cudaMemcpyHostToDevice, h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
      E.col[c]     = ColHost();
      E.col[c].st  = ST_RHS;
      E.col[c].rid = request_id;
      E.col[c].t0  = std::chrono::steady_clock::now();
      if (slot)
        *slot = c;
    });
  }

  int pibem_slots_step(pibem_handle *h, int32_t max_steps, int32_t *n_active, int32_t *n_done)
  {
    return guarded(h, [&] {
      if (!h->slots_open)
        throw Error(PIBEM_EINVAL, "pibem_slots_step before pibem_slots_open");
      FfGuard ff(h);
      Engine &E   = h->eng;
      bool    any = false;
      for (const auto &c : E.col)
        any = any || (c.st != ST_FREE && c.st != ST_DONE);
      if (any)
        engine_advance(h, max_steps);
      check_device_error(h);
      int act = 0, done = 0;
      for (const auto &c : E.col)
        {
          act += c.st != ST_FREE && c.st != ST_DONE;
          done += c.st == ST_DONE;
        }
      if (n_active)
        *n_active = act;
      if (n_done)
        *n_done = done;
    });
  }

  int pibem_slots_collect(pibem_handle *h, int64_t *request_id, double *phi, double *dphi_dn,
                          pibem_solve_stats *stats)
  {
    return guarded(h, [&] {
      if (!h->slots_open)
        throw Error(PIBEM_EINVAL, "pibem_slots_collect before pibem_slots_open");
      Engine &E = h->eng;
      int     c = -1;
      for (int k = 0; k < E.S; ++k)
        if (E.col[k].st == ST_DONE && (c < 0 || E.col[k].rid < E.col[c].rid))
          c = k;
      if (c < 0)
        throw Error(PIBEM_EAGAIN, "no finished request");
      const int64_t N = h->N();
      cudaStream_t  s = h->stream;
      HostIO        io{h};
      double       *dp = io.scratch(size_t(N)), *dd = io.scratch(size_t(N));
      // known entries from tmp_rhs, unknown ones from the solution
      PIBEM_CUDA(cudaMemcpyAsync(dp, E.tmp.p + int64_t(c) * N, sizeof(double) * N,
                                 cudaMemcpyDeviceToDevice, s));
      PIBEM_CUDA(cudaMemcpyAsync(dd, E.tmp.p + int64_t(c) * N, sizeof(double) * N,
                                 cudaMemcpyDeviceToDevice, s));
      launch_scatter(N, 1, E.x.p + int64_t(c) * N, h->d_dir.p, dp, dd, s);
      if (phi)
        PIBEM_CUDA(cudaMemcpyAsync(phi, dp, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
      if (dphi_dn)
        PIBEM_CUDA(cudaMemcpyAsync(dphi_dn, dd, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
      PIBEM_CUDA(cudaStreamSynchronize(s));
      const ColHost &C = E.col[c];
      if (request_id)
        *request_id = C.rid;
      if (stats)
        {
          stats->iterations        = C.iters;
          stats->refinement_steps  = E.mixed ? C.refine : 0;
          stats->fp64_matvecs      = C.c64;
          stats->fp32_matvecs      = C.c32;
          stats->relative_residual = C.rel;
          stats->seconds           = C.seconds;
        }
      const bool conv = C.rel <= h->prm.solver_tolerance;
      const double rel = C.rel;
      E.col[c] = ColHost();
      if (!conv)
        throw Error(PIBEM_ENOCONV, "request did not reach the tolerance (relative residual " +
                                     std::to_string(rel) + ")");
    });
  }

  static int projection(pibem_handle *h, int mode, int32_t R, const double *u, const double *dudn,
                        double *out)
  {
    return guarded(h, [&] {
      if (!h->mesh_ok)
        throw Error(PIBEM_EINVAL, "L2 projection before pibem_set_mesh");
      if (R < 1 || !out || (mode > 0 && !u) || (mode == 2 && !dudn))
        throw Error(PIBEM_EINVAL, "bad arguments");
      const int64_t N = h->N(), n = size_t(R) * N;
      HostIO        io{h};
      const double *du = mode > 0 ? io.in(u, n) : nullptr;
      const double *dd = mode == 2 ? io.in(dudn, n) : nullptr;
      double       *dout = io.scratch(size_t(3) * n);
      projection_dev(h, mode, R, du, dd, dout);
      PIBEM_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost,
                                 h->stream));
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int pibem_compute_normals(pibem_handle *h, double *normals)
  {
    return projection(h, 0, 1, nullptr, nullptr, normals);
  }

  int pibem_compute_surface_gradients(pibem_handle *h, int32_t R, const double *u, double *grad)
  {
    return projection(h, 1, R, u, nullptr, grad);
  }

  int pibem_compute_gradients(pibem_handle *h, int32_t R, const double *phi, const double *dphi_dn,
                              double *grad)
  {
    return projection(h, 2, R, phi, dphi_dn, grad);
  }

  int pibem_device_bytes(const pibem_handle *h, uint64_t *bytes)
  {
    if (!h || !bytes)
      return PIBEM_EINVAL;
    *bytes = uint64_t(h->device_bytes());
    return PIBEM_OK;
  }

  int pibem_setup_phases(pibem_handle *h, double *seconds)
  {
    return guarded(h, [&] {
      if (!seconds)
        throw Error(PIBEM_EINVAL, "null output");
      std::copy(h->setup_phase, h->setup_phase + PIBEM_SETUP_PHASES, seconds);
    });
  }

  int pibem_tree_info_get(pibem_handle *h, pibem_tree_info *info)
  {
    return guarded(h, [&] {
      if (!h->mesh_ok || !info)
        throw Error(PIBEM_EINVAL, "no mesh");
      info->n_boxes       = h->tree.nb;
      info->n_levels      = h->tree.L;
      info->n_leaves      = int(h->tree.childless.size());
      info->n_m2l_pairs   = h->plan.n_m2l;
      info->n_m2p_pairs   = h->plan.n_m2p;
      info->near_nnz      = pibem_near_nnz(h);
      info->p2m_rows      = int64_t(h->plan.prow_dof.size());
      info->n_quad_points = h->mesh.n_cells * h->nq;
      info->n_m2l_offsets = int(h->plan.offsets.size() / 3);
      info->setup_seconds = h->setup_seconds;
      info->octree_on_device = h->tree_on_host ? 0 : 1;
    });
  }

  int pibem_tree_boxes(pibem_handle *h, int32_t *level, int32_t *parent, int32_t *nchild,
                       double *pmin, double *delta, int32_t *n_nodes, int32_t *n_quads)
  {
    return guarded(h, [&] {
      if (!h->mesh_ok)
        throw Error(PIBEM_EINVAL, "no mesh");
      const Tree &t = h->tree;
      for (int b = 0; b < t.nb; ++b)
        {
          level[b]  = t.level[b];
          parent[b] = t.parent[b];
          nchild[b] = t.nchild[b];
          for (int k = 0; k < 3; ++k)
            pmin[3 * b + k] = t.pmin[3 * b + k];
          delta[b]   = t.delta[b];
          n_nodes[b] = t.nend[b] - t.nbeg[b];
          n_quads[b] = t.qend[b] - t.qbeg[b];
        }
    });
  }

  int pibem_tree_list_sublevels(pibem_handle *h, int32_t box)
  {
    if (!h || !h->mesh_ok || box < 0 || box >= h->tree.nb)
      return -1;
    return int(h->tree.nn[box].size());
  }

  int pibem_tree_list(pibem_handle *h, int32_t kind, int32_t box, int32_t sub, int32_t *out,
                      int32_t cap)
  {
    if (!h || !h->mesh_ok || box < 0 || box >= h->tree.nb || kind < 0 || kind > 2)
      return -1;
    const auto &L = kind == 0 ? h->tree.nn[box] : (kind == 1 ? h->tree.il[box] : h->tree.nil[box]);
    if (sub < 0 || sub >= int(L.size()))
      return -1;
    const auto &v = L[sub];
    for (int i = 0; i < int(v.size()) && i < cap; ++i)
      out[i] = v[i];
    return int(v.size());
  }

  int64_t pibem_near_nnz(pibem_handle *h)
  {
    if (!h || !h->mesh_ok)
      return -1;
    // distinct (row, col) pairs = sum of leaf block sizes (without row padding)
    const Plan &pl = h->plan;
    int64_t     s  = 0;
    for (size_t k = 0; k + 1 < pl.nrow_ptr.size(); ++k)
      s += (pl.nrow_ptr[k + 1] - pl.nrow_ptr[k]) * (pl.ncol_ptr[k + 1] - pl.ncol_ptr[k]);
    return s;
  }

  int pibem_near_export(pibem_handle *h, int32_t *rows, int32_t *cols, double *Nout, double *Dout)
  {
    return guarded(h, [&] {
      if (!h->mesh_ok)
        throw Error(PIBEM_EINVAL, "no mesh");
      const Plan         &pl = h->plan;
      const int64_t       nv = pl.nval_ptr.back();
      std::vector<double> Nv(nv), Dv(nv);
      h->d_N.download(Nv.data(), nv, h->stream);
      h->d_D.download(Dv.data(), nv, h->stream);
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
      const int64_t nnz = pibem_near_nnz(h);
      // rows sorted globally: collect (row, col, idx) and sort
      std::vector<std::pair<std::pair<int, int>, int64_t>> all;
      all.reserve(nv);
      for (size_t k = 0; k + 1 < pl.nrow_ptr.size(); ++k)
        {
          int64_t nc = pl.ncol_ptr[k + 1] - pl.ncol_ptr[k], ld = (nc + 3) / 4 * 4;
          for (int64_t r = pl.nrow_ptr[k]; r < pl.nrow_ptr[k + 1]; ++r)
            for (int64_t c = 0; c < nc; ++c)
              all.push_back({{pl.nrows[r], pl.ncols[pl.ncol_ptr[k] + c]},
                             pl.nval_ptr[k] + (r - pl.nrow_ptr[k]) * ld + c});
        }
      std::sort(all.begin(), all.end());
      for (int64_t i = 0; i < nnz; ++i)
        {
          rows[i] = all[i].first.first;
          cols[i] = all[i].first.second;
          Nout[i] = Nv[all[i].second];
          Dout[i] = Dv[all[i].second];
        }
    });
  }

  int pibem_quad_points(pibem_handle *h, double *pts)
  {
    return guarded(h, [&] {
      if (!h->mesh_ok)
        throw Error(PIBEM_EINVAL, "no mesh");
      h->d_qpts.download(pts, h->d_qpts.n, h->stream);
      PIBEM_CUDA(cudaStreamSynchronize(h->stream));
    });
  }

  int64_t pibem_launch_count(void) { return launch_count(); }

  int pibem_set_profiling(pibem_handle *h, int32_t on)
  {
    return guarded(h, [&] {
      if (on < 0 || on > 2)
        throw Error(PIBEM_EINVAL, "profiling mode must be 0, 1 or 2");
      h->timing         = on != 0;
      h->timing_hold_ns = on == 2 ? 400000 : 0;
    });
  }

  int pibem_phase_totals(pibem_handle *h, int32_t precision, double *ms7, int64_t *applications,
                         int32_t reset)
  {
    if (!h || precision < 0 || precision > 1)
      return PIBEM_EINVAL;
    if (ms7)
      for (int i = 0; i < 7; ++i)
        ms7[i] = h->phase_tot[precision][i];
    if (applications)
      *applications = h->phase_cnt[precision];
    if (reset)
      {
        for (int p = 0; p < 2; ++p)
          {
            for (int i = 0; i < 7; ++i)
              h->phase_tot[p][i] = 0;
            h->phase_cnt[p] = 0;
          }
      }
    return PIBEM_OK;
  }

  int pibem_last_phase_ms(pibem_handle *h, double *ms7)
  {
    if (!h || !ms7)
      return PIBEM_EINVAL;
    for (int i = 0; i < 7; ++i)
      ms7[i] = h->phase_ms[i];
    return PIBEM_OK;
  }
}

// ---------------------------------------------------------------------------
// Allocation-free FMM matvec (pibem_fmm_matvec_noalloc).
//
// For callers that must not allocate device memory while they run: every
// temporary of the call (multipole and local expansions, translation
// products, M2P values, Dirichlet flags and column modes) is carved out of the
// file-scope array below, which each GPU that loads the library holds until
// the process exits.  Host code must not take the array's name as a device
// address: the address is looked up once per device with cudaGetSymbolAddress
// (first call on that device, device current) and kept.  Successive calls share
// the array and find the previous call's contents; what must start at zero (the
// multipole expansions, the flags) is cleared by each call.  Calls whose work
// overlaps on the GPU race on the array.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_noalloc_scratch[PIBEM_NOALLOC_SCRATCH_BYTES / sizeof(double)];

namespace
{
  std::mutex g_noalloc_mutex;
  double    *g_noalloc_ptr[64] = {};

  double *noalloc_scratch(int device)
  {
    if (device < 0 || device >= 64)
      throw Error(PIBEM_EINVAL, "device ordinal out of range for the allocation-free scratch");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device])
      {
        void       *p  = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (rc != cudaSuccess || !p)
          throw Error(PIBEM_ECUDA, std::string("cudaGetSymbolAddress of the allocation-free scratch: ") +
                                     cudaGetErrorString(rc));
        g_noalloc_ptr[device] = static_cast<double *>(p);
      }
    return g_noalloc_ptr[device];
  }

  // The far-field launch sequence of far_field() on caller-provided buffers.
  void far_field_on(pibem_handle *h, OperatorDev<double> &op, int R, const uint8_t *dir,
                    const uint8_t *modes, const double *x, double *y, double *M, double *Lx,
                    double *Y)
  {
    const int    N = int(h->N());
    cudaStream_t s = h->stream;
    PIBEM_CUDA(cudaMemsetAsync(M, 0, size_t(h->tree.nb) * R * op.K * sizeof(double), s));
    launch_p2m_apply<double>(op, R, N, dir, modes, x, M, false, s);
    for (int l = h->tree.L; l >= 1; --l)
      launch_upward_level<double>(op, R, l, M, Y, s);
    launch_m2l_gemm<double>(op, R, M, Y, s);
    for (int l = 1; l <= h->tree.L; ++l)
      launch_downward_level<double>(op, R, l, Lx, Y, s);
    launch_m2p<double>(op, h->td, R, N, M, y, s);
    launch_l2p<double>(op, R, N, Lx, y, s);
  }
} // namespace

extern "C" int pibem_fmm_matvec_noalloc(pibem_handle *h, int32_t R, const double *d_phi,
                                        const double *d_dphi, double *d_outN, double *d_outD)
{
  return guarded(h, [&] {
    if (!h->mesh_ok)
      throw Error(PIBEM_EINVAL, "pibem_fmm_matvec_noalloc before pibem_set_mesh");
    if (R < 1 || !d_phi || !d_dphi || !d_outN || !d_outD)
      throw Error(PIBEM_EINVAL, "bad arguments");
    const int64_t N  = h->N();
    const int64_t K  = h->plan.K;
    const size_t  nM = size_t(h->tree.nb) * R * K;
    const size_t  nY = std::max<size_t>(1, size_t(h->op64.n_pairs) * R * K);
    const size_t  nS = std::max<size_t>(1, size_t(h->op64.n_m2p_items) * R);
    const size_t  nF = (size_t(N) + size_t(R) + 7) / 8; // flags, in doubles
    const size_t  need = (2 * nM + nY + nS + nF) * sizeof(double);
    if (need > PIBEM_NOALLOC_SCRATCH_BYTES)
      throw Error(PIBEM_EINVAL, "pibem_fmm_matvec_noalloc: this mesh and nrhs need " +
                                  std::to_string(need / (1024.0 * 1024.0)) +
                                  " MiB of scratch, more than the " +
                                  std::to_string(PIBEM_NOALLOC_SCRATCH_BYTES >> 20) + " MiB array");
    double      *M = noalloc_scratch(h->prm.device);
    double      *Lx = M + nM, *Y = Lx + nM, *S = Y + nY;
    uint8_t     *dir   = reinterpret_cast<uint8_t *>(S + nS);
    uint8_t     *modes = dir + N;
    cudaStream_t s     = h->stream;
    // a copy of the handle's operator view (host memory only) with the M2P
    // scratch pointed into the array; the handle itself is not modified.  The
    // far field is the plain FP64 one whatever the precision mode: ops_ff and
    // the tensor-core images of the view are not used by this call.
    OperatorDev<double> op = h->op64;
    op.m2p_scratch         = S;
    PIBEM_CUDA(cudaMemsetAsync(dir, 0, size_t(N), s));
    launch_near_spmv<double>(op, R, int(N), h->d_N.p, d_phi, d_outN, false, s);
    launch_near_spmv<double>(op, R, int(N), h->d_D.p, d_dphi, d_outD, false, s);
    PIBEM_CUDA(cudaMemsetAsync(modes, MODE_KER1, size_t(R), s));
    far_field_on(h, op, R, dir, modes, d_phi, d_outN, M, Lx, Y);
    PIBEM_CUDA(cudaMemsetAsync(modes, MODE_KER2, size_t(R), s));
    far_field_on(h, op, R, dir, modes, d_dphi, d_outD, M, Lx, Y);
    h->cnt64 += R;
  });
}
