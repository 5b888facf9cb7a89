// Internal declarations of the GB300 FMM-BEM library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pibem_gpu.h"

namespace pibem
{
  // Error raised inside the library; converted to a status code at the ABI.
  struct Error : std::runtime_error
  {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
  };

#define PIBEM_CUDA(call)                                                                       \
  do                                                                                           \
    {                                                                                          \
      cudaError_t e_ = (call);                                                                 \
      if (e_ != cudaSuccess)                                                                   \
        throw ::pibem::Error(e_ == cudaErrorMemoryAllocation ? PIBEM_ENOMEM_HBM : PIBEM_ECUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(e_));              \
    }                                                                                          \
  while (0)

  // Counts kernel launches of this library (all handles, all streams).
  void    note_launch(int64_t n = 1);
  int64_t launch_count();
  // Raise (never lower) a kernel's dynamic shared-memory limit on the current
  // device.  The limit is process-wide state of the function, and handles on
  // other host threads may launch the same kernel with other sizes at the same
  // time: lowering it under them would make their launches fail.
  void raise_smem_limit(const void *fn, size_t bytes);

  // Owning device buffer.
  template <typename T>
  struct DBuf
  {
    T     *p = nullptr;
    size_t n = 0;
    DBuf() {}
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release()
    {
      if (p)
        cudaFree(p);
      p = nullptr;
      n = 0;
    }
    // Grows only: a buffer keeps its capacity n once allocated.
    void alloc(size_t count)
    {
      if (count <= n && p)
        return;
      release();
      if (count == 0)
        return;
      PIBEM_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
      n = count;
    }
    void zero(cudaStream_t s)
    {
      if (n)
        PIBEM_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    void upload(const T *h, size_t count, cudaStream_t s)
    {
      alloc(count);
      if (count)
        PIBEM_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T> &v, cudaStream_t s) { upload(v.data(), v.size(), s); }
    void download(T *h, size_t count, cudaStream_t s) const
    {
      if (count)
        PIBEM_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    size_t bytes() const { return n * sizeof(T); }
  };

  // Page-locked host buffer (grow-only): small device -> host reads that the
  // host waits for (the Arnoldi step's Hessenberg column) skip the CUDA runtime's
  // staging copy of pageable memory.
  template <typename T>
  struct PinnedBuf
  {
    T     *p = nullptr;
    size_t n = 0;
    PinnedBuf() {}
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf()
    {
      if (p)
        cudaFreeHost(p);
    }
    void alloc(size_t count)
    {
      if (count <= n && p)
        return;
      if (p)
        cudaFreeHost(p);
      p = nullptr;
      n = 0;
      PIBEM_CUDA(cudaMallocHost((void **)&p, count * sizeof(T)));
      n = count;
    }
  };

  // ---------------------------------------------------------------------
  // Octree and interaction lists (host, built once per mesh).
  // Box ids follow the reference's numbering: level by level, parents in
  // order, children in the reference child order (bem_fma.cc:3811-3822).
  // ---------------------------------------------------------------------
  struct Tree
  {
    int                 L  = 0;
    int                 nb = 0;
    std::vector<int>    level, parent, nchild, child_first, digit;
    std::vector<int>    ic;    // 3 per box: lattice coordinates at the box level
    std::vector<double> pmin;  // 3 per box
    std::vector<double> delta; // per box
    std::vector<int>    nbeg, nend, qbeg, qend; // ranges in node_sorted / quad_sorted
    std::vector<int>    node_sorted, quad_sorted;
    std::vector<int>    startLevel, endLevel;
    std::vector<int>    childless; // reference childlessList order
    std::vector<char>   is_childless;
    std::vector<std::vector<int>> dofs_filled; // per level: boxes with nodes
    std::vector<int>    qbox; // (L+1) * Q: box of each quad point at each level (leaf if shallower)
    // lists[box][sub] sorted unique
    std::vector<std::vector<std::vector<int>>> nn, il, nil;
    std::vector<int>    node_leaf; // childless box of each node

    void center(int b, double c[3]) const
    {
      for (int k = 0; k < 3; ++k)
        c[k] = pmin[3 * b + k] + delta[b] / 2.;
    }
  };

  // The geometry the operator integrates over.  One body: the mesh itself.
  // Double body: the mesh (nodes 0..n_dofs-1, cells 0..n_cells_body-1)
  // followed by its reflection in the symmetry plane: node n_dofs + k is the
  // image of node k, cell n_cells_body + c the image of cell c with its
  // orientation reversed, so that its normal is the reflected normal.  Only
  // the mesh's own nodes are collocation points and unknowns; an image node
  // takes the value of its original (dof()).
  struct MeshHost
  {
    int64_t              n_nodes = 0, n_cells = 0;
    int64_t              n_dofs = 0, n_cells_body = 0;
    std::vector<double>  xyz;
    std::vector<int32_t> cells;
    std::vector<int32_t> dbl_off, dbl_ids; // always filled (each set includes the node)
    std::vector<int32_t> elem_off, elem_ids; // node -> cells CSR
    int32_t dof(int32_t v) const { return v < n_dofs ? v : int32_t(v - n_dofs); }
  };

  // Fills m (nodes, cells, double-node sets) from the mesh; with double_body
  // appends the reflection in z = z0 (source/bem_problem.cc:958-1135: points
  // z -> 2 z0 - z, normals n_z -> -n_z).  An image node's double-node set is
  // its original's set moved to the images: a node never shares a set with
  // an image, so reflected cells always take the regular Gauss rule, as in
  // the reference.
  void mirror_mesh(int64_t n_nodes, const double *xyz, int64_t n_cells, const int32_t *cells,
                   const std::vector<std::vector<int32_t>> &sets, bool double_body, double z0,
                   MeshHost &m);

  // Builds the octree and the near / interaction / non-interaction lists with
  // the reference semantics (bem_fma.cc:3615-4801).
  void build_tree(const MeshHost &mesh, const std::vector<double> &qpts, int nq, int levels,
                  int max_nodes, Tree &t);

  // ---------------------------------------------------------------------
  // Operator structure derived from the lists.
  // ---------------------------------------------------------------------
  struct NearEntry
  {
    int32_t  cell;
    int32_t  singular_ok; // 1: the intList part (Telles rule if singular)
    uint64_t qmask;       // quadrature points of the cell taken into account
    int32_t  lcol[4];     // local column of each cell dof in the leaf block
  };

  struct Plan
  {
    int p = 0, K = 0;
    // near field, per leaf with nodes
    std::vector<int32_t>  nleaf_box;          // box id
    std::vector<int64_t>  nrow_ptr, ncol_ptr, nent_ptr, nval_ptr;
    std::vector<int32_t>  nrows, ncols;       // node ids of rows / columns
    std::vector<NearEntry> entries;
    std::vector<int32_t>  gather_ptr, gather_ids; // per (leaf col): entry*4+j, offset by ncol_ptr
    std::vector<int32_t>  row_leaf;           // leaf index of each row position
    // P2M tables, per childless box with quad points
    std::vector<int32_t>  pleaf_box;
    std::vector<int64_t>  prow_ptr;
    std::vector<int32_t>  prow_dof;
    std::vector<int64_t>  pcontrib_ptr;
    std::vector<int32_t>  pcontrib_q;         // quad point id * 4 + j
    // L2P: per childless box with nodes, nodes listed
    std::vector<int32_t>  lleaf_box;
    std::vector<int64_t>  lnode_ptr;
    std::vector<int32_t>  lnode_ids;
    // M2M: per level (1..L) boxes of that level are children; parents contiguous
    // M2L: per level pairs grouped by target
    std::vector<int32_t>  m2l_tgt_ptr_level;  // per level: range into m2l_tgt
    std::vector<int32_t>  m2l_tgt;            // target boxes
    std::vector<int64_t>  m2l_src_ptr;        // per target
    std::vector<int32_t>  m2l_src, m2l_off;   // source box, offset id
    std::vector<int32_t>  offsets;            // distinct offsets, 3 per id
    // Batched translations.  One pair space q for M2L (all levels), M2M and
    // L2L (per level); pair q reads the expansion of box q_src[q] and applies
    // operator q_op[q] of the concatenated table [M2L offsets | 8 M2M | 8 L2L];
    // pairs are cut into chunks of <= 64 pairs sharing one operator.
    std::vector<int32_t>  q_src, q_op;
    std::vector<int32_t>  ch_start, ch_cnt, ch_op;
    int                   m2l_chunk_end = 0;            // chunks [0, m2l_chunk_end) are M2L
    std::vector<int32_t>  up_chunk_ptr, down_chunk_ptr; // per level l: chunk range
    // gathers: per level, boxes and the pairs summed into each (fixed order)
    std::vector<int32_t>  up_box_ptr, down_box_ptr;     // per level: range in up_box / down_box
    std::vector<int32_t>  up_box, down_box;
    std::vector<int64_t>  up_q_ptr, down_q_ptr;         // per listed box
    std::vector<int32_t>  up_q, down_q;
    // fused level passes: the children of each up_box entry by octant (-1:
    // none), 8 per entry; per down_box entry its octant and the parent whose
    // local expansion it receives by L2L (-1: none; then down_q has no L2L entry)
    std::vector<int32_t>  up_child8, down_par;
    std::vector<uint8_t>  down_oct;
    // target-major M2L products: slot of each M2L pair q (its index in
    // m2l_src), and per down_box entry the range of its slots
    std::vector<int32_t>  m2l_yslot, down_m2l_beg, down_m2l_end;
    // M2P pairs grouped by target
    std::vector<int32_t>  m2p_tgt;
    std::vector<int64_t>  m2p_src_ptr;
    std::vector<int32_t>  m2p_src;
    // L2L per level: boxes with nodes at levels >= 2
    std::vector<int32_t>  l2l_ptr_level, l2l_box;
    int64_t               n_m2l = 0, n_m2p = 0;
  };

  // The same tree built on the device (octree.cu) from the device copies of the
  // coordinates, quadrature points, double-node sets and node -> cells CSR;
  // false when a list does not fit its capacity (the caller then uses
  // build_tree).
  bool build_tree_device(const MeshHost &mesh, const double *d_xyz, const double *d_qpts, int nq,
                         int L, int max_nodes, const int32_t *d_dbl_off, const int32_t *d_dbl_ids,
                         const int32_t *d_elem_off, const int32_t *d_elem_ids, Tree &t,
                         cudaStream_t s);
  // chunk_pairs: the most M2L pairs of one operator in a tensor-core chunk
  void build_plan(const MeshHost &mesh, const Tree &t, int nq, int p, Plan &plan,
                  int chunk_pairs = 128);

  // Real-form translation operators (scaled expansions), row-major K x K.
  void build_m2m_ops(int p, std::vector<double> &ops8);
  void build_l2l_ops(int p, std::vector<double> &ops8);
  void build_m2l_op(int p, int dx, int dy, int dz, double *T);

  // Gauss-Legendre and Telles rules on [0,1]^2 (x index fastest).
  void gauss_rule_2d(int n, std::vector<double> &pts, std::vector<double> &w);
  void telles_rule_2d(int n, int vertex, std::vector<double> &pts, std::vector<double> &w);
} // namespace pibem
