/* pibem_gpu.h -- C ABI of the GB300 FMM-accelerated collocation BEM operator
 * (3-D Laplace, Q1 surface meshes) and the GMRES solve around it.
 *
 * It is the drop-in replacement for pi-BEM's BEMFMA<3> accelerator and for the
 * FMA branch of BEMProblem<3>:
 *   include/bem_fma.h:94-202         BEMFMA public interface
 *   source/bem_problem.cc:1139-1374  compute_alpha / vmult / compute_rhs /
 *                                    solve_system / solve (FMA branches)
 * Every entry point returns an int32 status (PIBEM_OK = 0); no C++ exception
 * crosses this boundary.  The message of the last failure of a handle is
 * available from pibem_last_error().
 *
 * Threading: a handle is used by one host thread at a time; several handles may
 * share the GPU.  Host arrays are owned by the caller and are read or written
 * only inside the call.  Device-pointer variants (suffix _device) are ordered
 * on the handle's stream (pibem_set_stream) and return before the work ends.
 */
#ifndef PIBEM_GPU_H
#define PIBEM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIBEM_OK 0
#define PIBEM_EINVAL 1      /* bad argument or call order */
#define PIBEM_ENOMEM_HBM 2  /* device allocation failed or HBM budget exceeded */
#define PIBEM_ENOCONV 3     /* GMRES did not reach the tolerance within max steps */
#define PIBEM_ETIMEDOUT 4   /* a bounded device wait gave up */
#define PIBEM_ECUDA 5       /* CUDA runtime error */
#define PIBEM_EAGAIN 6      /* request slots: no free slot / no finished request yet */

/* Arithmetic of the solve. */
#define PIBEM_PRECISION_FP64 0  /* plain path: every matvec in FP64 */
#define PIBEM_PRECISION_MIXED 1 /* FP32 operator inside GMRES + FP64-accurate refinement residual
                                   (float-float translations, FP64 elsewhere) */
#define PIBEM_PRECISION_FLOAT_FLOAT 2 /* every matvec FP64-accurate: FP64 near field and
                                         expansions, translations in FP32-pair arithmetic */

/* Engine of the FP32 translation GEMMs (M2L, M2M, L2L). */
#define PIBEM_M2L_TENSOR_CORE 0 /* tcgen05 3xTF32 where the order fits (p <= 10), else CUDA cores */
#define PIBEM_M2L_CUDA_CORE 1   /* FP32 FMA on CUDA cores */

typedef struct pibem_handle pibem_handle;

/* Parameter-file knobs of the reference (same names and defaults):
 *   BEMFMA<3>/Octree Params/Number of Octree Levels                      (10)
 *   BEMFMA<3>/Octree Params/Maximum Number of Collocation Points per
 *             Childless Block                                            (20)
 *   BEMFMA<3>/FMA Params/FMA Truncation Order                            (6)
 *   BEMProblem<3>/Quadrature rules/Quadrature order                      (4)
 *   BEMProblem<3>/Quadrature rules/Singular quadrature order             (5)
 *   BEMProblem<3>/Solver/Max steps, Tolerance
 *   BEMProblem<3>/Is external flow
 *   BEMProblem<3>/Symmetry plane z level                                 (0.0)
 *   BEMProblem<3>/Continuos gradient across edges                        (true)
 * (source/bem_fma.cc:65-103, source/bem_problem.cc:247-312), plus the keys of
 * the added subsection "GB300 Params". */
typedef struct pibem_params
{
  int32_t fma_truncation_order;          /* p, 1..10 */
  int32_t num_octree_levels;             /* 1..20 */
  int32_t max_nodes_per_childless_block; /* leaf size */
  int32_t quadrature_order;              /* QGauss order per direction, 1..8 */
  int32_t singular_quadrature_order;     /* Telles order per direction, 1..12 */
  int32_t solver_max_steps;              /* total GMRES iterations */
  double  solver_tolerance;              /* relative true residual ||b-Ax||/||b|| */
  int32_t gmres_restart;                 /* Krylov dimension (reference: 100) */
  int32_t is_external_flow;              /* 0 interior (alpha=-N1), 1 exterior (alpha=-1-N1) */
  int32_t precision_mode;                /* PIBEM_PRECISION_* */
  int32_t preconditioner;                /* 0 none, 1 leaf-block Jacobi (right), 2 ILU(0) of
                                            the near-field system matrix (right; the
                                            reference's FMA_preconditioner, bem_fma.cc:3080) */
  int32_t device;                        /* CUDA device ordinal */
  double  inner_tolerance;               /* mixed mode: inner FP32 GMRES tolerance */
  double  hbm_budget_gb;                 /* 0 = unlimited */
  int32_t m2l_engine;                    /* FP32 translations: PIBEM_M2L_* */
  /* Double body (BEMProblem::_assemble_system_double_body, bem_problem.cc:958-1135):
   * 1 adds to every collocation row the integrals over the mesh reflected in the
   * plane z = symmetry_plane_z_level (points z -> 2 z0 - z, normals n_z -> -n_z,
   * regular Gauss rule, values of the reflected node taken from its original).
   * 0 (default) is the one-body operator of the FMA branch. */
  int32_t double_body;
  double  symmetry_plane_z_level;
  /* "Continuos gradient across edges" (bem_problem.cc:277, default 1): the
   * constraint lines of Dirichlet-Dirichlet double nodes (see pibem_solve). */
  int32_t continuous_gradient;
  /* Tiles of the tensor-core FP32 M2L (tuning only; results do not change):
   * the most M2L pairs of one operator in a tile chunk (0 = 128; 16..128) and
   * the pipeline depth of the tile stages (0 = the deepest that fits in shared
   * memory; 2 or 3). */
  int32_t m2l_chunk_pairs;
  int32_t m2l_stages;
} pibem_params;

typedef struct pibem_solve_stats
{
  int32_t iterations;        /* GMRES iterations (inner iterations in mixed mode) */
  int32_t refinement_steps;  /* outer FP64 residual evaluations (mixed mode) */
  int32_t fp64_matvecs;      /* FP64 operator applications */
  int32_t fp32_matvecs;      /* FP32 operator applications */
  double  relative_residual; /* final ||b - A x|| / ||b|| (worst column), formed with the
                                FP64 operator (FP64-accurate one in mixed mode) after the
                                last correction */
  double  seconds;           /* wall time of the call */
} pibem_solve_stats;

typedef struct pibem_tree_info
{
  int32_t n_boxes, n_levels, n_leaves;
  int64_t n_m2l_pairs, n_m2p_pairs, near_nnz, p2m_rows, n_quad_points;
  int32_t n_m2l_offsets;
  double  setup_seconds;
  int32_t octree_on_device; /* 1: octree and lists built on the device, 0: on the host
                               (a list beyond the device builder's capacity) */
} pibem_tree_info;

/* Defaults of the reference parameter file. */
int pibem_params_default(pibem_params *params);
/* Parse the knobs above from the text of a deal.II .prm file
 * (subsection / set / end); unknown keys are ignored. */
int pibem_params_from_prm(pibem_params *params, const char *prm_text);

int         pibem_create(const pibem_params *params, pibem_handle **out);
int         pibem_destroy(pibem_handle *h);
const char *pibem_last_error(const pibem_handle *h);
/* cudaStream_t passed as void*; NULL selects the handle's own stream. */
int         pibem_set_stream(pibem_handle *h, void *stream);

/* Mesh: replaces BEMFMA::init_fma + generate_octree_blocking + direct_integrals
 * + multipole_integrals (bem_fma.cc:42-62, 3615, 108, 1609).
 *   xyz[3*n_nodes]        support points (DoF k at vertex k)
 *   cell_nodes[4*n_cells] Q1 cells, deal.II lexicographic vertex order
 *   double_offsets[n_nodes+1], double_ids: CSR of the double-node sets (each
 *                         set includes the node itself), both NULL if the mesh
 *                         has no double nodes. */
int pibem_set_mesh(pibem_handle *h, int64_t n_nodes, const double *xyz, int64_t n_cells,
                   const int32_t *cell_nodes, const int32_t *double_offsets,
                   const int32_t *double_ids);

/* Dirichlet mask (1 = Dirichlet node, 0 = Neumann node), the reference's
 * dirichlet_nodes vector (bem_problem.cc:315-411).  Computes alpha. */
int pibem_set_bc(pibem_handle *h, const uint8_t *dirichlet_mask);

/* BEMFMA::generate_multipole_expansions + multipole_matr_vect_products
 * (bem_fma.cc:1971, 2391): outN = N phi, outD = D dphi_dn, near field plus far
 * field, FP64.  nrhs vectors stored one after another (length n_nodes each). */
int pibem_fmm_matvec(pibem_handle *h, int32_t nrhs, const double *phi, const double *dphi_dn,
                     double *outN, double *outD);

/* BEMProblem::compute_alpha (bem_problem.cc:1139). */
int pibem_compute_alpha(pibem_handle *h, double *alpha);

/* BEMProblem::vmult (bem_problem.cc:1165): y = N(x.neu) - D(x.dir) + alpha.x.neu. */
int pibem_system_matvec(pibem_handle *h, int32_t nrhs, const double *x, double *y);

/* PreconditionILU::vmult on BEMFMA::FMA_preconditioner's matrix
 * (bem_fma.cc:3080-3411, applied in bem_problem.cc:1302-1318): z = P^-1 v for
 * nrhs vectors with the handle's preconditioner -- the ILU(0) of the near-field
 * system matrix (preconditioner 2), the leaf-block Jacobi inverses
 * (preconditioner 1; FP32 inverses in PRECISION_MIXED, FP64 otherwise), or
 * z = v (0).  Built by pibem_set_bc. */
int pibem_apply_preconditioner(pibem_handle *h, int32_t nrhs, const double *v, double *z);

/* BEMProblem::compute_rhs (bem_problem.cc:1220). */
int pibem_compute_rhs(pibem_handle *h, int32_t nrhs, const double *tmp_rhs, double *rhs);

/* BEMProblem::solve_system (bem_problem.cc:1267): rhs, GMRES from x0 = rhs,
 * scatter phi(i) = sol(i) on Neumann nodes, dphi_dn(i) = sol(i) on Dirichlet
 * nodes; the other entries of phi / dphi_dn are left as given.  With double
 * nodes the solve runs on the constrained system of compute_constraints
 * (bem_problem.cc:1377-1579) and ConstrainedOperator (constrained_matrix.h):
 * per double-node set, with i its first Dirichlet node (else its smallest id),
 *   i Neumann:            x_d = x_i for the set's other nodes d;
 *   i Dirichlet, d Neumann:   x_d = tmp_rhs_i;
 *   i, d Dirichlet (continuous_gradient): x_i and x_d are the normal
 *   derivatives given by the L2-projected normals and surface gradients of
 *   tmp_rhs (pibem_compute_normals / _surface_gradients).
 * pibem_system_matvec and pibem_compute_rhs stay unconstrained, as vmult and
 * compute_rhs are. */
int pibem_solve(pibem_handle *h, int32_t nrhs, double *phi, double *dphi_dn,
                const double *tmp_rhs, pibem_solve_stats *stats);

/* Same as pibem_solve with device pointers, stream-ordered. */
int pibem_solve_device(pibem_handle *h, int32_t nrhs, double *d_phi, double *d_dphi_dn,
                       const double *d_tmp_rhs, pibem_solve_stats *stats);

/* ---- request slots: continuous batching of solves on one mesh -------------
 * The serving form of pibem_solve (BEMProblem::solve, bem_problem.cc:1352-1374,
 * one solve per call there).  A handle opens max_slots slots; each submitted
 * right-hand side (tmp_rhs as in pibem_solve, with a caller's request id) takes
 * a free slot and runs the same algorithm as a column of pibem_solve.  Each
 * pibem_slots_step advances every slot from event to event (right-hand side,
 * residuals, refinement decisions: operator applications shared by the slots
 * that need them at that moment) and runs the Arnoldi steps of all slots in a
 * GMRES cycle on the device (one CUDA graph with a device-side loop condition)
 * until every one of them has ended its cycle, or for max_steps steps;
 * right-hand sides submitted between steps join at the next step.  A slot's arithmetic does not
 * depend on the other slots: its result equals what pibem_solve gives for that
 * right-hand side alone.  Finished requests are collected in request-id order
 * with the full phi / dphi_dn vectors (known entries from tmp_rhs) and their
 * own statistics.  Host arrays of n_nodes doubles; the work is ordered on the
 * handle's stream and every call returns after it.  pibem_solve is refused
 * while slots are open.
 *   pibem_slots_submit: PIBEM_EAGAIN when every slot is taken; *slot = the slot.
 *   pibem_slots_step:   max_steps > 0 bounds the Arnoldi steps of this call
 *                       (so that waiting submissions join soon: a slot in the
 *                       middle of a GMRES cycle resumes it at the next call);
 *                       *n_active = slots in progress, *n_done = finished ones
 *                       waiting to be collected.
 *   pibem_slots_collect: PIBEM_EAGAIN when none has finished; PIBEM_ENOCONV
 *                       (the results are written) when it stopped on the step
 *                       limit above the tolerance. */
int pibem_slots_open(pibem_handle *h, int32_t max_slots);
int pibem_slots_submit(pibem_handle *h, int64_t request_id, const double *tmp_rhs, int32_t *slot);
int pibem_slots_step(pibem_handle *h, int32_t max_steps, int32_t *n_active, int32_t *n_done);
int pibem_slots_collect(pibem_handle *h, int64_t *request_id, double *phi, double *dphi_dn,
                        pibem_solve_stats *stats);
int pibem_slots_close(pibem_handle *h);

/* Introspection for parity tests and logging. */
int pibem_tree_info_get(pibem_handle *h, pibem_tree_info *info);
/* Wall time in seconds of the phases of the last pibem_set_mesh, in the order:
 * mesh checks and quadrature points, octree and lists, operator plan, plan
 * upload, near-field integrals, P2M / L2P tables, translation operators, the
 * rest (the reference times its phases with Teuchos::TimeMonitor). */
#define PIBEM_SETUP_PHASES 8
int pibem_setup_phases(pibem_handle *h, double *seconds);
/* Box table: level, parent, number of children, pmin[3], delta, nodes, quad points. */
int pibem_tree_boxes(pibem_handle *h, int32_t *level, int32_t *parent, int32_t *nchild,
                     double *pmin, double *delta, int32_t *n_nodes, int32_t *n_quads);
/* List of a box: kind 0 nearNeigh, 1 intList, 2 nonIntList at sublevel sub.
 * Returns the size (copies at most cap ids), -1 on error. */
int pibem_tree_list(pibem_handle *h, int32_t kind, int32_t box, int32_t sub, int32_t *out,
                    int32_t cap);
int pibem_tree_list_sublevels(pibem_handle *h, int32_t box);
/* Near-field matrices as COO (rows, cols) sorted by row then column. */
int64_t pibem_near_nnz(pibem_handle *h);
int     pibem_near_export(pibem_handle *h, int32_t *rows, int32_t *cols, double *N, double *D);
/* Quadrature points of the mesh, cell-major (n_cells * nq points). */
int pibem_quad_points(pibem_handle *h, double *pts);
/* Phase timings of the last operator application, milliseconds, in the order
 * near, p2m, m2m (all levels), m2l (the batched M2L GEMM of all levels), l2l
 * (L2L and the sums of each box's products, all levels), m2p, l2p (7 values);
 * needs profiling on. */
int pibem_last_phase_ms(pibem_handle *h, double *ms7);
/* CUDA-event timing of the operator phases: 0 off (default), 1 on (event
 * records and one stream synchronisation per application), 2 on with a hold:
 * each application starts behind a 0.4 ms single-thread kernel, so that the
 * host has enqueued it before the GPU reaches the first phase event and the
 * phase times are GPU execution times without host launch gaps. */
int pibem_set_profiling(pibem_handle *h, int32_t on);
/* Phase times (ms, same order as pibem_last_phase_ms) summed over the operator
 * applications of the given precision (PIBEM_PRECISION_FP64: FP64 operator,
 * PIBEM_PRECISION_MIXED: FP32 operator) since the last reset, and their count. */
int pibem_phase_totals(pibem_handle *h, int32_t precision, double *ms7, int64_t *applications,
                       int32_t reset);
/* Number of CUDA kernels this library has launched so far (all handles). */
int64_t pibem_launch_count(void);
/* Device memory the handle holds now (resident operator, tree, plan and its
 * grow-only work buffers), in bytes.  No counterpart in the reference (its
 * operator lives in host memory); serving loops use it to keep a set of
 * resident meshes inside an HBM budget. */
int pibem_device_bytes(const pibem_handle *h, uint64_t *bytes);

/* ---- L2 projections onto the continuous Q1 space of the mesh -------------
 * The post-solve steps of BEMProblem (source/bem_problem.cc): the L2 projection
 * of a vector field g, u = M^-1 b with the consistent Q1 mass matrix M and
 * b_i = integral of phi_i g, per component, on the mesh's Gauss rule:
 *   compute_normals (:1998):           g = the cell normal;
 *   compute_surface_gradients (:1879): g = tangential gradient of the
 *                                      interpolated u;
 *   compute_gradients (:1747):         g = tangential gradient of phi + n dphi/dn.
 * Output: 3 values per node (x, y, z), node-major, R columns one after another.
 * Needs pibem_set_mesh only.  The reference solves with GMRES + AMG to its
 * solver tolerance; here CG with a Jacobi preconditioner runs to a relative
 * residual of 1e-13 (the same projection). */
int pibem_compute_normals(pibem_handle *h, double *normals);
int pibem_compute_surface_gradients(pibem_handle *h, int32_t R, const double *u, double *grad);
int pibem_compute_gradients(pibem_handle *h, int32_t R, const double *phi, const double *dphi_dn,
                            double *grad);

/* ---- mesh ingestion (host only; no GPU needed) ---------------------------
 * UCD (.inp) surface mesh, as ComputationalDomain::read_domain reads it with
 * GridIn::read_ucd (source/computational_domain.cc:280-287).  Call once with
 * xyz = cell_nodes = material_id = NULL to get the counts, then with arrays of
 * at least those sizes (*n_nodes, *n_cells give the capacities).  Only "quad"
 * cells are read; their counterclockwise UCD vertices are returned in deal.II
 * lexicographic order (v0, v1, v3, v2), node ids renumbered 0.. in file order.
 * On error pibem_mesh_io_error() has the message (per calling thread). */
int pibem_ucd_read(const char *path, int64_t *n_nodes, int64_t *n_cells, double *xyz,
                   int32_t *cell_nodes, int32_t *material_id);
const char *pibem_mesh_io_error(void);
/* Double-node sets: nodes closer than tol in every coordinate are one group;
 * node i's set (offsets[i]..offsets[i+1]) lists every member of its group,
 * itself included -- the double_nodes_set BEMProblem passes to init_fma
 * (source/bem_problem.cc:200), in the CSR form pibem_set_mesh takes.
 * offsets has n_nodes + 1 entries; *n_ids returns the total; ids may be NULL
 * (size query) or hold capacity entries (PIBEM_EINVAL if too small). */
int pibem_double_nodes(int64_t n_nodes, const double *xyz, double tol, int32_t *offsets,
                       int32_t *ids, int64_t capacity, int64_t *n_ids);
/* Dirichlet mask from cell material ids, as
 * BEMProblem::compute_dirichlet_and_neumann_dofs_vectors
 * (source/bem_problem.cc:315-411): a node is Dirichlet (1) when any of its cells
 * carries one of the n_dirichlet_ids material ids, else Neumann (0). */
int pibem_dirichlet_mask_from_materials(int64_t n_nodes, int64_t n_cells,
                                        const int32_t *cell_nodes, const int32_t *material_id,
                                        int32_t n_dirichlet_ids, const int32_t *dirichlet_ids,
                                        uint8_t *mask);

/* Allocation-free FMM matvec.  No counterpart in the reference.
 * Same result as pibem_fmm_matvec (outN = N phi, outD = D dphi_dn) in the FP64
 * and mixed precision modes -- its far field is always the plain FP64 one, so
 * in PIBEM_PRECISION_FLOAT_FLOAT mode (float-float translations) the two agree
 * to about 1e-12 relative instead -- but with device pointers and without
 * allocating any device memory during the call:
 * every temporary of the call lives in one file-scope device array of
 * PIBEM_NOALLOC_SCRATCH_BYTES that each GPU holds from library load to exit.
 * For callers that must not allocate at call time: applications that reserve
 * all device memory for themselves up front, and loops that cannot afford the
 * device-wide synchronisation that cudaMalloc / cudaFree imply.  The mesh must
 * be set up (pibem_set_mesh, which does allocate) beforehand.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.
 *  - Work is ordered on the handle's stream; the call returns before it ends.
 *  - All calls share the array and it keeps the last call's contents, so calls
 *    whose work overlaps on the GPU (other streams, other handles) race.
 *  - A mesh / nrhs whose temporaries exceed the array is rejected with
 *    PIBEM_EINVAL and a message giving the size it would need. */
#define PIBEM_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int pibem_fmm_matvec_noalloc(pibem_handle *h, int32_t nrhs, const double *d_phi,
                             const double *d_dphi_dn, double *d_outN, double *d_outD);

#ifdef __cplusplus
}
#endif
#endif
