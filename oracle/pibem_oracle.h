/* Oracle (test infrastructure only): a CPU restatement of pi-BEM's
 * FMM-accelerated collocation BEM operator, its dense collocation operator and
 * the solve around them.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it, and only to compare or time against it.
 *
 * Index conventions follow the reference: nodes are DoFs of FE_Q(1) on a
 * quadrilateral surface mesh, cell vertices in deal.II lexicographic order
 * (v0=(0,0), v1=(1,0), v2=(0,1), v3=(1,1) of the unit cell).
 */
#ifndef PIBEM_ORACLE_H
#define PIBEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_handle orc_handle;

orc_handle *orc_create(int trunc_order, int num_octree_levels, int max_nodes_per_leaf,
                       int quadrature_order, int singular_quadrature_order, int external_flow);
void        orc_destroy(orc_handle *h);
void        orc_set_threads(int n);

/* double_offsets/double_ids: CSR of the double-node sets (each set includes the
 * node itself); both NULL means every node is its own only double. */
int orc_set_mesh(orc_handle *h, int n_nodes, const double *xyz, int n_cells, const int *cells,
                 const int *double_offsets, const int *double_ids);
int orc_set_bc(orc_handle *h, const unsigned char *dirichlet_mask);
/* Double body for the dense operator (BEMProblem::_assemble_system_double_body,
 * bem_problem.cc:958-1135): every row adds the integrals over the mesh
 * reflected in z = z0.  The FMM functions keep the one-body operator of the
 * mesh they were given. */
int orc_set_double_body(orc_handle *h, int on, double z0);
/* Constraint lines applied by orc_solve as deal.II's ConstrainedOperator in
 * BEMProblem::solve_system (include/constrained_matrix.h, bem_problem.cc:1275-1283):
 * row rows[k] of the operator becomes x[rows[k]] - x[cols[k]] (cols[k] = -1: no
 * entry) and of the right-hand side g[k].  n = 0 clears them. */
int orc_set_constraints(orc_handle *h, int n, const int *rows, const int *cols, const double *g);

/* BEMFMA::generate_multipole_expansions + multipole_matr_vect_products. */
void orc_fmm_matvec(orc_handle *h, const double *phi, const double *dphi_dn, double *outN,
                    double *outD);
/* Dense collocation operator (one body), same quadrature rules as the FMM near field. */
void orc_dense_matvec(orc_handle *h, const double *phi, const double *dphi_dn, double *outN,
                      double *outD);
/* use_dense = 0: FMM operator, 1: dense operator for the three calls below. */
void orc_compute_alpha(orc_handle *h, int use_dense, double *alpha);
void orc_system_matvec(orc_handle *h, int use_dense, const double *alpha, const double *x,
                       double *y);
void orc_compute_rhs(orc_handle *h, int use_dense, const double *alpha, const double *tmp_rhs,
                     double *rhs);
/* BEMProblem::solve_system semantics with an own GMRES(restart); returns iterations. */
/* Preconditioner of orc_solve: 0 none (default), 1 right leaf-block Jacobi
 * (dense inverses of the near-field system matrix on each childless block's
 * own nodes, the GPU library's default), 2 right ILU(0) of the near-field
 * system matrix (BEMFMA::FMA_preconditioner, bem_fma.cc:3080-3411). */
void orc_set_preconditioner(orc_handle *h, int kind);
/* Builds the preconditioner `kind` (as above) with the FMM alpha and makes it
 * the handle's; returns the ILU's number of stored entries (0 otherwise). */
int64_t orc_preconditioner_build(orc_handle *h, int kind);
/* z = P^-1 v with the handle's preconditioner (v for none). */
void orc_preconditioner_apply(orc_handle *h, const double *v, double *z);
/* The ILU(0) factors in place in the CSR of the near-field system matrix:
 * ptr (n + 1), col, val (L below the diagonal with unit diagonal implied, U
 * from the diagonal on). */
void orc_ilu_factors(orc_handle *h, int64_t *ptr, int32_t *col, double *val);
int orc_solve(orc_handle *h, int use_dense, double *phi, double *dphi_dn, const double *tmp_rhs,
              double tol, int max_steps, int restart, double *final_rel_res);

/* Octree export. */
int  orc_num_blocks(orc_handle *h);
int  orc_num_levels(orc_handle *h);
void orc_level_range(orc_handle *h, int *start, int *end); /* L+1 entries each */
void orc_block_info(orc_handle *h, int *level, int *parent, int *nchild, double *pmin,
                    double *delta, int *n_nodes, int *n_quads);
int  orc_childless(orc_handle *h, int *out);
int  orc_list_sublevels(orc_handle *h, int block);
/* kind: 0 nearNeigh, 1 intList, 2 nonIntList.  Returns the size; copies up to cap. */
int  orc_list(orc_handle *h, int kind, int block, int sub, int *out, int cap);
int  orc_block_nodes(orc_handle *h, int block, int *out, int cap);

/* Near-field sparse matrices as COO (rows, cols sorted). */
long orc_near_nnz(orc_handle *h);
void orc_near_export(orc_handle *h, int *rows, int *cols, double *N, double *D);

/* Block expansions after the last orc_fmm_matvec; kind 0 M(Ker1) 1 M(Ker2) 2 L(Ker1) 3 L(Ker2);
 * out holds nblocks * (p+1)(p+2)/2 complex values as (re, im). */
void orc_block_expansions(orc_handle *h, int kind, double *out);

/* Quadrature data of the mesh (QGauss(quadrature_order) per cell). */
int  orc_num_quad_points(orc_handle *h);
void orc_quad_data(orc_handle *h, double *pts, double *normals, double *jxw);

/* Single-expansion primitives, same storage as the reference (complex, index n(n+1)/2+m). */
double orc_legendre(int n, int m, double x);
double orc_legendre_deriv(int n, int m, double x);
void   orc_p2m(int p, const double *c, int npts, const double *pts, const double *q, double *out);
void   orc_p2m_dipole(int p, const double *c, int npts, const double *pts, const double *normals,
                      const double *q, double *out);
void   orc_m2m(int p, const double *c_child, const double *coef, const double *c_parent,
               double *out);
void   orc_m2l(int p, const double *c_src, const double *coef, const double *c_tgt, double *out);
void   orc_l2l(int p, const double *c_parent, const double *coef, const double *c_child,
               double *out);
double orc_m2p(int p, const double *c, const double *coef, const double *x);
double orc_l2p(int p, const double *c, const double *coef, const double *x);

/* Quadrature rules on [0,1]^2 (n_out = number of points). */
int orc_gauss_rule(int n, double *pts, double *w);
int orc_telles_rule(int n, int vertex, double *pts, double *w);

#ifdef __cplusplus
}
#endif
#endif
