/*
 * fe_oracle.h -- CPU oracle for the pyoomph element residual/Jacobian
 * assembly path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and
 * the CPU-baseline leg of bench.py call it as the checker; the GPU product
 * never links or calls it.
 *
 * Restates, in plain C, what the reference does on this path:
 *   - mesh templates and node order (pyoomph/meshes/simplemeshes.py:225-305,
 *     src/meshtemplate.cpp:401-409,494-499,579-621,1378-1470,
 *     src/mesh2d.hpp:265-300)
 *   - global equation numbering (oomph mesh.cc:686-708, Node values in order,
 *     pinned values get no number)
 *   - shape functions and Gauss rules (oomph shape.h:607-650,
 *     Telements.h:569-680, integral.cc:50-206,355-369)
 *   - per-integration-point geometry through the metric tensor
 *     (src/elements.cpp:3593-3830, fill_shape_info_at_s)
 *   - element residual/Jacobian in the emission structure of the generated
 *     code (src/codegen.cpp:3912-4110, jitbridge_nohang.h:23-60) for the
 *     weak forms of equations/poisson.py:66-69 and
 *     equations/navier_stokes.py:303-345,481-503
 *   - global sparse assembly with vectors of (column,value) pairs, the
 *     per-contribution zero filter and first-insertion column order
 *     (oomph problem.cc:5332-5666)
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element types */
enum { OFE_Q2_QUAD = 0, OFE_P2_TRI = 1, OFE_Q2_HEX = 2 };
/* equations */
enum { OFE_EQ_POISSON = 0, OFE_EQ_NAVIER_STOKES_TH = 1, OFE_EQ_NONLINEAR_DIFFUSION = 2 };

/* Mesh sizes for a generator (nodes, elements, nodes per element). */
int ofe_mesh_sizes(int etype, int nx, int ny, int nz, int64_t *n_nodes, int64_t *n_elem,
                   int *nnode_el);
/*
 * Fill a structured mesh.  x: [n_nodes*dim], conn: [n_elem*nnode_el],
 * bmask: [n_nodes] boundary bits (1 left, 2 right, 4 bottom, 8 top,
 * 16 back, 32 front), is_vertex: [n_nodes] 1 for C1 (vertex) nodes.
 * split (P2 tri only): 0 = "left", 1 = "right".
 */
int ofe_mesh_fill(int etype, int nx, int ny, int nz, double lx, double ly, double lz, int split,
                  double *x, int32_t *conn, uint32_t *bmask, uint8_t *is_vertex);

/* Oracle assembly result (CSR in the reference's first-insertion order). */
typedef struct ofe_csr {
  int64_t n_dof;
  int64_t nnz;
  int32_t *rowptr;
  int32_t *colidx;
  double *vals;
  double *residual;
} ofe_csr;

/*
 * Assemble R (and J if with_jac) over all elements in mesh order.
 *   values: [n_nodes*nval] nodal values (pinned ones carry their BC value)
 *   eqn:    [n_nodes*nval] global equation numbers, -1 = pinned/absent
 *   params: equation parameters (see fe_oracle.c, equation section)
 *   zero_threshold: oomph's Numerical_zero_for_sparse_assembly (0.0 default;
 *     a negative value keeps every structural entry)
 * Returns NULL on error.
 */
ofe_csr *ofe_assemble(int etype, int eq, int64_t n_nodes, int dim, const double *x,
                      int64_t n_elem, const int32_t *conn, int nval, const double *values,
                      const int32_t *eqn, int64_t n_dof, const double *params, int nparams,
                      int with_jac, double zero_threshold);
void ofe_csr_free(ofe_csr *c);

/* The compressed-row insertion loop (with the zero filter) over given    */
/* element matrices: equations elem_eqn[n_elem][n], matrices Je[n_elem][n][n]. */
ofe_csr *ofe_pairs_from_elements(int64_t n_elem, int n, const int32_t *elem_eqn, const double *Je, int64_t n_dof,
                                 double zero_threshold);

/* Element-level R_e, J_e in the element's full local order (node-major,
 * values per node; absent values skipped).  Returns the local size. */
int ofe_element_res_jac(int etype, int eq, int dim, const double *x, const int32_t *conn_e,
                        int nval, const double *values, const uint8_t *is_vertex,
                        const double *params, int nparams, double *R, double *J);

/* Element mass matrix of the time-derivative term (coeff * int psi_i psi_j
 * between equal time-differentiated values), in the same local order.
 * Returns the local size. */
int ofe_element_mass(int etype, int eq, int dim, const double *x, const int32_t *conn_e, double coeff,
                     double *M);

/* Local-size helper: number of local values of one element. */
int ofe_element_nlocal(int etype, int eq, const int32_t *conn_e, int nval,
                       const uint8_t *is_vertex);

/* Shape/quadrature tables (for pinning against oomph's own tables). */
int ofe_n_intpt(int etype);
void ofe_intpt(int etype, int ipt, double *s, double *w);
void ofe_shape_c2(int etype, const double *s, double *psi, double *dpsids);
void ofe_shape_c1(int etype, const double *s, double *psi, double *dpsids);

#ifdef __cplusplus
}
#endif
#endif
