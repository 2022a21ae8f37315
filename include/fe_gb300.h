/*
 * fe_gb300.h -- C-ABI of the GB300 finite-element assembly engine
 * (libfe_gb300.so).  Plain pointers and sizes; no C++ or torch types.
 *
 * It replaces, for the residual/Jacobian hot path of pyoomph:
 *   - the element function table a JIT element library fills
 *     (JIT_ELEMENT_init / JITFuncSpec_Table_FiniteElement_t,
 *     src/jitbridge.h:329-499) and the per-element call
 *     ResidualAndJacobian[i](eleminfo, shapeinfo, R, J, M, flag)
 *     (src/jitbridge.h:285, called from src/elements.cpp:5104-5113):
 *     fe_code_compile + fe_problem_create take the generated element code
 *     and run it for every element of a domain in one launch;
 *   - the shape buffer callback fill_shape_buffer_for_point
 *     (src/elements.cpp:60, :3593-4270): computed on the device inside the
 *     element kernel from reference tables staged in shared memory;
 *   - the global assembly Problem::get_jacobian / get_residuals with the
 *     vectors-of-pairs sparse assembler (oomph problem.cc:3810-3930,
 *     4038-4165, 5332-5666) and pyoomph's Problem::get_jacobian /
 *     get_residuals (src/problem.cpp:902-965): fe_assemble;
 *   - the residual max-norm of the Newton loop (DoubleVector::max,
 *     double_vector.cc:611-629): fe_residual_max.
 *
 * Every function returns FE_OK (0) or an FE_ERR_* code; fe_last_error()
 * gives the message of the last failure on the calling thread.  No
 * exception crosses the boundary.  A problem handle is not thread-safe;
 * distinct handles may be used from distinct threads.
 */
#ifndef FE_GB300_H
#define FE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FE_OK = 0,
  FE_ERR_ARG = 1,     /* invalid argument */
  FE_ERR_CUDA = 2,    /* CUDA runtime/driver failure */
  FE_ERR_COMPILE = 3, /* nvrtc failed to compile element code */
  FE_ERR_NOMEM = 4,   /* device or host allocation refused */
  FE_ERR_STATE = 5,   /* call out of order */
  FE_ERR_DEVICE = 6,  /* a kernel reported an error in its status word */
  FE_ERR_NOGPU = 7,   /* no usable CUDA device */
  FE_ERR_SOLVER = 8   /* linear solver: not applicable, broke down or did not converge */
};

/* flags of fe_assemble */
enum {
  FE_ASSEMBLE_RESIDUAL = 1, /* fill R (Problem::get_residuals) */
  FE_ASSEMBLE_JACOBIAN = 2, /* fill the CSR values of J (Problem::get_jacobian) */
  FE_ASSEMBLE_VALUES_FROM_DOFS = 4, /* first scatter the dof vector into the nodal values */
  /* each in a call of its own: */
  FE_ASSEMBLE_MASS = 8,   /* J_vals receives the mass matrix dR/d(du/dt) (flag 2 of the
                             generated ResidualAndJacobian, jitbridge.h:285); code of a
                             transient form: fused code, or fixed-mesh code of a problem
                             created with n_history > 0 */
  FE_ASSEMBLE_DPARAM = 16, /* R receives dR/dp for the parameter of fe_problem_set_dparam
                             (dResidual{i}dParameter_{k}, codegen.cpp:4743-4760); fixed-mesh
                             and fused code */
  /* fixed-mesh code only, in a call of its own: */
  FE_ASSEMBLE_HVP = 32,    /* J_vals receives the Hessian-vector product
                              H(y)_ij = sum_k d2R_i/du_j du_k y_k for the direction of
                              fe_problem_set_direction (HessianVectorProduct{i},
                              jitbridge.h:286, codegen.cpp:3646) */
  /* with FE_ASSEMBLE_JACOBIAN or FE_ASSEMBLE_MASS: */
  FE_ASSEMBLE_ZERO_FILTER = 64 /* the matrix in the pattern of oomph's default sparse assembly,
                              which drops every element entry with |J_e(i,j)| <= threshold
                              (Problem::Numerical_zero_for_sparse_assembly, 0.0 by default,
                              problem.cc:110; per contribution, problem.cc:5520-5560): a slot
                              keeps the sum of its surviving contributions in element order,
                              a row's columns come in the order of their first surviving
                              insertion, and slots with none are dropped.  J_vals receives
                              the values in that pattern (at most nnz of them);
                              fe_problem_filtered_pattern gives its rowptr/colidx.  Meshes
                              without hanging values; not with fe_assemble_pipelined */
};

/* Jacobian value precision */
enum { FE_JAC_F64 = 0, FE_JAC_F32 = 1 };

typedef struct fe_code fe_code_t;       /* compiled element code (one domain) */
typedef struct fe_problem fe_problem_t; /* resident mesh + CSR + buffers */

/* Message of the last failing call on this thread ("" if none). */
const char *fe_last_error(void);

/* Library version string. */
const char *fe_version(void);

/* Device 0 properties; FE_ERR_NOGPU without a device. */
int fe_device_info(int *sm_count, int *cc_major, int *cc_minor, size_t *free_bytes,
                   size_t *total_bytes);

/*
 * Compile generated element code for sm_103a with nvrtc and load it.
 * Replaces CCompiler::compile + dlopen/dlsym("JIT_ELEMENT_init")
 * (pyoomph/generic/ccompiler.py:207-242, src/ccompiler.cpp:191-213).
 *   source       CUDA C source of one domain (from the code generator)
 *   kernel_name  extern "C" __global__ entry in that source
 *   include_dir  directory holding fe_device.cuh
 *   cache_dir    directory for cubin caching by source hash (may be NULL)
 *   log/log_cap  compiler log on failure (may be NULL)
 */
int fe_code_compile(const char *source, const char *kernel_name, const char *include_dir,
                    const char *cache_dir, fe_code_t **out, char *log, size_t log_cap);
void fe_code_destroy(fe_code_t *code);

/* Compile only (nvrtc -> cubin into cache_dir); needs no GPU.  cubin_bytes
 * receives the image size.  fe_code_compile reuses the cached image. */
int fe_code_build(const char *source, const char *kernel_name, const char *include_dir,
                  const char *cache_dir, size_t *cubin_bytes, char *log, size_t log_cap);

/* One domain: one element type, one compiled code. */
typedef struct fe_domain_desc {
  fe_code_t *code;
  int nnode_el;             /* nodes per element */
  int nlocal;               /* local values per element, node-major */
  int64_t n_elem;
  const int32_t *conn;      /* host [n_elem * nnode_el], global node numbers */
  const int32_t *local_node;/* host [nlocal]: element node slot of local value k */
  const int32_t *local_val; /* host [nlocal]: nodal value index of local value k */
  const double *tables;     /* host reference tables (layout fixed by the code) */
  int64_t n_tables;
  int elems_per_block;      /* launch shape chosen by the code generator / tuner */
  int threads_per_block;
  int smem_bytes;           /* dynamic shared memory per block */
  int64_t replica_elems;    /* > 0: the elements are replicas of a mesh of this many elements,
                               replica r reading params + r * params_stride (batched serving) */
} fe_domain_desc_t;

typedef struct fe_problem_desc {
  int dim;                  /* nodal dimension */
  int64_t n_nodes;
  int nval;                 /* values per node (max) */
  const double *x;          /* host [n_nodes * dim] nodal positions */
  const int32_t *eqn;       /* host [n_nodes * nval] equation numbers, -1 pinned/absent */
  int64_t n_dof;
  int n_domains;
  const fe_domain_desc_t *domains;
  int n_params;
  const double *params;     /* global parameters read by the element code */
  int jac_precision;        /* FE_JAC_F64 or FE_JAC_F32 */
  int params_stride;        /* parameters per replica (0 = one set for all elements) */
  int n_history;            /* previous time levels of the nodal values kept (BDF; the generated
                               code of a transient form reads levels 0 and 1 = u_{n-1}, u_{n-2}) */
  const double *x0;         /* host [n_nodes * dim] Lagrangian positions (NULL: = x) */
  int fused;                /* 1: every domain shares one fused code, run as one launch */
  /* hanging values (refined meshes; oomph's HangInfo, problem.cc / nodes.h:
   * a constrained value has no equation and equals sum_m w_m * master_m):
   * slot = node * nval + value index; masters are slots that do not hang */
  int64_t n_hang;
  const int64_t *hang_slot;   /* [n_hang] sorted */
  const int64_t *hang_ptr;    /* [n_hang + 1] */
  const int64_t *hang_master; /* [hang_ptr[n_hang]] */
  const double *hang_weight;  /* [hang_ptr[n_hang]] */
} fe_problem_desc_t;

/*
 * Upload the mesh, build the CSR pattern of the global Jacobian in the
 * reference's order (rows = equations; columns of a row in order of first
 * insertion over (element, local i, local j), every structural coupling
 * kept) and the per-slot contribution lists of the deterministic scatter.
 */
int fe_problem_create(const fe_problem_desc_t *desc, fe_problem_t **out);
void fe_problem_destroy(fe_problem_t *p);

/*
 * The same CSR pattern on the host only (no GPU; the domains' code may be
 * NULL).  Call with rowptr = colidx = NULL to get *nnz, then again with
 * buffers of n_dof+1 and nnz entries.
 */
int fe_pattern_host(const fe_problem_desc_t *desc, int64_t *nnz, int32_t *rowptr, int32_t *colidx);

int fe_problem_sizes(const fe_problem_t *p, int64_t *n_dof, int64_t *nnz);
/* Host copies of the CSR pattern. */
int fe_problem_pattern(const fe_problem_t *p, int32_t *rowptr, int32_t *colidx);
/* Device pointers of the resident CSR pattern. */
int fe_problem_pattern_device(const fe_problem_t *p, const int32_t **rowptr,
                              const int32_t **colidx);

/* Set all nodal values (incl. pinned boundary values) from a host array. */
int fe_problem_set_values(fe_problem_t *p, const double *values_host);
/* Read the nodal values back to the host. */
int fe_problem_get_values(const fe_problem_t *p, double *values_host);
/* Time history (implicit time stepping, MultiTimeStepper of
 * timestepper.hpp:46-108): level 0 is the previous step's values.
 * set_history writes one level from the host, get_history reads one back;
 * shift_history moves every level one step back and stores the current
 * values as level 0. */
int fe_problem_set_history(fe_problem_t *p, int level, const double *values_host);
int fe_problem_get_history(const fe_problem_t *p, int level, double *values_host);
int fe_problem_shift_history(fe_problem_t *p);
/* Overwrite the nodal positions (moving meshes keep them as dofs). */
int fe_problem_set_positions(fe_problem_t *p, const double *x_host);

/* Direction y (DEVICE dof vector, n_dof) of FE_ASSEMBLE_HVP assemblies. */
int fe_problem_set_direction(fe_problem_t *p, const double *y, void *stream);

/* Fused problems: launch the element kernel persistently (a grid of the
 * blocks the SMs hold at once, striding over all domains' element blocks)
 * instead of one block per element block.  Off by default. */
int fe_problem_set_persistent(fe_problem_t *p, int enable);

/* Parameter of the next FE_ASSEMBLE_DPARAM assembly (index into params). */
int fe_problem_set_dparam(fe_problem_t *p, int index);

/*
 * Element Jacobians contracted on the tensor cores (tcgen05, 3xTF32 split,
 * FP32 accumulation) for an FP32-Jacobian domain whose generated code writes
 * the pulled-back pointwise derivatives Dhat instead of J_e.  Replaces the
 * contraction loop of the reference's generated Jacobian
 * (write_generic_RJM_jacobian_contribution, codegen.cpp:1883-2258):
 *   J_e[i][j] = sum_q sum_p phi[q][pa[p]][i] Dhat_e[q][p] phi[q][pb[p]][j]
 * phi: HOST [nq][nc][n] reference basis (value and d/ds components at the
 * knots, local function order); pa/pb: HOST [npair] test/trial components.
 * n <= 32, nq <= 32, npair <= 32, nc <= 4, nq x (active test components)
 * <= 128.  fe_problem_set_tensor_contraction attaches it to a domain of a
 * problem (its kernel must be generated for it); fe_tc_contract runs it once
 * on caller buffers (DEVICE dhat [n_elem][nq][npair], jbuf [n_elem][n][n]).
 */
int fe_problem_set_tensor_contraction(fe_problem_t *p, int domain, int n, int nq, int nc, const double *phi, int npair,
                                      const int32_t *pa, const int32_t *pb);
int fe_tc_contract(const float *dhat, float *jbuf, int64_t n_elem, int n, int nq, int nc, const double *phi, int npair,
                   const int32_t *pa, const int32_t *pb, void *stream);

/*
 * Aggregation of the unknowns of a square CSR matrix (HOST arrays) for a
 * smoothed-aggregation multigrid preconditioner of the velocity block of a
 * saddle-point Jacobian (no counterpart on the reference's path, which
 * solves with SuperLU, pyoomph/solvers/scipy.py).  i and j are strongly
 * coupled when comp[i] == comp[j] and |a_ij| >= theta sqrt(|a_ii a_jj|).
 * Three passes in index order (deterministic): a free unknown whose strong
 * neighbours are all free starts an aggregate with them; a remaining
 * unknown joins the aggregate of its first aggregated strong neighbour; the
 * rest start aggregates with their free strong neighbours.  agg[i] in
 * [0, *n_agg).
 */
int fe_sa_aggregate(int64_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                    const int32_t *comp, double theta, int32_t *agg, int64_t *n_agg);

/* How the CSR values are summed from the element matrices (the reference's
 * scatter loop, problem.cc:5500-5560: each slot the sum of its element
 * contributions in element order).  FE_GATHER_SLOTS (default): a thread
 * per slot over the contribution lists, four slots per thread in flight.
 * FE_GATHER_TILES: a warp per tile of whole rows, the residual summed in
 * the same launch, each element-matrix row read once and coalesced; it
 * moves a third less DRAM traffic but is bound by latency at the occupancy
 * its registers allow, and measures faster on small meshes only.  Both give
 * the same bits.  The pipelined host assembly (fe_assemble_pipelined)
 * always sums per slot. */
enum { FE_GATHER_SLOTS = 0, FE_GATHER_TILES = 1 };
int fe_problem_set_gather(fe_problem_t *p, int mode);

/* Lanes per incidence of the tile gather in use, 0 when the per-slot gather
 * runs (FE_GATHER_SLOTS, hanging values, an element wider than 32 local
 * values, a row wider than 255 slots or with more element incidences than
 * a tile holds: 32, or 16 for elements wider than 16 local values); -1 for
 * a null problem. */
int fe_problem_gather_lanes(const fe_problem_t *p);

/* One level of the smoothed-aggregation hierarchy (host, threads), from the
 * n x n CSR matrix A (int32 indices) and its aggregates agg[n] in [0, n_agg)
 * (fe_sa_aggregate):
 *   lam = 1.1 x the largest eigenvalue of D^-1 A (12 power iterations from
 *         a fixed start; D = diag(A), nonzero),
 *   P   = P0 - (4/3)/lam D^-1 A P0   (n x n_agg; P0 the aggregation),
 *   Ac  = P^T A P                    (n_agg x n_agg).
 * Rows are computed independently and sum in a fixed order, columns
 * ascending: the level does not depend on the number of threads.  The
 * handle holds P and Ac until fe_sa_level_copy (rowptr n + 1 / n_agg + 1,
 * colidx and values of the sizes fe_sa_level_info reports); free it with
 * fe_sa_level_destroy.  Replaces the setup of the Newton systems' direct
 * solve (SuperLU, pyoomph/solvers/scipy.py) for Taylor-Hood Jacobians. */
typedef struct fe_sa_level fe_sa_level_t;
int fe_sa_level_build(int64_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                      const int32_t *agg, int64_t n_agg, fe_sa_level_t **out);
int fe_sa_level_info(const fe_sa_level_t *level, int64_t *nnz_p, int64_t *nnz_ac, double *lam);
int fe_sa_level_copy(const fe_sa_level_t *level, int32_t *p_rowptr, int32_t *p_colidx, double *p_vals,
                     int32_t *ac_rowptr, int32_t *ac_colidx, double *ac_vals);
void fe_sa_level_destroy(fe_sa_level_t *level);

/* One block of an n x n CSR matrix split by a label (0 or 1) per row and
 * column index: the rows labelled rl, in order, with their entries in
 * columns labelled cl; rows and columns renumbered within their label,
 * columns ascending within a row, b_slot[k] the entry's position in the
 * input (the saddle-point solver's A, Bt and B blocks of a Taylor-Hood
 * Jacobian).  *nnz is set first; with the three outputs NULL nothing else
 * is written, otherwise b_rowptr (rows labelled rl + 1), b_colidx and
 * b_slot (*nnz) are filled. */
int fe_csr_block(int64_t n, const int32_t *rowptr, const int32_t *colidx, const int8_t *label, int rl, int cl,
                 int64_t *nnz, int32_t *b_rowptr, int32_t *b_colidx, int64_t *b_slot);

/* One Arnoldi step of GMRES with classical Gram-Schmidt applied twice, on
 * DEVICE vectors: for the basis rows V[0..k] (n doubles each, row stride
 * ldv >= n; row k+1 receives the new vector) and w = A z (overwritten):
 * h = V w, w -= V^T h, h2 = V w, w -= V^T h2; hcol[j] = h[j] + h2[j] for
 * j <= k, hcol[k+1] = |w|, V[k+1] = w / |w|.  Reductions over fixed
 * chunks of rows in a fixed order (deterministic).  work: device scratch of
 * fe_gmres_cgs2_scratch(n, kmax) doubles, kmax >= k, k + 2 <= 128.
 * Ordered on `stream`.  The saddle-point solver's Arnoldi process (no
 * counterpart on the reference's path, which solves with SuperLU). */
int64_t fe_gmres_cgs2_scratch(int64_t n, int kmax);
int fe_gmres_cgs2(double *V, int64_t ldv, int64_t n, int k, double *w, double *hcol, double *work, void *stream);

/* Vector steps of the saddle-point solver's FP32 preconditioner (DEVICE
 * pointers, ordered on `stream`):
 *   fe_gather_cast_f32:  dst[i] = (float) src[idx[i]] (times scale[i] when
 *                        scale is not NULL), i < n;
 *   fe_sub_mul_f32:      t = a[i] - b[i] (b NULL: a[i]); c[i] = t (c not
 *                        NULL); x[i] = d[i] t;
 *   fe_scatter_cast_f64: dst[idx[i]] = (double) src[i]. */
int fe_gather_cast_f32(const double *src, const int64_t *idx, int64_t n, const float *scale, float *dst,
                       void *stream);
int fe_sub_mul_f32(const float *a, const float *b, const float *d, float *c, float *x, int64_t n, void *stream);
int fe_scatter_cast_f64(const float *src, const int64_t *idx, int64_t n, double *dst, void *stream);

/* Threshold of FE_ASSEMBLE_ZERO_FILTER assemblies (oomph's
 * Problem::Numerical_zero_for_sparse_assembly, problem.cc:110; default 0.0,
 * must be >= 0). */
int fe_problem_set_zero_threshold(fe_problem_t *p, double threshold);

/* The pattern of the last FE_ASSEMBLE_ZERO_FILTER assembly: waits for
 * `stream`, sets *nnz, and copies rowptr (n_dof + 1) and colidx (*nnz) to
 * rowptr/colidx (host or device pointers; either may be NULL).
 * FE_ERR_STATE before the first filtered assembly. */
int fe_problem_filtered_pattern(fe_problem_t *p, int64_t *nnz, int32_t *rowptr, int32_t *colidx, void *stream);

/* Update the global parameters (host array, n_params values). */
int fe_problem_set_params(fe_problem_t *p, const double *params_host);

/*
 * Assemble on the device.  dofs, R, J_vals are DEVICE pointers (R: n_dof
 * doubles; J_vals: nnz doubles or floats per jac_precision).  With
 * FE_ASSEMBLE_VALUES_FROM_DOFS the dof vector is first scattered into the
 * nodal values.  stream is a cudaStream_t (NULL = legacy default stream).
 * Asynchronous: errors reported by kernels surface at the next
 * fe_problem_check or synchronising call.
 */
int fe_assemble(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags,
                void *stream);

/*
 * Record one fe_assemble (these pointers and flags) as a CUDA graph, and
 * replay it: the Newton loop's assembly as a single graph launch instead of
 * four kernel launches (no counterpart in the reference, whose assembly is
 * a host loop; it replaces the launch sequence behind
 * Problem::get_jacobian, problem.cc:4038).  The graph reads the dof vector
 * and writes R / J_vals at the recorded addresses; parameters, history and
 * values set later through the other calls are read at replay time.
 * Capturing again replaces the recorded graph.
 */
int fe_problem_graph_capture(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags);
int fe_problem_graph_launch(fe_problem_t *p, void *stream);

/*
 * fe_assemble with HOST buffers, pipelined: the dof vector is copied in,
 * the elements run in nchunks consecutive ranges, and after each range the
 * rows it completed (every element touching them done) are gathered and
 * copied to the host on a second stream while the next range computes.  R
 * and J_vals are host buffers (pinned memory for overlap); results equal
 * fe_assemble's bit for bit.  Asynchronous on `stream`: the copies have
 * landed when the stream has completed.  Single-domain problems without
 * replicas; flags RESIDUAL, JACOBIAN, VALUES_FROM_DOFS.  Replaces the same
 * assembly calls as fe_assemble for a caller that keeps R and J on the host
 * (oomph's Problem::get_jacobian, problem.cc:4038-4165).
 */
int fe_assemble_pipelined(fe_problem_t *p, const double *dofs_host, double *R_host, void *J_host, int flags,
                          int nchunks, void *stream);

/* The same with HOST buffers: copies in, assembles, copies out, synchronises. */
int fe_assemble_host(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags);

/*
 * Device sparse kernels of the Newton linear solve (the reference solves on
 * the host with SuperLU, pyoomph/solvers/scipy.py, src/pybind/solver.cpp:105;
 * no counterpart on its assembly path).  DEVICE pointers: CSR rowptr/colidx
 * (the problem's resident pattern, fe_problem_pattern_device), values in
 * FE_JAC_F64 / FE_JAC_F32, FP64 vectors of length n.
 *   fe_csr_spmv:     y = A x; nnz = rowptr[n] (host copy): 4 lanes share
 *                    a row (32 when rows average over 128 entries), one
 *                    FMA per stored entry; the summation order depends only
 *                    on the row and that choice
 *   fe_csr_diagonal: diag[i] = A(i, i)
 */
int fe_csr_spmv(const int32_t *rowptr, const int32_t *colidx, const void *vals, int val_precision, const double *x,
                double *y, int64_t n, int64_t nnz, void *stream);
/* y = z + sc * w o (b - A x) for an FP64 CSR matrix (square or not; DEVICE
 * pointers), z, b, w each optional (NULL: 0, 0, 1): the damped-Jacobi,
 * residual and prolongation updates of the saddle-point solver's multigrid
 * cycle in one pass over the matrix (no counterpart on the reference's
 * path, which solves with SuperLU).  y must not alias x. */
int fe_csr_update(const int32_t *rowptr, const int32_t *colidx, const double *vals, const double *x, const double *b,
                  const double *z, const double *w, double sc, double *y, int64_t n, int64_t nnz, void *stream);
/* The same in FP32 (values and vectors): the saddle-point solver's FP32
 * multigrid cycle.  With b, z, w NULL and sc = -1 it is y = A x. */
int fe_csr_update_f32(const int32_t *rowptr, const int32_t *colidx, const float *vals, const float *x, const float *b,
                      const float *z, const float *w, float sc, float *y, int64_t n, int64_t nnz, void *stream);
int fe_csr_diagonal(const int32_t *rowptr, const int32_t *colidx, const void *vals, int val_precision, double *diag,
                    int64_t n, void *stream);

/*
 * Batched device Newton linear solve: Jacobi-preconditioned BiCGStab on the
 * `blocks` diagonal blocks of a stacked CSR matrix (block s owns rows
 * s*n/blocks .. (s+1)*n/blocks and couples only to them: the replicas of a
 * problem; blocks = 1 for one system).  Replaces the host SuperLU solve of
 * the reference's Newton step (pyoomph/solvers/scipy.py,
 * src/pybind/solver.cpp:105) for diffusion-type Jacobians.
 *
 * Every scalar and every reduction is per block, the reductions run over
 * fixed chunks of a block's rows in a fixed order, and a block stops at the
 * iteration its own residual reaches max(tol * ||b_s||_inf, atol) (atol:
 * an absolute floor, e.g. a fraction of a Newton tolerance; a block whose
 * ||b_s|| is already below it returns x_s = 0): a block's solution
 * is bit-identical whatever the other blocks hold.  Iterations run on the
 * solver's own stream (ordered after and before `stream` by events), in
 * blocks of check_every iterations replayed as one CUDA graph (use_graph);
 * the host reads the per-block state words between blocks.  A converged
 * block is confirmed by its true residual (<= 10 * target, else it
 * restarts); a breakdown restores the block's iterate from the last check
 * and restarts it (at most max_restarts times).
 *
 * create: DEVICE rowptr/colidx/vals stay owned by the caller and must stay
 *         valid (values may change between solves).
 * solve:  DEVICE b (n) and x (n, written for every block: inactive blocks
 *         get 0); HOST active[blocks] (NULL = all) and iterations[blocks]
 *         (may be NULL).  FE_ERR_SOLVER for a zero diagonal entry in an
 *         active block (saddle-point systems), a non-finite right-hand
 *         side, repeated breakdown or no convergence in maxiter.
 */
typedef struct fe_krylov fe_krylov_t;
int fe_krylov_create(const int32_t *rowptr, const int32_t *colidx, const void *vals, int val_precision, int64_t n,
                     int64_t nnz, int32_t blocks, int32_t check_every, int32_t use_graph, fe_krylov_t **out);
int fe_krylov_solve(fe_krylov_t *k, const double *b, const uint8_t *active, double tol, double atol,
                    int64_t maxiter, int32_t max_restarts, double *x, int64_t *iterations, void *stream);
/* y = A x (every row, DEVICE vectors of n) with the solver's matrix and
 * SpMV kernel (that of fe_csr_spmv).  Ordered on `stream`. */
int fe_krylov_matvec(fe_krylov_t *k, const double *x, double *y, void *stream);
/* kernel launches (graph nodes included), graph replays, restarts so far. */
int fe_krylov_info(const fe_krylov_t *k, int64_t *launches, int64_t *graph_replays, int64_t *restarts);
void fe_krylov_destroy(fe_krylov_t *k);

/* max |R| over n entries of a device vector, NaN -> +inf; result to host. */
int fe_residual_max(fe_problem_t *p, const double *R, int64_t n, double *out, void *stream);

/*
 * Allocation-free residual max-norm.  No counterpart in the reference: it is
 * an addition of this library for callers that cannot allocate device
 * memory.  fe_residual_max needs a problem handle, and creating one
 * allocates (mesh, CSR, element buffers).  A caller that only holds a
 * residual vector in device memory and may not call cudaMalloc -- for
 * example code that owns all device memory through its own pool, or code
 * that must not allocate between set-up and shutdown -- uses this instead.
 *
 * Same result as fe_residual_max: max |R[i]| over n entries of the device
 * vector R, NaN -> +inf, written to the host double *out; synchronises the
 * stream (cudaStream_t, NULL = legacy default stream).
 *
 * It allocates nothing: its scratch is a static device array of 256 KiB
 * that every GPU loading the library holds until the process exits.  n may
 * be at most fe_residual_max_noalloc_limit() (268,427,264 entries); larger
 * n is rejected with FE_ERR_ARG and a message.  The first call on a device
 * looks up the array's device address with that device current; make that
 * first call before any stream capture.  All calls share the array and the
 * last call's contents stay in it: calls that overlap on the GPU (other
 * streams or threads) race and must be serialised by the caller.
 */
int fe_residual_max_noalloc(const double *R, int64_t n, double *out, void *stream);
/* Largest n fe_residual_max_noalloc accepts. */
int64_t fe_residual_max_noalloc_limit(void);

/* x[i] -= dx[i] for device vectors (the Newton update). */
int fe_dof_update(fe_problem_t *p, double *x, const double *dx, int64_t n, void *stream);

/*
 * Element-level results of the last assembly of a domain (host copies):
 * R_e [n_elem][nlocal] doubles, J_e [n_elem][nlocal][nlocal] in the Jacobian
 * precision, local order node-major (either pointer may be NULL).  The
 * element residual/Jacobian R_e, J_e of GeneralisedElement::get_jacobian
 * (elements.h:990-999) that the reference checks against finite differences
 * (BulkElementBase::debug_analytical_jacobian, elements.cpp:5880).
 */
int fe_problem_element_buffers(fe_problem_t *p, int domain, double *R_e, void *J_e);

/* Synchronise the problem's work and report any kernel status error. */
int fe_problem_check(fe_problem_t *p);

/*
 * Stage tracing.  With timing enabled, fe_assemble records CUDA events on
 * its stream around its stages; fe_problem_stage_times synchronises,
 * returns the summed milliseconds per stage since the last query
 * (ms[0] dof scatter, ms[1] element kernels, ms[2] residual gather,
 * ms[3] Jacobian gather, ms[4] tensor-core contraction of the element
 * matrices; ms has room for 5) and the number of calls, and resets the sums.
 * The counterpart of oomph's Jacobian_setup_time (linear_solver.cc:884-894).
 */
int fe_problem_set_timing(fe_problem_t *p, int enable);
int fe_problem_stage_times(fe_problem_t *p, double *ms, int64_t *calls);

/*
 * Timeline of the last fe_assemble_pipelined call made with timing enabled:
 * per chunk k, milliseconds from the call's start to the end of its element
 * kernel (ms[3k]), of its gathers (ms[3k+1]) and of the copies of the rows
 * it completes (ms[3k+2]).  Synchronises on those events; returns the
 * number of chunks (0: no timed call), FE_ERR_ARG when cap < 3 x chunks.
 */
int fe_problem_pipeline_times(fe_problem_t *p, float *ms, int cap);

/*
 * Element streams of fe_assemble_pipelined: 1 (chunks in order on one
 * stream), 2 (consecutive chunks on alternating streams, which may run
 * concurrently) or 0 (automatic: one).  The values are the same bits
 * either way; two streams measured faster only for FP64 Jacobians, and
 * not reliably.
 */
int fe_problem_set_pipeline_streams(fe_problem_t *p, int n);

/* Number of element and scatter kernels one fe_assemble launches. */
int fe_problem_launch_count(const fe_problem_t *p, int flags);

#ifdef __cplusplus
}
#endif
#endif
