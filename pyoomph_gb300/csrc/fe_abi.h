// fe_abi.h -- argument block shared by the runtime (fe_gb300.cu) and the
// generated element kernels (compiled by nvrtc, which include fe_device.cuh).
// Plain types only: the same bytes are built on the host and read on the
// device through the kernel-parameter buffer.
#ifndef FE_ABI_H
#define FE_ABI_H

struct FeElemArgs {
  const double *x;      // [n_nodes * dim] nodal positions
  const int *conn;      // [n_elem * nnode] global node numbers
  const double *values; // [n_nodes * nval] nodal values
  const double *params; // global parameters
  const double *tables; // reference shape/quadrature tables of the element type
  double *rbuf;         // [n_elem * nlocal] element residuals
  void *jbuf;           // [n_elem * nlocal * nlocal] element Jacobians (f64 or f32)
  long long n_elem;
  int nval;
  int flag;             // 0: residual only, 1: residual and Jacobian
  int *status;          // device status word (0 = ok)
  long long replica_elems; // > 0: the domain is a stack of replicas of this many elements each
  int params_stride;       // parameters per replica (replica r reads params + r * params_stride)
  const double *hist;      // [n_hist][n_nodes * nval] nodal values of previous time levels
  const double *x0;        // [n_nodes * dim] Lagrangian (reference) positions
  int n_hist;
  long long hist_stride;    // entries per history level (n_nodes * nval)
  int aux;                  // flag 3: index of the parameter of dR/dp
  long long n_nodes;        // nodes of the problem (bounds of conn entries)
  const double *dir;        // flag 4: nodal values of the direction y of the Hessian-vector product
  float *dhat;              // [n_elem][nq][npair] pulled-back derivatives, written instead of J_e by
                            // kernels whose Jacobian is contracted on the tensor cores (fe_tc.cuh)
};

// One launch over several domains (bulk, interface, contact line ...): block
// b runs domain k for block_start[k] <= b < block_start[k+1].
#define FE_MAX_FUSED 4
struct FeFusedArgs {
  FeElemArgs d[FE_MAX_FUSED];
  int block_start[FE_MAX_FUSED + 1];
  int n_domains;
};

#endif
