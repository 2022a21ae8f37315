/*
 * fe_oracle.c -- CPU oracle for the pyoomph residual/Jacobian assembly path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this code, and only as
 * the checker or the timed CPU baseline.  The GPU product never calls it.
 *
 * Every function below cites the reference file:line whose behaviour it
 * restates (paths relative to the pyoomph project root; oomph-lib files are
 * under src/thirdparty/oomph-lib/include/).  See fe_oracle.h for the list.
 */
#include "fe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Quadrature tables.  The constants are the reference's own, digit for     */
/* digit, including the transposed digits ("...662941...") of some knots of */
/* Gauss<2,3> (integral.cc:84-102): parity at 1e-12 needs the same knots.   */
/* ------------------------------------------------------------------------ */

/* Gauss<2,3>: integral.cc:84-102 */
static const double GQ2_KNOT[9][2] = {
    {-0.774596669241483, -0.774596669241483}, {-0.774596669241483, 0.0},
    {-0.774596669241483, 0.774596662941483},  {0.0, -0.774596669241483},
    {0.0, 0.0},                               {0.0, 0.774596662941483},
    {0.774596662941483, -0.774596669241483},  {0.774596662941483, 0.0},
    {0.774596662941483, 0.774596662941483}};
static const double GQ2_W[9] = {(25.0 / 81.0), (40.0 / 81.0), (25.0 / 81.0),
                                (40.0 / 81.0), (64.0 / 81.0), (40.0 / 81.0),
                                (25.0 / 81.0), (40.0 / 81.0), (25.0 / 81.0)};

/* TGauss<2,3>: integral.cc:355-369 */
static const double GT2_KNOT[7][2] = {{0.1012865073235, 0.1012865073235},
                                      {0.7974269853531, 0.1012865073235},
                                      {0.1012865073235, 0.7974269853531},
                                      {0.4701420641051, 0.0597158717898},
                                      {0.4701420641051, 0.4701420641051},
                                      {0.0597158717898, 0.4701420641051},
                                      {0.3333333333333, 0.3333333333333}};
static const double GT2_W[7] = {0.5 * 0.1259391805448, 0.5 * 0.1259391805448,
                                0.5 * 0.1259391805448, 0.5 * 0.1323941527885,
                                0.5 * 0.1323941527885, 0.5 * 0.1323941527885,
                                0.5 * 0.225};

/* Gauss<3,3>: integral.cc:169-206 (knots on a 3x3x3 lexicographic grid,
 * last index fastest, 14 significant digits) */
static const double GH3_1D[3] = {-0.77459666924148, 0.0, 0.77459666924148};
static const double GH3_W[27] = {
    0.17146776406035, 0.27434842249657, 0.17146776406035, 0.27434842249657,
    0.43895747599451, 0.27434842249657, 0.17146776406035, 0.27434842249657,
    0.17146776406035, 0.27434842249657, 0.43895747599451, 0.27434842249657,
    0.43895747599451, 0.70233196159122, 0.43895747599451, 0.27434842249657,
    0.43895747599451, 0.27434842249657, 0.17146776406035, 0.27434842249657,
    0.17146776406035, 0.27434842249657, 0.43895747599451, 0.27434842249657,
    0.17146776406035, 0.27434842249657, 0.17146776406035};

int ofe_n_intpt(int etype) {
  switch (etype) {
  case OFE_Q2_QUAD: return 9;
  case OFE_P2_TRI: return 7;
  case OFE_Q2_HEX: return 27;
  }
  return 0;
}

void ofe_intpt(int etype, int ipt, double *s, double *w) {
  if (etype == OFE_Q2_QUAD) {
    s[0] = GQ2_KNOT[ipt][0]; s[1] = GQ2_KNOT[ipt][1]; *w = GQ2_W[ipt];
  } else if (etype == OFE_P2_TRI) {
    s[0] = GT2_KNOT[ipt][0]; s[1] = GT2_KNOT[ipt][1]; *w = GT2_W[ipt];
  } else {
    /* integral.cc:169: knot i = (k0[i/9], k1[(i/3)%3], k2[i%3]) */
    s[0] = GH3_1D[ipt / 9]; s[1] = GH3_1D[(ipt / 3) % 3]; s[2] = GH3_1D[ipt % 3];
    *w = GH3_W[ipt];
  }
}

/* ------------------------------------------------------------------------ */
/* Shape functions                                                           */
/* ------------------------------------------------------------------------ */
/* OneDimLagrange::shape<3>/dshape<3> (shape.h:633-650) */
static void lag3(double s, double *p, double *d) {
  p[0] = 0.5 * s * (s - 1.0); p[1] = 1.0 - s * s; p[2] = 0.5 * s * (s + 1.0);
  d[0] = s - 0.5; d[1] = -2.0 * s; d[2] = s + 0.5;
}
/* OneDimLagrange::shape<2>/dshape<2> (shape.h:607-620) */
static void lag2(double s, double *p, double *d) {
  p[0] = 0.5 * (1.0 - s); p[1] = 0.5 * (1.0 + s);
  d[0] = -0.5; d[1] = 0.5;
}

/* C2 space of the element.  dpsids is [n][dim]. */
void ofe_shape_c2(int etype, const double *s, double *psi, double *dpsids) {
  if (etype == OFE_Q2_QUAD) {
    /* QElement<2,3>: psi[3*i+j] = psi_s1[i]*psi_s0[j] (Qelements.h) */
    double p0[3], d0[3], p1[3], d1[3];
    lag3(s[0], p0, d0); lag3(s[1], p1, d1);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        int n = 3 * i + j;
        psi[n] = p1[i] * p0[j];
        dpsids[2 * n + 0] = p1[i] * d0[j];
        dpsids[2 * n + 1] = d1[i] * p0[j];
      }
  } else if (etype == OFE_P2_TRI) {
    /* TElementShape<2,3>::dshape_local (Telements.h:627-680) */
    double s2 = 1.0 - s[0] - s[1];
    psi[0] = 2.0 * s[0] * (s[0] - 0.5);
    psi[1] = 2.0 * s[1] * (s[1] - 0.5);
    psi[2] = 2.0 * s2 * (s2 - 0.5);
    psi[3] = 4.0 * s[0] * s[1];
    psi[4] = 4.0 * s[1] * s2;
    psi[5] = 4.0 * s2 * s[0];
    dpsids[0] = 4.0 * s[0] - 1.0;            dpsids[1] = 0.0;
    dpsids[2] = 0.0;                         dpsids[3] = 4.0 * s[1] - 1.0;
    dpsids[4] = 2.0 * (2.0 * s[0] - 1.5 + 2.0 * s[1]);
    dpsids[5] = 2.0 * (2.0 * s[0] - 1.5 + 2.0 * s[1]);
    dpsids[6] = 4.0 * s[1];                  dpsids[7] = 4.0 * s[0];
    dpsids[8] = -4.0 * s[1];                 dpsids[9] = 4.0 * (1.0 - s[0] - 2.0 * s[1]);
    dpsids[10] = 4.0 * (1.0 - 2.0 * s[0] - s[1]); dpsids[11] = -4.0 * s[0];
  } else {
    /* QElement<3,3>: psi[9*i+3*j+k] = psi_s2[i]*psi_s1[j]*psi_s0[k] */
    double p0[3], d0[3], p1[3], d1[3], p2[3], d2[3];
    lag3(s[0], p0, d0); lag3(s[1], p1, d1); lag3(s[2], p2, d2);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++) {
          int n = 9 * i + 3 * j + k;
          psi[n] = p2[i] * p1[j] * p0[k];
          dpsids[3 * n + 0] = p2[i] * p1[j] * d0[k];
          dpsids[3 * n + 1] = p2[i] * d1[j] * p0[k];
          dpsids[3 * n + 2] = d2[i] * p1[j] * p0[k];
        }
  }
}

/* C1 space of the element (vertex nodes).  elements.cpp:9274-9300 (quad),
 * :10097-10130 (tri), :11163 (brick). */
void ofe_shape_c1(int etype, const double *s, double *psi, double *dpsids) {
  if (etype == OFE_Q2_QUAD) {
    double p0[2], d0[2], p1[2], d1[2];
    lag2(s[0], p0, d0); lag2(s[1], p1, d1);
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        int n = 2 * i + j;
        psi[n] = p1[i] * p0[j];
        dpsids[2 * n + 0] = p1[i] * d0[j];
        dpsids[2 * n + 1] = d1[i] * p0[j];
      }
  } else if (etype == OFE_P2_TRI) {
    psi[0] = s[0]; psi[1] = s[1]; psi[2] = 1.0 - s[0] - s[1];
    dpsids[0] = 1.0; dpsids[1] = 0.0; dpsids[2] = 0.0; dpsids[3] = 1.0;
    dpsids[4] = -1.0; dpsids[5] = -1.0;
  } else {
    double p0[2], d0[2], p1[2], d1[2], p2[2], d2[2];
    lag2(s[0], p0, d0); lag2(s[1], p1, d1); lag2(s[2], p2, d2);
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) {
          int n = 4 * i + 2 * j + k;
          psi[n] = p2[i] * p1[j] * p0[k];
          dpsids[3 * n + 0] = p2[i] * p1[j] * d0[k];
          dpsids[3 * n + 1] = p2[i] * d1[j] * p0[k];
          dpsids[3 * n + 2] = d2[i] * p1[j] * p0[k];
        }
  }
}

static int etype_dim(int etype) { return etype == OFE_Q2_HEX ? 3 : 2; }
static int etype_nnode(int etype) {
  return etype == OFE_Q2_QUAD ? 9 : (etype == OFE_P2_TRI ? 6 : 27);
}
static int etype_nnode_c1(int etype) {
  return etype == OFE_Q2_QUAD ? 4 : (etype == OFE_P2_TRI ? 3 : 8);
}
/* get_node_index_C1_to_element: element-local indices of the C1 nodes */
static const int C1_IDX_QUAD[4] = {0, 2, 6, 8};
static const int C1_IDX_TRI[3] = {0, 1, 2};
static const int C1_IDX_HEX[8] = {0, 2, 6, 8, 18, 20, 24, 26};
static const int *c1_index(int etype) {
  return etype == OFE_Q2_QUAD ? C1_IDX_QUAD : (etype == OFE_P2_TRI ? C1_IDX_TRI : C1_IDX_HEX);
}
/* local C1 number of element node l, or -1 */
static int c1_of_node(int etype, int l) {
  const int *idx = c1_index(etype);
  for (int k = 0; k < etype_nnode_c1(etype); k++)
    if (idx[k] == l) return k;
  return -1;
}

/* ------------------------------------------------------------------------ */
/* Shape info at an integration point: the metric-tensor formulation of     */
/* BulkElementBase::fill_shape_info_at_s (elements.cpp:3593-3990) and the   */
/* weight of fill_shape_buffer_for_integration_point (elements.cpp:4573).   */
/* ------------------------------------------------------------------------ */
typedef struct {
  double w;              /* int_pt_weight = W * sqrt(det(g_ab)) */
  double x[3];           /* interpolated Eulerian position */
  double psi2[27];
  double dx2[27][3];     /* dx_shape_C2 */
  double psi1[8];
  double dx1[8][3];      /* dx_shape_C1 */
} shapeinfo_t;

static void fill_shape_info(int etype, const double *X /* [nnode][dim] */, int ipt,
                            shapeinfo_t *si) {
  const int dim = etype_dim(etype), nn = etype_nnode(etype), n1 = etype_nnode_c1(etype);
  double s[3] = {0, 0, 0}, W;
  ofe_intpt(etype, ipt, s, &W);
  double dps[27 * 3], dps1[8 * 3];
  ofe_shape_c2(etype, s, si->psi2, dps);
  ofe_shape_c1(etype, s, si->psi1, dps1);
  /* interpolated_t(j,i) += x(l,i) * dpsids(l,j) */
  double t[3][3] = {{0}};
  for (int l = 0; l < nn; l++)
    for (int i = 0; i < dim; i++)
      for (int j = 0; j < dim; j++) t[j][i] += X[l * dim + i] * dps[l * dim + j];
  double a[3][3];
  for (int al = 0; al < dim; al++)
    for (int be = 0; be < dim; be++) {
      a[al][be] = 0.0;
      for (int i = 0; i < dim; i++) a[al][be] += t[al][i] * t[be][i];
    }
  double aup[3][3], g[3][3], det_a;
  if (dim == 2) {
    det_a = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    aup[0][0] = a[1][1] / det_a;
    aup[0][1] = -a[0][1] / det_a;
    aup[1][0] = -a[1][0] / det_a;
    aup[1][1] = a[0][0] / det_a;
    for (int b = 0; b < 2; b++)
      for (int i = 0; i < 2; i++) g[b][i] = aup[0][b] * t[0][i] + aup[1][b] * t[1][i];
  } else {
    det_a = a[0][0] * a[1][1] * a[2][2] + a[0][1] * a[1][2] * a[2][0] +
            a[0][2] * a[1][0] * a[2][1] - a[0][0] * a[1][2] * a[2][1] -
            a[0][1] * a[1][0] * a[2][2] - a[0][2] * a[1][1] * a[2][0];
    aup[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det_a;
    aup[0][1] = -(a[0][1] * a[2][2] - a[0][2] * a[2][1]) / det_a;
    aup[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det_a;
    aup[1][0] = -(a[1][0] * a[2][2] - a[1][2] * a[2][0]) / det_a;
    aup[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det_a;
    aup[1][2] = -(a[0][0] * a[1][2] - a[0][2] * a[1][0]) / det_a;
    aup[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det_a;
    aup[2][1] = -(a[0][0] * a[2][1] - a[0][1] * a[2][0]) / det_a;
    aup[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det_a;
    for (int b = 0; b < 3; b++)
      for (int i = 0; i < 3; i++)
        g[b][i] = aup[0][b] * t[0][i] + aup[1][b] * t[1][i] + aup[2][b] * t[2][i];
  }
  const double J = sqrt(det_a);
  si->w = W * J;
  for (int i = 0; i < 3; i++) si->x[i] = 0.0;
  for (int l = 0; l < nn; l++)
    for (int i = 0; i < dim; i++) si->x[i] += X[l * dim + i] * si->psi2[l];
  for (int l = 0; l < nn; l++)
    for (int i = 0; i < dim; i++) {
      si->dx2[l][i] = 0.0;
      for (int b = 0; b < dim; b++) si->dx2[l][i] += g[b][i] * dps[l * dim + b];
    }
  for (int l = 0; l < n1; l++)
    for (int i = 0; i < dim; i++) {
      si->dx1[l][i] = 0.0;
      for (int b = 0; b < dim; b++) si->dx1[l][i] += g[b][i] * dps1[l * dim + b];
    }
}

/* ------------------------------------------------------------------------ */
/* Source term: a sum of Gaussians, f(x) = sum_k A_k exp(-|x-c_k|^2/(2w_k^2)) */
/* params layout: [ng, then per Gaussian: c_0..c_{dim-1}, w, A]             */
/* ------------------------------------------------------------------------ */
static double gauss_source(const double *params, int dim, const double *x) {
  int ng = (int)params[0];
  const double *p = params + 1;
  double f = 0.0;
  for (int k = 0; k < ng; k++) {
    double r2 = 0.0;
    for (int i = 0; i < dim; i++) {
      double d = x[i] - p[i];
      r2 += d * d;
    }
    double w = p[dim], A = p[dim + 1];
    f += A * exp(-r2 / (2.0 * w * w));
    p += dim + 2;
  }
  return f;
}

/* ------------------------------------------------------------------------ */
/* Element local layout: node-major, the values present at each node in     */
/* value order (C2 fields at every node, C1 fields at C1 nodes only).       */
/* This is oomph's nodal local numbering (elements.cc:694) before pinned    */
/* values are skipped.                                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nval;            /* values per node (max) */
  int nc2;             /* leading values that live on the C2 space */
  int n;               /* local size */
  int node[27 * 4];    /* node of local index */
  int val[27 * 4];     /* value index of local index */
  int loc[27][4];      /* local index of (node, value), -1 if absent */
} layout_t;

static void make_layout(int etype, int eq, layout_t *L) {
  const int nn = etype_nnode(etype);
  if (eq == OFE_EQ_NAVIER_STOKES_TH) { L->nval = 3; L->nc2 = 2; }
  else { L->nval = 1; L->nc2 = 1; }
  L->n = 0;
  for (int l = 0; l < nn; l++)
    for (int v = 0; v < L->nval; v++) {
      int present = (v < L->nc2) || (c1_of_node(etype, l) >= 0);
      if (present) {
        L->loc[l][v] = L->n;
        L->node[L->n] = l;
        L->val[L->n] = v;
        L->n++;
      } else {
        L->loc[l][v] = -1;
      }
    }
}

int ofe_element_nlocal(int etype, int eq, const int32_t *conn_e, int nval,
                       const uint8_t *is_vertex) {
  (void)conn_e; (void)nval; (void)is_vertex;
  layout_t L;
  make_layout(etype, eq, &L);
  return L.n;
}

/* ------------------------------------------------------------------------ */
/* Element residual/Jacobian, in the structure of the generated code:       */
/* gp loop -> shape info -> interpolation -> test loop (BEGIN_RESIDUAL) ->  */
/* shape loop (BEGIN_JACOBIAN).  R, J are caller-zeroed (elements.h:993).   */
/* ------------------------------------------------------------------------ */

/* Poisson, equations/poisson.py:66-69:
 *   weak(grad(u), grad(v)) - weak(f, v) */
static void rj_poisson(int etype, const double *X, const double *U /* [nnode] */,
                       const double *params, const layout_t *L, double *R, double *J,
                       int flag) {
  const int dim = etype_dim(etype), nn = etype_nnode(etype), nq = ofe_n_intpt(etype);
  const int n = L->n;
  shapeinfo_t si;
  for (int ipt = 0; ipt < nq; ipt++) {
    fill_shape_info(etype, X, ipt, &si);
    const double dx = si.w;
    double u = 0.0, gu[3] = {0, 0, 0};
    for (int l = 0; l < nn; l++) {
      u += U[l] * si.psi2[l];
      for (int i = 0; i < dim; i++) gu[i] += U[l] * si.dx2[l][i];
    }
    (void)u;
    const double f = gauss_source(params, dim, si.x);
    for (int lt = 0; lt < nn; lt++) {
      const int ie = L->loc[lt][0];
      double gg = 0.0;
      for (int i = 0; i < dim; i++) gg += gu[i] * si.dx2[lt][i];
      R[ie] += (gg - f * si.psi2[lt]) * dx;
      if (flag) {
        for (int ls = 0; ls < nn; ls++) {
          const int je = L->loc[ls][0];
          double gs = 0.0;
          for (int i = 0; i < dim; i++) gs += si.dx2[ls][i] * si.dx2[lt][i];
          J[ie * n + je] += gs * dx;
        }
      }
    }
  }
}

/* Nonlinear diffusion -div((1+u^2) grad u) = f:
 *   weak((1+u^2) grad(u), grad(v)) - weak(f, v) */
static void rj_nldiff(int etype, const double *X, const double *U, const double *params,
                      const layout_t *L, double *R, double *J, int flag) {
  const int dim = etype_dim(etype), nn = etype_nnode(etype), nq = ofe_n_intpt(etype);
  const int n = L->n;
  shapeinfo_t si;
  for (int ipt = 0; ipt < nq; ipt++) {
    fill_shape_info(etype, X, ipt, &si);
    const double dx = si.w;
    double u = 0.0, gu[3] = {0, 0, 0};
    for (int l = 0; l < nn; l++) {
      u += U[l] * si.psi2[l];
      for (int i = 0; i < dim; i++) gu[i] += U[l] * si.dx2[l][i];
    }
    const double k = 1.0 + u * u;
    const double f = gauss_source(params, dim, si.x);
    for (int lt = 0; lt < nn; lt++) {
      const int ie = L->loc[lt][0];
      double gg = 0.0;
      for (int i = 0; i < dim; i++) gg += gu[i] * si.dx2[lt][i];
      R[ie] += (k * gg - f * si.psi2[lt]) * dx;
      if (flag) {
        for (int ls = 0; ls < nn; ls++) {
          const int je = L->loc[ls][0];
          double gs = 0.0;
          for (int i = 0; i < dim; i++) gs += si.dx2[ls][i] * si.dx2[lt][i];
          J[ie * n + je] += (k * gs + 2.0 * u * si.psi2[ls] * gg) * dx;
        }
      }
    }
  }
}

/* Steady incompressible Navier-Stokes, Taylor-Hood (velocity C2, pressure C1),
 * equations/navier_stokes.py:303-345 (Stokes part) and :481-503 (advection):
 *   weak(2 mu sym(grad u) - p I, grad v) + weak(div u, q)
 *   + weak(rho (u.grad) u, v)
 * params: [rho, mu].  Values per node: 0 = u_x, 1 = u_y, 2 = p. */
static void rj_ns_th(int etype, const double *X, const double *U /* [nnode][3] */,
                     const double *params, const layout_t *L, double *R, double *J, int flag) {
  const int nn = etype_nnode(etype), n1 = etype_nnode_c1(etype), nq = ofe_n_intpt(etype);
  const int *c1 = c1_index(etype);
  const int n = L->n;
  const double rho = params[0], mu = params[1];
  shapeinfo_t si;
  for (int ipt = 0; ipt < nq; ipt++) {
    fill_shape_info(etype, X, ipt, &si);
    const double dx = si.w;
    double u[2] = {0, 0}, gu[2][2] = {{0, 0}, {0, 0}}, p = 0.0; /* gu[k][i] = d u_k / d x_i */
    for (int l = 0; l < nn; l++)
      for (int k = 0; k < 2; k++) {
        u[k] += U[l * 3 + k] * si.psi2[l];
        for (int i = 0; i < 2; i++) gu[k][i] += U[l * 3 + k] * si.dx2[l][i];
      }
    for (int l = 0; l < n1; l++) p += U[c1[l] * 3 + 2] * si.psi1[l];
    /* stress tau_ki = mu (du_k/dx_i + du_i/dx_k) - p delta_ki */
    double tau[2][2], adv[2];
    for (int k = 0; k < 2; k++) {
      for (int i = 0; i < 2; i++) tau[k][i] = mu * (gu[k][i] + gu[i][k]) - (k == i ? p : 0.0);
      adv[k] = rho * (u[0] * gu[k][0] + u[1] * gu[k][1]);
    }
    const double divu = gu[0][0] + gu[1][1];
    /* momentum test functions (C2) */
    for (int lt = 0; lt < nn; lt++) {
      for (int k = 0; k < 2; k++) {
        const int ie = L->loc[lt][k];
        R[ie] += (tau[k][0] * si.dx2[lt][0] + tau[k][1] * si.dx2[lt][1] + adv[k] * si.psi2[lt]) * dx;
        if (!flag) continue;
        /* d/d u_m at node ls */
        for (int ls = 0; ls < nn; ls++) {
          for (int m = 0; m < 2; m++) {
            const int je = L->loc[ls][m];
            double c = 0.0;
            /* viscous: mu (d(du_k/dx_i)/du_m + d(du_i/dx_k)/du_m) dphi/dx_i */
            for (int i = 0; i < 2; i++) {
              double dd = 0.0;
              if (m == k) dd += si.dx2[ls][i];
              if (m == i) dd += si.dx2[ls][k];
              c += mu * dd * si.dx2[lt][i];
            }
            /* advection: rho (psi u_m-part) */
            double dadv = rho * si.psi2[ls] * gu[k][m];
            if (m == k) dadv += rho * (u[0] * si.dx2[ls][0] + u[1] * si.dx2[ls][1]);
            c += dadv * si.psi2[lt];
            J[ie * n + je] += c * dx;
          }
        }
        /* d/d p at C1 node */
        for (int ls = 0; ls < n1; ls++) {
          const int je = L->loc[c1[ls]][2];
          J[ie * n + je] += -si.psi1[ls] * si.dx2[lt][k] * dx;
        }
      }
    }
    /* continuity test functions (C1) */
    for (int lt = 0; lt < n1; lt++) {
      const int ie = L->loc[c1[lt]][2];
      R[ie] += divu * si.psi1[lt] * dx;
      if (!flag) continue;
      for (int ls = 0; ls < nn; ls++)
        for (int m = 0; m < 2; m++) {
          const int je = L->loc[ls][m];
          J[ie * n + je] += si.dx2[ls][m] * si.psi1[lt] * dx;
        }
    }
  }
}

static int element_rj(int etype, int eq, int dim, const double *x, const int32_t *ce, int nval,
                      const double *values, const double *params, const layout_t *L,
                      double *R, double *J, int flag) {
  const int nn = etype_nnode(etype);
  double X[27 * 3], U[27 * 3];
  for (int l = 0; l < nn; l++) {
    for (int i = 0; i < dim; i++) X[l * dim + i] = x[(int64_t)ce[l] * dim + i];
    for (int v = 0; v < nval; v++) U[l * nval + v] = values[(int64_t)ce[l] * nval + v];
  }
  memset(R, 0, sizeof(double) * L->n);
  if (flag) memset(J, 0, sizeof(double) * L->n * L->n);
  switch (eq) {
  case OFE_EQ_POISSON: rj_poisson(etype, X, U, params, L, R, J, flag); break;
  case OFE_EQ_NONLINEAR_DIFFUSION: rj_nldiff(etype, X, U, params, L, R, J, flag); break;
  case OFE_EQ_NAVIER_STOKES_TH: rj_ns_th(etype, X, U, params, L, R, J, flag); break;
  default: return -1;
  }
  return L->n;
}

int ofe_element_res_jac(int etype, int eq, int dim, const double *x, const int32_t *conn_e,
                        int nval, const double *values, const uint8_t *is_vertex,
                        const double *params, int nparams, double *R, double *J) {
  (void)is_vertex; (void)nparams;
  layout_t L;
  make_layout(etype, eq, &L);
  if (L.nval != nval) return -1;
  return element_rj(etype, eq, dim, x, conn_e, nval, values, params, &L, R, J, 1);
}

/* Element mass matrix of the time-derivative term: M_e(i, j) = coeff *
 * int psi_i psi_j dx between equal time-differentiated values (the velocity
 * components for Navier-Stokes, coeff = rho: rho partial_t(u) of
 * navier_stokes.py:481-503 through generic.py:564; the field of a scalar
 * equation, coeff = temporal_factor: DiffusionEquation, poisson.py:153-180).
 * These forms are linear in du/dt with a coefficient independent of u, so
 * the transient element residual is R_e(u) + M_e udot_e and its Jacobian
 * J_e + w0 M_e, udot the BDF combination of the nodal time levels and w0
 * its weight of the current level; M_e is flag 2 of the generated code
 * (jitbridge.h:285). */
int ofe_element_mass(int etype, int eq, int dim, const double *x, const int32_t *conn_e, double coeff,
                     double *M) {
  layout_t L;
  make_layout(etype, eq, &L);
  const int nn = etype_nnode(etype), nq = ofe_n_intpt(etype), n = L.n;
  const int nt = eq == OFE_EQ_NAVIER_STOKES_TH ? 2 : 1;
  double X[27 * 3];
  for (int l = 0; l < nn; l++)
    for (int i = 0; i < dim; i++) X[l * dim + i] = x[(int64_t)conn_e[l] * dim + i];
  memset(M, 0, sizeof(double) * n * n);
  shapeinfo_t si;
  for (int ipt = 0; ipt < nq; ipt++) {
    fill_shape_info(etype, X, ipt, &si);
    for (int lt = 0; lt < nn; lt++)
      for (int ls = 0; ls < nn; ls++) {
        const double m = coeff * si.psi2[lt] * si.psi2[ls] * si.w;
        for (int k = 0; k < nt; k++) M[L.loc[lt][k] * n + L.loc[ls][k]] += m;
      }
  }
  return n;
}

/* ------------------------------------------------------------------------ */
/* Global assembly: Problem::sparse_assemble_row_or_column_compressed_with_ */
/* vectors_of_pairs (problem.cc:5332-5666), compressed-row branch.          */
/* Rows are vectors of (column, value); an element entry is skipped if      */
/* |value| <= zero_threshold; otherwise the row is searched linearly for    */
/* the column and either accumulated or appended.  The CSR keeps the row's  */
/* insertion order (problem.cc:5620-5660).                                  */
/* ------------------------------------------------------------------------ */
typedef struct { int32_t col; double val; } pair_t;
typedef struct { pair_t *p; int n, cap; } rowvec_t;

static void row_add(rowvec_t *r, int32_t col, double v) {
  for (int k = 0; k <= r->n; k++) {
    if (k == r->n) {
      if (r->n == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 16;
        r->p = (pair_t *)realloc(r->p, sizeof(pair_t) * r->cap);
      }
      r->p[r->n].col = col;
      r->p[r->n].val = v;
      r->n++;
      return;
    } else if (r->p[k].col == col) {
      r->p[k].val += v;
      return;
    }
  }
}

ofe_csr *ofe_assemble(int etype, int eq, int64_t n_nodes, int dim, const double *x,
                      int64_t n_elem, const int32_t *conn, int nval, const double *values,
                      const int32_t *eqn, int64_t n_dof, const double *params, int nparams,
                      int with_jac, double zero_threshold) {
  (void)n_nodes; (void)nparams;
  layout_t L;
  make_layout(etype, eq, &L);
  if (L.nval != nval || etype_dim(etype) != dim) return NULL;
  const int nn = etype_nnode(etype), n = L.n;
  ofe_csr *out = (ofe_csr *)calloc(1, sizeof(ofe_csr));
  out->n_dof = n_dof;
  out->residual = (double *)calloc((size_t)(n_dof > 0 ? n_dof : 1), sizeof(double));
  rowvec_t *rows = with_jac ? (rowvec_t *)calloc((size_t)(n_dof > 0 ? n_dof : 1), sizeof(rowvec_t)) : NULL;
  double *R = (double *)malloc(sizeof(double) * n);
  double *J = (double *)malloc(sizeof(double) * n * n);
  int32_t geq[27 * 4];
  for (int64_t e = 0; e < n_elem; e++) {
    const int32_t *ce = conn + e * nn;
    element_rj(etype, eq, dim, x, ce, nval, values, params, &L, R, J, with_jac);
    for (int i = 0; i < n; i++) geq[i] = eqn[(int64_t)ce[L.node[i]] * nval + L.val[i]];
    /* local dofs are the unpinned entries, in local order */
    for (int i = 0; i < n; i++) {
      const int32_t ei = geq[i];
      if (ei < 0) continue;
      out->residual[ei] += R[i];
      if (!with_jac) continue;
      for (int j = 0; j < n; j++) {
        const int32_t ej = geq[j];
        if (ej < 0) continue;
        const double v = J[i * n + j];
        if (fabs(v) > zero_threshold) row_add(&rows[ei], ej, v);
      }
    }
  }
  free(R);
  free(J);
  if (with_jac) {
    out->rowptr = (int32_t *)malloc(sizeof(int32_t) * (n_dof + 1));
    out->rowptr[0] = 0;
    for (int64_t i = 0; i < n_dof; i++) out->rowptr[i + 1] = out->rowptr[i] + rows[i].n;
    out->nnz = out->rowptr[n_dof];
    out->colidx = (int32_t *)malloc(sizeof(int32_t) * (out->nnz > 0 ? out->nnz : 1));
    out->vals = (double *)malloc(sizeof(double) * (out->nnz > 0 ? out->nnz : 1));
    for (int64_t i = 0; i < n_dof; i++) {
      int32_t o = out->rowptr[i];
      for (int k = 0; k < rows[i].n; k++) {
        out->colidx[o + k] = rows[i].p[k].col;
        out->vals[o + k] = rows[i].p[k].val;
      }
      free(rows[i].p);
    }
    free(rows);
  }
  return out;
}

/* The same compressed-row insertion loop over GIVEN element matrices:     */
/* elem_eqn[e * n + k] is the global equation of local value k of element  */
/* e (-1: none), Je[e * n * n + i * n + j] its element matrix.  Checks a   */
/* device compaction of the filtered pattern on the device's own element   */
/* matrices (no residual).                                                 */
ofe_csr *ofe_pairs_from_elements(int64_t n_elem, int n, const int32_t *elem_eqn, const double *Je, int64_t n_dof,
                                 double zero_threshold) {
  ofe_csr *out = (ofe_csr *)calloc(1, sizeof(ofe_csr));
  out->n_dof = n_dof;
  out->residual = (double *)calloc(1, sizeof(double));
  rowvec_t *rows = (rowvec_t *)calloc((size_t)(n_dof > 0 ? n_dof : 1), sizeof(rowvec_t));
  for (int64_t e = 0; e < n_elem; e++) {
    const int32_t *geq = elem_eqn + e * n;
    const double *J = Je + e * (int64_t)n * n;
    for (int i = 0; i < n; i++) {
      const int32_t ei = geq[i];
      if (ei < 0) continue;
      for (int j = 0; j < n; j++) {
        const int32_t ej = geq[j];
        if (ej < 0) continue;
        const double v = J[i * n + j];
        if (fabs(v) > zero_threshold) row_add(&rows[ei], ej, v);
      }
    }
  }
  out->rowptr = (int32_t *)malloc(sizeof(int32_t) * (n_dof + 1));
  out->rowptr[0] = 0;
  for (int64_t i = 0; i < n_dof; i++) out->rowptr[i + 1] = out->rowptr[i] + rows[i].n;
  out->nnz = out->rowptr[n_dof];
  out->colidx = (int32_t *)malloc(sizeof(int32_t) * (out->nnz > 0 ? out->nnz : 1));
  out->vals = (double *)malloc(sizeof(double) * (out->nnz > 0 ? out->nnz : 1));
  for (int64_t i = 0; i < n_dof; i++) {
    int32_t o = out->rowptr[i];
    for (int k = 0; k < rows[i].n; k++) {
      out->colidx[o + k] = rows[i].p[k].col;
      out->vals[o + k] = rows[i].p[k].val;
    }
    free(rows[i].p);
  }
  free(rows);
  return out;
}

void ofe_csr_free(ofe_csr *c) {
  if (!c) return;
  free(c->rowptr);
  free(c->colidx);
  free(c->vals);
  free(c->residual);
  free(c);
}

/* ------------------------------------------------------------------------ */
/* Mesh templates                                                           */
/* ------------------------------------------------------------------------ */
/* MeshTemplate::add_node_unique (meshtemplate.cpp:1378) deduplicates by     */
/* position through a kd-tree.  The structured templates here put every node */
/* on a half-cell lattice, so an exact lattice key gives the same answer.    */
typedef struct {
  int64_t *map;       /* lattice key -> node index (-1 = none) */
  int64_t n;          /* nodes created */
  int dim;
  double *x;
  uint32_t *bmask;
  uint8_t *is_vertex;
} builder_t;

static int64_t add_node(builder_t *b, int64_t key, const double *pos, uint32_t bm, int vertex) {
  if (b->map[key] >= 0) {
    int64_t i = b->map[key];
    /* intermediate nodes merge boundary info only while it is empty
     * (meshtemplate.cpp:1400-1418) */
    if (b->bmask[i] == 0) b->bmask[i] = bm;
    return i;
  }
  int64_t i = b->n++;
  b->map[key] = i;
  for (int d = 0; d < b->dim; d++) b->x[i * b->dim + d] = pos[d];
  b->bmask[i] = bm;
  b->is_vertex[i] = (uint8_t)vertex;
  return i;
}

int ofe_mesh_sizes(int etype, int nx, int ny, int nz, int64_t *n_nodes, int64_t *n_elem,
                   int *nnode_el) {
  if (nx < 1 || ny < 1) return -1;
  if (etype == OFE_Q2_QUAD) {
    *n_nodes = (int64_t)(2 * nx + 1) * (2 * ny + 1);
    *n_elem = (int64_t)nx * ny;
    *nnode_el = 9;
  } else if (etype == OFE_P2_TRI) {
    *n_nodes = (int64_t)(2 * nx + 1) * (2 * ny + 1);
    *n_elem = (int64_t)2 * nx * ny;
    *nnode_el = 6;
  } else if (etype == OFE_Q2_HEX) {
    if (nz < 1) return -1;
    *n_nodes = (int64_t)(2 * nx + 1) * (2 * ny + 1) * (2 * nz + 1);
    *n_elem = (int64_t)nx * ny * nz;
    *nnode_el = 27;
  } else {
    return -1;
  }
  return 0;
}

enum { B_LEFT = 1, B_RIGHT = 2, B_BOTTOM = 4, B_TOP = 8, B_BACK = 16, B_FRONT = 32 };

int ofe_mesh_fill(int etype, int nx, int ny, int nz, double lx, double ly, double lz, int split,
                  double *x, int32_t *conn, uint32_t *bmask, uint8_t *is_vertex) {
  int64_t n_nodes, n_elem;
  int nne;
  if (ofe_mesh_sizes(etype, nx, ny, nz, &n_nodes, &n_elem, &nne)) return -1;
  builder_t b;
  b.map = (int64_t *)malloc(sizeof(int64_t) * n_nodes);
  for (int64_t i = 0; i < n_nodes; i++) b.map[i] = -1;
  b.n = 0;
  b.dim = etype_dim(etype);
  b.x = x;
  b.bmask = bmask;
  b.is_vertex = is_vertex;
  const int64_t LX = 2 * nx + 1, LY = 2 * ny + 1;

  if (etype == OFE_Q2_QUAD || etype == OFE_P2_TRI) {
    /* RectangularQuadMesh.define_geometry (simplemeshes.py:225-305):
     * ix outer, iy inner; corners n00, n10, n01, n11. */
    const int ntri = (etype == OFE_P2_TRI);
    int32_t *c1 = (int32_t *)malloc(sizeof(int32_t) * n_elem * 4);
    int64_t ec = 0;
    for (int ix = 0; ix < nx; ix++)
      for (int iy = 0; iy < ny; iy++) {
        int64_t nd[4];
        for (int c = 0; c < 4; c++) {
          int px = c & 1, py = c >> 1;
          double pos[2] = {(double)(ix + px) * lx / nx + 0.0, (double)(iy + py) * ly / ny + 0.0};
          uint32_t bm = 0;
          /* boundaries: left ix==0 {n00,n01}, right ix==nx-1 {n10,n11},
           * bottom iy==0 {n00,n10}, top iy==ny-1 {n01,n11} */
          if (ix == 0 && px == 0) bm |= B_LEFT;
          if (ix == nx - 1 && px == 1) bm |= B_RIGHT;
          if (iy == 0 && py == 0) bm |= B_BOTTOM;
          if (iy == ny - 1 && py == 1) bm |= B_TOP;
          int64_t key = (int64_t)(2 * (ix + px)) + LX * (int64_t)(2 * (iy + py));
          nd[c] = add_node(&b, key, pos, 0, 1);
          b.bmask[nd[c]] |= bm;
        }
        if (!ntri) {
          int32_t *q = c1 + ec * 4;
          q[0] = (int32_t)nd[0]; q[1] = (int32_t)nd[1]; q[2] = (int32_t)nd[2]; q[3] = (int32_t)nd[3];
          ec++;
        } else {
          /* split "left": (n00,n10,n11),(n00,n11,n01); "right": (n01,n10,n11),(n00,n10,n01) */
          int32_t *t0 = c1 + ec * 4, *t1 = c1 + (ec + 1) * 4;
          if (split == 0) {
            t0[0] = (int32_t)nd[0]; t0[1] = (int32_t)nd[1]; t0[2] = (int32_t)nd[3];
            t1[0] = (int32_t)nd[0]; t1[1] = (int32_t)nd[3]; t1[2] = (int32_t)nd[2];
          } else {
            t0[0] = (int32_t)nd[2]; t0[1] = (int32_t)nd[1]; t0[2] = (int32_t)nd[3];
            t1[0] = (int32_t)nd[0]; t1[1] = (int32_t)nd[1]; t1[2] = (int32_t)nd[2];
          }
          ec += 2;
        }
      }
    /* C2 conversion per element in order (meshtemplate.cpp:401-409, 494-499) */
#define KEY2(a, bb) ((int64_t)((lat[a][0] + lat[bb][0]) / 2) + LX * (int64_t)((lat[a][1] + lat[bb][1]) / 2))
    for (int64_t e = 0; e < ec; e++) {
      int32_t *v = c1 + e * 4;
      int nv = ntri ? 3 : 4;
      int64_t lat[4][2];
      for (int k = 0; k < nv; k++) {
        /* recover lattice coordinates from the stored position */
        lat[k][0] = (int64_t)llround(x[v[k] * 2 + 0] / lx * nx * 2);
        lat[k][1] = (int64_t)llround(x[v[k] * 2 + 1] / ly * ny * 2);
      }
#define MID2(a, bb, out)                                                                 \
  do {                                                                                   \
    double pos[2] = {0.5 * (x[v[a] * 2 + 0] + x[v[bb] * 2 + 0]),                          \
                     0.5 * (x[v[a] * 2 + 1] + x[v[bb] * 2 + 1])};                         \
    out = add_node(&b, KEY2(a, bb), pos, b.bmask[v[a]] & b.bmask[v[bb]], 0);               \
  } while (0)
      int32_t *ce = conn + e * nne;
      if (!ntri) {
        int64_t n1, n3, n4, n5, n7;
        MID2(0, 1, n1);
        MID2(0, 2, n3);
        {
          double pos[2] = {0.25 * (x[v[0] * 2] + x[v[1] * 2] + x[v[2] * 2] + x[v[3] * 2]),
                           0.25 * (x[v[0] * 2 + 1] + x[v[1] * 2 + 1] + x[v[2] * 2 + 1] + x[v[3] * 2 + 1])};
          int64_t key = (int64_t)((lat[0][0] + lat[3][0]) / 2) + LX * (int64_t)((lat[0][1] + lat[3][1]) / 2);
          n4 = add_node(&b, key, pos, 0, 0);
        }
        MID2(1, 3, n5);
        MID2(2, 3, n7);
        ce[0] = v[0]; ce[1] = (int32_t)n1; ce[2] = v[1];
        ce[3] = (int32_t)n3; ce[4] = (int32_t)n4; ce[5] = (int32_t)n5;
        ce[6] = v[2]; ce[7] = (int32_t)n7; ce[8] = v[3];
      } else {
        int64_t n3, n4, n5;
        MID2(0, 1, n3);
        MID2(1, 2, n4);
        MID2(0, 2, n5);
        ce[0] = v[0]; ce[1] = v[1]; ce[2] = v[2];
        ce[3] = (int32_t)n3; ce[4] = (int32_t)n4; ce[5] = (int32_t)n5;
      }
#undef MID2
    }
#undef KEY2
    free(c1);
  } else {
    /* CuboidBrickMesh.define_geometry (simplemeshes.py:515-545):
     * ix, iy, iz loops; corners 000,100,010,110,001,101,011,111. */
    const int64_t LZ = 2 * nz + 1;
    (void)LZ;
    int32_t *c1 = (int32_t *)malloc(sizeof(int32_t) * n_elem * 8);
    int64_t ec = 0;
    for (int ix = 0; ix < nx; ix++)
      for (int iy = 0; iy < ny; iy++)
        for (int iz = 0; iz < nz; iz++) {
          int32_t *h = c1 + ec * 8;
          for (int c = 0; c < 8; c++) {
            int px = c & 1, py = (c >> 1) & 1, pz = c >> 2;
            double pos[3] = {(double)(ix + px) * lx / nx + 0.0, (double)(iy + py) * ly / ny + 0.0,
                             (double)(iz + pz) * lz / nz + 0.0};
            uint32_t bm = 0;
            if (ix == 0 && px == 0) bm |= B_LEFT;
            if (ix == nx - 1 && px == 1) bm |= B_RIGHT;
            if (iy == 0 && py == 0) bm |= B_BOTTOM;
            if (iy == ny - 1 && py == 1) bm |= B_TOP;
            if (iz == 0 && pz == 0) bm |= B_BACK;
            if (iz == nz - 1 && pz == 1) bm |= B_FRONT;
            int64_t key = (int64_t)(2 * (ix + px)) + LX * ((int64_t)(2 * (iy + py)) + LY * (int64_t)(2 * (iz + pz)));
            int64_t nd = add_node(&b, key, pos, 0, 1);
            b.bmask[nd] |= bm;
            h[c] = (int32_t)nd;
          }
          ec++;
        }
    /* C2 conversion (meshtemplate.cpp:579-621), in its call order */
    for (int64_t e = 0; e < ec; e++) {
      int32_t *v = c1 + e * 8;
      int64_t ni[27];
      int64_t lat[27][3];
      double P[27][3];
      const int corner_of[8] = {0, 2, 6, 8, 18, 20, 24, 26};
      for (int k = 0; k < 8; k++) {
        ni[corner_of[k]] = v[k];
        for (int d = 0; d < 3; d++) P[corner_of[k]][d] = x[v[k] * 3 + d];
        lat[corner_of[k]][0] = llround(P[corner_of[k]][0] / lx * nx * 2);
        lat[corner_of[k]][1] = llround(P[corner_of[k]][1] / ly * ny * 2);
        lat[corner_of[k]][2] = llround(P[corner_of[k]][2] / lz * nz * 2);
      }
      /* two-parent intermediate: out = mid(a, b) over element-local slots */
#define HMID(out, a, bb)                                                                    \
  do {                                                                                     \
    for (int d = 0; d < 3; d++) { P[out][d] = 0.5 * (P[a][d] + P[bb][d]); lat[out][d] = (lat[a][d] + lat[bb][d]) / 2; } \
    int64_t key = lat[out][0] + LX * (lat[out][1] + LY * lat[out][2]);                       \
    ni[out] = add_node(&b, key, P[out], b.bmask[ni[a]] & b.bmask[ni[bb]], 0);                  \
  } while (0)
      /* four-parent intermediate (face/body centre) */
#define HQUAD(out, a, bb, c, dd, bposs)                                                      \
  do {                                                                                      \
    for (int d = 0; d < 3; d++) { P[out][d] = 0.25 * (P[a][d] + P[bb][d] + P[c][d] + P[dd][d]); lat[out][d] = (lat[a][d] + lat[bb][d] + lat[c][d] + lat[dd][d]) / 4; } \
    int64_t key = lat[out][0] + LX * (lat[out][1] + LY * lat[out][2]);                        \
    uint32_t bm = (bposs) ? (b.bmask[ni[a]] & b.bmask[ni[bb]] & b.bmask[ni[c]] & b.bmask[ni[dd]]) : 0u; \
    ni[out] = add_node(&b, key, P[out], bm, 0);                                               \
  } while (0)
      HMID(1, 0, 2);
      HMID(3, 0, 6);
      HQUAD(4, 0, 2, 6, 8, 1);
      HMID(5, 2, 8);
      HMID(7, 6, 8);
      HMID(9, 0, 18);
      HMID(11, 2, 20);
      HMID(15, 6, 24);
      HMID(17, 8, 26);
      HMID(19, 18, 20);
      HMID(21, 18, 24);
      HQUAD(22, 18, 20, 24, 26, 1);
      HMID(23, 20, 26);
      HMID(25, 24, 26);
      HMID(10, 9, 11);
      HMID(12, 9, 15);
      HMID(14, 11, 17);
      HMID(16, 15, 17);
      /* ninds[13] = avg of corners 0,3,5,6 of the C1 brick = slots 0,8,20,24 */
      HQUAD(13, 0, 8, 20, 24, 0);
#undef HMID
#undef HQUAD
      int32_t *ce = conn + e * nne;
      for (int k = 0; k < 27; k++) ce[k] = (int32_t)ni[k];
    }
    free(c1);
  }
  free(b.map);
  return (b.n == n_nodes) ? 0 : -2;
}
