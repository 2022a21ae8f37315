// fe_device.cuh -- device helpers included by the generated element kernels
// (compiled at run time by nvrtc for sm_103a; no standard headers).
#ifndef FE_DEVICE_CUH
#define FE_DEVICE_CUH

#include "fe_abi.h"
#include "fe_df64.cuh"

// Bounds-checked build (compile the element code with -DFE_BOUNDS_CHECK=1):
// a connectivity entry outside [0, n_nodes) is replaced by node 0, and the
// kernel records status 2 with the element index instead of reading out of
// bounds.  The check the sanitizer would make, as an error word.
#if defined(FE_BOUNDS_CHECK) && FE_BOUNDS_CHECK
#define FE_CHECK_NODE(node, elem, args)                                          \
  do {                                                                           \
    if ((node) < 0 || (long long)(node) >= (args).n_nodes) {                     \
      atomicExch((args).status + 1, (int)(elem));                                \
      atomicExch((args).status, 2);                                              \
      (node) = 0;                                                                \
    }                                                                            \
  } while (0)
#else
#define FE_CHECK_NODE(node, elem, args) \
  do {                                  \
  } while (0)
#endif

// Geometry at one integration point through the metric tensor, the route of
// BulkElementBase::fill_shape_info_at_s (src/elements.cpp:3593-3990):
//   t[a][i]  = sum_l x_l,i dpsi_l/ds_a         (tangent vectors)
//   a_ab     = t_a . t_b,  aup = a^{-1}
//   g[b][i]  = sum_a aup(a,b) t[a][i]          ([g^{ab} g_a]_i)
//   J        = sqrt(det a_ab)
// so that d/dx_i = sum_b g[b][i] d/ds_b and the weight is W * J.
template <int DIM, int NN>
__device__ __forceinline__ void fe_metric_geometry(const double *__restrict__ X,
                                                   const double *__restrict__ dps,
                                                   double (&g)[DIM][DIM], double &J) {
  double t[DIM][DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a)
#pragma unroll
    for (int i = 0; i < DIM; ++i) t[a][i] = 0.0;
#pragma unroll
  for (int l = 0; l < NN; ++l)
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      const double xl = X[l * DIM + i];
#pragma unroll
      for (int a = 0; a < DIM; ++a) t[a][i] += xl * dps[l * DIM + a];
    }
  double am[DIM][DIM];
#pragma unroll
  for (int al = 0; al < DIM; ++al)
#pragma unroll
    for (int be = 0; be < DIM; ++be) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i) s += t[al][i] * t[be][i];
      am[al][be] = s;
    }
  double aup[DIM][DIM];
  double det;
  if constexpr (DIM == 1) {
    det = am[0][0];
    aup[0][0] = 1.0 / det;
  } else if constexpr (DIM == 2) {
    det = am[0][0] * am[1][1] - am[0][1] * am[1][0];
    const double idet = 1.0 / det;
    aup[0][0] = am[1][1] * idet;
    aup[0][1] = -am[0][1] * idet;
    aup[1][0] = -am[1][0] * idet;
    aup[1][1] = am[0][0] * idet;
  } else {
    det = am[0][0] * am[1][1] * am[2][2] + am[0][1] * am[1][2] * am[2][0] + am[0][2] * am[1][0] * am[2][1] -
          am[0][0] * am[1][2] * am[2][1] - am[0][1] * am[1][0] * am[2][2] - am[0][2] * am[1][1] * am[2][0];
    const double idet = 1.0 / det;
    aup[0][0] = (am[1][1] * am[2][2] - am[1][2] * am[2][1]) * idet;
    aup[0][1] = -(am[0][1] * am[2][2] - am[0][2] * am[2][1]) * idet;
    aup[0][2] = (am[0][1] * am[1][2] - am[0][2] * am[1][1]) * idet;
    aup[1][0] = -(am[1][0] * am[2][2] - am[1][2] * am[2][0]) * idet;
    aup[1][1] = (am[0][0] * am[2][2] - am[0][2] * am[2][0]) * idet;
    aup[1][2] = -(am[0][0] * am[1][2] - am[0][2] * am[1][0]) * idet;
    aup[2][0] = (am[1][0] * am[2][1] - am[1][1] * am[2][0]) * idet;
    aup[2][1] = -(am[0][0] * am[2][1] - am[0][1] * am[2][0]) * idet;
    aup[2][2] = (am[0][0] * am[1][1] - am[0][1] * am[1][0]) * idet;
  }
#pragma unroll
  for (int b = 0; b < DIM; ++b)
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < DIM; ++a) s += aup[a][b] * t[a][i];
      g[b][i] = s;
    }
  J = sqrt(det);
}

// Physical shape gradients dx[l][i] = sum_b g[b][i] dps[l][b] (dx_shape_*
// of the shape buffer), written in the Jacobian's precision T.
template <int DIM, int NN, typename T>
__device__ __forceinline__ void fe_phys_grad(const double (&g)[DIM][DIM], const double *__restrict__ dps,
                                             T *__restrict__ out) {
  T gl[DIM][DIM];
#pragma unroll
  for (int b = 0; b < DIM; ++b)
#pragma unroll
    for (int i = 0; i < DIM; ++i) gl[b][i] = (T)g[b][i];
#pragma unroll
  for (int l = 0; l < NN; ++l) {
    T d[DIM];
#pragma unroll
    for (int b = 0; b < DIM; ++b) d[b] = (T)dps[l * DIM + b];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      T s = (T)0;
#pragma unroll
      for (int b = 0; b < DIM; ++b) s += gl[b][i] * d[b];
      out[l * DIM + i] = s;
    }
  }
}

// Sum of n Gaussians A exp(-|x-c|^2 / (2 w^2)); parameters per Gaussian:
// c_0..c_{DIM-1}, w, A (contiguous).  A loop, not unrolled: it keeps the
// element kernel's register footprint independent of n.
template <int DIM>
__device__ __noinline__ double fe_gauss_sum(const double *__restrict__ Xq, const double *__restrict__ g, int n) {
  double f = 0.0;
#pragma unroll 1
  for (int k = 0; k < n; ++k, g += DIM + 2) {
    double r2 = 0.0;
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      const double d = Xq[i] - g[i];
      r2 += d * d;
    }
    const double w = g[DIM];
    f += g[DIM + 1] * exp(-r2 / (2.0 * w * w));
  }
  return f;
}

// d/dg_j of the same sum for one parameter, j = k (DIM + 2) + m of Gaussian
// k: m < DIM (centre c_m): A E (x_m - c_m) / w^2; m = DIM (width): A E r^2 /
// w^3; m = DIM + 1 (amplitude): E, with E = exp(-r^2 / (2 w^2)).
template <int DIM>
__device__ __noinline__ double fe_gauss_dparam(const double *__restrict__ Xq, const double *__restrict__ g, int j) {
  const int k = j / (DIM + 2), m = j - k * (DIM + 2);
  const double *gk = g + k * (DIM + 2);
  double r2 = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    const double d = Xq[i] - gk[i];
    r2 += d * d;
  }
  const double w = gk[DIM], e = exp(-r2 / (2.0 * w * w));
  if (m == DIM + 1) return e;
  const double a = gk[DIM + 1];
  if (m == DIM) return a * e * r2 / (w * w * w);
  return a * e * (Xq[m] - gk[m]) / (w * w);
}

// The same sum on an axis-aligned affine tensor-product element, separably:
// exp(-|x-c|^2/(2w^2)) = prod_d exp(-(x_d-c_d)^2/(2w^2)), and along axis d
// the knots take only three coordinates, so the element's factors
// T[k][d][i] are evaluated once per element (3 DIM exponentials per
// Gaussian instead of one per knot); qi = the knot's index along each axis.
template <int DIM>
__device__ __forceinline__ double fe_gauss_sep(const double *__restrict__ T, const int *__restrict__ qi,
                                               const double *__restrict__ g, int n) {
  double f = 0.0;
#pragma unroll 1
  for (int k = 0; k < n; ++k, g += DIM + 2, T += DIM * 3) {
    double p = g[DIM + 1];
#pragma unroll
    for (int d = 0; d < DIM; ++d) p *= T[d * 3 + qi[d]];
    f += p;
  }
  return f;
}

#endif
