"""Shared element-level cases: every kernel variant of the workloads
(geometry affine / per point, Jacobian FP64 / FP32) on a small mesh with a
random state, and the oracle's element residuals and matrices for it."""
import numpy as np

import oracle as O

KINDS = ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex", "nldiff_q2"]


def build(kind: str, geometry: str, prec: str, seed: int = 3, jref=None, transient: bool = False,
          residual: str = "fp64"):
    from pyoomph_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    T = W.wavy(0.03) if geometry == "general" else None
    if kind == "ns_th":
        P = W.navier_stokes_problem(N=[4, 3], transform=T, jacobian_precision=prec, transient=transient)
        et, eq, n3 = O.P2_TRI, O.EQ_NAVIER_STOKES_TH, (4, 3, 0)
        params = np.array([1.0, 0.01])
    else:
        et, dim, n3 = {"poisson_q2": (O.Q2_QUAD, 2, (4, 3, 0)), "poisson_p2": (O.P2_TRI, 2, (3, 4, 0)),
                       "nldiff_hex": (O.Q2_HEX, 3, (2, 2, 3)), "nldiff_q2": (O.Q2_QUAD, 2, (3, 3, 0))}[kind]
        gauss = W.draw_gaussians(seed, 8, dim)
        nx = list(n3[:dim])
        if kind.startswith("poisson"):
            P = W.poisson_problem(N=nx, gaussians=gauss, split="left" if et == O.P2_TRI else None, transform=T,
                                  jacobian_precision=prec, transient=transient)
            eq = O.EQ_POISSON
        else:
            P = W.nonlinear_diffusion_problem(N=nx, gaussians=gauss, dim=dim, transform=T, jacobian_precision=prec,
                                              transient=transient)
            eq = O.EQ_NONLINEAR_DIFFUSION
        params = O.gaussian_params(gauss)
    P.geometry = geometry if geometry == "general" else "auto"
    P.jacobian_reference = jref
    P.residual_precision = residual
    ks = P.lower()
    m = P.mesh
    values = P._values0.copy()
    free = P.eqn >= 0
    values[free] += rng.normal(0.0, 0.3, free.sum())
    nval = values.shape[1]
    Rr, Jr = [], []
    for e in range(m.n_elem):
        n = ks.layout.n
        R = np.zeros(n)
        J = np.zeros(n * n)
        O.lib().ofe_element_res_jac(et, eq, m.dim, O._ptr(np.ascontiguousarray(m.x)),
                                   O._ptr(np.ascontiguousarray(m.conn[e])), nval, O._ptr(np.ascontiguousarray(values)),
                                   None, O._ptr(np.ascontiguousarray(params)), len(params), O._ptr(R), O._ptr(J))
        Rr.append(R)
        Jr.append(J.reshape(n, n))
    return P, ks, values, np.array(Rr), np.array(Jr)


def relmax(a, b):
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - b)) / max(np.max(np.abs(b)), 1e-300))
