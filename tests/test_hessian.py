"""Hessian-vector products H(y)_ij = sum_k d2R_i/(du_j du_k) y_k of the
fixed-mesh kernels (pyoomph's HessianVectorProduct).  For the Navier-Stokes
and nonlinear-diffusion weak forms the Jacobian is at most quadratic in u,
so a central difference of the oracle's Jacobian along y is exact up to
rounding: that is the reference here."""
import numpy as np
import pytest

import oracle as O


def _oracle(kind, n, seed):
    from pyoomph_gb300 import workloads as W
    if kind == "ns":
        return O.navier_stokes_problem(O.mesh(O.P2_TRI, n, n), rho=1.0, mu=0.02)
    return O.poisson_problem(O.mesh(O.Q2_QUAD, n, n), W.draw_gaussians(seed, 16, 2), eq=O.EQ_NONLINEAR_DIFFUSION)


def _fd_hvp(OP, x, y, eps=1e-3):
    OP.set_dofs(x + eps * y)
    _, rp, ci, vp = O.assemble(OP, True, -1.0)
    OP.set_dofs(x - eps * y)
    _, rp2, ci2, vm = O.assemble(OP, True, -1.0)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    OP.set_dofs(x)
    return rp, ci, (vp - vm) / (2 * eps)


def _product(kind, n, prec):
    from pyoomph_gb300 import workloads as W
    if kind == "ns":
        P = W.navier_stokes_problem(N=n, Re=50.0, jacobian_precision=prec)
    else:
        P = W.nonlinear_diffusion_problem(N=n, seed=1, dim=2, jacobian_precision=prec)
    return P


@pytest.mark.parametrize("kind", ["ns", "nldiff"])
def test_emulated_hvp_matches_central_differences_of_the_oracle_jacobian(kind):
    import kernel_emulator as KE
    P = _product(kind, 3, "fp64")
    ks = P.lower()
    rng = np.random.default_rng(7)
    vals = P._values0.copy()
    free = P.eqn >= 0
    vals[free] += rng.normal(0.0, 0.3, free.sum())
    yv = np.zeros_like(vals)
    yv[free] = rng.normal(0.0, 1.0, free.sum())
    _, H, status = KE.run(ks, P.mesh.x, P.mesh.conn, vals, P.params, flag=4, direction=yv)
    assert not status.any()
    # the same element Hessian-vector products from two emulated Jacobians
    _, Jp, _ = KE.run(ks, P.mesh.x, P.mesh.conn, vals + 1e-3 * yv, P.params, flag=1)
    _, Jm, _ = KE.run(ks, P.mesh.x, P.mesh.conn, vals - 1e-3 * yv, P.params, flag=1)
    fd = (Jp - Jm) / 2e-3
    assert np.max(np.abs(H - fd)) <= 1e-9 * max(1.0, np.max(np.abs(fd)))


@pytest.mark.gpu
@pytest.mark.parametrize("kind,prec", [("ns", "fp64"), ("nldiff", "fp64"), ("nldiff", "fp32")])
def test_gpu_hvp_matches_the_oracle(kind, prec):
    P = _product(kind, 6, prec)
    P.initialise()
    OP = _oracle(kind, 6, 1)
    rng = np.random.default_rng(3)
    x = OP.dofs() + rng.normal(0.0, 0.2, OP.n_dof)
    y = rng.normal(0.0, 1.0, OP.n_dof)
    P.set_dofs(x)
    H = P.get_hessian_vector_product(y)
    rp, ci, ref = _fd_hvp(OP, x, y)
    prp, pci = P.pattern()
    assert np.array_equal(prp, rp) and np.array_equal(pci, ci)
    tol = 1e-9 if prec == "fp64" else 1e-5
    assert np.max(np.abs(H.data - ref)) <= tol * max(1.0, np.max(np.abs(ref)))
    # the Jacobian path is unaffected afterwards
    R, J = P.get_jacobian()
    OP.set_dofs(x)
    _, _, _, jv = O.assemble(OP, True, -1.0)
    assert np.max(np.abs(J.data - jv)) <= (1e-12 if prec == "fp64" else 1e-5) * np.max(np.abs(jv))
