"""Device Newton linear solve: CSR SpMV kernel and BiCGStab on the resident
Jacobian, against scipy / SuperLU and the oracle's Newton solution."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_spmv_and_diagonal_match_scipy(prec):
    import torch
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.linsolve import DeviceCSR
    P = W.navier_stokes_problem(N=10, jacobian_precision=prec)
    P.initialise()
    W.perturb_dofs(P, seed=1, sigma=1e-2)
    R, J = P.get_jacobian()
    A = DeviceCSR.of_problem(P)
    x = torch.as_tensor(np.random.default_rng(0).normal(size=P.n_dof), device="cuda")
    y = torch.empty_like(x)
    st = torch.cuda.current_stream().cuda_stream
    A.matvec(x, y, st)
    d = torch.empty_like(x)
    A.diagonal(d, st)
    ref = J @ x.cpu().numpy()
    assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-12 * np.max(np.abs(ref))
    assert np.array_equal(d.cpu().numpy(), J.diagonal())


def test_bicgstab_solves_a_poisson_jacobian():
    import scipy.sparse.linalg as spla
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.linsolve import DeviceCSR, bicgstab
    P = W.poisson_problem(N=24, seed=3)
    P.initialise()
    R, J = P.get_jacobian()
    x, its = bicgstab(DeviceCSR.of_problem(P), P.R_dev[:P.n_dof], tol=1e-13)
    ref = spla.splu(J.tocsc()).solve(R)
    assert np.max(np.abs(x.cpu().numpy() - ref)) <= 1e-10 * np.max(np.abs(ref))
    assert its > 0


def test_saddle_point_systems_are_refused():
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.linsolve import DeviceCSR, LinearSolverError, bicgstab
    P = W.navier_stokes_problem(N=6)
    P.initialise()
    P.get_jacobian()
    with pytest.raises(LinearSolverError, match="zero diagonal"):
        bicgstab(DeviceCSR.of_problem(P), P.R_dev[:P.n_dof])


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_device_newton_matches_the_oracle_solution(prec):
    from pyoomph_gb300 import workloads as W
    P = W.nonlinear_diffusion_problem(N=6, seed=2, jacobian_precision=prec)
    P.linear_solver = "bicgstab"
    P.newton_solver_tolerance = 1e-11
    P.max_newton_iterations = 20
    P.solve()
    OP = O.poisson_problem(O.mesh(O.Q2_HEX, 6, 6, 6), W.draw_gaussians(2, 16, 3), eq=O.EQ_NONLINEAR_DIFFUSION)
    O.newton(OP, tol=1e-11)
    x = OP.dofs()
    assert np.max(np.abs(P.get_dofs() - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))
    assert P.timings["krylov_iterations"] > 0
