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


def _replicated_poisson(side, reps, prec="fp64"):
    from pyoomph_gb300 import workloads as W
    P = W.poisson_problem(N=side, seed=0, jacobian_precision=prec)
    P.replicas = reps
    P.initialise()
    names = P.param_names
    for s in range(reps):
        g = W.draw_gaussians(11 + s, 8, 2)
        d = {}
        for k in range(g.shape[0]):
            d[f"g{k}_c0"], d[f"g{k}_c1"], d[f"g{k}_w"], d[f"g{k}_A"] = g[k]
        P.set_parameter_vector(np.array([d[nm] for nm in names]), replica=s)
    return P


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batched_blocks_are_independent_and_match_splu(prec):
    """Three replicas solved as one batch: each block matches SuperLU on its
    own block; a block's solution is bit-identical alone or with others, and
    with or without the CUDA graph."""
    import scipy.sparse.linalg as spla
    from pyoomph_gb300.linsolve import BatchedBiCGStab, DeviceCSR
    P = _replicated_poisson(12, 3, prec)
    R, J = P.get_jacobian()
    n = P.n_dof // 3
    A = DeviceCSR.of_problem(P)
    mix = BatchedBiCGStab(A, blocks=3)
    x, its = mix.solve(P.R_dev[:P.n_dof], active=[True, False, True], tol=1e-13)
    x = x.cpu().numpy().copy()
    assert mix.graph_replays > 0 and its[0] > 0 and its[1] == 0
    assert not x[1].any()
    for s in (0, 2):
        blk = slice(s * n, (s + 1) * n)
        ref = spla.splu(J[blk, blk].astype(np.float64).tocsc()).solve(R[blk])
        assert np.max(np.abs(x[s] - ref)) <= 1e-10 * np.max(np.abs(ref))
    alone, _ = BatchedBiCGStab(A, blocks=3).solve(P.R_dev[:P.n_dof], active=[True, False, False], tol=1e-13)
    assert np.array_equal(alone.cpu().numpy()[0], x[0])
    eager, _ = BatchedBiCGStab(A, blocks=3, graph=False).solve(P.R_dev[:P.n_dof], active=[True, False, True],
                                                               tol=1e-13)
    assert np.array_equal(eager.cpu().numpy(), x)
    # the Poisson Jacobian blocks are equal (the source only enters R): block
    # 0's right-hand side in slot 2 gives block 0's solution, bit for bit
    b2 = P.R_dev[:P.n_dof].clone().view(3, n)
    b2[2] = b2[0]
    moved, _ = BatchedBiCGStab(A, blocks=3).solve(b2, active=[False, True, True], tol=1e-13)
    assert np.array_equal(moved.cpu().numpy()[2], x[0])


def test_iteration_limit_is_an_error():
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.linsolve import BatchedBiCGStab, DeviceCSR, LinearSolverError
    P = W.poisson_problem(N=24, seed=3)
    P.initialise()
    P.get_jacobian()
    with pytest.raises(LinearSolverError, match="did not reach"):
        BatchedBiCGStab(DeviceCSR.of_problem(P)).solve(P.R_dev[:P.n_dof], tol=1e-13, maxiter=8)


def test_batched_solver_reused_across_newton_steps():
    """Problem.solve keeps one batched solver (one block per replica) across
    Newton steps; every replica converges to its own oracle solution."""
    from pyoomph_gb300 import workloads as W
    P = _replicated_poisson(10, 2)
    P.linear_solver = "bicgstab"
    P.newton_solver_tolerance = 1e-11
    P.solve()
    n = P.n_dof // 2
    x = P.get_dofs()
    for s in range(2):
        OP = O.poisson_problem(O.mesh(O.Q2_QUAD, 10, 10), W.draw_gaussians(11 + s, 8, 2))
        O.newton(OP, tol=1e-11)
        ref = OP.dofs()
        assert np.max(np.abs(x[s * n:(s + 1) * n] - ref)) <= 1e-10 * max(1.0, np.max(np.abs(ref)))
    assert P._krylov is not None and P._krylov.S == 2


def test_fp32_values_widen_exactly():
    """The SpMV widens FP32 values to FP64 with integer operations: on a
    diagonal matrix with x = 1 every value comes back exactly as numpy's
    float32 -> float64 conversion (normals at both ends of the range,
    subnormals, zeros, infinities, NaN)."""
    import torch
    from pyoomph_gb300.linsolve import DeviceCSR
    f = np.finfo(np.float32)
    special = np.array([0.0, -0.0, 1.0, -1.0, f.tiny, -f.tiny, f.max, -f.max, f.smallest_subnormal,
                        -3 * f.smallest_subnormal, f.tiny / 2, np.inf, -np.inf, np.nan, 1e-30, -7.25e30],
                       dtype=np.float32)
    vals32 = np.concatenate([special, np.random.default_rng(4).standard_normal(4096).astype(np.float32) *
                             np.float32(10.0) ** np.random.default_rng(5).integers(-30, 30, 4096)])
    vals32 = vals32.astype(np.float32)
    n = vals32.size
    rp = torch.arange(n + 1, dtype=torch.int32, device="cuda")
    ci = torch.arange(n, dtype=torch.int32, device="cuda")
    A = DeviceCSR(rp.data_ptr(), ci.data_ptr(), torch.as_tensor(vals32, device="cuda"), n, n)
    x = torch.ones(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    A.matvec(x, y, torch.cuda.current_stream().cuda_stream)
    assert np.array_equal(y.cpu().numpy(), vals32.astype(np.float64), equal_nan=True)


def test_non_finite_right_hand_side_is_an_error():
    import torch
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.linsolve import BatchedBiCGStab, DeviceCSR, LinearSolverError
    P = W.poisson_problem(N=8, seed=3)
    P.initialise()
    P.get_jacobian()
    b = P.R_dev[:P.n_dof].clone()
    b[5] = float("nan")
    with pytest.raises(LinearSolverError, match="non-finite"):
        BatchedBiCGStab(DeviceCSR.of_problem(P)).solve(b, tol=1e-13)
    # the solver object stays usable after the error
    K = BatchedBiCGStab(DeviceCSR.of_problem(P))
    with pytest.raises(LinearSolverError):
        K.solve(b)
    x, its = K.solve(P.R_dev[:P.n_dof], tol=1e-13)
    assert torch.isfinite(x).all() and its[0] > 0


def test_absolute_tolerance_is_per_block():
    """atol is an absolute floor per block: a block whose right-hand side is
    already below it returns x = 0 and takes no iteration; the others stop
    at max(tol |b_s|, atol), each independently of the others."""
    import torch
    from pyoomph_gb300.linsolve import BatchedBiCGStab, DeviceCSR
    P = _replicated_poisson(10, 2)
    P.get_jacobian()
    n = P.n_dof // 2
    b = P.R_dev[:P.n_dof].clone().view(2, n)
    b[1] *= 1e-14                       # block 1: |b| far below atol
    K = BatchedBiCGStab(DeviceCSR.of_problem(P), blocks=2)
    atol = 1e-9 * float(b[0].abs().max())
    x, its = K.solve(b, tol=1e-13, atol=atol)
    assert its[1] == 0 and not x[1].any()
    assert its[0] > 0
    # the true residual of block 0 meets the absolute floor (10x, the confirmation margin)
    y = torch.empty(P.n_dof, dtype=torch.float64, device="cuda")
    DeviceCSR.of_problem(P).matvec(x.reshape(-1), y, torch.cuda.current_stream().cuda_stream)
    r0 = (b[0] - y.view(2, n)[0]).abs().max()
    assert float(r0) <= 10 * atol
