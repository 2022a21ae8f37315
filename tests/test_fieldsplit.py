"""The device saddle-point solver (fieldsplit.py): GMRES with the block
upper-triangular preconditioner (smoothed-aggregation V-cycle on the
velocity block, pressure mass over the viscosity for the Schur complement)
on the resident Taylor-Hood Jacobian -- the systems the reference hands to
SuperLU on the host (pyoomph/solvers/scipy.py, src/pybind/solver.cpp:105).

Contract: the linear solve agrees with SuperLU on the same Jacobian; Newton
with it converges to max |R| < 1e-10 with FP64 and FP32 Jacobians, to the
oracle's solution within 1e-10; iteration counts stay flat as the mesh is
refined."""
import numpy as np
import pytest

import oracle as O


def test_pressure_lumped_mass_and_aggregates():
    """Host parts: the pressure space's lumped mass sums to the domain's
    area (P1 partition of unity; the pinned pressure dof has none); the
    aggregates cover every unknown, never mix components, and are
    reproducible."""
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300 import fieldsplit as F
    import scipy.sparse as sps
    P = W.navier_stokes_problem(N=6)
    P.lower()
    m = F.lumped_field_mass(P, "pressure")
    eqn = np.asarray(P.eqn).reshape(P.mesh.n_nodes, 3)
    pdofs = eqn[:, 2][eqn[:, 2] >= 0]
    assert np.all(m[pdofs] > 0)
    # the pinned pressure node's share is missing from the unit area
    assert 0.97 < m[pdofs].sum() < 1.0
    rng = np.random.default_rng(0)
    n = 400
    A = sps.random(n, n, density=0.02, random_state=1, format="csr") + sps.eye(n) * 4.0
    A = (A + A.T).tocsr()
    comp = rng.integers(0, 2, n).astype(np.int32)
    agg, na = F.aggregate(A, comp, 0.05)
    agg2, na2 = F.aggregate(A, comp, 0.05)
    assert na == na2 and np.array_equal(agg, agg2)
    assert agg.min() == 0 and agg.max() == na - 1 and na < n
    for a in range(na):
        assert np.unique(comp[agg == a]).size == 1


def test_native_block_split_and_multigrid_level_match_scipy():
    """Host parts of the set-up: fe_csr_block cuts the same blocks as scipy
    slicing, its slot map points at the right entries; fe_sa_level_build's
    prolongator and Galerkin operator equal the scipy products with the
    same spectral radius estimate (to rounding); a second build gives the
    same bits."""
    import scipy.sparse as sps
    from pyoomph_gb300 import fieldsplit as F
    rng = np.random.default_rng(3)
    n = 3000
    A = sps.random(n, n, density=0.004, random_state=2, format="csr")
    A = (A + A.T + sps.eye(n) * 6.0).tocsr()
    A.data += rng.normal(0.0, 1e-3, A.data.size)
    label = (rng.random(n) < 0.25).astype(np.int8)
    for rl in (0, 1):
        for cl in (0, 1):
            blk = F.csr_block(A.indptr, A.indices, label, rl, cl)
            rows, cols = np.flatnonzero(label == rl), np.flatnonzero(label == cl)
            ref = A[rows][:, cols].tocsr()
            ref.sort_indices()
            got = sps.csr_matrix((A.data[blk.slots], blk.indices, blk.indptr), shape=blk.shape)
            assert got.shape == ref.shape
            assert np.array_equal(got.indptr, ref.indptr) and np.array_equal(got.indices, ref.indices)
            assert np.array_equal(got.data, ref.data)
    comp = np.zeros(n, np.int32)
    agg, na = F.aggregate(A, comp, 0.05)
    Pn, Acn, lam = F.sa_level(A, agg, na)
    D = A.diagonal()
    ev = abs(sps.linalg.eigs(sps.diags(1.0 / D) @ A, k=1, which="LM", return_eigenvectors=False)[0])
    assert 1.0 * ev <= lam <= 1.15 * ev
    P0 = sps.csr_matrix((np.ones(n), (np.arange(n), agg)), shape=(n, na))
    Pr = (P0 - (4.0 / 3.0 / lam) * (sps.diags(1.0 / D) @ A @ P0)).tocsr()
    Acr = (Pr.T @ A @ Pr).tocsr()
    for got, ref in ((Pn, Pr), (Acn, Acr)):
        d = (got - ref).tocsr()
        assert abs(d).max() <= 1e-13 * abs(ref).max()
    P2, Ac2, lam2 = F.sa_level(A, agg, na)
    assert lam2 == lam and np.array_equal(P2.data, Pn.data) and np.array_equal(Ac2.data, Acn.data)


@pytest.mark.gpu
def test_linear_solve_matches_superlu():
    import scipy.sparse.linalg as spla
    import torch
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=20)
    P.initialise()
    W.perturb_dofs(P, seed=4, sigma=0.01)
    R, J = P.get_jacobian()
    S = P._fieldsplit_solver()
    x, its = S.solve(P.R_dev[:P.n_dof], tol=1e-11)
    ref = spla.splu(J.tocsc()).solve(R)
    err = np.max(np.abs(x.cpu().numpy() - ref)) / np.max(np.abs(ref))
    assert err <= 1e-8, (err, its)
    assert its < 200


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_newton_on_the_device_matches_the_oracle_solution(prec):
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=[24, 20], jacobian_precision=prec)
    P.linear_solver = "fieldsplit"
    P.newton_solver_tolerance = 1e-10
    P.max_newton_iterations = 20
    hist = P.solve()
    assert hist[-1] < 1e-10
    OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, 24, 20), rho=1.0, mu=0.01)
    O.newton(OP, tol=1e-10)
    x, x0 = P.get_dofs(), OP.dofs()
    assert np.max(np.abs(x - x0)) / np.max(np.abs(x0)) <= 1e-10


@pytest.mark.gpu
def test_iterations_do_not_grow_with_the_mesh():
    from pyoomph_gb300 import workloads as W
    counts = []
    for n in (16, 32, 64):
        P = W.navier_stokes_problem(N=n)
        P.initialise()
        W.perturb_dofs(P, seed=0, sigma=1e-3)
        P.assemble_device(with_jacobian=True)
        x, its = P._fieldsplit_solver().solve(P.R_dev[:P.n_dof], tol=1e-10)
        counts.append(its)
    assert max(counts) < 1.5 * min(counts) + 10, counts


@pytest.mark.gpu
def test_problems_without_a_constrained_field_are_refused():
    from pyoomph_gb300 import workloads as W
    P = W.poisson_problem(N=4)
    P.linear_solver = "fieldsplit"
    with pytest.raises(RuntimeError):
        P.solve()


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(1000, 0), (5000, 7), (300001, 40)])
def test_native_gram_schmidt_step_matches_torch_and_repeats(n, k):
    """fe_gmres_cgs2 against classical Gram-Schmidt twice written in torch
    (to rounding), and bit-identical when repeated."""
    import ctypes
    import torch
    from pyoomph_gb300 import _native as N
    L = N.load()
    g = torch.Generator(device="cuda").manual_seed(k + 1)
    m = 60
    V = torch.zeros((m + 1, n), dtype=torch.float64, device="cuda")
    Q, _ = torch.linalg.qr(torch.randn((n, k + 1), dtype=torch.float64, device="cuda", generator=g))
    V[:k + 1] = Q.T
    a = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    h = V[:k + 1] @ a
    w = a - V[:k + 1].T @ h
    h2 = V[:k + 1] @ w
    w -= V[:k + 1].T @ h2
    nw = torch.linalg.vector_norm(w)
    ref_h, ref_v = torch.cat([h + h2, nw.view(1)]), w / nw
    work = torch.empty(int(L.fe_gmres_cgs2_scratch(n, m)), dtype=torch.float64, device="cuda")
    outs = []
    for _ in range(2):
        Vc, wc = V.clone(), a.clone()
        hc = torch.zeros(m + 1, dtype=torch.float64, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        N.check(L.fe_gmres_cgs2(ctypes.c_void_p(Vc.data_ptr()), n, n, k, ctypes.c_void_p(wc.data_ptr()),
                                ctypes.c_void_p(hc.data_ptr()), ctypes.c_void_p(work.data_ptr()), ctypes.c_void_p(st)))
        torch.cuda.synchronize()
        outs.append((hc[:k + 2].clone(), Vc[k + 1].clone()))
    assert torch.max(torch.abs(outs[0][0] - ref_h)) <= 1e-12 * torch.max(torch.abs(ref_h))
    assert torch.max(torch.abs(outs[0][1] - ref_v)) <= 1e-12
    assert torch.equal(outs[0][0].view(torch.int64), outs[1][0].view(torch.int64))
    assert torch.equal(outs[0][1].view(torch.int64), outs[1][1].view(torch.int64))
