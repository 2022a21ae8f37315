"""Refined meshes with hanging nodes (one level of quadtree refinement of a
Q2 mesh): mesh, hang info, numbering and the weighted CSR pattern against an
independent oracle restatement; assembly and Newton on the GPU."""
import numpy as np
import pytest

import hang_oracle as H
from pyoomph_gb300 import _native as N
from pyoomph_gb300.equations import DirichletBC, NonlinearDiffusionEquation, PoissonEquation
from pyoomph_gb300.meshes import RefinedQuadMesh
from pyoomph_gb300.problem import Problem
from pyoomph_gb300.workloads import draw_gaussians

REGIONS = {"half": lambda x, y: x < 0.5, "corner": lambda x, y: x < 0.5 and y > 0.25,
           "ring": lambda x, y: 0.1 < (x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.2}


def _problem(n, region, eq="poisson", seed=5, prec="fp64"):
    g = draw_gaussians(seed, 8, 2)
    P = Problem()
    P.jacobian_precision = prec
    P += RefinedQuadMesh(N=n, refine=REGIONS[region])
    E = PoissonEquation if eq == "poisson" else NonlinearDiffusionEquation
    P += (E(source=g) + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    HP = H.HangProblem(n, REGIONS[region], g, eq=H.O.EQ_POISSON if eq == "poisson" else H.O.EQ_NONLINEAR_DIFFUSION)
    return P, HP


@pytest.mark.parametrize("region", list(REGIONS))
def test_refined_mesh_numbering_and_pattern_match_the_oracle(region):
    P, HP = _problem(6, region)
    P.lower()
    assert np.array_equal(P.mesh.x, HP.x) and np.array_equal(P.mesh.conn, HP.conn)
    assert P.mesh.hang == HP.hang and len(HP.hang) > 0
    assert np.array_equal(P.eqn[:, 0], HP.eqn)
    rp, ci = P.host_pattern()
    _, orp, oci, _ = HP.assemble()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


def test_bad_hang_info_is_rejected():
    P, _ = _problem(4, "half")
    P.lower()
    h0 = int(P.hang_slots[0])
    # a master that hangs itself
    P.hang_master = P.hang_master.copy()
    P.hang_master[0] = int(P.hang_slots[1])
    with pytest.raises(N.FeError, match="hangs itself"):
        P.host_pattern()
    # a hanging value that still has an equation
    P2, _ = _problem(4, "half")
    P2.lower()
    P2.eqn = P2.eqn.copy()
    P2.eqn.reshape(-1)[int(P2.hang_slots[0])] = 0
    with pytest.raises(N.FeError, match="has an equation"):
        P2.host_pattern()
    assert h0 >= 0


@pytest.mark.gpu
@pytest.mark.parametrize("eq,prec", [("poisson", "fp64"), ("nldiff", "fp64"), ("nldiff", "fp32")])
def test_gpu_assembly_with_hanging_nodes_matches_the_oracle(eq, prec):
    P, HP = _problem(6, "ring", eq=eq, prec=prec)
    P.initialise()
    rng = np.random.default_rng(2)
    d = rng.normal(0.0, 0.3, P.n_dof)
    P.set_dofs(d)
    R, J = P.get_jacobian()
    HP.set_dofs(d)
    Ro, orp, oci, ov = HP.assemble()
    rp, ci = P.pattern()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.max(np.abs(R - Ro)) <= 1e-12 * np.max(np.abs(Ro))
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert np.max(np.abs(J.data - ov)) <= tol * np.max(np.abs(ov))


@pytest.mark.gpu
def test_gpu_newton_on_a_refined_mesh_matches_the_oracle():
    P, HP = _problem(6, "corner", eq="nldiff")
    P.newton_solver_tolerance = 1e-11
    P.solve()
    x = HP.newton(tol=1e-11)
    assert np.max(np.abs(P.get_dofs() - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))
    # hanging values follow their masters
    v = P.get_values()[:, 0]
    for h, ms in P.mesh.hang.items():
        assert abs(v[h] - sum(w * v[m] for m, w in ms)) < 1e-14


@pytest.mark.gpu
def test_refinement_improves_a_manufactured_solution():
    """-lap u = 2 pi^2 sin(pi x) sin(pi y), u = 0 on the boundary: refining
    half of the mesh (with hanging nodes on the interface) lowers the
    integrated squared error, in total and in the refined half.  (Nodal
    errors are no measure here: uniform Q2 meshes superconverge at the
    nodes, a refined mesh does not.)"""
    import sympy as sp
    from pyoomph_gb300 import expressions as E
    from pyoomph_gb300.meshes import RectangularQuadMesh
    f = 2 * sp.pi ** 2 * sp.sin(sp.pi * E.X[0]) * sp.sin(sp.pi * E.X[1])
    errs = {}
    for name, mesh in (("coarse", RectangularQuadMesh(N=6)), ("refined", RefinedQuadMesh(N=6))):
        P = Problem()
        P += mesh
        P += (PoissonEquation(source=f) + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
        P.newton_solver_tolerance = 1e-12
        P.solve()
        et = P.mesh.etype
        t = et.tables()
        X = P.mesh.x[P.mesh.conn]
        v = P.get_values()[:, 0][P.mesh.conn]
        tot = left = 0.0
        for q in range(et.nq):
            xq = np.einsum("eli,l->ei", X, t["PSI2"][q])
            tq = np.einsum("eli,la->eai", X, t["DPS2"][q])
            det = np.abs(tq[:, 0, 0] * tq[:, 1, 1] - tq[:, 0, 1] * tq[:, 1, 0])
            e2 = t["W"][q] * det * (v @ t["PSI2"][q] - np.sin(np.pi * xq[:, 0]) * np.sin(np.pi * xq[:, 1])) ** 2
            tot += e2.sum()
            left += e2[xq[:, 0] < 0.5].sum()
        errs[name] = (tot, left)
    assert errs["refined"][0] < errs["coarse"][0]
    assert errs["refined"][1] < 0.25 * errs["coarse"][1]
