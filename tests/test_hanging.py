"""Refined meshes with hanging nodes (one level of quadtree refinement of a
Q2 mesh): mesh, hang info, numbering and the weighted CSR pattern against an
independent oracle restatement; assembly and Newton on the GPU."""
import numpy as np
import pytest

import hang_oracle as H
from pyoomph_gb300 import _native as N
from pyoomph_gb300.equations import DirichletBC, NonlinearDiffusionEquation, PoissonEquation
from pyoomph_gb300.meshes import AdaptiveQuadMesh, RefinedQuadMesh
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


def _around(px, py, n):
    """Refine the cells that contain (px, py), at every level."""
    return lambda x, y, level: abs(x - px) < 0.5 / n / 2 ** level and abs(y - py) < 0.5 / n / 2 ** level


# multi-level refinements without 2:1 balance: "point" refines towards a
# point just inside a base-cell corner, so that three levels meet and some
# masters hang themselves (completed recursively)
LEVELS = {"point": (4, lambda n: _around(0.26, 0.26, n), 4),
          "ring": (4, lambda n: (lambda x, y, l: abs(np.hypot(x - 0.5, y - 0.5) - 0.3) < 0.2 / 2 ** l), 3),
          "two_points": (6, lambda n: (lambda x, y, l: _around(0.2, 0.7, n)(x, y, l) or _around(0.55, 0.3, n)(x, y, l)), 3)}


def _problem_levels(case, eq="poisson", seed=5, prec="fp64"):
    n, mk, L = LEVELS[case]
    g = draw_gaussians(seed, 8, 2)
    P = Problem()
    P.jacobian_precision = prec
    P += AdaptiveQuadMesh(N=n, refine=mk(n), max_level=L)
    E = PoissonEquation if eq == "poisson" else NonlinearDiffusionEquation
    P += (E(source=g) + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    HP = H.HangProblem(n, mk(n), g, eq=H.O.EQ_POISSON if eq == "poisson" else H.O.EQ_NONLINEAR_DIFFUSION,
                       max_level=L)
    return P, HP


@pytest.mark.parametrize("case", list(LEVELS))
def test_multilevel_mesh_numbering_and_pattern_match_the_oracle(case):
    """Several refinement levels: leaves in tree order, first-encounter
    node numbering (oomph's reorder_nodes), hang infos completed through
    hanging masters (oomph's complete_hanging_nodes), equation numbers and
    the weighted CSR pattern, all against the oracle's geometric
    restatement."""
    P, HP = _problem_levels(case)
    P.lower()
    assert np.array_equal(P.mesh.conn, HP.conn)
    assert np.max(np.abs(P.mesh.x - HP.x)) <= 1e-15
    assert P.mesh.hang == HP.hang and len(HP.hang) > 0
    assert np.array_equal(P.eqn[:, 0], HP.eqn)
    rp, ci = P.host_pattern()
    _, orp, oci, _ = HP.assemble()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    if case == "point":
        assert max(len(v) for v in HP.hang.values()) == 5       # masters of masters
    for h, ms in P.mesh.hang.items():                               # linear fields are reproduced
        assert abs(sum(w for _, w in ms) - 1.0) < 1e-14
        assert np.allclose(sum(w * P.mesh.x[m] for m, w in ms), P.mesh.x[h], atol=1e-14, rtol=0)


HANG_FIXTURES = ["hang_point_4_L4", "hang_ring_4_L3", "hang_two_points_6_L3"]


def _plan_predicate(plan):
    keys = {(int(l), round(float(cx), 12), round(float(cy), 12)) for l, cx, cy in plan}
    return lambda x, y, level: (level, round(float(x), 12), round(float(y), 12)) in keys


@pytest.mark.parametrize("name", HANG_FIXTURES)
def test_multilevel_refinement_matches_oomph(name):
    """Against oomph-lib's own quadtree refinement, hanging nodes and
    assembly (fixtures from oracle/_ref/oomph_hang_driver, compiled from the
    reference tree: tests/golden/make_golden.py): node positions, elements
    (tree order), first-encounter numbering, equation numbers and the
    structural CSR pattern bit-exact; the completed hang infos equal as
    sets of (master, weight), and in oomph's order wherever oomph's node
    addresses follow the order of creation (the "point" case throughout);
    the oracle's residual and Jacobian values within 1e-13 of oomph's."""
    import os
    G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hang", name + ".npz"))
    N_, L = int(G["N"]), int(G["L"])
    chosen = _plan_predicate(G["plan"])
    g = G["gaussians"]
    P = Problem()
    P += AdaptiveQuadMesh(N=N_, refine=chosen, max_level=L)
    P += (PoissonEquation(source=g) + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    P.lower()
    assert np.array_equal(P.mesh.conn, G["conn"])
    assert np.max(np.abs(P.mesh.x - G["x"])) <= 1e-15
    assert np.array_equal(P.eqn[:, 0] >= 0, G["eqn"] >= 0)
    assert np.array_equal(P.eqn[:, 0][G["eqn"] >= 0], G["eqn"][G["eqn"] >= 0])
    ref = {int(h): [(int(m), float(w)) for m, w in zip(G["hang_master"][a:b], G["hang_weight"][a:b])]
           for h, a, b in zip(G["hang_node"], G["hang_ptr"][:-1], G["hang_ptr"][1:])}
    assert sorted(ref) == sorted(P.mesh.hang)
    assert all(sorted(ref[h]) == sorted(P.mesh.hang[h]) for h in ref)
    out_of_order = sum(ref[h] != P.mesh.hang[h] for h in ref)
    if name.startswith("hang_point"):
        assert out_of_order == 0
    # oomph's heap reuse puts a few masters out of creation order: 8 of 256
    # hang infos in the ring case, 4 of 48 in the two-point case
    assert out_of_order <= 0.1 * len(ref)
    rp, ci = P.host_pattern()
    assert np.array_equal(rp, G["rowptr"]) and np.array_equal(ci, G["colidx"])
    HP = H.HangProblem(N_, chosen, g, max_level=L)
    HP.set_dofs(G["dofs"])
    Ro, orp, oci, ov = HP.assemble()
    assert np.array_equal(orp, G["rowptr"]) and np.array_equal(oci, G["colidx"])
    assert np.max(np.abs(Ro - G["R"])) <= 1e-13 * np.max(np.abs(G["R"]))
    assert np.max(np.abs(ov - G["vals"])) <= 1e-13 * np.max(np.abs(G["vals"]))


def test_completion_restates_oomph():
    """complete_hanging against the oracle's literal restatement on a
    hand-made chain: c hangs on (a, b), b hangs on (a, d); weights multiply,
    repeats add, zero weights drop."""
    from pyoomph_gb300.meshes import complete_hanging
    hang = {2: [(0, 0.25), (1, 0.75)], 1: [(0, 0.5), (3, 0.5)], 5: [(4, 1.0), (2, 0.0)]}
    got = complete_hanging(hang)
    assert got == H._complete(hang)
    assert got[2] == [(0, 0.625), (3, 0.375)] and got[1] == [(0, 0.5), (3, 0.5)] and got[5] == [(4, 1.0)]


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


@pytest.mark.gpu
@pytest.mark.parametrize("case,eq,prec", [("point", "poisson", "fp64"), ("two_points", "nldiff", "fp64"),
                                          ("ring", "nldiff", "fp32")])
def test_gpu_multilevel_assembly_matches_the_oracle(case, eq, prec):
    """Several levels, masters completed through hanging masters: R, the
    CSR pattern and J from the device against the oracle's hanging-node
    assembly."""
    P, HP = _problem_levels(case, eq=eq, prec=prec)
    P.initialise()
    d = np.random.default_rng(4).normal(0.0, 0.3, P.n_dof)
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
def test_gpu_newton_on_a_multilevel_mesh_matches_the_oracle():
    P, HP = _problem_levels("two_points", eq="nldiff")
    P.newton_solver_tolerance = 1e-11
    P.solve()
    x = HP.newton(tol=1e-11)
    assert np.max(np.abs(P.get_dofs() - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))
    v = P.get_values()[:, 0]
    for h, ms in P.mesh.hang.items():
        assert abs(v[h] - sum(w * v[m] for m, w in ms)) < 1e-14


# Taylor-Hood (Q2 velocity, Q1 pressure) on refined meshes: the pressure of
# a vertex strictly inside a coarser leaf's edge -- the edge's middle node
# too -- hangs linearly on the edge's two end vertices
NS_LEVELS = {"half_L1": (4, lambda x, y, l: x < 0.5, 1), "point_L3": (4, lambda x, y, l: _around(0.26, 0.26, 4)(x, y, l), 3)}


def _ns_problem_levels(case, prec="fp64"):
    from pyoomph_gb300.equations import NavierStokesEquations, PressureFixation
    from pyoomph_gb300.workloads import lid_velocity
    n, refine, L = NS_LEVELS[case]
    P = Problem()
    P.jacobian_precision = prec
    P += AdaptiveQuadMesh(N=n, refine=refine, max_level=L)
    eqs = NavierStokesEquations(mass_density=1.0, dynamic_viscosity=0.01)
    eqs += DirichletBC(velocity_x=lid_velocity, velocity_y=0.0) @ "top"
    eqs += DirichletBC(velocity_x=0.0, velocity_y=0.0) @ ["left", "right", "bottom"]
    eqs += PressureFixation("pressure", 0.0)
    P += eqs @ "domain"
    return P, H.HangNSProblem(n, refine, L, rho=1.0, mu=0.01)


@pytest.mark.parametrize("case", list(NS_LEVELS))
def test_taylor_hood_hanging_pressure_numbering_and_pattern_match_the_oracle(case):
    P, HP = _ns_problem_levels(case)
    P.lower()
    assert np.array_equal(P.mesh.conn, HP.conn)
    assert P.mesh.hang == HP.hang and P.mesh.hang_c1 == HP.hang_c1 and len(HP.hang_c1) > 0
    # the middle node of a coarse edge: velocity free, pressure hanging
    mids = [h for h in HP.hang_c1 if h not in HP.hang]
    assert mids
    for h, ms in P.mesh.hang_c1.items():        # linear fields are reproduced
        assert abs(sum(w for _, w in ms) - 1.0) < 1e-14
        assert np.allclose(sum(w * P.mesh.x[m] for m, w in ms), P.mesh.x[h], atol=1e-14, rtol=0)
        assert all(HP.isv[m] for m, _ in ms)
    assert np.array_equal(P.eqn, HP.eqn)
    rp, ci = P.host_pattern()
    _, orp, oci, _ = HP.assemble()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(NS_LEVELS))
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_taylor_hood_hanging_assembly_and_newton_match_the_oracle(case, prec):
    P, HP = _ns_problem_levels(case, prec)
    P.initialise()
    rng = np.random.default_rng(3)
    d = rng.normal(0.0, 0.05, P.n_dof)
    P.set_dofs(d)
    HP.set_dofs(d)
    R, J = P.get_jacobian()
    Ro, orp, oci, ov = HP.assemble()
    assert np.array_equal(J.indptr, orp) and np.array_equal(J.indices, oci)
    assert np.max(np.abs(R - Ro)) <= 1e-12 * np.max(np.abs(Ro))
    jtol = 1e-12 if prec == "fp64" else 1e-5
    assert np.max(np.abs(J.data - ov)) <= jtol * np.max(np.abs(ov))
    # Newton from rest to max |R| < 1e-10; the hanging values follow their masters
    P.set_dofs(np.zeros(P.n_dof))
    HP.set_dofs(np.zeros(HP.n_dof))
    P.newton_solver_tolerance = 1e-10
    hist = P.solve()
    assert hist[-1] < 1e-10
    x0 = HP.newton(tol=1e-10)
    assert np.max(np.abs(P.get_dofs() - x0)) <= 1e-9 * max(1.0, np.max(np.abs(x0)))
    v = P.get_values()
    for h, ms in P.mesh.hang_c1.items():
        assert abs(v[h, 2] - sum(w * v[m, 2] for m, w in ms)) <= 1e-13 * max(1.0, np.max(np.abs(v[:, 2])))
