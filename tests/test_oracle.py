"""The CPU oracle against the reference's own oomph-lib output (golden
fixtures made by tests/golden/make_golden.py from oracle/_ref), and the
oracle's own invariants: FD-certified element Jacobians (the method of
BulkElementBase::debug_analytical_jacobian, elements.cpp:5880-5920) and
mesh/numbering counts."""
import glob
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(glob.glob(os.path.join(GOLD, "*_*.npz")))
CASES = [c for c in CASES if not c.endswith("oomph_tables.npz")]


def _problem(g):
    m = O.Mesh(int(g["etype"]), g["x"].shape[1], g["x"], g["conn"], g["bmask"], g["is_vertex"])
    return O.Problem(mesh=m, eq=int(g["eq"]), nval=g["values"].shape[1], nvalue=g["nvalue"],
                     pinned=g["pinned"], values=g["values"].copy(), params=g["params"])


def test_tables_match_oomph():
    T = np.load(os.path.join(GOLD, "oomph_tables.npz"))
    for et in (O.Q2_QUAD, O.P2_TRI, O.Q2_HEX):
        mine = O.oracle_tables(et)
        for k in ("s", "w", "psi", "dpsi"):
            assert np.array_equal(mine[k], T[f"{et}_{k}"]), (et, k)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_mesh_and_numbering_match_reference(path):
    g = np.load(path)
    m = O.mesh(int(g["etype"]), int(g["nx"]), int(g["ny"]), int(g["nz"]), split=int(g["split"]))
    assert np.array_equal(m.conn, g["conn"])
    assert np.array_equal(m.x, g["x"])
    assert np.array_equal(m.bmask, g["bmask"])
    P = _problem(g)
    assert np.array_equal(P.eqn, g["eqn"])


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_structural_csr_bit_exact_and_values(path):
    g = np.load(path)
    P = _problem(g)
    R, rp, ci, v = O.assemble(P, True, -1.0)
    assert np.array_equal(rp, g["rowptr_st"])
    assert np.array_equal(ci, g["colidx_st"])
    scale = np.max(np.abs(g["vals_st"]))
    assert np.max(np.abs(v - g["vals_st"])) <= 1e-12 * scale
    assert np.max(np.abs(R - g["R"])) <= 1e-12 * np.max(np.abs(g["R"]))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_zero_filter_pattern(path):
    """With the default filter (|J_e(i,j)| > 0.0) the pattern depends on which
    analytically-zero entries round to exactly 0.0.  Where the element forms
    have no such entries (Poisson, nonlinear diffusion) it is bit-exact;
    for Taylor-Hood only the entries that survive in both can be compared."""
    g = np.load(path)
    P = _problem(g)
    R, rp, ci, v = O.assemble(P, True, 0.0)
    if int(g["eq"]) != O.EQ_NAVIER_STOKES_TH:
        assert np.array_equal(rp, g["rowptr_zf"])
        assert np.array_equal(ci, g["colidx_zf"])
    else:
        # the same set of large entries, to rounding
        import scipy.sparse as sp
        n = P.n_dof
        A = sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()
        B = sp.csr_matrix((g["vals_zf"], g["colidx_zf"], g["rowptr_zf"]), shape=(n, n)).toarray()
        assert np.max(np.abs(A - B)) <= 1e-12 * np.max(np.abs(B))


@pytest.mark.parametrize("etype,eq", [(O.Q2_QUAD, O.EQ_NONLINEAR_DIFFUSION), (O.P2_TRI, O.EQ_NAVIER_STOKES_TH),
                                      (O.Q2_HEX, O.EQ_NONLINEAR_DIFFUSION)])
def test_element_jacobian_by_finite_differences(etype, eq):
    rng = np.random.default_rng(7)
    m = O.mesh(etype, 2, 2, 2)
    if eq == O.EQ_NAVIER_STOKES_TH:
        P = O.navier_stokes_problem(m)
        P.set_dofs(P.dofs() + rng.normal(0, 0.3, P.n_dof))
    else:
        g = np.hstack([rng.uniform(0, 1, (4, m.dim)), rng.uniform(0.05, 0.2, (4, 1)), rng.normal(0, 1, (4, 1))])
        P = O.poisson_problem(m, g, eq=eq)
        P.set_dofs(rng.normal(0, 0.5, P.n_dof))
    R, rp, ci, v = O.assemble(P, True, -1.0)
    import scipy.sparse as sp
    J = sp.csr_matrix((v, ci, rp), shape=(P.n_dof, P.n_dof)).toarray()
    x0 = P.dofs()
    eps = 1e-7
    Jfd = np.zeros_like(J)
    for j in range(P.n_dof):
        xp = x0.copy(); xp[j] += eps
        P.set_dofs(xp)
        Rp = O.assemble(P, False)
        xm = x0.copy(); xm[j] -= eps
        P.set_dofs(xm)
        Rm = O.assemble(P, False)
        Jfd[:, j] = (Rp - Rm) / (2 * eps)
    P.set_dofs(x0)
    assert np.max(np.abs(J - Jfd)) <= 1e-6 * np.max(np.abs(J))


def test_mesh_sizes_of_the_workloads():
    """Node/dof counts quoted for the workloads: 64x64 Q2 = 16,641 nodes /
    16,129 free; 48^3 Q2 hex = 912,673 nodes."""
    m = O.mesh(O.Q2_QUAD, 64, 64)
    assert m.x.shape[0] == 16641
    P = O.poisson_problem(m, np.array([[0.5, 0.5, 0.1, 1.0]]))
    assert P.n_dof == 16129
    n, e, k = [O.ctypes.c_int64(), O.ctypes.c_int64(), O.ctypes.c_int()]
    O.lib().ofe_mesh_sizes(O.Q2_HEX, 48, 48, 48, O.ctypes.byref(n), O.ctypes.byref(e), O.ctypes.byref(k))
    assert n.value == 912673 and e.value == 110592


@pytest.mark.parametrize("kind", ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex"])
@pytest.mark.parametrize("threshold", [0.0, -1.0, 0.05])
def test_vectors_of_pairs_restatement_matches_the_c_assembler(kind, threshold):
    """oracle.vectors_of_pairs (the insertion loop over given element
    matrices) gives the C oracle's CSR bit for bit, with and without the
    zero filter: it can check the device's filtered compaction on the
    product's own element matrices."""
    import element_cases as C
    from pyoomph_gb300 import workloads as W
    P, ks, values, Rr, Jr = C.build(kind, "affine", "fp64")
    m = P.mesh
    if kind == "ns_th":
        OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, 4, 3), rho=1.0, mu=0.01)
    else:
        et, nx, dim = {"poisson_q2": (O.Q2_QUAD, (4, 3, 0), 2), "poisson_p2": (O.P2_TRI, (3, 4, 0), 2),
                       "nldiff_hex": (O.Q2_HEX, (2, 2, 3), 3)}[kind]
        eq = O.EQ_POISSON if kind.startswith("poisson") else O.EQ_NONLINEAR_DIFFUSION
        OP = O.poisson_problem(O.mesh(et, *nx), W.draw_gaussians(3, 8, dim), eq=eq)
    assert np.array_equal(OP.eqn, np.asarray(P.eqn).reshape(OP.eqn.shape))
    OP.values[:] = values
    R0, rp0, ci0, v0 = O.assemble(OP, True, threshold)
    lay = ks.layout
    eqns = OP.eqn[m.conn[:, lay.node], lay.val]
    rp, ci, v = O.vectors_of_pairs(eqns, Jr, OP.n_dof, threshold)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0) and np.array_equal(v, v0)
