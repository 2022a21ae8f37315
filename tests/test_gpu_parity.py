"""GPU parity: the CUDA assembly (through the C-ABI library) against the
reference's own oomph-lib output (golden fixtures) and the CPU oracle.

Contract (fp64 path): CSR rowptr/colidx bit-exact (structural pattern in
first-insertion order), residual and Jacobian entries within 1e-12 of the
max norm, converged Newton solutions within 1e-10.  FP32-Jacobian path:
residual as above; Jacobian within 1e-5 relative (max norm) of the FP64
oracle; Newton converges to the FP64 solution within 1e-10.
"""
import glob
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = [c for c in sorted(glob.glob(os.path.join(GOLD, "*_*.npz"))) if not c.endswith("oomph_tables.npz")]
RTOL = 1e-12
JTOL32 = 1e-5
STOL = 1e-10


def _product_for(g):
    from pyoomph_gb300 import workloads as W
    et, eq = int(g["etype"]), int(g["eq"])
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    if eq == O.EQ_NAVIER_STOKES_TH:
        P = W.navier_stokes_problem(N=[nx, ny], Re=1.0 / float(g["params"][1]),
                                    split="left" if int(g["split"]) == 0 else "right")
    else:
        dim = 3 if et == O.Q2_HEX else 2
        gauss = g["params"][1:].reshape(int(g["params"][0]), dim + 2)
        if eq == O.EQ_POISSON:
            P = W.poisson_problem(N=[nx, ny], gaussians=gauss, split=None if et == O.Q2_QUAD else "left")
        else:
            P = W.nonlinear_diffusion_problem(N=[nx, ny, nz] if dim == 3 else [nx, ny], gaussians=gauss, dim=dim)
    P.initialise()
    return P


def _relmax(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_golden_reference_parity(path):
    g = np.load(path)
    P = _product_for(g)
    assert np.array_equal(P.eqn, g["eqn"])
    P.set_values(g["values"])
    R, J = P.get_jacobian()
    assert np.array_equal(J.indptr, g["rowptr_st"])
    assert np.array_equal(J.indices, g["colidx_st"])
    assert _relmax(J.data, g["vals_st"]) <= RTOL
    assert _relmax(R, g["R"]) <= RTOL


@pytest.mark.parametrize("prec", ["fp64", "df64"])
@pytest.mark.parametrize("kind", ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex", "nldiff_q2"])
def test_random_state_vs_oracle(kind, prec):
    """Full CSR assembly (pattern bit-exact, values within 1e-12) for the FP64
    Jacobian and for the double-float contraction (df64)."""
    from pyoomph_gb300 import workloads as W
    rng = np.random.default_rng(11)
    if kind == "ns_th":
        P = W.navier_stokes_problem(N=[9, 7], jacobian_precision=prec)
        P.initialise()
        m = O.mesh(O.P2_TRI, 9, 7)
        OP = O.navier_stokes_problem(m, rho=1.0, mu=0.01)
        x = OP.dofs() + rng.normal(0, 0.1, OP.n_dof)
    else:
        if kind == "nldiff_hex":
            et, dim, nx = O.Q2_HEX, 3, [3, 4, 2]
        elif kind == "poisson_p2":
            et, dim, nx = O.P2_TRI, 2, [11, 6]
        else:
            et, dim, nx = O.Q2_QUAD, 2, [12, 9]
        gauss = W.draw_gaussians(3, 8, dim)
        eq = O.EQ_POISSON if kind.startswith("poisson") else O.EQ_NONLINEAR_DIFFUSION
        if eq == O.EQ_POISSON:
            P = W.poisson_problem(N=nx, gaussians=gauss, split="left" if et == O.P2_TRI else None,
                                  jacobian_precision=prec)
        else:
            P = W.nonlinear_diffusion_problem(N=nx, gaussians=gauss, dim=dim, jacobian_precision=prec)
        P.initialise()
        m = O.mesh(et, *(nx + [0] * (3 - len(nx))))
        OP = O.poisson_problem(m, gauss, eq=eq)
        x = rng.normal(0, 0.5, OP.n_dof)
    assert P.n_dof == OP.n_dof and np.array_equal(P.eqn, OP.eqn)
    OP.set_dofs(x)
    P.set_dofs(x)
    R0, rp, ci, v = O.assemble(OP, True, -1.0)
    R, J = P.get_jacobian()
    assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
    assert _relmax(J.data, v) <= RTOL
    assert _relmax(R, R0) <= RTOL
    # residual-only assembly gives the same residual
    assert np.array_equal(P.get_residuals(), R)


def test_assembly_is_deterministic():
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=[10, 10])
    P.initialise()
    W.perturb_dofs(P, seed=5, sigma=0.05)
    R1, J1 = P.get_jacobian()
    R2, J2 = P.get_jacobian()
    assert np.array_equal(R1, R2) and np.array_equal(J1.data, J2.data)


@pytest.mark.parametrize("kind", ["nldiff_hex", "ns_th"])
def test_fp32_jacobian_error_vs_fp64_oracle(kind):
    from pyoomph_gb300 import workloads as W
    rng = np.random.default_rng(5)
    if kind == "ns_th":
        P = W.navier_stokes_problem(N=[8, 8], jacobian_precision="fp32")
        P.initialise()
        OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, 8, 8), rho=1.0, mu=0.01)
        x = OP.dofs() + rng.normal(0, 0.1, OP.n_dof)
    else:
        gauss = W.draw_gaussians(4, 16, 3)
        P = W.nonlinear_diffusion_problem(N=4, gaussians=gauss, jacobian_precision="fp32")
        P.initialise()
        OP = O.poisson_problem(O.mesh(O.Q2_HEX, 4, 4, 4), gauss, eq=O.EQ_NONLINEAR_DIFFUSION)
        x = rng.normal(0, 0.5, OP.n_dof)
    OP.set_dofs(x)
    P.set_dofs(x)
    R0, rp, ci, v = O.assemble(OP, True, -1.0)
    R, J = P.get_jacobian()
    assert J.data.dtype == np.float32
    assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
    err = _relmax(J.data.astype(np.float64), v)
    assert err <= JTOL32, err
    assert _relmax(R, R0) <= RTOL


def test_newton_poisson_matches_oracle_solution():
    from pyoomph_gb300 import workloads as W
    gauss = W.draw_gaussians(0, 8, 2)
    P = W.poisson_problem(N=16, gaussians=gauss)
    P.newton_solver_tolerance = 1e-10
    hist = P.solve()
    assert hist[-1] < 1e-10
    OP = O.poisson_problem(O.mesh(O.Q2_QUAD, 16, 16), gauss)
    O.newton(OP, tol=1e-10)
    assert _relmax(P.get_dofs(), OP.dofs()) <= STOL


@pytest.mark.parametrize("prec", ["fp64", "fp32", "df64", "fp32:df64", "df64:df64"])
def test_newton_navier_stokes_matches_oracle_solution(prec):
    """Newton on NS 8x8 to max|R| < 1e-10 with every Jacobian precision and,
    after the colon, the double-float residual path: the same solution as
    the oracle's FP64 Newton."""
    from pyoomph_gb300 import workloads as W
    jp, _, rp = prec.partition(":")
    P = W.navier_stokes_problem(N=[8, 8], jacobian_precision=jp)
    P.residual_precision = rp or "fp64"
    P.newton_solver_tolerance = 1e-10
    P.max_newton_iterations = 20
    hist = P.solve()
    assert hist[-1] < 1e-10
    OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, 8, 8), rho=1.0, mu=0.01)
    O.newton(OP, tol=1e-10)
    assert _relmax(P.get_dofs(), OP.dofs()) <= STOL


def test_newton_nonlinear_diffusion_fp32_converges_to_fp64_solution():
    from pyoomph_gb300 import workloads as W
    gauss = W.draw_gaussians(1, 16, 3) * np.array([1, 1, 1, 1, 20.0])
    P64 = W.nonlinear_diffusion_problem(N=3, gaussians=gauss)
    P64.newton_solver_tolerance = 1e-10
    P64.solve()
    P32 = W.nonlinear_diffusion_problem(N=3, gaussians=gauss, jacobian_precision="fp32")
    P32.newton_solver_tolerance = 1e-10
    P32.max_newton_iterations = 20
    P32.solve()
    assert _relmax(P32.get_dofs(), P64.get_dofs()) <= STOL
    OP = O.poisson_problem(O.mesh(O.Q2_HEX, 3, 3, 3), gauss, eq=O.EQ_NONLINEAR_DIFFUSION)
    O.newton(OP, tol=1e-10)
    assert _relmax(P64.get_dofs(), OP.dofs()) <= STOL


@pytest.mark.parametrize("kind", ["ns_th", "nldiff_hex", "poisson_q2"])
def test_curved_mesh_general_geometry_vs_oracle(kind):
    """Non-affine (curved) elements take the per-integration-point geometry
    path; the affine shortcut must not be selected."""
    from pyoomph_gb300 import workloads as W
    rng = np.random.default_rng(21)
    T = W.wavy(0.03)
    if kind == "ns_th":
        P = W.navier_stokes_problem(N=[7, 6], transform=T)
        P.initialise()
        m = O.mesh(O.P2_TRI, 7, 6)
        m.x = T(m.x.copy())
        OP = O.navier_stokes_problem(m, rho=1.0, mu=0.01)
        x = OP.dofs() + rng.normal(0, 0.1, OP.n_dof)
    else:
        et, dim, nx = (O.Q2_HEX, 3, [3, 2, 3]) if kind == "nldiff_hex" else (O.Q2_QUAD, 2, [6, 5])
        gauss = W.draw_gaussians(8, 8, dim)
        if kind == "nldiff_hex":
            P = W.nonlinear_diffusion_problem(N=nx, gaussians=gauss, transform=T)
            eq = O.EQ_NONLINEAR_DIFFUSION
        else:
            P = W.poisson_problem(N=nx, gaussians=gauss, transform=T)
            eq = O.EQ_POISSON
        P.initialise()
        m = O.mesh(et, *(nx + [0] * (3 - len(nx))))
        m.x = T(m.x.copy())
        OP = O.poisson_problem(m, gauss, eq=eq)
        x = rng.normal(0, 0.5, OP.n_dof)
    assert not P.affine
    OP.set_dofs(x)
    P.set_dofs(x)
    R0, rp, ci, v = O.assemble(OP, True, -1.0)
    R, J = P.get_jacobian()
    assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
    assert _relmax(J.data, v) <= RTOL
    assert _relmax(R, R0) <= RTOL


def test_structured_workloads_take_the_affine_path():
    from pyoomph_gb300 import workloads as W
    for P in (W.poisson_problem(N=4), W.navier_stokes_problem(N=4), W.nonlinear_diffusion_problem(N=2)):
        P.lower()
        assert P.affine


@pytest.mark.parametrize("jref", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("geometry", ["affine", "general"])
@pytest.mark.parametrize("kind", ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex", "nldiff_q2"])
def test_element_level_parity_every_kernel_variant(kind, geometry, prec, jref):
    """Element residuals/matrices straight from the GPU element buffers
    (fe_problem_element_buffers) against the oracle's, for every variant
    (Jacobian contracted in physical or in reference coordinates)."""
    import element_cases as C
    P, ks, values, Rr, Jr = C.build(kind, geometry, prec, jref=jref)
    P.initialise()
    P.set_values(values)
    P.get_jacobian()
    Re, Je = P.element_buffers()
    assert C.relmax(Re, Rr) <= RTOL
    assert C.relmax(Je, Jr) <= (RTOL if prec == "fp64" else JTOL32)


def test_custom_assembler_drop_in_contract():
    """GB300Assembler through pyoomph's CustomAssemblyBase contract: float64
    residual, CSR with int32 indptr/indices and float64 data, dofs taken
    from the host problem's get_current_dofs()."""
    from pyoomph_gb300 import GB300Assembler, workloads as W

    class HostProblem:  # stands for the pyoomph Problem
        def __init__(self, x):
            self.x = x

        def get_current_dofs(self):
            return self.x, None

    gauss = W.draw_gaussians(2, 8, 2)
    eng = W.poisson_problem(N=6, gaussians=gauss)
    asm = GB300Assembler(eng)
    asm.initialize()
    x = np.random.default_rng(1).normal(size=eng.n_dof)
    asm._set_problem(HostProblem(x))
    R = asm.get_residuals_and_jacobian(False)
    R2, J = asm.get_residuals_and_jacobian(True)
    assert R.dtype == np.float64 and J.data.dtype == np.float64
    assert J.indptr.dtype == np.int32 and J.indices.dtype == np.int32
    assert np.array_equal(R, R2)
    OP = O.poisson_problem(O.mesh(O.Q2_QUAD, 6, 6), gauss)
    OP.set_dofs(x)
    R0, rp, ci, v = O.assemble(OP, True, -1.0)
    assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
    assert _relmax(J.data, v) <= RTOL and _relmax(R, R0) <= RTOL


@pytest.mark.parametrize("geometry", ["affine", "general"])
@pytest.mark.parametrize("kind", ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex", "nldiff_q2"])
def test_df64_element_level_parity(kind, geometry):
    """The double-float Jacobian's element matrices from the GPU element
    buffers against the oracle's, within the FP64 contract."""
    import element_cases as C
    P, ks, values, Rr, Jr = C.build(kind, geometry, "df64")
    P.initialise()
    P.set_values(values)
    P.get_jacobian()
    Re, Je = P.element_buffers()
    assert C.relmax(Re, Rr) <= RTOL
    assert C.relmax(Je, Jr) <= RTOL


@pytest.mark.parametrize("jac", ["fp32", "df64"])
@pytest.mark.parametrize("geometry", ["affine", "general"])
def test_df64_residual_element_level_parity(geometry, jac):
    """The double-float residual path (interpolation, pointwise residual and
    test-function contraction on the FP32 pipes) from the GPU element
    buffers against the oracle's element residuals, within the FP64
    contract; the Jacobian keeps its own precision's contract."""
    import element_cases as C
    P, ks, values, Rr, Jr = C.build("ns_th", geometry, jac, residual="df64")
    assert "_rdf" in ks.name
    P.initialise()
    P.set_values(values)
    P.get_jacobian()
    Re, Je = P.element_buffers()
    assert C.relmax(Re, Rr) <= RTOL
    assert C.relmax(Je, Jr) <= (RTOL if jac == "df64" else 1e-5)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_thread_count_changes_rounding_only(prec):
    """Every phase of the element kernel is a block-strided loop, so any
    thread count gives the same element values up to the compiler's choice
    of fused multiply-adds: one thread per row, the default max(knots,
    ceil(rows/2)) per element, and fewer threads than knots."""
    from pyoomph_gb300 import workloads as W
    out = {}
    for thr in (None, 480, 96):
        P = W.navier_stokes_problem(N=[12, 10], jacobian_precision=prec)
        P.elems_per_block = 32
        P.threads_per_block = thr
        P.initialise()
        W.perturb_dofs(P, seed=5, sigma=1e-2)
        assert P.kernel.threads == (256 if thr is None else thr)
        R, J = P.get_jacobian()
        out[thr] = (R, J.data.astype(np.float64))
    R0, J0 = out[None]
    for thr in (480, 96):
        R, J = out[thr]
        assert _relmax(R, R0) <= 1e-14 and _relmax(J, J0) <= (1e-14 if prec == "fp64" else 1e-6)
