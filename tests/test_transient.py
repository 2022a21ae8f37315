"""Time-dependent forms on fixed meshes: partial_t terms with BDF weights
(pyoomph's DiffusionEquation, poisson.py:153-180, and the rho partial_t(u)
of Navier-Stokes, navier_stokes.py:481-503), the mass matrix (flag 2 of the
generated ResidualAndJacobian, jitbridge.h:285) and the BDF1/BDF2 time
stepping of Problem.unsteady_newton_solve.

These forms are linear in du/dt with a coefficient c independent of u, so
the oracle's transient element residual is R_e(u) + M_e udot_e and its
Jacobian J_e + w0 M_e, with M_e = c int psi_i psi_j (ofe_element_mass) and
udot the BDF combination of the nodal time levels."""
import numpy as np
import pytest

import element_cases as C
import oracle as O

# BDF2 with a variable step (dt = 0.1 after 0.07)
_OM = 0.1 / 0.07
W_BDF2 = ((1.0 + 2.0 * _OM) / ((1.0 + _OM) * 0.1), -(1.0 + _OM) / 0.1, _OM * _OM / ((1.0 + _OM) * 0.1))


def _oracle_mass(kind, P, ks):
    et = {"ns_th": O.P2_TRI, "poisson_q2": O.Q2_QUAD, "poisson_p2": O.P2_TRI, "nldiff_hex": O.Q2_HEX,
          "nldiff_q2": O.Q2_QUAD}[kind]
    eq = {"ns_th": O.EQ_NAVIER_STOKES_TH, "poisson_q2": O.EQ_POISSON, "poisson_p2": O.EQ_POISSON,
          "nldiff_hex": O.EQ_NONLINEAR_DIFFUSION, "nldiff_q2": O.EQ_NONLINEAR_DIFFUSION}[kind]
    coeff = 1.0  # rho = 1 (Navier-Stokes), temporal factor 1
    m = P.mesh
    n = ks.layout.n
    out = []
    for e in range(m.n_elem):
        M = np.zeros(n * n)
        O.lib().ofe_element_mass(et, eq, m.dim, O._ptr(np.ascontiguousarray(m.x)),
                                 O._ptr(np.ascontiguousarray(m.conn[e])), coeff, O._ptr(M))
        out.append(M.reshape(n, n))
    return np.array(out)


def _local(ks, conn, nodal):
    """Nodal values [n_nodes, nval] -> element-local vectors [E, nloc]."""
    lay = ks.layout
    return nodal[conn[:, lay.node], lay.val]


@pytest.mark.parametrize("geometry", ["affine", "general"])
@pytest.mark.parametrize("kind,prec", [(k, "fp64") for k in C.KINDS] + [("ns_th", "df64"), ("poisson_q2", "fp32"),
                                                                       ("nldiff_hex", "df64")])
def test_emulated_transient_element_matches_oracle(kind, geometry, prec):
    import kernel_emulator as KE
    P, ks, values, Rr, Jr = C.build(kind, geometry, prec, transient=True)
    assert ks.pointwise.transient and P.param_names[-3:] == ["_bdf_w0", "_bdf_w1", "_bdf_w2"]
    m = P.mesh
    rng = np.random.default_rng(11)
    hist = np.stack([values + rng.normal(0.0, 0.2, values.shape), values + rng.normal(0.0, 0.2, values.shape)])
    params = P.params.copy()
    params[-3:] = W_BDF2
    rb, jb, st = KE.run(ks, m.x, m.conn, values, params, flag=1, hist=hist)
    assert not st.any()
    _, mb, st = KE.run(ks, m.x, m.conn, values, params, flag=2, hist=hist)
    assert not st.any()
    Me = _oracle_mass(kind, P, ks)
    udot = W_BDF2[0] * values + W_BDF2[1] * hist[0] + W_BDF2[2] * hist[1]
    ue = _local(ks, m.conn, udot)
    Rt = Rr + np.einsum("eij,ej->ei", Me, ue)
    Jt = Jr + W_BDF2[0] * Me
    jtol = 1e-5 if prec == "fp32" else 1e-12
    assert C.relmax(rb, Rt) <= 1e-12
    assert C.relmax(jb, Jt) <= jtol
    assert C.relmax(mb, Me) <= jtol
    # the time term is really there: the transient residual differs from the steady one
    assert C.relmax(Rr, Rt) > 1e-3


def test_steady_lowering_drops_the_time_derivative():
    """A steady problem generates the steady kernel (no history, no BDF
    weights), even where the form has partial_t terms (Navier-Stokes)."""
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=4)
    ks = P.lower()
    assert not ks.pointwise.transient and "_bdf_w0" not in P.param_names and "sUt" not in ks.source
    Pt = W.navier_stokes_problem(N=4, transient=True)
    kt = Pt.lower()
    assert kt.pointwise.transient and "sUt" in kt.source and kt.name != ks.name
    # BDF weights: BDF1, and BDF2 reproducing d/dt of a quadratic in time exactly
    from pyoomph_gb300.ale import bdf_weights
    w = bdf_weights(2, 0.1, 0.07)
    t = np.array([0.17, 0.07, 0.0])
    f = 3.0 + 2.0 * t - 5.0 * t * t
    assert abs(np.dot(w, f) - (2.0 - 10.0 * 0.17)) < 1e-12
    assert np.allclose(bdf_weights(1, 0.1), (10.0, -10.0, 0.0))


def _engine_and_oracle(kind, prec, n=6):
    from pyoomph_gb300 import workloads as W
    if kind == "ns":
        P = W.navier_stokes_problem(N=n, Re=50.0, jacobian_precision=prec, transient=True)
        OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, n, n), rho=1.0, mu=0.02)
        et, eq = O.P2_TRI, O.EQ_NAVIER_STOKES_TH
    elif kind == "poisson":
        g = W.draw_gaussians(4, 8, 2)
        P = W.poisson_problem(N=n, gaussians=g, jacobian_precision=prec, transient=True)
        OP = O.poisson_problem(O.mesh(O.Q2_QUAD, n, n), g)
        et, eq = O.Q2_QUAD, O.EQ_POISSON
    else:
        g = W.draw_gaussians(4, 16, 3)
        P = W.nonlinear_diffusion_problem(N=3, gaussians=g, jacobian_precision=prec, transient=True)
        OP = O.poisson_problem(O.mesh(O.Q2_HEX, 3, 3, 3), g, eq=O.EQ_NONLINEAR_DIFFUSION)
        et, eq = O.Q2_HEX, O.EQ_NONLINEAR_DIFFUSION
    return P, OP, et, eq


def _oracle_time_term(P, et, eq, udot):
    """Global sum_e M_e udot_e (free rows) and the free-free block of the
    assembled mass matrix, dense (small meshes)."""
    m, lay = P.mesh, P.kernel.layout
    n = lay.n
    R = np.zeros(P.n_dof)
    M = np.zeros((P.n_dof, P.n_dof))
    for e in range(m.n_elem):
        Me = np.zeros(n * n)
        O.lib().ofe_element_mass(et, eq, m.dim, O._ptr(np.ascontiguousarray(m.x)),
                                 O._ptr(np.ascontiguousarray(m.conn[e])), 1.0, O._ptr(Me))
        Me = Me.reshape(n, n)
        g = P.eqn[m.conn[e, lay.node], lay.val]
        r = Me @ udot[m.conn[e, lay.node], lay.val]
        f = g >= 0
        np.add.at(R, g[f], r[f])
        M[np.ix_(g[f], g[f])] += Me[np.ix_(f, f)]
    return R, M


@pytest.mark.gpu
@pytest.mark.parametrize("kind,prec", [("poisson", "fp64"), ("ns", "fp64"), ("ns", "df64"), ("hex", "fp64"),
                                       ("hex", "fp32")])
def test_gpu_transient_assembly_matches_oracle(kind, prec):
    P, OP, et, eq = _engine_and_oracle(kind, prec)
    P.initialise()
    rng = np.random.default_rng(8)
    free = P.eqn >= 0
    levels = []
    for _ in range(3):
        v = P._values0.copy()
        v[free] += rng.normal(0.0, 0.3, free.sum())
        levels.append(v)
    P.set_values(levels[0])
    P.set_history_values(0, levels[1])
    P.set_history_values(1, levels[2])
    P.set_parameters(**dict(zip(["_bdf_w0", "_bdf_w1", "_bdf_w2"], W_BDF2)))
    R, J = P.get_jacobian()
    Mm = P.get_mass_matrix()
    x = P.get_dofs()
    OP.set_dofs(x)
    R0, rp, ci, v0 = O.assemble(OP, True, -1.0)
    prp, pci = P.pattern()
    assert np.array_equal(prp, rp) and np.array_equal(pci, ci)
    udot = W_BDF2[0] * levels[0] + W_BDF2[1] * levels[1] + W_BDF2[2] * levels[2]
    Rt, Md = _oracle_time_term(P, et, eq, udot)
    rows = np.repeat(np.arange(P.n_dof), np.diff(rp))
    Mv = Md[rows, ci]
    jtol = 1e-5 if prec == "fp32" else 1e-12
    assert C.relmax(R, R0 + Rt) <= 1e-12
    assert C.relmax(J.data, v0 + W_BDF2[0] * Mv) <= jtol
    assert np.array_equal(Mm.indptr, rp) and np.array_equal(Mm.indices, ci)
    assert C.relmax(Mm.data, Mv) <= jtol


@pytest.mark.gpu
def test_gpu_heat_equation_known_answer_second_order_in_time():
    """du/dt = Laplace(u) on the unit square, u = 0 on the boundary,
    u(0) = sin(pi x) sin(pi y): u(t) = exp(-2 pi^2 t) sin(pi x) sin(pi y).
    Through unsteady_newton_solve (BDF1 first step, BDF2 after), the error
    at t = 0.1 is the time scheme's own: the same recurrence applied to the
    one mode, y' = -2 pi^2 y, gives it to within the (Q2, h = 1/24) spatial
    error -- 6.6e-4 and 1.3e-4 for 10 and 20 steps, second order
    (ratio -> 4 as dt -> 0; 4.97 at lambda dt = 0.2)."""
    from pyoomph_gb300 import DiffusionEquation, DirichletBC, Problem, RectangularQuadMesh
    errs = []
    for nsteps in (10, 20):
        P = Problem()
        P += RectangularQuadMesh(N=24)
        P += (DiffusionEquation() + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
        P.initialise()
        x = P.mesh.x
        u0 = (np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1]))[:, None]
        P.set_values(u0)
        dt = 0.1 / nsteps
        for _ in range(nsteps):
            hist = P.unsteady_newton_solve(dt)
            assert hist[-1] < 1e-10
        assert P.is_transient and abs(P.time - 0.1) < 1e-12
        exact = np.exp(-2.0 * np.pi ** 2 * 0.1) * u0[:, 0]
        errs.append(np.max(np.abs(P.get_values()[:, 0] - exact)))
    lam = 2.0 * np.pi ** 2
    for nsteps, err in zip((10, 20), errs):
        dt = 0.1 / nsteps
        y = [1.0, 1.0]
        for k in range(nsteps):
            w = (1.0 / dt, -1.0 / dt, 0.0) if k == 0 else (1.5 / dt, -2.0 / dt, 0.5 / dt)
            y.append(-(w[1] * y[-1] + w[2] * y[-2]) / (w[0] + lam))
        model = abs(y[-1] - np.exp(-lam * 0.1))
        assert abs(err - model) <= 0.01 * model, (nsteps, err, model)


def test_generalized_eigensolver_host_logic():
    """(-J) v = lambda M v: the shift-invert branch agrees with the dense
    one; rows without mass (constraints) give infinite eigenvalues that the
    dense branch drops; eigenpairs satisfy the equation."""
    import scipy.sparse as sps
    from pyoomph_gb300.problem import solve_generalized_eigenproblem
    n = 40
    h = 1.0 / (n + 1)
    K = sps.diags([-np.ones(n - 1), 2 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]) / h     # 1D P1 stiffness
    M = sps.diags([np.ones(n - 1), 4 * np.ones(n), np.ones(n - 1)], [-1, 0, 1]) * h / 6   # and mass
    J = K.tocsr()                       # du/dt = u'' -> J = K, eigenvalues of -K: -(k pi)^2 approx
    ev_d, vec_d = solve_generalized_eigenproblem(J, M.tocsr(), 0)
    ev_s, vec_s = solve_generalized_eigenproblem(J, M.tocsr(), 4, shift=0.0)
    assert np.allclose(ev_s, ev_d[:4], rtol=1e-10)
    assert abs(ev_d[0].real + np.pi ** 2) < 1e-2 * np.pi ** 2
    for lam, v in zip(ev_s, vec_s):
        assert np.linalg.norm(-J @ v - lam * (M @ v)) <= 1e-8 * np.linalg.norm(J @ v)
    # a constraint row (no mass) has an infinite eigenvalue
    M2 = M.tolil()
    M2[0, :] = 0.0
    ev2, _ = solve_generalized_eigenproblem(J, M2.tocsr(), 0)
    assert np.all(np.isfinite(ev2)) and len(ev2) == n - 1


@pytest.mark.gpu
def test_gpu_eigenvalues_of_the_laplacian():
    """The heat equation on the unit square with u = 0 on the boundary: the
    leading eigenvalues of (-J) v = lambda M v approximate -pi^2 (k^2 + l^2)
    (-2 pi^2, -5 pi^2 twice, -8 pi^2).  Q2 elements with the 3 x 3 Gauss
    rule are the exact tensor product of 1D P2 ones (stiffness
    (1/3h)[7 -8 1; -8 16 -8; 1 -8 7], mass (h/30)[4 2 -1; 2 16 2; -1 2 4]),
    so the discrete eigenvalues are exactly -(mu_k + mu_l) of the 1D P2
    problem: checked to 1e-9, and to the continuous ones within 5e-5."""
    import scipy.linalg as sla
    from pyoomph_gb300 import DiffusionEquation, DirichletBC, Problem, RectangularQuadMesh
    P = Problem()
    P += RectangularQuadMesh(N=16)
    P += (DiffusionEquation() + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    P.initialise()
    ev, vec = P.solve_eigenproblem(4, shift=0.0)
    N, h = 16, 1.0 / 16
    Ke = np.array([[7, -8, 1], [-8, 16, -8], [1, -8, 7]]) / (3 * h)
    Me = np.array([[4, 2, -1], [2, 16, 2], [-1, 2, 4]]) * h / 30
    K1, M1 = np.zeros((2 * N + 1, 2 * N + 1)), np.zeros((2 * N + 1, 2 * N + 1))
    for e in range(N):
        ix = np.ix_([2 * e, 2 * e + 1, 2 * e + 2], [2 * e, 2 * e + 1, 2 * e + 2])
        K1[ix] += Ke
        M1[ix] += Me
    mu = np.sort(sla.eigh(K1[1:-1, 1:-1], M1[1:-1, 1:-1], eigvals_only=True))
    discrete = -np.array([mu[0] + mu[0], mu[0] + mu[1], mu[0] + mu[1], mu[1] + mu[1]])
    assert np.max(np.abs(ev.real - discrete) / np.abs(discrete)) < 1e-9, (ev, discrete)
    exact = -np.pi ** 2 * np.array([2.0, 5.0, 5.0, 8.0])
    assert np.max(np.abs(ev.real - exact) / np.abs(exact)) < 5e-5, ev
    assert np.max(np.abs(ev.imag)) < 1e-8
    assert vec.shape == (4, P.n_dof) and np.array_equal(P.get_last_eigenvalues(), ev)


def test_assembler_last_mass_and_jacobian_host_logic():
    """GB300Assembler.get_last_mass_and_jacobian_matrices (pyoomph's hook,
    read by its Lyapunov-exponent tool): nothing before a Jacobian or for a
    steady engine; the last J and the engine's mass matrix otherwise."""
    import scipy.sparse as sps
    from pyoomph_gb300 import GB300Assembler

    class Engine:
        is_transient = False
        n_dof = 2

        def initialise(self):
            pass

        def set_dofs(self, x):
            pass

        def get_jacobian(self):
            return np.zeros(2), sps.csr_matrix(np.array([[2.0, 0.0], [1.0, 3.0]], dtype=np.float32))

        def get_mass_matrix(self):
            return sps.identity(2, format="csr")

    eng = Engine()
    asm = GB300Assembler(eng)
    assert asm.get_last_mass_and_jacobian_matrices() == (None, None)
    _, J = asm.get_residuals_and_jacobian(True)
    assert J.data.dtype == np.float64 and J.indptr.dtype == np.int32
    assert asm.get_last_mass_and_jacobian_matrices() == (None, None)      # steady engine
    eng.is_transient = True
    M, J2 = asm.get_last_mass_and_jacobian_matrices()
    assert J2 is J and (M != sps.identity(2)).nnz == 0
    asm.invalidate_cache()
    assert asm.get_last_mass_and_jacobian_matrices() == (None, None)


def _time_form_problem(source):
    from pyoomph_gb300 import DirichletBC, Equations, Problem, RectangularQuadMesh, grad, var_and_test, weak

    class Heat(Equations):
        def define_fields(self):
            self.define_scalar_field("u", "C2")

        def define_residuals(self):
            u, v = var_and_test("u")
            self.add_residual(weak(grad(u), grad(v)) - weak(source(), v))

    P = Problem()
    P += RectangularQuadMesh(N=3)
    P += (Heat() + DirichletBC(u=0.0) @ ["left", "right"]) @ "domain"
    return P


def test_emulated_time_symbol_reads_the_time_parameter():
    """var("time") is a run-time parameter: the kernel of a form with
    sin(t) x y at t = 0.3 gives the residual of the form with the number
    sin(0.3) in its place."""
    import kernel_emulator as KE
    import sympy as sp
    from pyoomph_gb300 import expressions as E
    from pyoomph_gb300 import var
    Pt = _time_form_problem(lambda: sp.sin(var("time")) * E.X[0] * E.X[1])
    Pt.time = 0.3
    kt = Pt.lower()
    assert Pt.param_names == ["_time"] and Pt.params[0] == 0.3
    Pc = _time_form_problem(lambda: sp.Float(np.sin(0.3)) * E.X[0] * E.X[1])
    kc = Pc.lower()
    m = Pt.mesh
    vals = Pt._values0 + np.random.default_rng(1).normal(0.0, 0.2, Pt._values0.shape)
    rt, jt, st = KE.run(kt, m.x, m.conn, vals, Pt.params)
    rc, jc, sc = KE.run(kc, m.x, m.conn, vals, np.zeros(1))
    assert not st.any() and not sc.any()
    assert np.max(np.abs(rt - rc)) <= 1e-14 * np.max(np.abs(rc)) and np.array_equal(jt, jc)
    # another time, another source
    p2 = Pt.params.copy()
    p2[0] = 1.1
    r2, _, _ = KE.run(kt, m.x, m.conn, vals, p2)
    assert np.max(np.abs(r2 - rt)) > 1e-3


def test_time_dependent_dirichlet_values(monkeypatch):
    """Dirichlet values given as f(x, y, t=...) are evaluated at lowering
    (at Problem.time) and again by set_time, which uploads the nodal
    values; constant and time-independent values stay as they are."""
    from pyoomph_gb300 import DirichletBC, PoissonEquation, Problem, RectangularQuadMesh
    from pyoomph_gb300 import problem as PR
    P = Problem()
    P += RectangularQuadMesh(N=4)
    P += (PoissonEquation() + DirichletBC(u=lambda x, y, t: np.sin(np.pi * x) * np.exp(-t)) @ "top" +
          DirichletBC(u=lambda x, y: x) @ "bottom" + DirichletBC(u=2.0) @ "left") @ "domain"
    P.time = 0.5
    P.lower()
    top = P.mesh.boundaries["top"] & ~P.mesh.boundaries["left"]
    x = P.mesh.x
    assert np.allclose(P._values0[top, 0], np.sin(np.pi * x[top, 0]) * np.exp(-0.5))
    assert len(P._timed_bcs) == 1
    uploads = []

    class Lib:
        def fe_problem_set_values(self, h, ptr):
            uploads.append(np.ctypeslib.as_array((PR.ctypes.c_double * P._values0.size).from_address(ptr)).copy())
            return 0

    monkeypatch.setattr(PR.N, "load", lambda: Lib())
    P._initialised, P._h = True, object()
    P.set_time(1.25)
    assert P.time == 1.25 and len(uploads) == 1
    up = uploads[0].reshape(P._values0.shape)
    assert np.allclose(up[top, 0], np.sin(np.pi * x[top, 0]) * np.exp(-1.25))
    bottom = P.mesh.boundaries["bottom"] & ~P.mesh.boundaries["left"]
    assert np.allclose(up[bottom, 0], x[bottom, 0])
    b = P.mesh.boundaries
    assert np.all(up[b["left"] & ~b["top"] & ~b["bottom"], 0] == 2.0)
    assert np.array_equal(up[~top, 0], P._values0[~top, 0])       # only the timed values change
    P._initialised, P._h = False, None


def test_bdf_weights_are_the_references():
    """pyoomph's MultiTimeStepper::set_weights (src/timestepper.cpp:32-52):
    BDF1 1/dt, -1/dt; BDF2 1/dt + 1/(dt+dtp), -(dt+dtp)/(dt dtp),
    dt/((dt+dtp) dtp) -- the same expressions, so the same bits; and
    consistent with d/dt of quadratics in time."""
    from pyoomph_gb300.ale import bdf_weights
    import ale_oracle as AO
    rng = np.random.default_rng(0)
    for _ in range(200):
        dt, dtp = 10.0 ** rng.uniform(-5, 0, 2)
        ref = (1.0 / dt + 1.0 / (dt + dtp), -(dt + dtp) / (dt * dtp), dt / ((dt + dtp) * dtp))
        assert bdf_weights(2, dt, dtp) == ref == AO.bdf_weights(2, dt, dtp)
        assert bdf_weights(1, dt) == (1.0 / dt, -1.0 / dt, 0.0)
        t = np.array([dt + dtp, dtp, 0.0])
        f = 1.0 + 3.0 * t - 2.0 * t * t
        assert abs(np.dot(ref, f) - (3.0 - 4.0 * (dt + dtp))) <= 1e-9 * max(1.0, 1.0 / dt)


def test_run_steps_to_the_output_times_and_the_end():
    """Problem.run's time loop (host logic; the step itself stubbed): steps
    of `timestep`, shortened to land on every output time and on the end
    time; outputs at the start and at every outstep; the Newton settings of
    the call restored afterwards."""
    from pyoomph_gb300 import workloads as W
    P = W.poisson_problem(N=4, transient=True)
    steps, outs = [], []

    def fake_step(dt):
        steps.append(dt)
        P.time += dt

    P.unsteady_newton_solve = fake_step
    t = P.run(1.0, 0.3, outstep=0.25, output=lambda p: outs.append(round(p.time, 12)),
              newton_solver_tolerance=1e-3)
    assert abs(t - 1.0) < 1e-12 and P.newton_solver_tolerance == 1e-8
    assert outs == [0.0, 0.25, 0.5, 0.75, 1.0]
    assert np.allclose(steps, [0.25, 0.25, 0.25, 0.25])        # the output interval caps the step
    steps.clear()
    outs.clear()
    P.run(1.3, 0.1, outstep=True, output=lambda p: outs.append(round(p.time, 12)))
    assert len(steps) == 3 and abs(sum(steps) - 0.3) < 1e-12 and len(outs) == 4
    steps.clear()
    P.run(2.0, numouts=4)                                        # step = output interval
    assert np.allclose(steps, [0.175] * 4)
    with pytest.raises(ValueError):
        P.run(3.0, 0.1, outstep=0.5, numouts=3)
    with pytest.raises(NotImplementedError):
        P.run(3.0, 0.1, spatial_adapt=1)
    # temporal_error: the adaptive step answers with the next step size
    steps.clear()
    P.adaptive_unsteady_newton_solve = lambda dt, eps: (fake_step(dt), 2.0 * dt)[1]
    P.run(P.time + 0.7, 0.1, temporal_error=1e-4)
    assert np.allclose(steps, [0.1, 0.2, 0.4])          # doubling steps, the last one cut to the end time


def test_history_levels_keep_hanging_values_consistent(monkeypatch):
    """set_history_values constrains the hanging values of the level it
    uploads (the device interpolates the current values only)."""
    from pyoomph_gb300 import DiffusionEquation, DirichletBC, Problem
    from pyoomph_gb300 import problem as PR
    from pyoomph_gb300.meshes import RefinedQuadMesh
    P = Problem()
    P.transient = True
    P += RefinedQuadMesh(N=4)
    P += (DiffusionEquation() + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    P.lower()
    assert P.is_transient and len(P.hang_slots) > 0
    got = []

    class Lib:
        def fe_problem_set_history(self, h, level, ptr):
            got.append(np.ctypeslib.as_array((PR.ctypes.c_double * P.mesh.n_nodes).from_address(ptr)).copy())
            return 0

    monkeypatch.setattr(PR.N, "load", lambda: Lib())
    P._h = object()
    v = np.random.default_rng(0).normal(size=(P.mesh.n_nodes, 1))
    P.set_history_values(0, v)
    up = got[0]
    for h, ms in P.mesh.hang.items():
        assert abs(up[h] - sum(w * up[m] for m, w in ms)) < 1e-14
    free = np.ones(P.mesh.n_nodes, dtype=bool)
    free[list(P.mesh.hang)] = False
    assert np.array_equal(up[free], v[free, 0])
    P._h = None


def test_steady_solve_of_a_transient_problem_zeroes_the_bdf_weights():
    """Problem.solve is the steady solve also for a transient problem (the
    BDF weights are 0 during its Newton loop and restored after); a time
    step keeps them."""
    from pyoomph_gb300 import workloads as W
    P = W.poisson_problem(N=4, transient=True)
    P.lower()
    k = [P.param_names.index(n) for n in ("_bdf_w0", "_bdf_w1", "_bdf_w2")]
    P.params[k] = (3.0, -4.0, 1.0)
    seen = []
    P.initialise = lambda: None

    def set_parameters(replica=None, **kw):
        for n, v in kw.items():
            P.params[P.param_names.index(n)] = v

    P.set_parameters = set_parameters
    P._newton = lambda: seen.append(P.params[k].copy()) or [0.0]
    P.solve()
    assert np.array_equal(seen[0], np.zeros(3)) and np.array_equal(P.params[k], (3.0, -4.0, 1.0))
