"""Pseudo-arclength continuation (pyoomph's Problem.arclength_continuation,
problem.py:3508) round the fold of the Bratu problem
-Laplace(u) = lambda exp(u), u = 0 on the boundary: the path from
(lambda, u) = (0, 0) turns at lambda* = 3.513830719 on the unit interval and
at lambda* = 6.808124 on the unit square.  The continuation needs J and
dR/dlambda (the kernels' parameter derivative, flag 3)."""
import numpy as np
import pytest

from pyoomph_gb300.continuation import ContinuationError, arclength_step, fold_from_three


def _follow_to_fold(step_fn, p_of, max_steps=60):
    """Step until the parameter turns; the fold from a parabola through the
    last three points (s, p)."""
    s, pts, state = 0.0, [], None
    for _ in range(max_steps):
        state = step_fn(state)
        s += state.ds
        pts.append((s, p_of(state)))
        if state.dp < 0.0:
            break
    else:
        raise AssertionError("no fold reached")
    (s0, p0), (s1, p1), (s2, p2) = pts[-3:]
    return fold_from_three([s0, s1, s2], [p0, p1, p2]), pts


class _Bratu1D:
    """Finite differences: -(u[i-1] - 2u[i] + u[i+1])/h^2 - lambda exp(u[i])."""

    def __init__(self, n):
        import scipy.sparse as sps
        self.n_dof = n
        self.h = 1.0 / (n + 1)
        self.K = sps.diags([-np.ones(n - 1), 2 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]).tocsr() / self.h ** 2
        self.u = np.zeros(n)
        self.lam = 0.0

    def get_dofs(self):
        return self.u.copy()

    def set_dofs(self, x):
        self.u = np.array(x, dtype=np.float64)

    def get_parameter(self):
        return self.lam

    def set_parameter(self, v):
        self.lam = float(v)

    def residual_and_jacobian(self):
        import scipy.sparse as sps
        e = np.exp(self.u)
        return self.K @ self.u - self.lam * e, (self.K - sps.diags(self.lam * e)).tocsr()

    def parameter_derivative(self):
        return -np.exp(self.u)


def test_continuation_rounds_the_fold_of_the_1d_bratu_problem():
    ops = _Bratu1D(200)
    ds = [0.5]

    def step(state):
        new, ds[0] = arclength_step(ops, state, ds[0], tol=1e-10, max_ds=0.5)
        step.last = new
        return new

    lam_fold, pts = _follow_to_fold(step, lambda st: st.p0)
    print("1D Bratu fold", lam_fold, "after", len(pts), "steps")
    assert abs(lam_fold - 3.513830719) < 2e-3, (lam_fold, pts[-4:])
    # every point on the path solves R = 0
    R, _ = ops.residual_and_jacobian()
    assert np.max(np.abs(R)) < 1e-8
    # beyond the fold the path continues on the upper branch: lambda falls, u grows
    lam, umax = [pts[-1][1]], [np.max(ops.get_dofs())]
    st = step.last
    for _ in range(3):
        st, ds[0] = arclength_step(ops, st, ds[0], tol=1e-10, max_ds=0.5)
        lam.append(st.p0)
        umax.append(np.max(st.u0))
    assert np.all(np.diff(lam) < 0) and np.all(np.diff(umax) > 0), (lam, umax)


def test_failed_step_restores_the_last_point():
    ops = _Bratu1D(50)
    u0, p0 = ops.get_dofs(), ops.get_parameter()
    with pytest.raises(ContinuationError):
        # no Newton iteration allowed and a step far off the path: halving cannot rescue it
        arclength_step(ops, None, 5.0, tol=1e-12, max_newton_iterations=0, min_ds=1.0)
    assert np.array_equal(ops.get_dofs(), u0) and ops.get_parameter() == p0


@pytest.mark.gpu
def test_gpu_continuation_finds_the_fold_of_the_2d_bratu_problem():
    from pyoomph_gb300 import DirichletBC, Equations, Problem, RectangularQuadMesh, exp, grad, var_and_test, weak

    class Bratu(Equations):
        def define_fields(self):
            self.define_scalar_field("u", "C2")

        def define_residuals(self):
            u, v = var_and_test("u")
            lam = self.set_parameter("lambda", 0.0)
            self.add_residual(weak(grad(u), grad(v)) - weak(lam * exp(u), v))

    P = Problem()
    P += RectangularQuadMesh(N=12)
    P += (Bratu() + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    P.newton_solver_tolerance = 1e-10
    P.initialise()
    ds = [0.5]

    def step(state):
        ds[0] = P.arclength_continuation("lambda", ds[0], max_ds=0.5)
        return P._arclength

    lam_fold, pts = _follow_to_fold(step, lambda st: st.p0)
    assert abs(lam_fold - 6.808124) < 2e-3, (lam_fold, pts[-4:])
    assert np.max(np.abs(P.get_residuals())) < 1e-9
