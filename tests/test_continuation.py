"""Pseudo-arclength continuation (pyoomph's Problem.arclength_continuation,
problem.py:3508) round the fold of the Bratu problem
-Laplace(u) = lambda exp(u), u = 0 on the boundary: the path from
(lambda, u) = (0, 0) turns at lambda* = 3.513830719 on the unit interval and
at lambda* = 6.808124 on the unit square.  The continuation needs J and
dR/dlambda (the kernels' parameter derivative, flag 3)."""
import numpy as np
import pytest

from pyoomph_gb300.continuation import ContinuationError, arclength_step, locate_fold


def _follow_to_fold(step_fn, max_steps=60):
    """Step until the parameter turns; returns the states before and after."""
    prev, state = None, None
    for _ in range(max_steps):
        prev, state = state, step_fn(state)
        if state.dp < 0.0:
            return prev, state
    raise AssertionError("no fold reached")


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


@pytest.mark.parametrize("max_ds", [0.25, 0.5, 1.0])
def test_continuation_rounds_the_fold_of_the_1d_bratu_problem(max_ds):
    """Finite differences, 200 points: the discrete fold, 3.51378547, lies
    4.5e-5 below the continuum's 3.513830719 (second order in h); located
    by bisection to 1e-8 whatever the step sizes that reached it."""
    ops = _Bratu1D(200)
    ds = [0.5]

    def step(state):
        new, ds[0] = arclength_step(ops, state, ds[0], tol=1e-10, max_ds=max_ds)
        return new

    before, after = _follow_to_fold(step)
    # beyond the fold the path continues on the upper branch: lambda falls, u grows
    lam, umax, st = [after.p0], [np.max(after.u0)], after
    for _ in range(3):
        st, ds[0] = arclength_step(ops, st, ds[0], tol=1e-10, max_ds=max_ds)
        lam.append(st.p0)
        umax.append(np.max(st.u0))
    assert np.all(np.diff(lam) < 0) and np.all(np.diff(umax) > 0), (lam, umax)
    fold = locate_fold(ops, before, after.ds, tol=1e-10)
    print("1D Bratu fold", fold.p0, "max_ds", max_ds)
    assert abs(fold.p0 - 3.51378547) < 1e-8 and 3e-5 < 3.513830719 - fold.p0 < 6e-5
    R, _ = ops.residual_and_jacobian()
    assert np.max(np.abs(R)) < 1e-8 and abs(fold.dp) < 1e-2


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

    _follow_to_fold(step)
    lam_fold = P.locate_fold()
    print("2D Bratu fold", lam_fold)
    assert abs(lam_fold - 6.808124) < 1e-3, lam_fold
    assert np.max(np.abs(P.get_residuals())) < 1e-9
