"""Adaptive BDF2 (oomph-lib's adaptive_unsteady_newton_solve with BDF<2>'s
predictor and error weights) on a linear system whose implicit step is
solved exactly: the global error follows the tolerance, the steps grow as
the solution decays, a step that is too large is rejected and redone."""
import numpy as np
import pytest

from pyoomph_gb300.ale import bdf_weights
from pyoomph_gb300.timestepping import AdaptiveState, adaptive_step, error_weight, predictor


class _ODE:
    """u' = -lam u (two decoupled modes), BDF1 then BDF2, solved exactly."""

    def __init__(self, lam=(1.0, 3.0)):
        self.lam = np.array(lam)
        self.u = np.array([1.0, 0.5])
        self.h = [self.u.copy(), self.u.copy()]
        self.steps, self.dtp, self.w, self.t, self.rejected = 0, None, None, 0.0, 0

    def step(self, dt):
        w = bdf_weights(1 if self.steps == 0 else 2, dt, self.dtp)
        new = -(w[1] * self.u + w[2] * self.h[0]) / (w[0] + self.lam)
        self.h = [self.u.copy(), self.h[0]]
        self.u, self.steps, self.dtp, self.w, self.t = new, self.steps + 1, dt, w, self.t + dt

    def dofs(self):
        return self.u.copy()

    def snapshot(self):
        return self.u.copy(), [x.copy() for x in self.h], self.steps, self.dtp, self.w, self.t

    def restore(self, s):
        self.rejected += 1
        self.u, self.h, self.steps, self.dtp, self.w, self.t = s[0].copy(), [x.copy() for x in s[1]], *s[2:]

    def weights(self):
        return self.w

    def exact(self):
        return np.array([1.0, 0.5]) * np.exp(-self.lam * self.t)


def _integrate(eps, dt0, T=2.0):
    ode = _ODE()
    st = AdaptiveState(ode.dofs())
    dt, dts = dt0, []
    while ode.t < T - 1e-12:
        taken, dt = adaptive_step(ode, st, min(dt, T - ode.t), eps)
        dts.append(taken)
    return ode, dts


def test_global_error_follows_the_tolerance():
    errs, nsteps = [], []
    for eps in (1e-4, 1e-6):
        ode, dts = _integrate(eps, 1e-3)
        errs.append(np.max(np.abs(ode.u - ode.exact())))
        nsteps.append(len(dts))
    assert errs[1] < errs[0] / 10 and nsteps[1] > nsteps[0]
    assert errs[1] < 1e-4


def test_steps_grow_and_large_steps_are_rejected():
    ode, dts = _integrate(1e-6, 0.05)
    # the first step has no estimate; the second, tried at 0.05, errs ~1e-3 and is redone shorter
    assert dts[0] == 0.05 and ode.rejected >= 1 and dts[1] < 0.05
    ode, dts = _integrate(1e-5, 1e-3)
    assert dts[-2] > 4 * dts[2]                         # the decaying solution allows longer steps
    assert all(b <= 4.0 * a + 1e-15 for a, b in zip(dts[:-2], dts[1:-1]))


def test_predictor_and_error_weight_formulas():
    """The predictor is exact for quadratics in time; the error weight of
    constant steps is 4/10 (BDF2's Milne constant against this predictor)."""
    dt, dtp = 0.3, 0.2
    f = lambda t: 2.0 - t + 0.7 * t * t
    st = AdaptiveState(np.array([f(0.0)]), np.array([f(-dtp)]), np.array([-1.0 + 1.4 * 0.0]), dtp)
    assert abs(predictor(st, dt)[0] - f(dt)) < 1e-14
    assert error_weight(0.1, 0.1) == pytest.approx(4.0 / 10.0)


def test_error_norm_counts_only_scaled_values():
    """pyoomph's norm: sum of scale * err^2 over the values with a non-zero
    scale, divided by their count (src/mesh.cpp:1783-1843)."""
    from pyoomph_gb300.timestepping import error_norm
    e = np.array([1.0, 2.0, 3.0, 4.0])
    assert error_norm(e, None) == pytest.approx(np.sqrt(np.mean(e * e)))
    s = np.array([1.0, 0.0, 2.0, 0.0])
    assert error_norm(e, s) == pytest.approx(np.sqrt((1.0 + 2.0 * 9.0) / 2.0))
    assert error_norm(e, np.zeros(4)) == 0.0


@pytest.mark.gpu
def test_gpu_adaptive_steps_match_a_fixed_step_replay():
    """The Problem adapter of adaptive stepping on the device: a step
    rejected for its error and a step whose Newton solve fails are undone
    from the host copies of the time levels; a fixed step in between makes
    the stepper restart from the current point.  Every accepted state equals
    a replay of the same step sizes by plain unsteady_newton_solve."""
    from pyoomph_gb300 import DiffusionEquation, DirichletBC, Problem, RectangularQuadMesh
    from pyoomph_gb300.problem import NewtonSolverError

    def make():
        P = Problem()
        P += RectangularQuadMesh(N=12)
        P += (DiffusionEquation() + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
        P.initialise()
        x = P.mesh.x
        u0 = (np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1])
              + 0.3 * np.sin(3 * np.pi * x[:, 0]) * np.sin(2 * np.pi * x[:, 1]))[:, None]
        P.set_values(u0)
        return P

    P = make()
    calls, failed = [0], []
    newton = P._newton

    def flaky_newton():
        calls[0] += 1
        if calls[0] == 3:               # the third attempt may not iterate: NewtonSolverError
            keep = P.max_newton_iterations
            P.max_newton_iterations = 0
            try:
                return newton()
            except NewtonSolverError:
                failed.append(calls[0])
                raise
            finally:
                P.max_newton_iterations = keep
        return newton()

    P._newton = flaky_newton
    taken, states = [], []
    dt = 0.05                           # lambda dt ~ 1: the first estimated step is far too long
    while P.time < 0.12 - 1e-12:
        dt = P.adaptive_unsteady_newton_solve(min(dt, 0.12 - P.time), 1e-4)
        taken.append(P.dt_prev)
        states.append(P.get_dofs())
    P.unsteady_newton_solve(0.01)       # a fixed step: the adaptive state is stale afterwards
    taken.append(0.01)
    states.append(P.get_dofs())
    while P.time < 0.3 - 1e-12:
        dt = P.adaptive_unsteady_newton_solve(min(dt, 0.3 - P.time), 1e-4)
        taken.append(P.dt_prev)
        states.append(P.get_dofs())
    assert failed == [3]
    assert calls[0] > len(taken) + 1    # at least one step was also rejected for its error
    Q = make()
    for k, h in enumerate(taken):
        Q.unsteady_newton_solve(h)
        ref = Q.get_dofs()
        assert np.max(np.abs(states[k] - ref)) <= 1e-12 * np.max(np.abs(ref)), k
    assert abs(Q.time - P.time) < 1e-14 and Q.steps_done == P.steps_done


def test_temporal_error_scales_per_field():
    """Problem.set_temporal_error_factor: the scale of every dof of a field;
    fields without a factor count with scale 0 once any field has one."""
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=3)
    P.lower()
    assert P._temporal_error_scales() is None
    P.set_temporal_error_factor("velocity_x", 2.0)
    s = P._temporal_error_scales()
    eqn = np.asarray(P.eqn).reshape(P.mesh.n_nodes, 3)
    ux = eqn[:, 0][eqn[:, 0] >= 0]
    assert np.all(s[ux] == 2.0) and np.count_nonzero(s) == ux.size
    P.set_temporal_error_factor("nonexistent", 1.0)
    with pytest.raises(KeyError):
        P._temporal_error_scales()
