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
