"""Pseudo-arclength continuation in a global parameter (pyoomph's
Problem.arclength_continuation, problem.py:3508, which calls oomph-lib's
Problem::arc_length_step_solve).

A step from the last converged point (u0, p0) with unit tangent (u', p')
(norm theta^2 |u'|^2 + p'^2 = 1, theta^2 = 1 / n_dof: the dofs count by
their mean square) solves

    R(u, p) = 0,    theta^2 u'.(u - u0) + p' (p - p0) - ds = 0

by Newton from the predictor (u0 + ds u', p0 + ds p').  The bordered
system is solved by block elimination with one factorisation of the
Jacobian J = dR/du per iteration and two right-hand sides (-R and -dR/dp):
Keller's method.  The new tangent is z = -J^-1 dR/dp, p' = 1/sqrt(1 +
theta^2 |z|^2), u' = p' z, oriented to continue the previous one (the sign
of theta^2 u'_old.u'_new + p'_old p'_new), which carries the path round a
fold, where p' changes sign.  The step adapts as oomph-lib's does: a step
that converged in fewer Newton iterations than desired grows the next one
(at most x2, at most max_ds); a failed step is halved and retried down to
min_ds.

The algorithm only needs the four operations of ``ContinuationOps``: the
Problem supplies them from device assembly (R and J from fe_assemble, dR/dp
from the kernels' flag 3), a test can supply them from any small model.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np


class ContinuationError(RuntimeError):
    pass


class ContinuationOps:
    """What a continuation step calls (host arrays)."""
    n_dof: int

    def get_dofs(self) -> np.ndarray: ...
    def set_dofs(self, x: np.ndarray) -> None: ...
    def get_parameter(self) -> float: ...
    def set_parameter(self, v: float) -> None: ...
    def residual_and_jacobian(self):
        """(R, J as a scipy sparse matrix) at the current dofs and parameter."""
    def parameter_derivative(self) -> np.ndarray:
        """dR/dp at the current dofs and parameter."""


@dataclass
class ContinuationState:
    u0: np.ndarray
    p0: float
    du: np.ndarray
    dp: float
    theta2: float
    newton_iterations: int = 0
    ds: float = 0.0            # the step that reached this point


def _factor(J):
    import scipy.sparse.linalg as spla
    return spla.splu(J.tocsc().astype(np.float64))


def tangent(ops: ContinuationOps, theta2: float, prev: Optional[ContinuationState] = None):
    """Unit tangent (u', p') at the current point; p' > 0 without a
    previous tangent, else oriented along it."""
    _, J = ops.residual_and_jacobian()
    z = _factor(J).solve(-ops.parameter_derivative())
    dp = 1.0 / np.sqrt(1.0 + theta2 * float(z @ z))
    du = dp * z
    if prev is not None and theta2 * float(prev.du @ du) + prev.dp * dp < 0.0:
        du, dp = -du, -dp
    return du, dp


def arclength_step(ops: ContinuationOps, state: Optional[ContinuationState], ds: float, *,
                   tol: float = 1e-8, max_newton_iterations: int = 10, min_ds: float = 1e-8,
                   max_ds: Optional[float] = None, desired_newton_iterations: int = 3):
    """One continuation step of (signed) length ds from the current solved
    point.  Returns (new state, next ds)."""
    if state is None:
        theta2 = 1.0 / max(ops.n_dof, 1)
        du, dp = tangent(ops, theta2)
        state = ContinuationState(ops.get_dofs().copy(), ops.get_parameter(), du, dp, theta2)
    th = state.theta2
    while True:
        u = state.u0 + ds * state.du
        p = state.p0 + ds * state.dp
        converged = False
        its = 0
        for its in range(max_newton_iterations + 1):
            ops.set_dofs(u)
            ops.set_parameter(p)
            R, J = ops.residual_and_jacobian()
            g = th * float(state.du @ (u - state.u0)) + state.dp * (p - state.p0) - ds
            if not np.all(np.isfinite(R)):
                break
            if max(float(np.max(np.abs(R))) if R.size else 0.0, abs(g)) < tol:
                converged = True
                break
            if its == max_newton_iterations:
                break
            lu = _factor(J)
            a = lu.solve(-R)
            b = lu.solve(-ops.parameter_derivative())
            den = state.dp + th * float(state.du @ b)
            if den == 0.0 or not np.isfinite(den):
                break
            dlam = -(g + th * float(state.du @ a)) / den
            u = u + a + dlam * b
            p = p + dlam
        if converged:
            break
        ds = 0.5 * ds
        if abs(ds) < min_ds:
            ops.set_dofs(state.u0)
            ops.set_parameter(state.p0)
            raise ContinuationError(f"arclength step failed down to ds = {2 * ds:.3e}")
    du, dp = tangent(ops, th, state)
    new = ContinuationState(u.copy(), p, du, dp, th, its, ds)
    grow = min(2.0, desired_newton_iterations / max(its, 1))
    nds = ds * max(grow, 1.0) if its <= desired_newton_iterations else ds * grow
    if max_ds is not None and abs(nds) > max_ds:
        nds = float(np.sign(nds)) * max_ds
    return new, nds


def locate_fold(ops: ContinuationOps, before: ContinuationState, ds: float, *, rel_tol: float = 1e-6,
                **step_kw) -> ContinuationState:
    """The turning point between `before` and the point a step ds from it,
    whose tangents' parameter components p' differ in sign: bisection on
    the step length from `before`, each trial a full corrector solve, until
    the bracket is rel_tol * |ds| wide.  The parameter is stationary there,
    so its error is quadratic in the bracket.  Leaves ops at the returned
    point (the last trial on the near side)."""
    if before.dp == 0.0:
        return before
    lo, hi = 0.0, float(ds)
    best = before
    step_kw = dict(step_kw)
    step_kw.pop("max_ds", None)
    while abs(hi - lo) > rel_tol * abs(ds):
        mid = 0.5 * (lo + hi)
        st, _ = arclength_step(ops, before, mid, **step_kw)
        if st.ds != mid:               # the step was shortened to converge
            mid = st.ds
        if np.sign(st.dp) == np.sign(before.dp):
            lo, best = mid, st
        else:
            hi = mid
    ops.set_dofs(best.u0)
    ops.set_parameter(best.p0)
    return best
