"""Adaptive BDF2 time stepping (pyoomph's run(temporal_error=...), which
calls oomph-lib's Problem::adaptive_unsteady_newton_solve, problem.cc:
11280-11500, with BDF<2>'s predictor and error weights, timesteppers.cc:
252-395, and pyoomph's temporal error norm, src/problem.cpp:660-670 and
src/mesh.cpp:1783-1830).

After a step of size dt from t_n (previous step dtp):

* the predictor is the explicit extrapolation
  u_p = (1 - r^2) u_n + r^2 u_{n-1} + (1 + r) dt u'_n,  r = dt / dtp,
  u'_n the BDF derivative at t_n (the weights of the step that reached it);
* the error of a value is E (u_{n+1} - u_p), E = (1 + q)^2 / (1 + 3q +
  4q^2 + 2q^3), q = dtp / dt; the norm is pyoomph's: sqrt(sum_k s_k e_k^2 /
  #{k : s_k != 0}) over the free values k, s_k the temporal error scale of
  the value's field (set_temporal_error_factor in pyoomph, whose default
  scale is 0; ``AdaptiveState.scales`` None means scale 1 for every value);
* the step is rescaled by f = (eps / max(error, 1e-12))^(1/3): rejected
  (and redone with f dt) when error > eps or f <= 0.8, the next step f dt
  at most 4 dt; dt stays in [1e-12, 1e12].  A Newton failure rejects the
  step and halves it.

The first step (BDF1: no derivative at the start yet) is taken without an
estimate.  The algorithm only needs ``AdaptiveOps``; the Problem
provides them (time levels restored from host snapshots on rejection).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

DTSF_MAX_INCREASE = 4.0
DTSF_MIN_DECREASE = 0.8
MINIMUM_DT = 1e-12
MAXIMUM_DT = 1e12
NONCONVERGENCE_FACTOR = 0.5


class AdaptiveOps:
    """What an adaptive step calls."""

    def step(self, dt: float) -> None:
        """One implicit BDF step (BDF1 first); raises on Newton failure."""

    def dofs(self) -> np.ndarray: ...
    def snapshot(self): ...
    def restore(self, snap) -> None: ...
    def weights(self) -> tuple:
        """The BDF weights of the last step (w0, w1, w2)."""


@dataclass
class AdaptiveState:
    u_n: np.ndarray
    u_nm1: Optional[np.ndarray] = None
    udot_n: Optional[np.ndarray] = None
    dt_n: Optional[float] = None
    steps: int = 0
    last_error: Optional[float] = None
    # temporal error scale of every dof (None: 1 for every dof)
    scales: Optional[np.ndarray] = None


def error_norm(err: np.ndarray, scales: Optional[np.ndarray]) -> float:
    """pyoomph's temporal error norm (src/mesh.cpp:1783-1843 per mesh,
    src/problem.cpp:660-670 summed): the root of the scale-weighted mean
    square over the values whose field has a non-zero scale."""
    if scales is None:
        return float(np.sqrt(np.mean(err * err))) if err.size else 0.0
    n = int(np.count_nonzero(scales))
    return float(np.sqrt(np.sum(scales * err * err) / n)) if n else 0.0


def predictor(st: AdaptiveState, dt: float) -> np.ndarray:
    r = dt / st.dt_n
    return (1.0 - r * r) * st.u_n + r * r * st.u_nm1 + (1.0 + r) * dt * st.udot_n


def error_weight(dt: float, dtp: float) -> float:
    q = dtp / dt
    return (1.0 + q) ** 2 / (1.0 + 3.0 * q + 4.0 * q ** 2 + 2.0 * q ** 3)


def adaptive_step(ops: AdaptiveOps, st: AdaptiveState, dt: float, epsilon: float,
                  newton_error=Exception, max_tries: int = 50):
    """One accepted step from the state's point; returns (dt taken, next
    dt).  Updates the state."""
    for _ in range(max_tries):
        snap = ops.snapshot()
        try:
            ops.step(dt)
        except newton_error:
            ops.restore(snap)
            dt *= NONCONVERGENCE_FACTOR
            if dt < MINIMUM_DT:
                raise
            continue
        u = ops.dofs()
        factor, reject = 1.0, False
        if st.udot_n is not None and st.u_nm1 is not None:
            err = error_weight(dt, st.dt_n) * (u - predictor(st, dt))
            error = max(error_norm(err, st.scales), 1e-12)
            st.last_error = error
            factor = (epsilon / error) ** (1.0 / 3.0)
            reject = error > epsilon
        new_dt = factor * dt
        if factor > DTSF_MAX_INCREASE:
            new_dt = DTSF_MAX_INCREASE * dt
        elif not reject and factor <= DTSF_MIN_DECREASE:
            reject = True
        if new_dt < MINIMUM_DT:
            raise RuntimeError(f"time step would fall below {MINIMUM_DT}")
        new_dt = min(new_dt, MAXIMUM_DT)
        if reject:
            ops.restore(snap)
            dt = new_dt
            continue
        w = ops.weights()
        udot = w[0] * u + w[1] * st.u_n + (w[2] * st.u_nm1 if st.u_nm1 is not None else 0.0)
        st.u_nm1, st.u_n, st.udot_n, st.dt_n = st.u_n, u, udot, dt
        st.steps += 1
        return dt, new_dt
    raise RuntimeError("adaptive step: no acceptable step size found")
