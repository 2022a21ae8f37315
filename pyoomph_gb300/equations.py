"""Equations: the user-facing weak-form classes, mirroring pyoomph's
``Equations`` API (``pyoomph/generic/codegen.py``: ``BaseEquations`` :287,
``define_scalar_field`` :2037, ``define_vector_field`` :2054,
``add_residual`` :777) and the predefined forms used by the workloads:

* ``PoissonEquation`` -- ``pyoomph/equations/poisson.py:33-72``:
  ``weak(coeff*grad(u), grad(v)) - weak(f, v)``;
* ``NavierStokesEquations`` (Taylor-Hood: velocity C2, pressure C1) --
  ``navier_stokes.py:148-345`` (stress ``2 mu sym(grad u) - p I``,
  continuity ``weak(div u, q)``) and ``:481-503`` (advection
  ``weak(rho (u.grad)u, v)``);
* ``NonlinearDiffusionEquation`` -- ``-div((1+u^2) grad u) = f``, written
  with the same building blocks.

Boundary conditions: ``DirichletBC`` (``pyoomph/meshes/bcs.py:304``) pins
values on a named boundary; ``PressureFixation`` pins the pressure of the
first node of the first element (``PressureFixationTaylorHood``,
``navier_stokes.py:55-85``).
"""
from __future__ import annotations

from typing import Callable, Dict, List, Optional, Sequence, Tuple, Union

import numpy as np
import sympy as sp

from . import expressions as E
from .expressions import (div, dot, grad, identity_matrix, material_derivative, partial_t, sym, testfunction,
                          var, var_and_test, weak)

SPACE_ORDER = {"C2TB": 0, "C2": 1, "C1TB": 2, "C1": 3}


class EquationPart:
    """Base of things that can be combined with ``+`` and restricted with ``@``."""

    def __add__(self, other: "EquationPart") -> "CombinedEquations":
        return CombinedEquations([self, other])

    def __matmul__(self, where: Union[str, Sequence[str]]) -> "Restricted":
        return Restricted(self, [where] if isinstance(where, str) else list(where))


class CombinedEquations(EquationPart):
    def __init__(self, parts: List[EquationPart]):
        self.parts: List[EquationPart] = []
        for p in parts:
            if isinstance(p, CombinedEquations):
                self.parts += p.parts
            else:
                self.parts.append(p)

    def __add__(self, other):
        return CombinedEquations(self.parts + [other])


class Restricted(EquationPart):
    def __init__(self, eq: EquationPart, where: List[str]):
        self.eq = eq
        self.where = where


class Equations(EquationPart):
    """Base class of bulk equations.  Subclasses implement
    ``define_fields`` (calling ``define_scalar_field`` /
    ``define_vector_field``) and ``define_residuals`` (calling
    ``add_residual``)."""

    def __init__(self):
        self._fields: List[Tuple[str, str]] = []
        self._residual = sp.Integer(0)
        self._params: Dict[str, float] = {}

    # -- fields --------------------------------------------------------
    def define_scalar_field(self, name: str, space: str, **_ignored) -> None:
        if space not in ("C2", "C1"):
            raise ValueError(f"space {space!r} not supported (C2, C1)")
        self._fields.append((name, space))
        E.REG.field(name)

    def define_vector_field(self, name: str, space: str, **_ignored) -> None:
        comps = [f"{name}_{c}" for c in "xyz"[:E.dimension()]]
        E.register_vector_field(name, comps)
        for c in comps:
            self.define_scalar_field(c, space)

    def define_fields(self) -> None:
        pass

    # -- residuals -----------------------------------------------------
    def add_residual(self, expr) -> None:
        self._residual = self._residual + sp.sympify(expr)

    def define_residuals(self) -> None:
        pass

    # -- parameters ----------------------------------------------------
    def set_parameter(self, name: str, value: float) -> sp.Symbol:
        self._params[name] = float(value)
        return E.parameter(name)

    def parameter_values(self) -> Dict[str, float]:
        return dict(self._params)

    def information(self) -> str:
        return type(self).__name__


def _source_expr(eq: "Equations", source):
    """A source given as an array of Gaussians [n, dim+2] (centre..., width,
    amplitude) becomes sum_k A_k exp(-|x-c_k|^2/(2 w_k^2)) with its numbers
    as run-time parameters; any other value is used as is."""
    if isinstance(source, np.ndarray):
        g = np.asarray(source, dtype=np.float64)
        dim = E.dimension()
        if g.ndim != 2 or g.shape[1] != dim + 2:
            raise ValueError(f"Gaussian source must be [n, {dim + 2}]")
        for k in range(g.shape[0]):
            for i in range(dim):
                eq.set_parameter(f"g{k}_c{i}", g[k, i])
            eq.set_parameter(f"g{k}_w", g[k, dim])
            eq.set_parameter(f"g{k}_A", g[k, dim + 1])
        return E.gaussian_source(g.shape[0], dim)
    return source


class PoissonEquation(Equations):
    """-div(coeff*grad(u)) = f  (pyoomph/equations/poisson.py:33-72)."""

    def __init__(self, name: str = "u", *, space: str = "C2", source=None, coefficient=1):
        super().__init__()
        self.name = name
        self.space = space
        self.source = source
        self.coefficient = coefficient

    def define_fields(self):
        self.define_scalar_field(self.name, self.space)

    def define_residuals(self):
        u, u_test = var_and_test(self.name)
        self.add_residual(weak(self.coefficient * grad(u), grad(u_test)))
        if self.source is not None:
            self.add_residual(-weak(_source_expr(self, self.source), u_test))


class DiffusionEquation(PoissonEquation):
    """temporal_factor partial_t(u) - div(diffusivity grad(u)) = f
    (pyoomph/equations/poisson.py:153-180): the Poisson form plus
    weak(temporal_factor partial_t(u), v)."""

    def __init__(self, name: str = "u", *, space: str = "C2", source=None, diffusivity=1, temporal_factor=1):
        super().__init__(name, space=space, source=source, coefficient=diffusivity)
        self.temporal_factor = temporal_factor

    def define_residuals(self):
        super().define_residuals()
        u, v = var_and_test(self.name)
        self.add_residual(weak(self.temporal_factor * partial_t(u), v))


class NonlinearDiffusionEquation(Equations):
    """temporal_factor partial_t(u) - div((1+u^2) grad u) = f (steady by
    default: temporal_factor 0)."""

    def __init__(self, name: str = "u", *, space: str = "C2", source=None, temporal_factor=0):
        super().__init__()
        self.name = name
        self.space = space
        self.source = source
        self.temporal_factor = temporal_factor

    def define_fields(self):
        self.define_scalar_field(self.name, self.space)

    def define_residuals(self):
        u, v = var_and_test(self.name)
        self.add_residual(weak((1 + u * u) * grad(u), grad(v)))
        if self.source is not None:
            self.add_residual(-weak(_source_expr(self, self.source), v))
        if self.temporal_factor:
            self.add_residual(weak(self.temporal_factor * partial_t(u), v))


class StokesEquations(Equations):
    """Stokes flow, Taylor-Hood (navier_stokes.py:148-345): the total stress
    2 mu sym(grad u) - p I tested with grad(v), and weak(div(u), q)."""

    def __init__(self, *, dynamic_viscosity: float = 1.0, velocity_name: str = "velocity",
                 pressure_name: str = "pressure", mode: str = "TH"):
        super().__init__()
        if mode != "TH":
            raise ValueError("only Taylor-Hood (TH) is implemented")
        self.mu = dynamic_viscosity
        self.velocity_name = velocity_name
        self.pressure_name = pressure_name

    def define_fields(self):
        self.define_vector_field(self.velocity_name, "C2")
        self.define_scalar_field(self.pressure_name, "C1")

    def saddle_point(self):
        """(constrained field, parameter scaling its Schur complement): the
        pressure, whose diagonal block is zero, and the viscosity (the
        device saddle-point solver approximates the Schur complement by the
        pressure mass over it)."""
        return self.pressure_name, "dynamic_viscosity"

    def define_residuals(self):
        u, v = var_and_test(self.velocity_name)
        p, q = var_and_test(self.pressure_name)
        mu = self.set_parameter("dynamic_viscosity", self.mu)
        stress = 2 * mu * sym(grad(u)) - identity_matrix() * p
        self.add_residual(weak(stress, grad(v)))
        self.add_residual(weak(div(u), q))


class NavierStokesEquations(StokesEquations):
    """Incompressible Navier-Stokes (navier_stokes.py:481-503): Stokes part
    plus weak(rho (partial_t u + (u.grad) u), v); the partial_t term
    vanishes in a steady solve."""

    def __init__(self, *, mass_density: float = 1.0, dynamic_viscosity: float = 1.0, **kw):
        super().__init__(dynamic_viscosity=dynamic_viscosity, **kw)
        self.rho = mass_density

    def define_residuals(self):
        super().define_residuals()
        u, v = var_and_test(self.velocity_name)
        rho = self.set_parameter("mass_density", self.rho)
        self.add_residual(weak(rho * material_derivative(u, u), v))


class BoundaryCondition(EquationPart):
    pass


class DirichletBC(BoundaryCondition):
    """Pin fields on a boundary: DirichletBC(u=0) or a callable of the
    position, e.g. velocity_x=lambda x, y: 16*x**2*(1-x)**2
    (pyoomph/meshes/bcs.py:304)."""

    def __init__(self, **values):
        self.values: Dict[str, Union[float, Callable]] = values


class PressureFixation(BoundaryCondition):
    """Pin the pressure at node 0 of element 0 (PressureFixationTaylorHood,
    navier_stokes.py:55-85)."""

    def __init__(self, name: str = "pressure", value: Optional[float] = 0.0):
        self.name = name
        self.value = value


def flatten(eq: EquationPart, where: Optional[List[str]] = None):
    """Yield (part, boundary-list-or-None) pairs of a combined tree."""
    if isinstance(eq, CombinedEquations):
        for p in eq.parts:
            yield from flatten(p, where)
    elif isinstance(eq, Restricted):
        yield from flatten(eq.eq, eq.where)
    else:
        yield eq, where
