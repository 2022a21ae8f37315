"""The problem-level assembly plugin, mirroring pyoomph's
``CustomAssemblyBase`` (``pyoomph/generic/assembly.py:36-88``) and its use
by ``Problem.set_custom_assembler`` / ``get_custom_residuals_jacobian``
(``pyoomph/generic/problem.py:1711-1745``).

``GB300Assembler`` is the drop-in: a pyoomph ``Problem`` that calls
``set_custom_assembler(GB300Assembler(engine_problem))`` gets its residual
and CSR Jacobian from the GPU engine, in the reference's equation numbering
and CSR order, with the dtypes pyoomph asserts (float64 residual, int32
indptr/indices, float64 data).  The host problem's current dofs are read
with ``get_current_dofs()[0]`` each call, as pyoomph's own assemblers do.
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple, Union

import numpy as np


def _reference_base():
    """pyoomph's own CustomAssemblyBase (pyoomph/generic/assembly.py:36) when
    pyoomph imports here, so that the assembler is an instance of the class
    pyoomph's Problem.set_custom_assembler expects; None otherwise."""
    try:
        from pyoomph.generic.assembly import CustomAssemblyBase as base  # type: ignore
        return base
    except Exception:
        return None


class _LocalCustomAssemblyBase:
    """The plugin contract of pyoomph's CustomAssemblyBase, for hosts where
    pyoomph itself does not import."""

    def __init__(self) -> None:
        self.problem = None

    def _set_problem(self, problem) -> None:
        self.problem = problem

    def has_custom_solve_routine(self) -> bool:
        return False

    def custom_solve_routine(self, solve_Jx_b: Callable[[np.ndarray], np.ndarray], b: np.ndarray) -> np.ndarray:
        raise NotImplementedError("Custom solve routine not implemented")

    def invalidate_cache(self) -> None:
        pass

    def actions_after_adapt(self) -> None:
        self.invalidate_cache()

    def actions_after_remeshing(self) -> None:
        self.invalidate_cache()

    def actions_after_equation_numbering(self) -> None:
        self.invalidate_cache()

    def actions_after_setting_initial_condition(self) -> None:
        self.invalidate_cache()

    def actions_after_successful_newton_solve(self) -> None:
        pass

    def initialize(self) -> None:
        pass

    def finalize(self) -> None:
        pass

    def get_residuals_and_jacobian(self, require_jacobian: bool, dparameter: Optional[str] = None):
        raise RuntimeError("Must be implemented")

    def get_last_mass_and_jacobian_matrices(self):
        return None, None


CustomAssemblyBase = _reference_base() or _LocalCustomAssemblyBase


def numbering_fingerprint(eqn) -> str:
    """A hash of an equation-number table [n_nodes, nval] (int32)."""
    import hashlib
    return hashlib.sha1(np.ascontiguousarray(eqn, dtype=np.int32).tobytes()).hexdigest()[:16]


class GB300Assembler(CustomAssemblyBase):
    """Residual and CSR Jacobian from the GB300 engine.

    ``engine`` is a ``pyoomph_gb300.Problem`` describing the same mesh and
    weak form as the host problem (same equation numbering, which
    ``check_numbering`` verifies against the host problem when it is set).
    If the host problem is not set, the engine's own dof state is
    assembled."""

    def __init__(self, engine, device_linear_solve: bool = False, mesh_name: str = "domain") -> None:
        super().__init__()
        self.engine = engine
        self.device_linear_solve = bool(device_linear_solve)
        self.mesh_name = mesh_name
        self._last_J = None
        self._numbering_checked = False

    def check_numbering(self) -> None:
        """Refuse a host problem numbered differently from the engine: its
        number of equations (pyoomph's Problem.ndof) and, where the host
        exposes its mesh (Problem.get_mesh(name).nodes(), Node.nvalue,
        Node.eqn_number), the equation of every nodal value, which fixes the
        CSR rows and columns.  A mismatch would otherwise assemble a
        different system without any error."""
        P = self.problem
        if P is None:
            return
        self.engine.lower()
        nd = P.ndof() if callable(getattr(P, "ndof", None)) else None
        if nd is not None and int(nd) != self.engine.n_dof:
            raise RuntimeError(f"host problem has {nd} equations, the engine {self.engine.n_dof}")
        getm = getattr(P, "get_mesh", None)
        if not callable(getm):
            return
        mesh = getm(self.mesh_name)
        if mesh is None or not hasattr(mesh, "nodes"):
            return
        eqn = np.asarray(self.engine.eqn).reshape(self.engine.mesh.n_nodes, len(self.engine.fields))
        host = np.full_like(eqn, -1)
        k = -1
        for k, node in enumerate(mesh.nodes()):
            if k >= eqn.shape[0]:
                raise RuntimeError(f"host mesh {self.mesh_name!r} has more nodes than the engine's")
            nv = min(int(node.nvalue()), eqn.shape[1])
            for vi in range(nv):
                host[k, vi] = int(node.eqn_number(vi))
        if k + 1 != eqn.shape[0]:
            raise RuntimeError(f"host mesh {self.mesh_name!r} has {k + 1} nodes, the engine {eqn.shape[0]}")
        if numbering_fingerprint(host) != numbering_fingerprint(eqn):
            bad = np.argwhere(host != eqn)[0]
            raise RuntimeError(f"equation numbering differs from the host problem's (first at node {bad[0]}, "
                               f"value {bad[1]}: host {host[tuple(bad)]}, engine {eqn[tuple(bad)]})")
        self._numbering_checked = True

    def has_custom_solve_routine(self) -> bool:
        return self.device_linear_solve

    def custom_solve_routine(self, solve_Jx_b, b):
        """J x = b for pyoomph's Newton step (assembly.py:47-50 of pyoomph)
        on the device: the engine's native BiCGStab on the Jacobian of the
        last assembly, still resident.  A matrix the solver refuses
        (saddle-point systems) raises LinearSolverError: construct the
        assembler without device_linear_solve to keep pyoomph's own solver."""
        return np.ascontiguousarray(self.engine.solve_linear_device(np.asarray(b, dtype=np.float64)),
                                    dtype=np.float64)

    def initialize(self) -> None:
        self.check_numbering()
        self.engine.initialise()

    def actions_after_equation_numbering(self) -> None:
        self.invalidate_cache()
        self.check_numbering()

    def _sync_dofs(self) -> None:
        if self.problem is not None and hasattr(self.problem, "get_current_dofs"):
            dofs = np.asarray(self.problem.get_current_dofs()[0], dtype=np.float64)
            if dofs.shape[0] != self.engine.n_dof:
                raise RuntimeError(f"host problem has {dofs.shape[0]} dofs, engine {self.engine.n_dof}")
            self.engine.set_dofs(dofs)

    def _sync_params(self) -> None:
        """Copy the host problem's global parameters that the engine's weak
        form reads (by name: pyoomph's Problem.get_global_parameter_names /
        get_global_parameter(name).value, src/pybind/problem.cpp:515-517)
        into the engine when they changed, e.g. under arclength
        continuation."""
        if self.problem is None or not hasattr(self.problem, "get_global_parameter_names"):
            return
        stride = len(self.engine.param_names)
        changed = {}
        for name in self.problem.get_global_parameter_names():
            if name in self.engine.param_names:
                v = float(self.problem.get_global_parameter(name).value)
                if v != self.engine.params[self.engine.param_names.index(name) % stride]:
                    changed[name] = v
        if changed:
            self.engine.set_parameters(**changed)

    def get_residuals_and_jacobian(self, require_jacobian: bool, dparameter: Optional[str] = None
                                   ) -> Union[np.ndarray, Tuple[np.ndarray, "object"]]:
        """R (float64[n]), or (R, J) with J a CSR matrix of int32 indices and
        float64 values; with ``dparameter`` and no Jacobian, dR/dp of that
        global parameter (problem.py:1739-1744 of pyoomph asks for it so; a
        Jacobian derived by a parameter is refused there as here)."""
        if dparameter is not None and require_jacobian:
            raise RuntimeError("Cannot derive custom Jacobian with respect to a parameter yet")
        self.engine.initialise()
        self._sync_params()
        self._sync_dofs()
        if dparameter is not None:
            return np.ascontiguousarray(self.engine.get_parameter_derivative(dparameter), dtype=np.float64)
        if not require_jacobian:
            return np.ascontiguousarray(self.engine.get_residuals(), dtype=np.float64)
        R, J = self.engine.get_jacobian()
        J.data = J.data.astype(np.float64, copy=False)
        J.indptr = J.indptr.astype(np.int32, copy=False)
        J.indices = J.indices.astype(np.int32, copy=False)
        self._last_J = J
        return np.ascontiguousarray(R, dtype=np.float64), J

    def get_last_mass_and_jacobian_matrices(self):
        """(M, J): J as returned by the last Jacobian assembly, M = dR/d(du/dt)
        from the engine's mass-matrix assembly at the current state
        (pyoomph's hook, assembly.py:87, read by utils/lyapunov.py:83).
        (None, None) before any Jacobian or for a steady engine: the caller
        then assembles them itself."""
        if self._last_J is None or not getattr(self.engine, "is_transient", False):
            return None, None
        return self.engine.get_mass_matrix(), self._last_J

    def invalidate_cache(self) -> None:
        self._last_J = None
