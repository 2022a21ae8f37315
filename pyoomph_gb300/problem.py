"""Problem: the drop-in counterpart of pyoomph's ``Problem`` for the
residual/Jacobian path (``pyoomph/generic/problem.py``: ``Problem`` :343,
``initialise`` :2430, ``assemble_jacobian`` :711, ``solve`` :4721; Newton
defaults :409-411).

``initialise`` generates the meshes, numbers the equations
(oomph ``Mesh::assign_global_eqn_numbers``, ``mesh.cc:686-708``: nodes in
order, values in order, pinned values skipped), lowers the weak form to a
CUDA element kernel (``codegen.generate_kernel``), JIT-compiles it for
sm_103a and creates the resident device problem through the C-ABI.

``solve`` is ``Problem::newton_solve`` (``problem.cc:8986-9300``): residual
max-norm (NaN -> inf), stop below ``newton_solver_tolerance``, otherwise
assemble R and J on the GPU, solve J dx = R (SuperLU through scipy, the
reference's default serial solver, or a caller-supplied solver), x -= dx.
"""
from __future__ import annotations

import contextlib
import ctypes
import time
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
import sympy as sp

from . import _native as N
from . import expressions as E
from .codegen import BDF_PARAMS, KernelSpec, Pointwise, differentiate, generate_kernel, time_derivative_symbols
from .equations import (SPACE_ORDER, BoundaryCondition, DirichletBC, EquationPart, Equations,
                        PressureFixation, flatten)
from .meshes import MeshData, MeshTemplate


def _sm_count() -> int:
    """Streaming multiprocessors of device 0 (152 on GB300; also the value
    used where no device is visible, so that the generated kernels are the
    same with and without one)."""
    global _SMS
    if _SMS is None:
        try:
            n = ctypes.c_int()
            _SMS = n.value if N.load().fe_device_info(ctypes.byref(n), None, None, None, None) == 0 else 152
        except Exception:
            _SMS = 152
    return _SMS


_SMS = None


def mesh_is_axis_aligned(mesh: MeshData, rtol: float = 1e-14) -> bool:
    """True if every element's reference axis a maps onto physical axis a
    alone (the affine map's Jacobian dx/ds is diagonal at the element
    centre, off-diagonal entries below rtol of the diagonal): the
    structured rectangle and cuboid meshes.  Tensor-product elements of such
    a mesh take three coordinates per axis at their 3^dim Gauss points."""
    et = mesh.etype
    if et.name not in ("Q2_QUAD", "Q2_HEX"):
        return False
    _, d1 = et.shape_c1(np.zeros(mesh.dim))
    Xv = mesh.x[mesh.conn[:, list(et.c1_index)]]                 # [E, vertices, D]
    A = np.einsum("eld,la->eda", Xv, d1)                        # [E, physical, reference]
    diag = np.abs(np.einsum("edd->ed", A))
    off = np.abs(A).sum(axis=2) - diag
    return bool(np.all(off <= rtol * diag) and np.all(diag > 0))


def mesh_is_affine(mesh: MeshData, rtol: float = 1e-12) -> bool:
    """True if every element's map from reference to physical coordinates is
    affine: the tangent vectors dx/ds are the same at all integration points
    and the vertex (C1) interpolation reproduces the position.  Such elements
    get their geometry computed once per element instead of once per
    integration point (the values differ only by rounding)."""
    et = mesh.etype
    t = et.tables()
    X = mesh.x[mesh.conn]                                   # [E, NN, D]
    dps = t["DPS2"]                                         # [Q, NN, D]
    scale = np.max(np.abs(mesh.x)) + 1e-300
    E = X.shape[0]
    for lo in range(0, E, 65536):
        Xb = X[lo:lo + 65536]
        tq = np.einsum("eli,qla->eqai", Xb, dps)            # tangents at every point
        if np.max(np.abs(tq - tq[:, :1])) > rtol * np.max(np.abs(tq[:, :1]) + 1e-300) * 10:
            return False
        x2 = np.einsum("eli,ql->eqi", Xb, t["PSI2"])
        x1 = np.einsum("eli,ql->eqi", Xb[:, list(et.c1_index)], t["PSI1"])
        if np.max(np.abs(x2 - x1)) > 1e-13 * scale:
            return False
    return True


_KERNEL_CACHE: Dict[tuple, KernelSpec] = {}
_CODE_CACHE: Dict[str, "N.Code"] = {}


def nvtx_range(name: str):
    """NVTX range around a host-side stage (assembly, linear solve) for
    timeline profilers; a no-op context when torch has no CUDA."""
    import contextlib
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.nvtx.range(name)
    except Exception:
        pass
    return contextlib.nullcontext()


def _bc_takes_time(fn) -> bool:
    import inspect
    try:
        return "t" in inspect.signature(fn).parameters
    except (TypeError, ValueError):
        return False


def _bc_value(fn, x: np.ndarray, k: int, ncomp: int, t: float):
    """A Dirichlet value function at nodes x [n, dim]: fn(x0, x1[, x2]) or,
    time-dependent, fn(x0, x1[, x2], t=...); a vector field's function
    returns one array per component."""
    args = [x[:, d] for d in range(x.shape[1])]
    v = fn(*args, t=t) if _bc_takes_time(fn) else fn(*args)
    return v[k] if isinstance(v, (tuple, list)) and ncomp > 1 else v


def solve_generalized_eigenproblem(J, M, n: int, shift=0.0, sort: bool = True, which: str = "LM", v0=None,
                                   target=None):
    """(-J) v = lambda M v for sparse J, M (host): all eigenpairs densely when
    n covers the system, else n of them by shift-invert Arnoldi about
    `shift` (scipy's eigs, as pyoomph's scipy eigensolver, solvers/scipy.py:166-190).
    Sorted by descending real part, or by distance to `target`; infinite
    eigenvalues (rows without mass: constraints, pressure) dropped in the
    dense branch.  Returns (eigenvalues, eigenvectors as rows)."""
    import scipy.linalg as sla
    import scipy.sparse.linalg as spla_
    A = -J.astype(np.float64)
    N_ = A.shape[0]
    if n <= 0 or n >= N_ - 1:
        ev, vec = sla.eig(A.toarray(), b=M.toarray())
        keep = np.isfinite(ev)
        ev, vec = ev[keep], vec[:, keep]
    else:
        ev, vec = spla_.eigs(A.tocsc(), k=n, M=M.tocsc(), sigma=shift, which=which, v0=v0)
    if sort:
        order = np.argsort(np.abs(ev - target)) if target is not None else np.argsort(-ev.real, kind="stable")
        ev, vec = ev[order], vec[:, order]
    if n > 0:
        ev, vec = ev[:n], vec[:, :n]
    return ev, vec.T


class _ProblemContinuationOps:
    """The continuation's operations on a Problem (device assembly)."""

    def __init__(self, P: "Problem", name: str):
        self.P, self.name = P, name
        self.n_dof = P.n_dof
        self.k = P.param_names.index(name)

    def get_dofs(self):
        return self.P.get_dofs()

    def set_dofs(self, x):
        self.P.set_dofs(x)

    def get_parameter(self):
        return float(self.P.params[self.k])

    def set_parameter(self, v):
        self.P.set_parameters(**{self.name: float(v)})

    def residual_and_jacobian(self):
        R, J = self.P.get_jacobian()
        return np.asarray(R, dtype=np.float64), J

    def parameter_derivative(self):
        return self.P.get_parameter_derivative(self.name)


class _ProblemAdaptiveOps:
    """The adaptive stepper's operations on a Problem; the two previous time
    levels are kept on the host to undo a rejected step."""

    def __init__(self, P: "Problem", prev):
        self.P, self.prev = P, list(prev)

    def step(self, dt):
        # the nodal values before the step: the snapshot the stepper took
        # just before this call holds them
        self._before = self._last_snapshot[0]
        self.P.unsteady_newton_solve(dt)

    def dofs(self):
        return self.P.get_dofs()

    def snapshot(self):
        P = self.P
        k = [P.param_names.index(n) for n in BDF_PARAMS]
        self._last_snapshot = (P.get_values(), P.get_dofs(), list(self.prev), P.time, P.steps_done, P.dt_prev,
                               P.params[k].copy())
        return self._last_snapshot

    def restore(self, s):
        P = self.P
        vals, dofs, prev, t, steps, dtp, w = s
        P.set_values(vals)
        P.set_dofs(dofs)
        P.set_history_values(0, prev[0])
        P.set_history_values(1, prev[1])
        P.steps_done, P.dt_prev = steps, dtp
        P.set_parameters(**dict(zip(BDF_PARAMS, w)))
        P.set_time(t)
        self.prev = list(prev)

    def accepted(self):
        self.prev = [self._before, self.prev[0]]

    def weights(self):
        P = self.P
        return tuple(float(P.params[P.param_names.index(n)]) for n in BDF_PARAMS)


class NewtonSolverError(RuntimeError):
    """Raised when Newton diverges or exceeds its iteration cap
    (oomph's NewtonSolverError, problem.cc:9298)."""


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise N.FeError(N.FE_ERR_NOGPU, "pyoomph_gb300 needs a CUDA GPU (none visible)")
    return torch


@dataclass
class AssemblyStats:
    n_elem: int
    n_dof: int
    nnz: int
    n_contrib: int


class Problem:
    def __init__(self):
        self._meshes: List[MeshTemplate] = []
        self._equations: List[EquationPart] = []
        self.max_residuals = 1e10
        self.max_newton_iterations = 10
        self.newton_solver_tolerance = 1e-8
        # "fp64"; "fp32": FP32 Jacobian, FP64 residual; "df64": FP64 Jacobian
        # values contracted in double-float (~2^-48) on the FP32 pipes
        self.jacobian_precision = "fp64"
        # "fp64"; "df64": the residual path (interpolation, pointwise
        # residual, test-function contraction) in double-float on the FP32
        # pipes, for FP32 and df64 Jacobians of steady forms whose pointwise
        # terms are rational (Gaussian sources evaluated in FP64)
        self.residual_precision = "fp64"
        self.elems_per_block: Optional[int] = None
        # threads per block of the element kernel (None: one per local row
        # of the block's elements; fewer run the rows in rounds)
        self.threads_per_block: Optional[int] = None
        # "auto": detect affine elements (constant geometry per element) on the host
        self.geometry = "auto"
        # > 1: a stack of independent copies of the problem assembled together
        self.replicas = 1
        self.linear_solver: Optional[Callable] = None
        # compile the element code with device-side bounds checks (status word 2)
        self.bounds_check = False
        # contract the Jacobian in reference coordinates (None: the generator's
        # default, on for 3D elements)
        self.jacobian_reference: Optional[bool] = None
        # contract FP32 element Jacobians on the tensor cores (None: where the
        # generator supports it and it pays, the Q2 hex's 27 x 27 matrices)
        self.tensor_cores: Optional[bool] = None
        # resident blocks per SM the element kernel's registers are bounded
        # for (__launch_bounds__ minimum; None: the generator's choice, 0:
        # no bound)
        self.min_blocks_per_sm: Optional[int] = None
        # linear_solver = "bicgstab": J dx = R solved on the device (linsolve.py)
        # to this relative tolerance; "fieldsplit": saddle-point systems
        # (Taylor-Hood) on the device (fieldsplit.py: GMRES, block-triangular
        # multigrid preconditioner) to fieldsplit_forcing; None: SuperLU on the
        # host (the reference's default)
        self.linear_solver_tolerance = 1e-13
        # Gaussian source terms on axis-aligned affine Q2 meshes: evaluate the
        # per-axis factors once per element (3 dim exponentials per Gaussian
        # instead of one per knot); the values differ from the per-knot
        # evaluation by rounding only
        self.separable_source = True
        # absolute floor of the device solve's residual (0: relative only);
        # e.g. 0.1 x newton_solver_tolerance for an inexact Newton step
        self.linear_solver_atol = 0.0
        # "fieldsplit" (saddle-point GMRES, fieldsplit.py): each Newton step
        # solves to the relative tolerance fieldsplit_forcing, an inexact
        # Newton step whose linear error stays below the quadratic term
        # (fieldsplit.newton_forcing), never below fieldsplit_min_tolerance
        # (the 2-norm residual of a Krylov solve of these systems stalls near
        # cond x eps)
        self.fieldsplit_forcing = 1e-5
        self.fieldsplit_min_tolerance = 1e-11
        self.saddle_point = None
        # time-dependent solve: the weak form's partial_t terms are kept (BDF
        # weights of the step as parameters, two previous time levels on the
        # device); False: they vanish (the steady ResidualAndJacobianSteady
        # of pyoomph's generated code).  Switched on by the first
        # unsteady_newton_solve.
        self.transient = False
        self.is_transient = False      # set by lower(): the lowered form keeps partial_t terms
        self.time = 0.0
        self.steps_done = 0
        self.dt_prev: Optional[float] = None
        # bumped by every write of the state from outside a time step (dofs,
        # values, history levels, a rebuild); the adaptive stepper's host
        # copies of the time levels are valid only while it is unchanged
        self._state_generation = 0
        # oomph's Problem::Numerical_zero_for_sparse_assembly for the
        # matrices get_jacobian returns: None = the structural pattern (every
        # coupling kept, the fast path); a threshold >= 0 = the reference's
        # value-dependent pattern (its default is 0.0)
        self.numerical_zero_for_sparse_assembly: Optional[float] = None
        # assemble only the elements [lo, hi) of the mesh, with the global
        # numbering (oomph's First_el_for_assembly / Last_el_plus_one_for_
        # assembly split, problem.cc:5354-5358): R and J hold this range's
        # contributions; distributed.py completes the sum across ranks
        self.element_range: Optional[Tuple[int, int]] = None
        # temporal error scale per field name (set_temporal_error_factor)
        self.temporal_error_factors: Dict[str, float] = {}
        self.verbose = False
        self._initialised = False
        self.newton_history: List[float] = []
        self.timings: Dict[str, float] = {}

    # -- building ------------------------------------------------------
    def add_mesh(self, mesh: MeshTemplate) -> None:
        if len(self._meshes) >= 1:
            raise NotImplementedError("one bulk domain per problem")
        self._meshes.append(mesh)

    def add_equations(self, eqs: EquationPart) -> None:
        self._equations.append(eqs)

    def __iadd__(self, other):
        if isinstance(other, MeshTemplate):
            self.add_mesh(other)
        elif isinstance(other, EquationPart):
            self.add_equations(other)
        else:
            raise TypeError(f"cannot add {type(other).__name__} to a Problem")
        return self

    # -- initialise ----------------------------------------------------
    def lower(self) -> KernelSpec:
        """Generate the mesh and the element kernel source (no GPU needed):
        fields in nodal-value order, the summed weak form, its pointwise
        derivatives and the CUDA kernel (codegen.generate_kernel)."""
        if getattr(self, "kernel", None) is not None:
            return self.kernel
        t0 = time.perf_counter()
        if not self._meshes:
            raise RuntimeError("no mesh added")
        tmpl = self._meshes[0]
        mesh = tmpl.generate()
        self.mesh: MeshData = mesh
        E.set_dimension(mesh.dim)
        bulk: List[Equations] = []
        bcs: List[Tuple[BoundaryCondition, Optional[List[str]]]] = []
        for eq in self._equations:
            for part, where in flatten(eq):
                if isinstance(part, Equations):
                    bulk.append(part)
                elif isinstance(part, BoundaryCondition):
                    bcs.append((part, where))
                else:
                    raise TypeError(type(part).__name__)
        if not bulk:
            raise RuntimeError("no bulk equations")
        self._bcs = bcs
        self.saddle_point = next((b.saddle_point() for b in bulk if hasattr(b, "saddle_point")), None)
        fields: List[Tuple[str, str]] = []
        integrand = 0
        params: Dict[str, float] = {}
        for b in bulk:
            b._fields, b._residual = [], 0
            b.define_fields()
            fields += b._fields
        for b in bulk:
            b.define_residuals()
            integrand = integrand + b._residual
            params.update(b.parameter_values())
        dsyms = time_derivative_symbols(fields)
        self.is_transient = bool(self.transient) and any(sp.sympify(integrand).has(s_) for s_ in dsyms)
        if not self.is_transient and hasattr(integrand, "subs"):
            integrand = integrand.subs({s_: 0 for s_ in dsyms})
        # nodal value order: by space (C2TB, C2, C1TB, C1), then definition order
        # (codegen.cpp:2367-2380, 2795-2810)
        order = sorted(range(len(fields)), key=lambda i: (SPACE_ORDER[fields[i][1]], i))
        fields = [fields[i] for i in order]
        self.fields = fields
        self.field_index = {n: i for i, (n, _) in enumerate(fields)}
        # parameters referenced by the integrand, in a stable order
        used = sorted({s.name[2:] for s in (integrand.free_symbols if hasattr(integrand, "free_symbols") else [])
                       if s.name.startswith("P_")}, key=E.parameter_order_key)
        if E.TIME_PARAM in used:
            params[E.TIME_PARAM] = float(self.time)
        missing = [p for p in used if p not in params]
        if missing:
            raise RuntimeError(f"parameters without values: {missing}")
        if self.is_transient:
            # the BDF weights of the step, last (set by unsteady_newton_solve)
            used = used + list(BDF_PARAMS)
            params.update({k: 0.0 for k in BDF_PARAMS})
        self.param_names = used
        self.params = np.array([params[p] for p in used], dtype=np.float64)
        t1 = time.perf_counter()
        jp = self.jacobian_precision
        if jp in ("fp64", "f64", "double"):
            kprec = "f64"
        elif jp in ("fp32", "f32", "float"):
            kprec = "f32"
        elif jp == "df64":
            kprec = "df64"   # FP64 storage; contraction in double-float on the FP32 pipes
        else:
            raise ValueError(f"jacobian_precision must be fp64, fp32 or df64, not {jp!r}")
        rp = self.residual_precision
        if rp not in ("fp64", "f64", "double", "df64"):
            raise ValueError(f"residual_precision must be fp64 or df64, not {rp!r}")
        rprec = "df64" if rp == "df64" else "f64"
        prec = "f32" if kprec == "f32" else "f64"   # storage of the Jacobian values
        self._prec = prec
        self._kprec = kprec
        if self.geometry == "auto":
            self.affine = mesh_is_affine(mesh)
        else:
            self.affine = self.geometry == "affine"
        # the kernel depends on the weak form, element type, precision and
        # geometry kind only -- not on the mesh size: cache it per process
        gsep = bool(self.separable_source and self.affine and mesh_is_axis_aligned(mesh))
        key = (mesh.etype.name, tuple(fields), str(integrand), tuple(used), kprec, self.affine, gsep,
               self.is_transient, self.tensor_cores, self.min_blocks_per_sm, rprec, self.threads_per_block,
               self.elems_per_block, self.jacobian_reference)
        ks = _KERNEL_CACHE.get(key)
        if ks is None:
            pw = differentiate(fields, mesh.dim, integrand, used)
            ks = generate_kernel(mesh.etype, pw, kprec, epb=self.elems_per_block, affine=self.affine,
                                 jref=self.jacobian_reference, gauss_sep=gsep, tc=self.tensor_cores,
                                 min_blocks=self.min_blocks_per_sm, residual_precision=rprec,
                                 threads=self.threads_per_block)
            _KERNEL_CACHE[key] = ks
        if self.elems_per_block is None and int(self.replicas) == 1:
            # balance the waves: with W = ceil(E / (SMs x EPB)) waves of one
            # block per SM, EPB' = ceil(E / (SMs x W)) fills every wave as
            # evenly (small meshes: Poisson Q2 64^2, 4,096 elements, 32 per
            # block = 128 blocks on 152 SMs; 27 per block = one full wave,
            # 10% faster on GB300; large meshes keep their shape).  Not for
            # replicated problems: serving classes of many sizes then share
            # one kernel instead of compiling one per size.
            sms = _sm_count()
            lo_, hi_ = self._element_slice()
            n_el = max(1, hi_ - lo_)
            waves = -(-n_el // (sms * ks.epb))
            epb = max(1, -(-n_el // (sms * waves)))
            if epb < ks.epb:
                key2 = key[:-2] + (epb, self.jacobian_reference)
                ks2 = _KERNEL_CACHE.get(key2)
                if ks2 is None:
                    ks2 = generate_kernel(mesh.etype, differentiate(fields, mesh.dim, integrand, used), kprec,
                                          epb=epb, affine=self.affine, jref=self.jacobian_reference,
                                          gauss_sep=gsep, tc=self.tensor_cores, min_blocks=self.min_blocks_per_sm,
                                          residual_precision=rprec, threads=self.threads_per_block)
                    _KERNEL_CACHE[key2] = ks2
                ks = ks2
        self.kernel: KernelSpec = ks
        self.timings.update(setup_mesh_s=t1 - t0, codegen_s=time.perf_counter() - t1)
        # nodal values, pins and equation numbers
        nval = len(fields)
        n = mesh.n_nodes
        present = np.zeros((n, nval), dtype=bool)
        for f, (_, sp_) in enumerate(fields):
            present[:, f] = True if sp_ == "C2" else mesh.is_vertex
        pinned = np.zeros((n, nval), dtype=bool)
        values = np.zeros((n, nval))
        self._timed_bcs = []     # (node mask, value index, callable, component, components) of f(x, ..., t=)
        for bc, where in bcs:
            if isinstance(bc, DirichletBC):
                if where is None:
                    raise RuntimeError("DirichletBC needs a boundary: DirichletBC(...) @ 'left'")
                mask = np.zeros(n, dtype=bool)
                for w in where:
                    if w not in mesh.boundaries:
                        raise KeyError(f"unknown boundary {w!r}; have {list(mesh.boundaries)}")
                    mask |= mesh.boundaries[w]
                for name, val in bc.values.items():
                    names = E.REG.vector_fields.get(name, [name])
                    for k, fname in enumerate(names):
                        f = self.field_index[fname]
                        m = mask & present[:, f]
                        pinned[m, f] = True
                        if callable(val):
                            values[m, f] = _bc_value(val, mesh.x[m], k, len(names), self.time)
                            if _bc_takes_time(val):
                                self._timed_bcs.append((m, f, val, k, len(names)))
                        elif val is not None:
                            vv = val[k] if isinstance(val, (tuple, list)) else val
                            values[m, f] = vv
            elif isinstance(bc, PressureFixation):
                f = self.field_index[bc.name]
                node0 = int(mesh.conn[0, 0])
                pinned[node0, f] = True
                if bc.value is not None:
                    values[node0, f] = bc.value
        R = int(self.replicas)
        if R > 1:
            # a stack of independent copies of the mesh (batched serving):
            # replica r's nodes follow replica r-1's, so its equations are a
            # contiguous block and the Jacobian is block diagonal
            self.base_mesh = mesh
            self.base_n_nodes, self.base_n_elem = n, mesh.n_elem
            mesh = MeshData(mesh.etype, np.tile(mesh.x, (R, 1)),
                            (mesh.conn[None, :, :] + (np.arange(R) * n)[:, None, None]).reshape(-1, mesh.conn.shape[1]).astype(np.int32),
                            np.tile(mesh.is_vertex, R), {k: np.tile(v, R) for k, v in mesh.boundaries.items()})
            self.mesh = mesh
            present, pinned, values = np.tile(present, (R, 1)), np.tile(pinned, (R, 1)), np.tile(values, (R, 1))
            n = mesh.n_nodes
            self.replica_elems = self.base_n_elem
            self.params_stride = len(self.params)
            self.params = np.tile(self.params, R)
        # hanging values (refined meshes): constrained, no equation; each is the
        # weighted sum of its masters (oomph's HangInfo)
        self.hang_slots = np.zeros(0, dtype=np.int64)
        self.hang_ptr = np.zeros(1, dtype=np.int64)
        self.hang_master = np.zeros(0, dtype=np.int64)
        self.hang_weight = np.zeros(0)
        constrained = np.zeros((n, nval), dtype=bool)
        if getattr(mesh, "hang", None):
            if R > 1:
                raise NotImplementedError("replicas of meshes with hanging nodes")
            if any(sp_ not in ("C2", "C1") for _, sp_ in fields):
                raise NotImplementedError("hanging nodes with fields other than C2 and C1")
            if any(sp_ == "C1" for _, sp_ in fields) and getattr(mesh, "hang_c1", None) is None:
                raise NotImplementedError("this mesh has no hang infos of its C1 values")
            # each field hangs by the interpolation of its space: C2 values on
            # the coarse edge's three nodes, C1 values on its two vertices
            slots, ptr, mas, wts = [], [0], [], []
            for f, (_, sp_) in enumerate(fields):
                for h, ms in (mesh.hang if sp_ == "C2" else mesh.hang_c1).items():
                    if not present[h, f]:
                        continue
                    slots.append(h * nval + f)
                    for m, w in ms:
                        mas.append(m * nval + f)
                        wts.append(w)
                    ptr.append(len(mas))
                    constrained[h, f] = True
            order = np.argsort(slots, kind="stable")
            ptr_a = np.array(ptr, dtype=np.int64)
            lens = np.diff(ptr_a)
            mas_a, wts_a = np.array(mas, dtype=np.int64), np.array(wts)
            new_m, new_w, new_p = [], [], [0]
            for k in order:
                new_m.append(mas_a[ptr_a[k]:ptr_a[k + 1]])
                new_w.append(wts_a[ptr_a[k]:ptr_a[k + 1]])
                new_p.append(new_p[-1] + lens[k])
            self.hang_slots = np.array(slots, dtype=np.int64)[order]
            self.hang_ptr = np.array(new_p, dtype=np.int64)
            self.hang_master = np.concatenate(new_m).astype(np.int64)
            self.hang_weight = np.concatenate(new_w)
            flat_v = values.reshape(-1)
            for k, s_ in enumerate(self.hang_slots):
                a, b = self.hang_ptr[k], self.hang_ptr[k + 1]
                flat_v[s_] = np.dot(self.hang_weight[a:b], flat_v[self.hang_master[a:b]])
        free = present & ~pinned & ~constrained
        eqn = np.full((n, nval), -1, dtype=np.int32)
        flat = free.reshape(-1)
        self.n_dof = int(flat.sum())
        eqn.reshape(-1)[flat] = np.arange(self.n_dof, dtype=np.int32)
        self.eqn = eqn
        self.present = present
        self.pinned = pinned
        self._values0 = values
        return self.kernel

    def initialise(self) -> None:
        if self._initialised:
            return
        torch = _torch()
        self.lower()
        mesh, fields, prec = self.mesh, self.fields, self._prec
        n, nval, values, eqn = mesh.n_nodes, len(fields), self._values0, self.eqn
        t2 = time.perf_counter()
        ckey = self.kernel.name + ("+bounds" if self.bounds_check else "")
        self.code = _CODE_CACHE.get(ckey)
        if self.code is None:
            src = ("#define FE_BOUNDS_CHECK 1\n" if self.bounds_check else "") + self.kernel.source
            self.code = N.Code(src, self.kernel.name)
            _CODE_CACHE[ckey] = self.code
        t3 = time.perf_counter()
        # device problem
        L = N.load()
        desc, self._domains, self._keep = self._descriptors(with_code=True)
        h = ctypes.c_void_p()
        N.check(L.fe_problem_create(ctypes.byref(desc), ctypes.byref(h)))
        self._h = h
        if self.kernel.tc_pairs:
            pa, pb, phi = self.tensor_contraction_tables()
            N.check(L.fe_problem_set_tensor_contraction(h, 0, self.kernel.layout.n, mesh.etype.nq, mesh.dim + 1,
                                                        phi.ctypes.data, len(pa), pa.ctypes.data, pb.ctypes.data))
        N.check(L.fe_problem_set_values(h, values.ctypes.data))
        nd = ctypes.c_int64()
        nnz = ctypes.c_int64()
        N.check(L.fe_problem_sizes(h, ctypes.byref(nd), ctypes.byref(nnz)))
        self.nnz = nnz.value
        self._jdtype = torch.float64 if prec == "f64" else torch.float32
        dev = torch.device("cuda")
        self.x_dev = torch.zeros(self.n_dof, dtype=torch.float64, device=dev)
        self.R_dev = torch.zeros(max(self.n_dof, 1), dtype=torch.float64, device=dev)
        self.J_dev = torch.zeros(max(self.nnz, 1), dtype=self._jdtype, device=dev)
        self._krylov = None   # device linear solver state, bound to J_dev
        self._fieldsplit = None
        self.x_dev.copy_(torch.from_numpy(self._dofs_from_values(values)))
        self._state_generation += 1           # a new device problem
        t4 = time.perf_counter()
        self.timings.update(jit_s=t3 - t2, device_setup_s=t4 - t3)
        self._initialised = True

    def tensor_contraction_tables(self):
        """The tables of the tensor-core contraction (codegen.tc_tables)."""
        from .codegen import tc_tables
        return tc_tables(self.kernel)

    def _element_slice(self) -> Tuple[int, int]:
        """The elements this problem assembles: all, or element_range."""
        if self.element_range is None:
            return 0, self.mesh.n_elem
        lo, hi = (int(v) for v in self.element_range)
        if not 0 <= lo <= hi <= self.mesh.n_elem:
            raise ValueError(f"element_range {self.element_range} outside [0, {self.mesh.n_elem}]")
        if int(self.replicas) != 1:
            raise NotImplementedError("element ranges of replicated problems")
        return lo, hi

    def _descriptors(self, with_code: bool):
        mesh = self.mesh
        lay = self.kernel.layout
        lo, hi = self._element_slice()
        keep = dict(
            conn=np.ascontiguousarray(mesh.conn[lo:hi], dtype=np.int32),
            lnode=np.ascontiguousarray(lay.node, dtype=np.int32),
            lval=np.ascontiguousarray(lay.val, dtype=np.int32),
            tables=np.ascontiguousarray(self.kernel.tables, dtype=np.float64),
            x=np.ascontiguousarray(mesh.x, dtype=np.float64),
            eqn=np.ascontiguousarray(self.eqn),
            params=np.ascontiguousarray(self.params if len(self.params) else np.zeros(1)),
            hs=np.ascontiguousarray(self.hang_slots, dtype=np.int64),
            hp=np.ascontiguousarray(self.hang_ptr, dtype=np.int64),
            hm=np.ascontiguousarray(self.hang_master if self.hang_master.size else np.zeros(1, np.int64)),
            hw=np.ascontiguousarray(self.hang_weight if self.hang_weight.size else np.zeros(1)),
        )
        k = keep
        dd = N.DomainDesc(self.code.handle if with_code else None, mesh.etype.nnode, lay.n, hi - lo,
                          k["conn"].ctypes.data, k["lnode"].ctypes.data, k["lval"].ctypes.data,
                          k["tables"].ctypes.data, k["tables"].size, self.kernel.epb, self.kernel.threads,
                          self.kernel.smem_bytes, getattr(self, "replica_elems", 0))
        doms = (N.DomainDesc * 1)(dd)
        desc = N.ProblemDesc(mesh.dim, mesh.n_nodes, len(self.fields), k["x"].ctypes.data, k["eqn"].ctypes.data,
                             self.n_dof, 1, doms, len(self.params), k["params"].ctypes.data,
                             N.FE_JAC_F64 if self._prec == "f64" else N.FE_JAC_F32,
                             getattr(self, "params_stride", 0), 2 if self.is_transient else 0, None, 0,
                             int(self.hang_slots.size), k["hs"].ctypes.data, k["hp"].ctypes.data,
                             k["hm"].ctypes.data, k["hw"].ctypes.data)
        return desc, doms, keep

    def host_pattern(self) -> Tuple[np.ndarray, np.ndarray]:
        """The CSR pattern built on the host only (fe_pattern_host; no GPU)."""
        self.lower()
        desc, doms, keep = self._descriptors(with_code=False)
        L = N.load()
        nnz = ctypes.c_int64()
        N.check(L.fe_pattern_host(ctypes.byref(desc), ctypes.byref(nnz), None, None))
        rp = np.zeros(self.n_dof + 1, dtype=np.int32)
        ci = np.zeros(max(nnz.value, 1), dtype=np.int32)
        N.check(L.fe_pattern_host(ctypes.byref(desc), None, rp.ctypes.data, ci.ctypes.data))
        return rp, ci[:nnz.value]

    def _dofs_from_values(self, values: np.ndarray) -> np.ndarray:
        x = np.zeros(self.n_dof)
        m = self.eqn >= 0
        x[self.eqn[m]] = values[m]
        return x

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.load().fe_problem_destroy(self._h)
                self._h = None
        except Exception:
            pass

    # -- state ---------------------------------------------------------
    def get_dofs(self) -> np.ndarray:
        return self.x_dev.cpu().numpy()

    def set_dofs(self, x: np.ndarray) -> None:
        torch = _torch()
        self.x_dev.copy_(torch.as_tensor(np.asarray(x, dtype=np.float64)))
        self._state_generation += 1

    def set_values(self, values: np.ndarray) -> None:
        """Set every nodal value [n_nodes, nval] (pinned ones included) and
        the dof vector that goes with it."""
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(self.mesh.n_nodes, len(self.fields))
        N.check(N.load().fe_problem_set_values(self._h, v.ctypes.data))
        self.set_dofs(self._dofs_from_values(v))

    def set_history_values(self, level: int, values: np.ndarray) -> None:
        """Nodal values [n_nodes, nval] of a previous time level of a
        transient problem (0: u_{n-1}, 1: u_{n-2}); unsteady_newton_solve
        fills them itself."""
        if not self.is_transient:
            raise RuntimeError("a steady problem keeps no time levels")
        v = np.array(values, dtype=np.float64).reshape(self.mesh.n_nodes, len(self.fields))
        # hanging values follow their masters at every time level (the
        # device constrains the current values only)
        flat = v.reshape(-1)
        for k, s_ in enumerate(self.hang_slots):
            a, b = self.hang_ptr[k], self.hang_ptr[k + 1]
            flat[s_] = np.dot(self.hang_weight[a:b], flat[self.hang_master[a:b]])
        N.check(N.load().fe_problem_set_history(self._h, int(level), v.ctypes.data))
        self._state_generation += 1

    def get_history_values(self, level: int) -> np.ndarray:
        """Nodal values [n_nodes, nval] of a previous time level (0: u_{n-1},
        1: u_{n-2}) as the device holds them."""
        if not self.is_transient:
            raise RuntimeError("a steady problem keeps no time levels")
        v = np.zeros((self.mesh.n_nodes, len(self.fields)))
        N.check(N.load().fe_problem_get_history(self._h, int(level), v.ctypes.data))
        return v

    def get_current_dofs(self):
        """pyoomph's accessor: (dof vector, pinned values)."""
        return self.get_dofs(), self._values0[self.pinned].copy() if hasattr(self, "pinned") else None

    def set_current_dofs(self, dofs) -> None:
        self.set_dofs(np.asarray(dofs, dtype=np.float64))

    def set_custom_assembler(self, assembler) -> None:
        """pyoomph's Problem.set_custom_assembler (problem.py:1711): the
        assembler then provides residuals and Jacobians to solve()."""
        if getattr(self, "_custom_assembler", None) is not None:
            self._custom_assembler.finalize()
        self._custom_assembler = assembler
        if assembler is not None:
            assembler._set_problem(self)
            assembler.initialize()

    def get_values(self) -> np.ndarray:
        """Nodal values [n_nodes, nval] (after the last assembly's dof scatter)."""
        v = np.zeros((self.mesh.n_nodes, len(self.fields)))
        N.check(N.load().fe_problem_get_values(self._h, v.ctypes.data))
        return v

    def set_parameters(self, replica: Optional[int] = None, **kw) -> None:
        """Set global parameters by name (of one replica, or of all)."""
        stride = len(self.param_names)
        reps = range(int(self.replicas)) if replica is None else [replica]
        for k, v in kw.items():
            j = self.param_names.index(k)
            for r in reps:
                self.params[r * stride + j] = float(v)
        self._keep["params"][:len(self.params)] = self.params
        N.check(N.load().fe_problem_set_params(self._h, self._keep["params"].ctypes.data))

    def set_parameter_vector(self, values: np.ndarray, replica: Optional[int] = None) -> None:
        """Set every global parameter (array in param_names order)."""
        stride = len(self.param_names)
        v = np.asarray(values, dtype=np.float64).reshape(stride)
        reps = range(int(self.replicas)) if replica is None else [replica]
        for r in reps:
            self.params[r * stride:(r + 1) * stride] = v
        self._keep["params"][:len(self.params)] = self.params
        N.check(N.load().fe_problem_set_params(self._h, self._keep["params"].ctypes.data))

    def pattern(self) -> Tuple[np.ndarray, np.ndarray]:
        rp = np.zeros(self.n_dof + 1, dtype=np.int32)
        ci = np.zeros(max(self.nnz, 1), dtype=np.int32)
        N.check(N.load().fe_problem_pattern(self._h, rp.ctypes.data, ci.ctypes.data))
        return rp, ci[:self.nnz]

    # -- assembly (device) ----------------------------------------------
    def assemble_device(self, with_jacobian: bool = True, stream=None, zero_threshold: Optional[float] = None) -> None:
        """R (and CSR J values) into self.R_dev / self.J_dev from self.x_dev.
        zero_threshold: J in oomph's zero-filtered pattern instead (its
        rowptr/colidx from fe_problem_filtered_pattern)."""
        torch = _torch()
        flags = N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_VALUES_FROM_DOFS
        if with_jacobian:
            flags |= N.FE_ASSEMBLE_JACOBIAN
        if zero_threshold is not None and with_jacobian:
            N.check(N.load().fe_problem_set_zero_threshold(self._h, float(zero_threshold)))
            flags |= N.FE_ASSEMBLE_ZERO_FILTER
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(),
                                     self.J_dev.data_ptr(), flags, ctypes.c_void_p(st)))

    def assemble_host(self, x_host, R_host, J_host, with_jacobian: bool = True, chunks: int = 8, stream=None) -> None:
        """Assemble from a host dof vector into host R / CSR values
        (fe_assemble_pipelined: the copies of finished rows overlap the
        element chunks still computing).  Pass pinned tensors/arrays;
        asynchronous on the stream."""
        import torch
        flags = N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_VALUES_FROM_DOFS
        if with_jacobian:
            flags |= N.FE_ASSEMBLE_JACOBIAN
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream

        def ptr(a):
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        N.check(N.load().fe_assemble_pipelined(self._h, ptr(x_host), ptr(R_host), ptr(J_host), flags, int(chunks),
                                               ctypes.c_void_p(st)))

    def capture_assembly(self, with_jacobian: bool = True) -> None:
        """Record the assembly from x_dev into R_dev / J_dev as a CUDA graph
        (fe_problem_graph_capture); assemble_graph replays it."""
        flags = N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_VALUES_FROM_DOFS
        if with_jacobian:
            flags |= N.FE_ASSEMBLE_JACOBIAN
        N.check(N.load().fe_problem_graph_capture(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(),
                                                  self.J_dev.data_ptr(), flags))

    def assemble_graph(self, stream=None) -> None:
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_problem_graph_launch(self._h, ctypes.c_void_p(st)))

    def launch_count(self, with_jacobian: bool = True, zero_filter: bool = False) -> int:
        """Kernel launches of one assembly from the dof vector (R, and J when
        asked; ``zero_filter``: J in the reference's value-dependent pattern)."""
        flags = N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_VALUES_FROM_DOFS
        if with_jacobian:
            flags |= N.FE_ASSEMBLE_JACOBIAN
        if zero_filter:
            flags |= N.FE_ASSEMBLE_ZERO_FILTER
        return N.load().fe_problem_launch_count(self._h, flags)

    def set_stage_timing(self, enable: bool) -> None:
        N.check(N.load().fe_problem_set_timing(self._h, int(enable)))

    def set_pipeline_streams(self, n: int) -> None:
        """Element streams of ``assemble_host``: 1, 2 (consecutive chunks on
        alternating streams, which may run concurrently) or 0 (automatic:
        one).  Same bits either way."""
        N.check(N.load().fe_problem_set_pipeline_streams(self._h, int(n)))

    def pipeline_times(self) -> np.ndarray:
        """Timeline of the last ``assemble_host`` call made with stage timing
        on: per chunk, ms from its start to the end of the chunk's element
        kernel, of its gathers and of the copies of the rows it completes
        (array [chunks, 3]; empty when no timed call was made)."""
        buf = np.zeros(3 * 1024, dtype=np.float32)
        n = N.load().fe_problem_pipeline_times(self._h, buf.ctypes.data, buf.size)
        N.check(min(n, 0))
        return buf[:3 * n].reshape(n, 3).astype(np.float64)

    def stage_times(self):
        """Summed ms per stage (dof scatter, element kernels, residual gather,
        Jacobian gather, tensor-core contraction) since the last call, and
        the number of assemblies."""
        ms = np.zeros(5)
        calls = ctypes.c_int64()
        N.check(N.load().fe_problem_stage_times(self._h, ms.ctypes.data, ctypes.byref(calls)))
        return ms, calls.value

    def element_buffers(self):
        """(R_e [E, nloc], J_e [E, nloc, nloc]) of the last assembly."""
        lo, hi = self._element_slice()
        E, n = hi - lo, self.kernel.layout.n
        R = np.zeros((E, n))
        J = np.zeros((E, n, n), dtype=np.float64 if self._prec == "f64" else np.float32)
        N.check(N.load().fe_problem_element_buffers(self._h, 0, R.ctypes.data, J.ctypes.data))
        return R, J

    def check(self) -> None:
        N.check(N.load().fe_problem_check(self._h))

    # -- the reference-facing calls --------------------------------------
    def get_residuals(self) -> np.ndarray:
        """Problem::get_residuals (problem.cc:3810): R at the current dofs."""
        self.initialise()
        self.assemble_device(with_jacobian=False)
        self.check()
        return self.R_dev[:self.n_dof].cpu().numpy()

    def get_jacobian(self):
        """Problem::get_jacobian (problem.cc:4038): (R, scipy CSR J).  With
        numerical_zero_for_sparse_assembly set (oomph's default is 0.0), J
        has the reference's value-dependent pattern: element entries with
        |J_e(i,j)| <= the threshold are left out (problem.cc:5520-5560);
        otherwise (None) the structural pattern of every coupling."""
        import scipy.sparse as sp
        self.initialise()
        thr = self.numerical_zero_for_sparse_assembly
        if thr is None:
            self.assemble_device(with_jacobian=True)
            self.check()
            R = self.R_dev[:self.n_dof].cpu().numpy()
            rp, ci = self.pattern()
            vals = self.J_dev[:self.nnz].cpu().numpy()
            return R, sp.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))
        R, rp, ci, vals = self.assemble_filtered(float(thr))
        return R, sp.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))

    def assemble_filtered(self, threshold: float = 0.0):
        """R and J in oomph's zero-filtered pattern (fe_assemble with
        FE_ASSEMBLE_ZERO_FILTER): (R, rowptr, colidx, values) on the host."""
        torch = _torch()
        self.initialise()
        L = N.load()
        N.check(L.fe_problem_set_zero_threshold(self._h, float(threshold)))
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        flags = (N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_JACOBIAN | N.FE_ASSEMBLE_VALUES_FROM_DOFS
                 | N.FE_ASSEMBLE_ZERO_FILTER)
        N.check(L.fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(), self.J_dev.data_ptr(), flags,
                              st))
        self.check()
        nnz = ctypes.c_int64()
        rp = np.zeros(self.n_dof + 1, dtype=np.int32)
        N.check(L.fe_problem_filtered_pattern(self._h, ctypes.byref(nnz), rp.ctypes.data, None, st))
        ci = np.zeros(max(nnz.value, 1), dtype=np.int32)
        N.check(L.fe_problem_filtered_pattern(self._h, None, None, ci.ctypes.data, st))
        R = self.R_dev[:self.n_dof].cpu().numpy()
        vals = self.J_dev[:nnz.value].cpu().numpy()
        return R, rp, ci[:nnz.value], vals

    def get_parameter_derivative(self, name: str) -> np.ndarray:
        """dR/dp of one global parameter at the current dofs
        (dResidual{i}dParameter_{k} of pyoomph's generated code,
        codegen.cpp:4743-4760; used by continuation and bifurcation
        tracking).  With replicas, each replica's residual by its own copy
        of the parameter."""
        torch = _torch()
        self.initialise()
        if name not in self.param_names:
            raise KeyError(f"unknown parameter {name!r}; have {self.param_names}")
        N.check(N.load().fe_problem_set_dparam(self._h, self.param_names.index(name)))
        st = torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(), self.J_dev.data_ptr(),
                                     N.FE_ASSEMBLE_DPARAM | N.FE_ASSEMBLE_VALUES_FROM_DOFS, ctypes.c_void_p(st)))
        self.check()
        return self.R_dev[:self.n_dof].cpu().numpy()

    def get_hessian_vector_product(self, y: np.ndarray):
        """H(y)_ij = sum_k d2R_i/(du_j du_k) y_k at the current dofs, in the
        Jacobian's CSR pattern (pyoomph's HessianVectorProduct, used by
        bifurcation tracking).  Leaves J_dev holding H(y)."""
        import scipy.sparse as sp
        torch = _torch()
        self.initialise()
        st = torch.cuda.current_stream().cuda_stream
        yd = torch.as_tensor(np.asarray(y, dtype=np.float64), device=self.x_dev.device)
        N.check(N.load().fe_problem_set_direction(self._h, yd.data_ptr(), ctypes.c_void_p(st)))
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(), self.J_dev.data_ptr(),
                                     N.FE_ASSEMBLE_HVP | N.FE_ASSEMBLE_VALUES_FROM_DOFS, ctypes.c_void_p(st)))
        self.check()
        rp, ci = self.pattern()
        vals = self.J_dev[:self.nnz].cpu().numpy().astype(np.float64)
        return sp.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))

    def assemble_jacobian(self):
        """pyoomph's Problem.assemble_jacobian (problem.py:711)."""
        return self.get_jacobian()

    def residual_max(self) -> float:
        out = ctypes.c_double()
        torch = _torch()
        N.check(N.load().fe_residual_max(self._h, self.R_dev.data_ptr(), self.n_dof, ctypes.byref(out),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return out.value

    # -- Newton ----------------------------------------------------------
    def _solve_linear(self, R: np.ndarray) -> np.ndarray:
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        rp, ci = self._pattern_cache
        vals = self.J_dev[:self.nnz].cpu().numpy().astype(np.float64)
        A = sp.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))
        if callable(self.linear_solver):
            return self.linear_solver(A, R)
        return spla.splu(A.tocsc()).solve(R)

    def _fieldsplit_solver(self):
        """The device saddle-point solver of this problem (fieldsplit.py),
        built at the first solve: the constrained field and the viscosity
        scaling its Schur complement come from the equations
        (StokesEquations.saddle_point)."""
        if self.saddle_point is None:
            raise RuntimeError("linear_solver='fieldsplit' needs equations with a constrained field "
                               "(Stokes / Navier-Stokes)")
        field, scale_param = self.saddle_point
        scale = float(self.params[self.param_names.index(scale_param)])
        if getattr(self, "_fieldsplit", None) is None:
            from .fieldsplit import SaddlePointSolver
            self._fieldsplit = SaddlePointSolver(self, field, scale)
        # the hierarchy belongs to the parameters it was built for: new
        # parameters (another viscosity, another request) rebuild it at the
        # next solve
        self._fieldsplit.renew_if_changed(tuple(np.asarray(self.params, dtype=float)), scale)
        return self._fieldsplit

    def solve_linear_device(self, b: np.ndarray) -> np.ndarray:
        """x with J x = b, J the Jacobian of the last assembly (resident on
        the device), by the native batched BiCGStab (linsolve.py) to
        linear_solver_tolerance; raises LinearSolverError where the solver
        refuses the matrix or does not converge."""
        torch = _torch()
        from .linsolve import BatchedBiCGStab, DeviceCSR
        if getattr(self, "_krylov", None) is None:
            self._krylov = BatchedBiCGStab(DeviceCSR.of_problem(self), blocks=self.replicas)
        bd = torch.as_tensor(np.ascontiguousarray(b, dtype=np.float64), device=self.x_dev.device)
        x, _ = self._krylov.solve(bd, tol=self.linear_solver_tolerance, atol=self.linear_solver_atol)
        return x.view(-1)[:self.n_dof].cpu().numpy()

    # -- time stepping ---------------------------------------------------
    def unsteady_newton_solve(self, dt: float) -> List[float]:
        """One implicit time step of size dt (pyoomph's
        Problem.unsteady_newton_solve): the current values become the
        previous time level (and the previous one the one before), the BDF
        weights of the step are set -- BDF1 on the first step, BDF2 with
        variable steps after it (the degraded start of pyoomph's BDF2,
        timestepper.hpp:46-108) -- and Newton solves for the new level.
        The first call on a steady problem switches it to its transient form
        (a new kernel; the dofs are kept).  Returns the Newton residual
        history."""
        from .ale import bdf_weights
        if dt <= 0.0:
            raise ValueError("dt must be positive")
        if not self.transient:
            self.make_transient()
        self.initialise()
        if not self.is_transient:
            raise RuntimeError("the weak form has no time derivative (partial_t)")
        self.assemble_device(with_jacobian=False)      # nodal values = the current dofs
        N.check(N.load().fe_problem_shift_history(self._h))
        if self.steps_done == 0:
            N.check(N.load().fe_problem_shift_history(self._h))   # both levels = the initial state
        w = bdf_weights(1 if self.steps_done == 0 else 2, dt, self.dt_prev)
        self.set_parameters(**dict(zip(BDF_PARAMS, w)))
        self.set_time(self.time + dt)            # var("time") and timed boundary values at t_{n+1}
        hist = self._newton()
        self.steps_done += 1
        self.dt_prev = dt
        return hist

    def run(self, endtime: float, timestep: Optional[float] = None, *, outstep=None, numouts: Optional[int] = None,
            out_initially: Optional[bool] = None, newton_solver_tolerance: Optional[float] = None,
            max_newton_iterations: Optional[int] = None, starttime: Optional[float] = None,
            temporal_error=None, spatial_adapt: int = 0, output: Optional[Callable] = None) -> float:
        """Integrate to `endtime` with unsteady_newton_solve (pyoomph's
        Problem.run, problem.py:4873, without spatial adaptivity; with
        temporal_error, adaptive steps, adaptive_unsteady_newton_solve):
        steps of `timestep` (default: the output interval),
        shortened to land on every output time and on `endtime`; `output`
        (a callable taking the problem) at the start (out_initially) and at
        every multiple of `outstep` (or numouts evenly spaced outputs;
        outstep=True: after every step).  Returns the final time."""
        if spatial_adapt:
            raise NotImplementedError("spatial adaptivity is not built")
        if outstep is not None and outstep is not False and numouts is not None:
            raise ValueError("outstep and numouts cannot both be given")
        if starttime is not None:
            self.set_time(float(starttime))
        t0 = float(self.time)
        endtime = float(endtime)
        if numouts is not None:
            outstep = (endtime - t0) / max(int(numouts), 1)
        every = outstep is True
        if outstep is None or outstep is False or every:
            ostep = None
        else:
            ostep = float(outstep)
        if timestep is None:
            if ostep is None:
                raise ValueError("give a timestep (or an outstep to derive it from)")
            timestep = ostep
        dt = float(timestep)
        if dt <= 0.0:
            raise ValueError("timestep must be positive")
        if out_initially is None:
            out_initially = outstep is not False and outstep is not None or numouts is not None
        keep = (self.newton_solver_tolerance, self.max_newton_iterations)
        if newton_solver_tolerance is not None:
            self.newton_solver_tolerance = float(newton_solver_tolerance)
        if max_newton_iterations is not None:
            self.max_newton_iterations = int(max_newton_iterations)
        if temporal_error is not None and float(temporal_error) <= 0.0:
            temporal_error = None            # pyoomph: no positive tolerance = fixed steps
        eps = 1e-12 * max(1.0, abs(endtime))
        try:
            if output is not None and out_initially:
                output(self)
            k_out = 1
            while self.time < endtime - eps:
                step = min(dt, endtime - self.time)
                if ostep is not None:
                    t_out = t0 + k_out * ostep
                    if t_out < self.time + step - eps:
                        step = t_out - self.time
                if temporal_error is not None:
                    dt = self.adaptive_unsteady_newton_solve(step, float(temporal_error))
                else:
                    self.unsteady_newton_solve(step)
                if output is not None and (every or (ostep is not None and
                                                     abs(self.time - (t0 + k_out * ostep)) <= eps)):
                    output(self)
                if ostep is not None and self.time >= t0 + k_out * ostep - eps:
                    k_out += 1
        finally:
            self.newton_solver_tolerance, self.max_newton_iterations = keep
        return float(self.time)

    def set_time(self, t: float) -> None:
        """Set the current time: the parameter var("time") reads and the
        Dirichlet values given as functions with a keyword ``t``
        (re-evaluated at the pinned nodes and uploaded; the free values keep
        the current dofs)."""
        self.time = float(t)
        if not self._initialised:
            return
        if E.TIME_PARAM in self.param_names:
            self.set_parameters(**{E.TIME_PARAM: self.time})
        if getattr(self, "_timed_bcs", None):
            R = int(self.replicas)
            n0 = self.mesh.n_nodes // R
            vals = self._values0
            for m, f, fn, k, ncomp in self._timed_bcs:
                v = _bc_value(fn, self.mesh.x[:n0][m[:n0]], k, ncomp, self.time)
                vals[:n0][m[:n0], f] = v
                for r in range(1, R):
                    vals[r * n0:(r + 1) * n0][m[:n0], f] = v
            N.check(N.load().fe_problem_set_values(self._h, np.ascontiguousarray(vals).ctypes.data))

    def adaptive_unsteady_newton_solve(self, dt_desired: float, epsilon: float) -> float:
        """One accepted time step with temporal error control (oomph-lib's
        Problem::adaptive_unsteady_newton_solve; the algorithm is in
        timestepping.py): a step whose error exceeds epsilon is undone (the
        time levels restored from host copies) and redone shorter.  Returns
        the suggested next step; the step taken is self.dt_prev.  Adaptive
        stepping starts at the first step of a problem."""
        from .timestepping import AdaptiveState, adaptive_step
        if not self.transient:
            self.make_transient()
        self.initialise()
        ad = getattr(self, "_adaptive", None)
        key = (self.steps_done, self.time, self._state_generation)
        if ad is not None and ad[2] != key:
            # the state changed since the last adaptive step (a fixed step, new
            # dofs/values/history, a rebuild): the stepper's host copies are
            # stale, so it restarts from the current point (no error estimate
            # for the next step, as for the first one)
            ad = None
        if ad is None:
            self.assemble_device(with_jacobian=False)
            v0 = self.get_values()
            if self.steps_done:
                prev = [self.get_history_values(0), self.get_history_values(1)]
            else:
                prev = [v0, v0]
            ad = (AdaptiveState(self.get_dofs(), scales=self._temporal_error_scales()),
                  _ProblemAdaptiveOps(self, prev), None)
        st, ops, _ = ad
        _, nxt = adaptive_step(ops, st, float(dt_desired), float(epsilon), newton_error=NewtonSolverError)
        ops.accepted()
        self._adaptive = (st, ops, (self.steps_done, self.time, self._state_generation))
        return nxt

    def set_temporal_error_factor(self, field: str, factor: float) -> None:
        """The scale of a field in the temporal error norm of adaptive time
        stepping (pyoomph's Equations.set_temporal_error_factor).  pyoomph
        counts only fields given a factor (default 0); here, while no field
        has one, every field counts with scale 1."""
        self.temporal_error_factors[field] = float(factor)

    def _temporal_error_scales(self) -> Optional[np.ndarray]:
        if not self.temporal_error_factors:
            return None
        names = [n for n, _ in self.fields]
        unknown = set(self.temporal_error_factors) - set(names)
        if unknown:
            raise KeyError(f"temporal error factors of unknown fields {sorted(unknown)}; have {names}")
        eqn = np.asarray(self.eqn).reshape(self.mesh.n_nodes, len(self.fields))
        s = np.zeros(self.n_dof)
        for j, f in enumerate(names):
            col = eqn[:, j]
            s[col[col >= 0]] = self.temporal_error_factors.get(f, 0.0)
        return s

    def make_transient(self) -> None:
        """Keep the partial_t terms from now on.  An initialised problem is
        rebuilt with its transient kernel; its dofs carry over."""
        if self.transient:
            return
        dofs = self.get_dofs() if self._initialised else None
        self.transient = True
        if self._initialised:
            if getattr(self, "_h", None):
                N.load().fe_problem_destroy(self._h)
                self._h = None
            self._initialised = False
        self.kernel = None
        self.initialise()
        if dofs is not None:
            self.set_dofs(dofs)

    def get_mass_matrix(self):
        """The mass matrix M = dR/d(du/dt) on the Jacobian's CSR pattern (flag
        2 of pyoomph's generated ResidualAndJacobian; the eigenproblem
        J v = lambda M v of Problem.get_eigenvalues).  A steady problem is
        switched to its transient form first."""
        import scipy.sparse as sps
        torch = _torch()
        if not self.transient:
            self.make_transient()
        self.initialise()
        M = torch.zeros_like(self.J_dev)
        st = torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(), M.data_ptr(),
                                     N.FE_ASSEMBLE_MASS | N.FE_ASSEMBLE_VALUES_FROM_DOFS, ctypes.c_void_p(st)))
        self.check()
        rp, ci = self.pattern()
        return sps.csr_matrix((M[:self.nnz].cpu().numpy().astype(np.float64), ci, rp),
                              shape=(self.n_dof, self.n_dof))

    def arclength_continuation(self, parameter: str, step: float, *, max_ds: Optional[float] = None,
                               max_newton_iterations: Optional[int] = None,
                               newton_solver_tolerance: Optional[float] = None,
                               min_ds: Optional[float] = None) -> float:
        """One pseudo-arclength step of (signed) length `step` in a global
        parameter from the current solution (pyoomph's
        Problem.arclength_continuation, problem.py:3508; the algorithm is in
        continuation.py).  R and J come from the device assembly, dR/dp from
        the kernels' parameter derivative.  Consecutive calls with the same
        parameter continue along the path (the tangent is kept); returns the
        suggested next step.  reset_arc_length_parameters() forgets the
        path."""
        from .continuation import arclength_step
        self.initialise()
        if int(self.replicas) != 1:
            raise NotImplementedError("continuation of replicated problems")
        if parameter not in self.param_names:
            raise KeyError(f"unknown parameter {parameter!r}; have {self.param_names}")
        st = self._arclength if getattr(self, "_arclength_param", None) == parameter else None
        self._arclength_prev = st
        with self._steady():            # continuation of steady states
            new, nds = arclength_step(
                _ProblemContinuationOps(self, parameter), st, float(step),
                tol=self.newton_solver_tolerance if newton_solver_tolerance is None else newton_solver_tolerance,
                max_newton_iterations=self.max_newton_iterations if max_newton_iterations is None
                else max_newton_iterations,
                min_ds=1e-8 if min_ds is None else min_ds, max_ds=max_ds)
        self._arclength, self._arclength_param = new, parameter
        self.assemble_device(with_jacobian=False)      # nodal values at the new point
        return nds

    def reset_arc_length_parameters(self) -> None:
        self._arclength = self._arclength_param = self._arclength_prev = None

    def locate_fold(self, rel_tol: float = 1e-6) -> float:
        """After an arclength step that passed a fold (the parameter turned):
        bisect that step down to the turning point, leave the problem there
        and return the parameter's value (continuation.locate_fold)."""
        from .continuation import locate_fold
        prev, last = getattr(self, "_arclength_prev", None), getattr(self, "_arclength", None)
        if prev is None or last is None or np.sign(prev.dp) == np.sign(last.dp):
            raise RuntimeError("the last arclength step did not pass a fold")
        with self._steady():
            st = locate_fold(_ProblemContinuationOps(self, self._arclength_param), prev, last.ds, rel_tol=rel_tol,
                             tol=self.newton_solver_tolerance, max_newton_iterations=self.max_newton_iterations)
        self._arclength = st
        self.assemble_device(with_jacobian=False)
        return st.p0

    def solve_eigenproblem(self, n: int, shift=0.0, sort: bool = True, which: str = "LM", v0=None,
                           target=None):
        """Eigenvalues lambda and eigenvectors v of (-J) v = lambda M v at the
        current dofs, J the steady Jacobian and M the mass matrix, both
        assembled on the device (pyoomph's Problem.solve_eigenproblem with
        its scipy eigensolver: solvers/generic.py:377-383 negates J,
        solvers/scipy.py:166-190 solves shift-inverted).  Returns
        (eigenvalues [n], eigenvectors [n, n_dof]), also kept for
        get_last_eigenvalues / get_last_eigenvectors."""
        M = self.get_mass_matrix()
        with self._steady():            # the steady Jacobian
            _, J = self.get_jacobian()
        ev, vec = solve_generalized_eigenproblem(J, M, n, shift=shift, sort=sort, which=which, v0=v0,
                                                 target=target)
        self._last_eigen = (ev, vec)
        return ev, vec

    def get_last_eigenvalues(self) -> np.ndarray:
        return self._last_eigen[0] if getattr(self, "_last_eigen", None) else np.zeros(0, dtype=complex)

    def get_last_eigenvectors(self) -> np.ndarray:
        return self._last_eigen[1] if getattr(self, "_last_eigen", None) else np.zeros((0, 0), dtype=complex)

    def solve(self, **_ignored) -> List[float]:
        """Stationary Newton solve; returns the residual max-norm history.
        A transient problem is solved for its steady state (BDF weights 0
        during the solve: pyoomph's ResidualAndJacobianSteady); its time
        stepping state is kept."""
        self.initialise()
        with self._steady():
            return self._newton()

    @contextlib.contextmanager
    def _steady(self):
        """The steady form for the block (a transient problem's BDF weights
        0, restored after)."""
        if not self.is_transient:
            yield
            return
        idx = [self.param_names.index(k) for k in BDF_PARAMS]
        keep = self.params[idx].copy()
        self.set_parameters(**{k: 0.0 for k in BDF_PARAMS})
        try:
            yield
        finally:
            self.set_parameters(**dict(zip(BDF_PARAMS, keep)))

    def _newton(self) -> List[float]:
        """Newton on R(u) = 0 with the parameters as set (a time step when
        the BDF weights are)."""
        torch = _torch()
        self._pattern_cache = self.pattern()
        hist = []
        t_asm = 0.0
        t_lin = 0.0
        t0 = time.perf_counter()
        self.assemble_device(with_jacobian=False)
        hist.append(self.residual_max())
        it = 0
        while hist[-1] >= self.newton_solver_tolerance:
            if it >= self.max_newton_iterations:
                raise NewtonSolverError(f"max Newton iterations ({self.max_newton_iterations}) reached; "
                                        f"residuals {hist}")
            if hist[-1] > self.max_residuals:
                raise NewtonSolverError(f"max residuals ({self.max_residuals}) exceeded: {hist}")
            ta = time.perf_counter()
            device_solve = self.linear_solver in ("bicgstab", "fieldsplit")
            with nvtx_range("fe_assemble R+J"):
                self.assemble_device(with_jacobian=True)
                self.check()
                R = None if device_solve else self.R_dev[:self.n_dof].cpu().numpy()
            tb = time.perf_counter()
            with nvtx_range("linear solve"):
                if self.linear_solver == "fieldsplit":
                    # an inexact Newton step (the forcing term), and no more
                    # accuracy than the Newton criterion can see (a target
                    # below the attainable accuracy of a small late-step
                    # residual would stall)
                    from .fieldsplit import newton_forcing
                    dxd, its = self._fieldsplit_solver().solve(
                        self.R_dev[:self.n_dof],
                        tol=newton_forcing(self.fieldsplit_forcing, self.fieldsplit_min_tolerance),
                        atol=max(self.linear_solver_atol, 1e-3 * self.newton_solver_tolerance))
                    self.timings["krylov_iterations"] = self.timings.get("krylov_iterations", 0) + int(its)
                elif device_solve:
                    from .linsolve import BatchedBiCGStab, DeviceCSR
                    if getattr(self, "_krylov", None) is None:
                        # one block per replica: each replica's solve is its own
                        self._krylov = BatchedBiCGStab(DeviceCSR.of_problem(self), blocks=self.replicas)
                    dx2, its = self._krylov.solve(self.R_dev[:self.n_dof], tol=self.linear_solver_tolerance,
                                                  atol=self.linear_solver_atol)
                    dxd = dx2.view(-1)
                    self.timings["krylov_iterations"] = self.timings.get("krylov_iterations", 0) + int(its.max())
                else:
                    dx = self._solve_linear(R)
            tc = time.perf_counter()
            if not device_solve:
                dxd = torch.as_tensor(dx, device=self.x_dev.device)
            N.check(N.load().fe_dof_update(self._h, self.x_dev.data_ptr(), dxd.data_ptr(), self.n_dof,
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
            self.assemble_device(with_jacobian=False)
            hist.append(self.residual_max())
            t_asm += tb - ta
            t_lin += tc - tb
            it += 1
            if self.verbose:
                print(f"Newton iteration {it}: max residual {hist[-1]:.3e}")
        self.assemble_device(with_jacobian=False)  # leaves the nodal values at the solution
        self.check()
        self.newton_history = hist
        self.timings.update(newton_total_s=time.perf_counter() - t0, newton_assembly_s=t_asm,
                            newton_linear_solve_s=t_lin, newton_iterations=it)
        return hist
