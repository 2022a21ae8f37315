"""Weak-form expression language, mirroring the names of pyoomph's
``pyoomph.expressions`` (``generic.py``: ``var`` :137, ``grad`` :355,
``weak`` :394, ``testfunction`` :647, ``material_derivative`` :564;
``__init__.py:453`` ``var_and_test``) on top of sympy.

A field value at an integration point is a sympy symbol; its spatial
gradient is a vector of symbols.  ``weak(a, b)`` is the integrand
``a : b`` times the coordinate-system measure (``2*pi*r`` for the
axisymmetric system, ``expressions/coordsys.py:428-432``).  The code
generator differentiates the summed integrand with respect to the test
and trial components to obtain the pointwise residual coefficients and
their Jacobian -- the role GiNaC plays in the reference.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple, Union

import sympy as sp

Expr = Union[sp.Expr, sp.MatrixBase, float, int]

# coordinate symbols x0, x1, x2 (Eulerian position at the integration point;
# on moving meshes these are the values of the position fields mesh_x/y/z)
X = sp.symbols("x0:3", real=True)
# Lagrangian (reference) coordinates and the interface normal
LAG = sp.symbols("XL0:3", real=True)
NORMAL = sp.symbols("N0:3", real=True)
MESH_FIELDS = ("mesh_x", "mesh_y", "mesh_z")


class _Registry:
    """Symbols of the fields, their gradients and test functions."""

    def __init__(self):
        self.value: Dict[str, sp.Symbol] = {}
        self.grad: Dict[str, Tuple[sp.Symbol, ...]] = {}
        self.test: Dict[str, sp.Symbol] = {}
        self.test_grad: Dict[str, Tuple[sp.Symbol, ...]] = {}
        self.params: Dict[str, sp.Symbol] = {}
        self.vector_fields: Dict[str, List[str]] = {}
        self.lgrad: Dict[str, Tuple[sp.Symbol, ...]] = {}
        self.test_lgrad: Dict[str, Tuple[sp.Symbol, ...]] = {}
        self.dt: Dict[str, sp.Symbol] = {}

    def field(self, name: str):
        if name not in self.value:
            self.value[name] = sp.Symbol(f"U_{name}", real=True)
            self.grad[name] = tuple(sp.Symbol(f"U_{name}__x{i}", real=True) for i in range(3))
            self.test[name] = sp.Symbol(f"T_{name}", real=True)
            self.test_grad[name] = tuple(sp.Symbol(f"T_{name}__x{i}", real=True) for i in range(3))
            self.lgrad[name] = tuple(sp.Symbol(f"U_{name}__L{i}", real=True) for i in range(3))
            self.test_lgrad[name] = tuple(sp.Symbol(f"T_{name}__L{i}", real=True) for i in range(3))
            self.dt[name] = sp.Symbol(f"U_{name}__t", real=True)
        return self.value[name]


REG = _Registry()
_DIM = [2]


def set_dimension(dim: int) -> None:
    _DIM[0] = dim


def dimension() -> int:
    return _DIM[0]


def register_vector_field(name: str, comps: List[str]) -> None:
    REG.vector_fields[name] = comps


TIME_PARAM = "_time"


def var(name: str) -> Expr:
    """Field value (scalar symbol, or a column vector for a vector field).
    ``time``: the current time; ``mesh``/``coordinate``: the Eulerian position; ``lagrangian``: the
    reference position; ``normal``: the outward unit normal (interfaces)."""
    if name in REG.vector_fields:
        return sp.Matrix([REG.field(c) for c in REG.vector_fields[name]])
    if name == "time":
        # the time of the solve (t_{n+1} within a time step): a run-time
        # parameter the time stepper sets
        return parameter(TIME_PARAM)
    if name in ("coordinate", "mesh"):
        return sp.Matrix(X[:dimension()])
    if name == "lagrangian":
        return sp.Matrix(LAG[:dimension()])
    if name == "normal":
        return sp.Matrix(NORMAL[:dimension()])
    if name.startswith("coordinate_"):
        return X["xyz".index(name[-1])]
    return REG.field(name)


def testfunction(name: str) -> Expr:
    if name == "mesh":
        comps = list(MESH_FIELDS[:dimension()])
        for c in comps:
            REG.field(c)
        return sp.Matrix([REG.test[c] for c in comps])
    if name in REG.vector_fields:
        comps = REG.vector_fields[name]
        for c in comps:
            REG.field(c)
        return sp.Matrix([REG.test[c] for c in comps])
    REG.field(name)
    return REG.test[name]


def var_and_test(name: str):
    return var(name), testfunction(name)


def parameter(name: str) -> sp.Symbol:
    """A global parameter (read from the parameter array at run time)."""
    if name not in REG.params:
        REG.params[name] = sp.Symbol(f"P_{name}", real=True)
    return REG.params[name]


def mesh_velocity() -> Expr:
    """d x / d t at fixed Lagrangian position (BDF weights of the step)."""
    return sp.Matrix([REG.dt[REG.field(c) and c] for c in MESH_FIELDS[:dimension()]])


def partial_t(f: Expr) -> Expr:
    """Time derivative at fixed node of a field (or vector of fields)."""
    if isinstance(f, sp.MatrixBase):
        return sp.Matrix([partial_t(c) for c in f])
    f = sp.sympify(f)
    out = sp.Integer(0)
    for s_ in f.free_symbols:
        nm = s_.name
        if nm.startswith("U_") and "__" not in nm:
            out += sp.diff(f, s_) * REG.dt[nm[2:]]
        elif s_ in X:
            out += sp.diff(f, s_) * REG.dt[MESH_FIELDS[X.index(s_)]]
    return out


def _d_dL(e: sp.Expr, i: int) -> sp.Expr:
    """d/dxi_i (Lagrangian) of a pointwise expression."""
    e = sp.sympify(e)
    out = sp.Integer(0)
    for s_ in e.free_symbols:
        de = sp.diff(e, s_)
        if de == 0:
            continue
        nm = s_.name
        if nm.startswith("U_") and "__" not in nm:
            out += de * REG.lgrad[nm[2:]][i]
        elif nm.startswith("T_") and "__" not in nm:
            out += de * REG.test_lgrad[nm[2:]][i]
        elif s_ in X:
            out += de * REG.lgrad[MESH_FIELDS[X.index(s_)]][i]
        elif s_ in LAG:
            out += de * (1 if LAG.index(s_) == i else 0)
        elif nm.startswith("P_"):
            continue
        else:
            raise NotImplementedError(f"Lagrangian derivative of {nm} is not supported")
    return out


def _d_dx(e: sp.Expr, i: int) -> sp.Expr:
    """d/dx_i of a pointwise expression by the chain rule through the
    field symbols (value -> gradient component) and the coordinates."""
    e = sp.sympify(e)
    out = sp.Integer(0)
    for s in e.free_symbols:
        de = sp.diff(e, s)
        if de == 0:
            continue
        nm = s.name
        if nm.startswith("U_") and "__x" not in nm:
            out += de * REG.grad[nm[2:]][i]
        elif nm.startswith("T_") and "__x" not in nm:
            out += de * REG.test_grad[nm[2:]][i]
        elif s in X:
            out += de * (1 if X.index(s) == i else 0)
        elif nm.startswith("P_"):
            continue
        else:
            raise NotImplementedError(f"second derivatives of {nm} are not supported")
    return out


def grad(e: Expr, lagrangian: bool = False, coordsys=None) -> Expr:
    """Gradient.  Scalar -> column vector g_i = d e/dx_i; vector u ->
    matrix G[i, j] = d u_j / d x_i (pyoomph's convention).  With
    ``lagrangian`` the derivatives are with respect to the reference
    position.  In the axisymmetric system a 2-vector (u_r, u_z) has the 3x3
    gradient with the hoop entry G[2, 2] = u_r / r."""
    d = dimension()
    dd = _d_dL if lagrangian else _d_dx
    cs = coordsys or _COORDSYS[0]
    if isinstance(e, sp.MatrixBase):
        G = sp.Matrix(d, e.shape[0], lambda i, j: dd(e[j], i))
        if isinstance(cs, AxisymmetricCoordinateSystem) and e.shape[0] == 2:
            r = LAG[0] if lagrangian else X[0]
            G3 = sp.zeros(3, 3)
            G3[:2, :2] = G
            G3[2, 2] = e[0] / r
            return G3
        return G
    return sp.Matrix([dd(e, i) for i in range(d)])


def div(u: Expr, coordsys=None) -> sp.Expr:
    """Divergence (axisymmetric: + u_r / r)."""
    d = dimension()
    cs = coordsys or _COORDSYS[0]
    out = sum(_d_dx(u[i], i) for i in range(d))
    if isinstance(cs, AxisymmetricCoordinateSystem):
        out += u[0] / X[0]
    return out


def transpose(A: sp.MatrixBase) -> sp.MatrixBase:
    return A.T


def sym(A: sp.MatrixBase) -> sp.MatrixBase:
    return (A + A.T) / 2


def identity_matrix(n: int = None) -> sp.MatrixBase:
    return sp.eye(n or dimension())


def trace(A: sp.MatrixBase) -> sp.Expr:
    return A.trace()


def dot(a: Expr, b: Expr) -> Expr:
    """Contraction of the last index of a with the first of b."""
    if isinstance(a, sp.MatrixBase) and isinstance(b, sp.MatrixBase):
        if a.shape[1] == 1 and b.shape[1] == 1:
            return (a.T * b)[0, 0]
        if a.shape[1] == 1:  # vector . matrix
            return (a.T * b).T
        return a * b
    return a * b


def material_derivative(f: Expr, velocity: Expr) -> Expr:
    """partial_t f + (u . grad) f (generic.py:564); the partial_t term
    vanishes in a steady solve."""
    return partial_t(f) + dot(velocity, grad(f))


class CoordinateSystem:
    def measure(self) -> sp.Expr:
        return sp.Integer(1)


class CartesianCoordinateSystem(CoordinateSystem):
    pass


class AxisymmetricCoordinateSystem(CoordinateSystem):
    """dx = 2*pi*r dr dz with r = x0 (coordsys.py:428-432)."""

    def measure(self) -> sp.Expr:
        return 2 * sp.pi * X[0]


_COORDSYS = [CartesianCoordinateSystem()]


def set_coordinate_system(cs: CoordinateSystem) -> None:
    _COORDSYS[0] = cs


class LagrangianIntegrand:
    """An integrand over the reference (Lagrangian) configuration (``Weak``)."""

    def __init__(self, expr):
        self.expr = sp.sympify(expr)

    def __mul__(self, c):
        return LagrangianIntegrand(self.expr * c)

    __rmul__ = __mul__

    def __neg__(self):
        return LagrangianIntegrand(-self.expr)


def Weak(a: Expr, b: Expr, coordinate_system: CoordinateSystem = None) -> LagrangianIntegrand:
    """a : b integrated over the Lagrangian configuration dX."""
    cs = coordinate_system or CartesianCoordinateSystem()
    A, B = (sp.Matrix(a), sp.Matrix(b)) if isinstance(a, sp.MatrixBase) or isinstance(b, sp.MatrixBase) else (a, b)
    if isinstance(A, sp.MatrixBase):
        if A.shape != B.shape:
            raise ValueError(f"Weak: shape mismatch {A.shape} vs {B.shape}")
        prod = sum(A[i] * B[i] for i in range(len(A)))
    else:
        prod = sp.sympify(A) * sp.sympify(B)
    meas = 2 * sp.pi * LAG[0] if isinstance(cs, AxisymmetricCoordinateSystem) else 1
    return LagrangianIntegrand(prod * meas)


def weak(a: Expr, b: Expr, coordinate_system: CoordinateSystem = None) -> sp.Expr:
    """Integrand a : b (full contraction) times the measure."""
    cs = coordinate_system or _COORDSYS[0]
    if isinstance(a, sp.MatrixBase) or isinstance(b, sp.MatrixBase):
        A = sp.Matrix(a)
        B = sp.Matrix(b)
        if A.shape != B.shape:
            raise ValueError(f"weak: shape mismatch {A.shape} vs {B.shape}")
        prod = sum(A[i] * B[i] for i in range(len(A)))
    else:
        prod = sp.sympify(a) * sp.sympify(b)
    return prod * cs.measure()


def exp(e: Expr) -> sp.Expr:
    return sp.exp(e)


def square_mag(v: Sequence) -> sp.Expr:
    return sum(c * c for c in v)


class GaussianSum(sp.Function):
    """sum_k A_k exp(-|x - c_k|^2 / (2 w_k^2)) over n Gaussians whose
    centres, widths and amplitudes are the parameters g{k}_c{i}, g{k}_w,
    g{k}_A (stored contiguously per Gaussian).  Arguments: the coordinate
    symbols, n, dim, then the parameter symbols in array order.  The code
    generator prints it as a call of the
    device loop fe_gauss_sum<dim>, which keeps the kernel small; it depends
    on the position only, so its derivative with respect to any field is 0."""

    def fdiff(self, argindex=1):
        raise NotImplementedError("GaussianSum has no coordinate derivative (fixed meshes only)")


def gaussian_source(n: int, dim: int) -> sp.Expr:
    ps = []
    for k in range(n):
        for i in range(dim):
            ps.append(parameter(f"g{k}_c{i}"))
        ps.append(parameter(f"g{k}_w"))
        ps.append(parameter(f"g{k}_A"))
    return GaussianSum(*X[:dim], sp.Integer(n), sp.Integer(dim), *ps)


_GAUSS_RE = __import__("re").compile(r"^g(\d+)_(c(\d)|w|A)$")


def parameter_order_key(name: str):
    """Array order of the global parameters: the Gaussian groups first,
    each Gaussian's c_0..c_{d-1}, w, A contiguous; then the rest by name."""
    m = _GAUSS_RE.match(name)
    if m:
        comp = {"w": 10, "A": 11}.get(m.group(2), int(m.group(3)) if m.group(3) is not None else 0)
        return (0, int(m.group(1)), comp, "")
    return (1, 0, 0, name)
