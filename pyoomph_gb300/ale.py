"""Moving meshes (pseudo-solid ALE), interface and point elements, implicit
time stepping, and the fused multi-domain element kernel.

This is the device counterpart of the parts of pyoomph that an
axisymmetric sessile droplet uses:

* positions as unknowns (the ``mesh_x``/``mesh_y`` fields of a domain with
  ``_coordinates_as_dofs``) with the shape derivatives of the Jacobian --
  ``int_pt_weights_d_coords`` and ``d_dx_shape_dcoord`` of the shape buffer
  (``src/jitbridge.h:175-190``, computed in ``src/elements.cpp:3051-3140``)
  -- folded here into per-point coefficients of the element Jacobian and
  never materialised;
* integrals over the reference configuration (``Weak``; the pseudo-elastic
  mesh of ``pyoomph/equations/ALE.py:97-147``);
* 1D interface elements (``InterfaceTElementLine1dC2``,
  ``src/elements.hpp:2074``, geometry ``elements.cpp:13685``, normals
  ``:4259-4265``) and 0D contact-line elements;
* BDF1/BDF2 time derivatives from previous time levels (``MultiTimeStepper``
  weights, degraded to BDF1 on the first step, ``elements.cpp:4588-4640``);
* all domains of a problem evaluated in ONE launch: blocks are dispatched to
  the bulk, interface and contact-line element code by block index.

Position derivatives (Eulerian integrals; X_{m,b} = coordinate b of node m,
all follow from the chain rule):

* weight:           d(w J)/dX = w J dpsi_m/dx_b  (bulk and surface alike);
* test gradient:    d(dphi_l/dx_a)/dX = -(dphi_l/dx_b)(dpsi_m/dx_a)  (bulk);
* field gradient:   d(du/dx_a)/dX = -(du/dx_b)(dpsi_m/dx_a)  (bulk);
* on a line in 2D with unit tangent tau and s_l = (dpsi_l/ds)/|dx/ds|
  (so the surface gradient is tau s_l):
  d(tau_a s_l)/dX = s_l s_m (delta_ab - 2 tau_a tau_b),
  dn_i/dX = (R_ib - n_i tau_b) s_m for the outward normal n = R tau,
  R = [[0, 1], [-1, 0]] (elements ordered counterclockwise);
* explicit positions (the axisymmetric 2 pi r, the mesh velocity) are the
  values of the position fields and differentiate like any field.
"""
from __future__ import annotations

import ctypes
import hashlib
import math
import re
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import sympy as sp

from . import _native as N
from . import expressions as E
from .codegen import _emit
from .meshes import RectangularQuadMesh
from .problem import nvtx_range
from .spaces import GAUSS_T2_KNOTS, GAUSS_T2_WEIGHTS, P2_TRI

# TGauss<1,3> (oomph integral.cc:311-316) and TElement<1,3> shapes (Telements.h:347-366)
_TG1_KNOTS = np.array([[0.5 * (-0.774596669241483 + 1.0)], [0.5], [0.5 * (0.774596669241483 + 1.0)]])
_TG1_WEIGHTS = np.array([5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0])


def line3_shape(s):
    s0 = s[0]
    psi = np.array([2.0 * (s0 - 1.0) * (s0 - 0.5), 4.0 * (1.0 - s0) * s0, 2.0 * (s0 - 0.5) * s0])
    dps = np.array([[4.0 * s0 - 3.0], [4.0 - 8.0 * s0], [4.0 * s0 - 1.0]])
    return psi, dps


def line2_shape(s):
    return np.array([1.0 - s[0], s[0]]), np.array([[-1.0], [1.0]])


@dataclass
class DomainType:
    """Element geometry of one domain kind: reference element dimension,
    nodes, C1 (vertex) nodes and the quadrature rule."""
    name: str
    el_dim: int
    nnode: int
    c1_index: Tuple[int, ...]
    knots: np.ndarray
    weights: np.ndarray

    @property
    def nq(self) -> int:
        return len(self.weights)

    @property
    def ed(self) -> int:
        """Stored derivative directions (at least 1, zeros for points)."""
        return max(1, self.el_dim)

    def shapes(self):
        nq, nn, n1, d = self.nq, self.nnode, len(self.c1_index), self.ed
        psi2, dps2 = np.zeros((nq, nn)), np.zeros((nq, nn, d))
        psi1, dps1 = np.zeros((nq, n1)), np.zeros((nq, n1, d))
        for q in range(nq):
            if self.name == "P2_TRI":
                psi2[q], dps2[q] = P2_TRI.shape_c2(self.knots[q])
                psi1[q], dps1[q] = P2_TRI.shape_c1(self.knots[q])
            elif self.name == "P2_LINE":
                psi2[q], dps2[q] = line3_shape(self.knots[q])
                psi1[q], dps1[q] = line2_shape(self.knots[q])
            else:
                psi2[q], psi1[q] = 1.0, 1.0
        return psi2, dps2, psi1, dps1

    def tables(self) -> np.ndarray:
        """Packed: weights, C2 shapes, C2 local derivatives, C1 shapes, C1 derivatives."""
        psi2, dps2, psi1, dps1 = self.shapes()
        return np.concatenate([self.weights, psi2.ravel(), dps2.ravel(), psi1.ravel(), dps1.ravel()])


TRI6 = DomainType("P2_TRI", 2, 6, (0, 1, 2), GAUSS_T2_KNOTS, GAUSS_T2_WEIGHTS)
LINE3 = DomainType("P2_LINE", 1, 3, (0, 2), _TG1_KNOTS, _TG1_WEIGHTS)
POINT1 = DomainType("POINT", 0, 1, (0,), np.zeros((1, 1)), np.ones(1))


# ---------------------------------------------------------------------------
# equations
# ---------------------------------------------------------------------------
AXI = E.AxisymmetricCoordinateSystem()


class ALEEquations:
    """Weak-form contributions of one domain ('bulk', 'interface' or
    'point'): an Eulerian integrand (``weak``) and a Lagrangian one
    (``Weak``), both linear in the test functions."""
    domain = "bulk"

    def __init__(self):
        self.fields: List[Tuple[str, str]] = []
        self.rE = sp.Integer(0)
        self.rL = sp.Integer(0)
        self.param_values: Dict[str, float] = {}

    def define_scalar_field(self, name: str, space: str) -> None:
        self.fields.append((name, space))
        E.REG.field(name)

    def define_vector_field(self, name: str, space: str) -> None:
        comps = [f"{name}_{c}" for c in "xyz"[:E.dimension()]]
        E.register_vector_field(name, comps)
        for c in comps:
            self.define_scalar_field(c, space)

    def add_residual(self, expr) -> None:
        if isinstance(expr, E.LagrangianIntegrand):
            self.rL = self.rL + expr.expr
        else:
            self.rE = self.rE + sp.sympify(expr)

    def set_parameter(self, name: str, value: float) -> sp.Symbol:
        self.param_values[name] = float(value)
        return E.parameter(name)

    def define_fields(self) -> None:
        pass

    def define_residuals(self) -> None:
        pass


class AxisymmetricStokesEquations(ALEEquations):
    """Stokes flow in (r, z) on Taylor-Hood elements
    (``navier_stokes.py:303-345``: weak(stress, grad(v)) + weak(div u, q);
    axisymmetric: 3x3 velocity gradient with the hoop entry u_r/r,
    div u += u_r/r, dx = 2 pi r)."""

    def __init__(self, dynamic_viscosity: float = 1.0):
        super().__init__()
        self.mu = dynamic_viscosity

    def define_fields(self):
        self.define_vector_field("velocity", "C2")
        self.define_scalar_field("pressure", "C1")

    def define_residuals(self):
        u, v = E.var_and_test("velocity")
        p, q = E.var_and_test("pressure")
        mu = self.set_parameter("dynamic_viscosity", self.mu)
        stress = 2 * mu * E.sym(E.grad(u, coordsys=AXI)) - E.identity_matrix(3) * p
        self.add_residual(E.weak(stress, E.grad(v, coordsys=AXI), AXI))
        self.add_residual(E.weak(E.div(u, AXI), q, AXI))


class PseudoElasticMesh(ALEEquations):
    """Pseudo-solid mesh motion (``ALE.py:97-147``): linear elasticity of the
    displacement x - X over the reference configuration, cartesian,
    mu = E/(2(1+nu)), lambda' = 2 mu lambda / (lambda + 2 mu)."""

    def __init__(self, E_: float = 1.0, nu: float = 0.3):
        super().__init__()
        self.E_ = E_
        self.nu = nu

    def define_fields(self):
        for c in E.MESH_FIELDS[:E.dimension()]:
            self.define_scalar_field(c, "C2")

    def define_residuals(self):
        Em, nu = sp.nsimplify(self.E_), sp.nsimplify(self.nu)
        mu = Em / 2 / (1 + nu)
        lm = Em * nu / (1 + nu) / (1 - 2 * nu)
        lm = 2 * mu * lm / (lm + 2 * mu)
        cart = E.CartesianCoordinateSystem()
        x, xt = E.var("mesh"), E.testfunction("mesh")
        X = E.var("lagrangian")

        def eps(w):
            return E.sym(E.grad(w, lagrangian=True, coordsys=cart))

        def sig(w):
            return lm * E.trace(eps(w)) * E.identity_matrix(2) + 2 * mu * eps(w)

        self.add_residual(E.Weak(sig(x - X), eps(xt)))


class FreeSurface(ALEEquations):
    """Free surface on a moving mesh (``NavierStokesFreeSurface``,
    ``navier_stokes.py:605-676``): weak((xdot - u).n, l_test)
    - weak(l, n.x_test) + weak(sigma, div_s v)."""
    domain = "interface"

    def __init__(self, surface_tension: float = 1.0, kinbc_name: str = "_kin_bc"):
        super().__init__()
        self.sigma = surface_tension
        self.kin = kinbc_name

    def define_fields(self):
        self.define_scalar_field(self.kin, "C2")

    def define_residuals(self):
        n = E.var("normal")
        u, v = E.var_and_test("velocity")
        xt = E.testfunction("mesh")
        lam, lt = E.var_and_test(self.kin)
        sigma = self.set_parameter("surface_tension", self.sigma)
        self.add_residual(E.weak(E.dot(E.mesh_velocity() - u, n), lt, AXI))
        self.add_residual(-E.weak(lam, E.dot(n, xt), AXI))
        comps = E.REG.vector_fields["velocity"]
        div_s = sum(E.REG.test_grad[c][i] for i, c in enumerate(comps)) + v[0] / E.X[0]
        self.add_residual(E.weak(sigma, div_s, AXI))


class ContactAngle(ALEEquations):
    """Contact line on the substrate z = 0 (``NavierStokesContactAngle``,
    ``navier_stokes.py:1025-1088``): weak(sigma, m.v) with
    m = sin(theta) n_wall + cos(theta) t_wall, n_wall = (0, 1) and the wall
    tangent pointing into the drop, t_wall = (-1, 0)."""
    domain = "point"

    def __init__(self, contact_angle: float, surface_tension: float = 1.0):
        super().__init__()
        self.theta = contact_angle
        self.sigma = surface_tension

    def define_residuals(self):
        _, v = E.var_and_test("velocity")
        th = self.set_parameter("contact_angle", self.theta)
        sigma = self.set_parameter("surface_tension", self.sigma)
        m = sp.Matrix([-sp.cos(th), sp.sin(th)])
        self.add_residual(E.weak(sigma, E.dot(m, v), AXI))


# ---------------------------------------------------------------------------
# code generation
# ---------------------------------------------------------------------------
@dataclass
class DomainCode:
    """One domain of a fused kernel: its element type, fields and integrands,
    and (after generation) its local layout and launch shape."""
    dtype: DomainType
    fields: List[Tuple[str, str, int, bool]]   # (name, space, nodal value index, is_position)
    rE: sp.Expr
    rL: sp.Expr
    layout_node: List[int] = field(default_factory=list)
    layout_val: List[int] = field(default_factory=list)
    nloc: int = 0
    epb: int = 1
    smem: int = 0
    nk: int = 0
    rows_needed: int = 0
    flops: float = 0.0          # FP64 operations per element (FMA = 2), counted from the generated code
    flops32: float = 0.0        # FP32 operations per element (the Jacobian contraction of the f32 variant)
    flops_df64: float = 0.0     # FP64-equivalent operations of the df64 variant's contraction

    def layout(self):
        """Local order: the nodal values node by node (fields in order), then
        the positions node by node -- oomph's order for solid elements
        (nodal data, then ``assign_solid_local_eqn_numbers``)."""
        dt = self.dtype
        lnode, lval, slot = [], [], {}
        for group in (False, True):
            for l in range(dt.nnode):
                for f, (_, space, vi, isp) in enumerate(self.fields):
                    if isp != group or (space == "C1" and l not in dt.c1_index):
                        continue
                    slot[(f, l)] = len(lnode)
                    lnode.append(l)
                    lval.append(vi)
        return lnode, lval, slot


def _ops(c_expr: str) -> int:
    """Binary arithmetic operations in a generated C expression."""
    return c_expr.count(" * ") + c_expr.count(" + ") + c_expr.count(" - ")


def _sub_nodes(dc: DomainCode, f: int) -> List[int]:
    return list(dc.dtype.c1_index) if dc.fields[f][1] == "C1" else list(range(dc.dtype.nnode))


def _domain_source(k: int, dc: DomainCode, dim: int, params: List[str], nval: int, nh: int,
                   smem_budget: int, nthreads_cap: int, f32: bool = False, df64: bool = False,
                   rows_per_thread: int = 1) -> str:
    """Device namespace dom{k} with ``run(a, blk, smem)`` evaluating one block
    of elements of this domain: stage tables and nodal data (phase 0), one
    thread per (element, knot) for geometry, interpolation and the pointwise
    weak form (phase A), one thread per (element, row) for R_e and J_e
    (phase B).  With ``f32`` the Jacobian coefficients, the shape values and
    gradients they are contracted with, and the accumulation are single
    precision; geometry, pointwise weak form and residual stay FP64."""
    dt = dc.dtype
    ed, EDs = dt.el_dim, dt.ed
    nn, nq, c1 = dt.nnode, dt.nq, dt.c1_index
    n1 = len(c1)
    d = dim
    fields = dc.fields
    nf = len(fields)
    NCU, NCT = 2 + 2 * d, 1 + 2 * d
    pos_f = {nm: f for f, (nm, _, _, isp) in enumerate(fields) if isp}
    mesh_f = [pos_f.get(E.MESH_FIELDS[b], -1) for b in range(d)]
    moving = all(m >= 0 for m in mesh_f)
    bdf0 = params.index("__bdf0") if "__bdf0" in params else -1

    def tci(f, c):
        return f * NCT + c

    def ici(f, c):
        return f * NCU + c

    # ---- symbols -> component slots
    usym, tsym = {}, {}
    for f, (nm, _, _, _) in enumerate(fields):
        usym[E.REG.value[nm]] = ici(f, 0)
        for i in range(d):
            usym[E.REG.grad[nm][i]] = ici(f, 1 + i)
            usym[E.REG.lgrad[nm][i]] = ici(f, 1 + d + i)
            tsym[E.REG.test_grad[nm][i]] = tci(f, 1 + i)
            tsym[E.REG.test_lgrad[nm][i]] = tci(f, 1 + d + i)
        usym[E.REG.dt[nm]] = ici(f, 1 + 2 * d)
        tsym[E.REG.test[nm]] = tci(f, 0)
    subs = {E.X[b]: E.REG.value[E.MESH_FIELDS[b]] for b in range(d)} if moving else {}
    IE = sp.sympify(dc.rE).xreplace(subs)
    IL = sp.sympify(dc.rL).xreplace(subs)
    if ed < d and IL != 0:
        raise NotImplementedError("Lagrangian integrals on interface/point domains")
    tsyms = (IE + IL).free_symbols
    if (bdf0 < 0 or nh == 0) and any(s_ in usym and usym[s_] % NCU == 1 + 2 * d for s_ in tsyms):
        raise ValueError("time derivatives need the BDF weight parameters and history levels")
    allowed = set(usym) | set(tsym) | set(E.LAG) | set(E.NORMAL) | set(E.X) | {E.parameter(p) for p in params}
    for s_ in tsyms:
        if s_ not in allowed:
            raise ValueError(f"symbol {s_} is not defined on this domain")
    ntc = nf * NCT
    tlist = [None] * ntc
    for s_, i in tsym.items():
        tlist[i] = s_
    rEc = [sp.diff(IE, t) if t is not None else sp.Integer(0) for t in tlist]
    rLc = [sp.diff(IL, t) if t is not None else sp.Integer(0) for t in tlist]
    for t in tlist:
        if t is not None and any(sp.diff(c, t) != 0 for c in rEc + rLc if c != 0):
            raise ValueError("the weak form must be linear in the test functions")
    ulist = [None] * (nf * NCU)
    for s_, i in usym.items():
        ulist[i] = s_
    DE, DL, DN = {}, {}, {}
    for tc in range(ntc):
        for ic, us in enumerate(ulist):
            if us is None:
                continue
            if rEc[tc] != 0:
                v = sp.diff(rEc[tc], us)
                if v != 0:
                    DE[(tc, ic)] = v
            if rLc[tc] != 0:
                v = sp.diff(rLc[tc], us)
                if v != 0:
                    DL[(tc, ic)] = v
        if ed == 1 and rEc[tc] != 0:
            for i in range(d):
                v = sp.diff(rEc[tc], E.NORMAL[i])
                if v != 0:
                    DN[(tc, i)] = v
    # ---- printed names
    names = {s_: f"U[{i}]" for s_, i in usym.items()}
    for i in range(3):
        names[E.LAG[i]] = f"XL[{i}]"
        names[E.NORMAL[i]] = f"Nn[{i}]"
        names[E.X[i]] = f"Xq[{i}]"
    for j, p in enumerate(params):
        names[E.parameter(p)] = f"P[{j}]"
    # ---- residual coefficients and Jacobian coefficient terms
    rEn = {tc: j for j, tc in enumerate(tc for tc in range(ntc) if rEc[tc] != 0)}
    rLn = {tc: j for j, tc in enumerate(tc for tc in range(ntc) if rLc[tc] != 0)}
    eE = {key: j for j, key in enumerate(DE)}
    eL = {key: j for j, key in enumerate(DL)}
    eN = {key: j for j, key in enumerate(DN)}
    terms: Dict[Tuple[int, int], List[str]] = {}

    def add(key, s_):
        terms.setdefault(key, []).append(s_)

    for key, j in eE.items():
        add(key, f"wE * dE[{j}]")
    for key, j in eL.items():
        add(key, f"wL * dL[{j}]")
    if moving and ed >= 1:
        for b in range(d):
            fb = mesh_f[b]

            def kron(a):
                return "1.0" if a == b else "0.0"

            for tc, j in rEn.items():                       # weight
                add((tc, ici(fb, 1 + b)), f"wE * rE[{j}]")
            if ed == d:
                for tf in range(nf):                          # test gradients
                    for a in range(d):
                        j = rEn.get(tci(tf, 1 + a))
                        if j is not None:
                            add((tci(tf, 1 + b), ici(fb, 1 + a)), f"-wE * rE[{j}]")
                for (tc, ic), j in eE.items():                # field gradients
                    f, c = divmod(ic, NCU)
                    if 1 <= c <= d:
                        add((tc, ici(fb, c)), f"-wE * dE[{j}] * U[{ici(f, 1 + b)}]")
            else:
                for tf in range(nf):                          # surface test gradients
                    js = [rEn.get(tci(tf, 1 + a)) for a in range(d)]
                    if all(j is None for j in js):
                        continue
                    Kb = " + ".join(f"rE[{js[a]}] * ({kron(a)} - 2.0 * tau[{a}] * tau[{b}])"
                                    for a in range(d) if js[a] is not None)
                    for c in range(d):
                        for e2 in range(d):
                            add((tci(tf, 1 + c), ici(fb, 1 + e2)), f"wE * ({Kb}) * tau[{c}] * tau[{e2}]")
                grouped: Dict[Tuple[int, int], List[Tuple[int, int]]] = {}
                for (tc, ic), j in eE.items():                # surface field gradients
                    f, c = divmod(ic, NCU)
                    if 1 <= c <= d:
                        grouped.setdefault((tc, f), []).append((c - 1, j))
                for (tc, f), lst in grouped.items():
                    us = " + ".join(f"tau[{c}] * U[{ici(f, 1 + c)}]" for c in range(d))
                    K = " + ".join(f"dE[{j}] * ({kron(a)} - 2.0 * tau[{a}] * tau[{b}])" for a, j in lst)
                    for e2 in range(d):
                        add((tc, ici(fb, 1 + e2)), f"wE * ({K}) * ({us}) * tau[{e2}]")
                Rm = [[0.0, 1.0], [-1.0, 0.0]]
                for (tc, i), j in eN.items():                 # normal
                    for e2 in range(d):
                        add((tc, ici(fb, 1 + e2)),
                            f"wE * dN[{j}] * ({Rm[i][b]!r} - Nn[{i}] * tau[{b}]) * tau[{e2}]")
    keys = sorted(terms)
    NK = max(1, len(keys))
    dc.nk = len(keys)
    # interpolated components the pointwise code and the Jacobian terms read
    used_u = set()
    for e_ in rEc + rLc:
        used_u |= {usym[s_] for s_ in sp.sympify(e_).free_symbols if s_ in usym}
    for key in keys:
        for t_ in terms[key]:
            used_u |= {int(m_) for m_ in re.findall(r"U\[(\d+)\]", t_)}
    used_t = set(rEn) | set(rLn) | {tc for tc, _ in keys}
    lagr = (any(d + 1 <= u_ % NCU <= 2 * d for u_ in used_u) or any(d + 1 <= t_ % NCT for t_ in used_t)
            or any(d + 1 <= ic % NCU <= 2 * d for _, ic in keys))
    # ---- local layout
    lnode, lval, slot = dc.layout()
    nloc = len(lnode)
    dc.layout_node, dc.layout_val, dc.nloc = lnode, lval, nloc
    rows_f = [None] * nloc
    for (f, l), i in slot.items():
        rows_f[i] = (f, _sub_nodes(dc, f).index(l))
    # ---- shared memory plan (doubles)
    tabd = nq + nq * nn + nq * nn * EDs + nq * n1 + nq * n1 * EDs
    # the Jacobian contraction reads copies in its own type: float (f32) or
    # double-float pairs (df64, 8 bytes) of the shape values, the gradients
    # and the coefficients; FP64 reads the FP64 originals
    lowp = f32 or df64
    lt = "fe_df64" if df64 else "float"
    per8 = 1 if df64 else 2                           # low-precision values per 8 bytes
    tabf = nq * (nn + n1) if lowp else 0               # copies of the shape values
    tabfd = (tabf + per8 - 1) // per8
    QB = 2 * nn * d + 2 * n1 * d + ntc + (0 if lowp else NK) + 4
    FQB = NK + 2 * nn * d + 2 * n1 * d if lowp else 0  # per knot: C, dx, dX, dx1, dX1
    if f32:
        FQB += FQB % 2
    per_el = nn * nval * (1 + nh) + nn * d + nq * QB + nq * FQB // per8
    # threads per element: one per knot or per `rows_per_thread` rows, the
    # larger (the row phase then takes several rounds; every phase is a
    # block-strided loop)
    per_thr = max(nq, -(-nloc // max(1, int(rows_per_thread))))
    epb = 1
    for e_ in range(1, 65):
        if e_ * per_thr > nthreads_cap or (tabd + tabfd + e_ * per_el) * 8 > smem_budget:
            break
        epb = e_
    dc.epb = epb
    dc.smem = ((tabd + tabfd + epb * per_el) * 8 + 15) // 16 * 16
    dc.rows_needed = epb * per_thr
    # ---- source
    L: List[str] = []
    w = L.append
    w(f"namespace dom{k} {{")
    w(f"constexpr int NN = {nn}, NQ = {nq}, N1 = {n1}, ED = {EDs}, DIM = {d}, NVAL = {nval}, NH = {nh};")
    w(f"constexpr int NTC = {ntc}, NK = {NK}, NLOC = {nloc}, EPB = {epb};")
    w(f"constexpr int TABD = {tabd}, TABFD = {tabfd}, QB = {QB}, FQB = {FQB}, PER_EL = {per_el};")
    w("__device__ __forceinline__ void pointwise(const double* __restrict__ U, const double* __restrict__ Xq,")
    w("    const double* __restrict__ XL, const double* __restrict__ Nn, const double* __restrict__ P,")
    w("    const double* __restrict__ tau, double wE, double wL, double* __restrict__ rc, jreal* __restrict__ C,")
    w("    int flag, int dparam) {")
    w(f"  double rE[{max(1, len(rEn))}], rL[{max(1, len(rLn))}];")
    w(f"  double dE[{max(1, len(eE))}], dL[{max(1, len(eL))}], dN[{max(1, len(eN))}];")
    w("  (void)U; (void)Xq; (void)XL; (void)Nn; (void)P; (void)tau; (void)rE; (void)rL; (void)dE; (void)dL; (void)dN;")
    exprs, outs = [], []
    for tc, j in rEn.items():
        exprs.append(rEc[tc])
        outs.append(f"rE[{j}]")
    for tc, j in rLn.items():
        exprs.append(rLc[tc])
        outs.append(f"rL[{j}]")
    for key, j in eE.items():
        exprs.append(DE[key])
        outs.append(f"dE[{j}]")
    for key, j in eL.items():
        exprs.append(DL[key])
        outs.append(f"dL[{j}]")
    for key, j in eN.items():
        exprs.append(DN[key])
        outs.append(f"dN[{j}]")
    fl_point = 0
    if exprs:
        repl, red = sp.cse(exprs, symbols=sp.numbered_symbols("t_"), optimizations="basic")
        fl_point = sum(sp.count_ops(e) for _, e in repl) + sum(sp.count_ops(e) for e in red)
    fl_point += sum(_ops(" + ".join(terms[key])) for key in keys) + 2 * ntc
    if exprs:
        body = _emit(exprs, names, False, outs, "  ")
        dlines = [ln for ln in body if ln.strip().startswith(("dE[", "dL[", "dN["))]
        rlines = [ln for ln in body if not ln.strip().startswith(("dE[", "dL[", "dN["))]
        L.extend(rlines)
        w("  if (flag == 1 || flag == 2) {")
        L.extend("  " + ln for ln in dlines)
        w("  }")
    for tc in range(ntc):
        parts = []
        if tc in rEn:
            parts.append(f"wE * rE[{rEn[tc]}]")
        if tc in rLn:
            parts.append(f"wL * rL[{rLn[tc]}]")
        w(f"  rc[{tc}] = {' + '.join(parts) if parts else '0.0'};")
    w("  if (flag == 1 || flag == 2) {")
    for kk, key in enumerate(keys):
        w(f"    C[{kk}] = (jreal)({' + '.join(terms[key])});")
    w("  }")
    # flag 3: residual coefficients differentiated by one global parameter
    w("  if (flag == 3) {")
    w("    (void)dparam;")
    w(f"    for (int k = 0; k < {ntc}; ++k) rc[k] = 0.0;")
    w("    switch (dparam) {")
    for j, pn in enumerate(params):
        psym = E.parameter(pn)
        pex, pouts = [], []
        for tc in range(ntc):
            dEp = sp.diff(rEc[tc], psym) if rEc[tc] != 0 else sp.Integer(0)
            dLp = sp.diff(rLc[tc], psym) if rLc[tc] != 0 else sp.Integer(0)
            if dEp != 0 or dLp != 0:
                pex.append(dEp * sp.Symbol("WE") + dLp * sp.Symbol("WL"))
                pouts.append(f"rc[{tc}]")
        if not pex:
            continue
        w(f"    case {j}: {{")
        pn_names = dict(names)
        pn_names[sp.Symbol("WE")] = "wE"
        pn_names[sp.Symbol("WL")] = "wL"
        L.extend(_emit(pex, pn_names, False, pouts, "      "))
        w("      break; }")
    w("    default: break;")
    w("    }")
    w("  }")
    w("}")
    rowof = [slot[(f, l)] for f in range(nf) for l in _sub_nodes(dc, f)]
    w(f"__constant__ int c_rowof[NLOC] = {{{', '.join(map(str, rowof))}}};")
    w("__device__ __forceinline__ void run(const FeElemArgs& a, int blk, double* __restrict__ sW) {")
    w("  double* sPsi2 = sW + NQ;")
    w("  double* sDps2 = sPsi2 + NQ * NN;")
    w("  double* sPsi1 = sDps2 + NQ * NN * ED;")
    w("  double* sDps1 = sPsi1 + NQ * N1;")
    w("  double* sE = sW + TABD + TABFD;")
    w(f"  {lt}* sPsi2f = reinterpret_cast<{lt}*>(sW + TABD); {lt}* sPsi1f = sPsi2f + NQ * NN;")
    w("  (void)sPsi2f; (void)sPsi1f;")
    w("  const long long e0 = (long long)blk * EPB;")
    w("  const long long rem = a.n_elem - e0;")
    w("  const int nel = rem < EPB ? (int)rem : EPB;")
    w("  const int flag = a.flag;")
    w("  const double* __restrict__ P = a.params;")
    w("  (void)P; (void)sDps1;")
    w("  for (int k = threadIdx.x; k < TABD; k += FE_NT) sW[k] = a.tables[k];")
    if lowp:
        w(f"  for (int k = threadIdx.x; k < NQ * NN; k += FE_NT) sPsi2f[k] = ({lt})a.tables[NQ + k];")
        w(f"  for (int k = threadIdx.x; k < NQ * N1; k += FE_NT) sPsi1f[k] = ({lt})a.tables[NQ + NQ * NN * (1 + ED) + k];")
    if bdf0 >= 0:
        w(f"  const jreal w0j = (jreal)P[{bdf0}]; (void)w0j;")
    w("  for (int k = threadIdx.x; k < nel * NN; k += FE_NT) {")
    w("    const int el = k / NN, l = k - el * NN;")
    w("    long long node = a.conn[(e0 + el) * NN + l];")
    w("    FE_CHECK_NODE(node, e0 + el, a);")
    w("    double* eb = sE + el * PER_EL;")
    w("    for (int v = 0; v < NVAL; ++v) eb[l * NVAL + v] = a.values[node * NVAL + v];")
    w("    for (int h = 0; h < NH; ++h)")
    w("      for (int v = 0; v < NVAL; ++v)")
    w("        eb[(1 + h) * NN * NVAL + l * NVAL + v] = h < a.n_hist ? a.hist[h * a.hist_stride + node * NVAL + v] : 0.0;")
    w("    for (int i = 0; i < DIM; ++i) eb[(1 + NH) * NN * NVAL + l * DIM + i] = a.x0[node * DIM + i];")
    w("  }")
    w("  __syncthreads();")
    w("  for (int p = threadIdx.x; p < nel * NQ; p += FE_NT) {")
    w("    const int el = p / NQ, q = p - el * NQ;")
    w("    const double* Uv = sE + el * PER_EL;")
    w("    const double* X0 = Uv + (1 + NH) * NN * NVAL;")
    w("    double* qb = sE + el * PER_EL + (1 + NH) * NN * NVAL + NN * DIM + q * QB;")
    w("    double* dx = qb; double* dX = dx + NN * DIM; double* dx1 = dX + NN * DIM; double* dX1 = dx1 + N1 * DIM;")
    if lowp:
        w("    double* rc = dX1 + N1 * DIM; double* misc = rc + NTC;")
        w(f"    {lt}* C = reinterpret_cast<{lt}*>(sE + el * PER_EL + (1 + NH) * NN * NVAL + NN * DIM + NQ * QB) + q * FQB;")
        w(f"    {lt}* fdx = C + NK; {lt}* fdX = fdx + NN * DIM; {lt}* fdx1 = fdX + NN * DIM; {lt}* fdX1 = fdx1 + N1 * DIM;")
        w("    (void)fdX; (void)fdX1;")
    else:
        w("    double* rc = dX1 + N1 * DIM; double* C = rc + NTC; double* misc = C + NK;")
    w("    const double* ps = sPsi2 + q * NN;")
    w("    const double* dps = sDps2 + q * NN * ED;")
    w("    const double* dps1 = sDps1 + q * N1 * ED;")
    w("    double Xe[NN * DIM];")
    if moving:
        w("    for (int l = 0; l < NN; ++l) {")
        for b in range(d):
            w(f"      Xe[l * DIM + {b}] = Uv[l * NVAL + {fields[mesh_f[b]][2]}];")
        w("    }")
    else:
        w("    for (int l = 0; l < NN; ++l) for (int i = 0; i < DIM; ++i) "
          "Xe[l * DIM + i] = a.x[(long long)a.conn[(e0 + el) * NN + l] * DIM + i];")
    w("    double g[ED][DIM], gl[ED][DIM];")
    w("    for (int b = 0; b < ED; ++b) for (int i = 0; i < DIM; ++i) { g[b][i] = 0.0; gl[b][i] = 0.0; }")
    w("    double wE = sW[q], wL = 0.0;")
    w("    double tau[2] = {0.0, 0.0}, Nn[3] = {0.0, 0.0, 0.0};")
    if ed == d:
        w("    { double J; fe_metric_geometry<DIM, NN>(Xe, dps, g, J); wE = sW[q] * J;")
        w("      if (!(J > 0.0)) atomicExch(a.status, 1); }")
        if lagr:
            w("    { double J; fe_metric_geometry<DIM, NN>(X0, dps, gl, J); wL = sW[q] * J; }")
    elif ed == 1:
        if d != 2:
            raise NotImplementedError("line elements are implemented in 2D")
        w("    { double t0 = 0.0, t1 = 0.0;")
        w("      for (int l = 0; l < NN; ++l) { t0 += Xe[l * DIM] * dps[l]; t1 += Xe[l * DIM + 1] * dps[l]; }")
        w("      const double am = t0 * t0 + t1 * t1; const double J = sqrt(am);")
        w("      if (!(J > 0.0)) atomicExch(a.status, 1);")
        w("      wE = sW[q] * J; tau[0] = t0 / J; tau[1] = t1 / J; Nn[0] = tau[1]; Nn[1] = -tau[0];")
        w("      g[0][0] = t0 / am; g[0][1] = t1 / am; }")
    w("    for (int l = 0; l < NN; ++l) for (int i = 0; i < DIM; ++i) {")
    w("      double s1 = 0.0;")
    w("      for (int b = 0; b < ED; ++b) s1 += g[b][i] * dps[l * ED + b];")
    w("      dx[l * DIM + i] = s1;" + (f" fdx[l * DIM + i] = ({lt})s1;" if lowp else "") + " }")
    w("    for (int l = 0; l < N1; ++l) for (int i = 0; i < DIM; ++i) {")
    w("      double s1 = 0.0;")
    w("      for (int b = 0; b < ED; ++b) s1 += g[b][i] * dps1[l * ED + b];")
    w("      dx1[l * DIM + i] = s1;" + (f" fdx1[l * DIM + i] = ({lt})s1;" if lowp else "") + " }")
    if lagr:
        w("    for (int l = 0; l < NN; ++l) for (int i = 0; i < DIM; ++i) {")
        w("      double s2 = 0.0;")
        w("      for (int b = 0; b < ED; ++b) s2 += gl[b][i] * dps[l * ED + b];")
        w("      dX[l * DIM + i] = s2;" + (f" fdX[l * DIM + i] = ({lt})s2;" if lowp else "") + " }")
        w("    for (int l = 0; l < N1; ++l) for (int i = 0; i < DIM; ++i) {")
        w("      double s2 = 0.0;")
        w("      for (int b = 0; b < ED; ++b) s2 += gl[b][i] * dps1[l * ED + b];")
        w("      dX1[l * DIM + i] = s2;" + (f" fdX1[l * DIM + i] = ({lt})s2;" if lowp else "") + " }")
    w(f"    double U[{nf * NCU}];")
    w(f"    for (int c = 0; c < {nf * NCU}; ++c) U[c] = 0.0;")
    interp = 0
    for f, (nm, space, vi, _) in enumerate(fields):
        b0 = ici(f, 0)
        want = [c for c in range(NCU) if b0 + c in used_u]
        if not want:
            continue
        tder = bdf0 >= 0 and nh > 0 and (1 + 2 * d) in want
        nodes = list(range(nn)) if space == "C2" else list(c1)
        for s_, l in enumerate(nodes):
            psv = f"ps[{l}]" if space == "C2" else f"sPsi1[q * N1 + {s_}]"
            gxv = (lambda i: f"dx[{l * d + i}]") if space == "C2" else (lambda i: f"dx1[{s_ * d + i}]")
            gXv = (lambda i: f"dX[{l * d + i}]") if space == "C2" else (lambda i: f"dX1[{s_ * d + i}]")
            w(f"    {{ const double u = Uv[{l} * NVAL + {vi}];")
            for c in want:
                if c == 0:
                    w(f"      U[{b0}] += u * {psv};")
                elif c <= d:
                    w(f"      U[{b0 + c}] += u * {gxv(c - 1)};")
                elif c <= 2 * d:
                    w(f"      U[{b0 + c}] += u * {gXv(c - 1 - d)};")
                interp += 2 if c <= 2 * d else 0
            if tder:
                hs = " + ".join(f"P[{bdf0 + 1 + h}] * Uv[{(1 + h) * nn * nval + l * nval + vi}]" for h in range(nh))
                w(f"      U[{b0 + 1 + 2 * d}] += (P[{bdf0}] * u + {hs}) * {psv};")
                interp += 2 * (nh + 1) + 2
            w("    }")
    w("    double Xq[3] = {0.0, 0.0, 0.0}, XL[3] = {0.0, 0.0, 0.0};")
    w("    for (int l = 0; l < NN; ++l) for (int i = 0; i < DIM; ++i) "
      "{ Xq[i] += Xe[l * DIM + i] * ps[l]; XL[i] += X0[l * DIM + i] * ps[l]; }")
    w("    pointwise(U, Xq, XL, Nn, P, tau, wE, wL, rc, C, flag, a.aux);")
    w("    misc[0] = tau[0]; misc[1] = tau[1];")
    w("  }")
    w("  __syncthreads();")
    # threads take rows field by field (all elements' rows of field 0, then
    # field 1, ...) so that a warp runs one test field's code
    nsubs = [len(_sub_nodes(dc, f)) for f in range(nf)]
    w("  for (int p = threadIdx.x; p < EPB * NLOC; p += FE_NT) {")
    w("    int tf, el, ts, i;")
    off = 0
    roff = 0
    for f in range(nf):
        cond = "if" if f == 0 else "} else if"
        hi = off + epb * nsubs[f]
        w(f"    {cond} (p < {hi}) {{")
        w(f"      tf = {f}; el = (p - {off}) / {nsubs[f]}; ts = (p - {off}) - el * {nsubs[f]}; i = c_rowof[{roff} + ts];")
        off = hi
        roff += nsubs[f]
    w("    } else { tf = 0; el = EPB; ts = 0; i = 0; }")
    w("    if (el >= nel) continue;")
    w("    const double* ebq = sE + el * PER_EL + (1 + NH) * NN * NVAL + NN * DIM;")
    w("    double Racc = 0.0;")
    w("    jreal Jr[NLOC];")
    w("    for (int c = 0; c < NLOC; ++c) Jr[c] = (jreal)0;")
    w("    switch (tf) {")
    fl_rows_r = fl_rows_j = 0
    for tf in range(nf):
        tsp = fields[tf][1]
        w(f"    case {tf}: {{")
        w("      for (int q = 0; q < NQ; ++q) {")
        w("        const double* qb = ebq + q * QB;")
        w("        const double* dx = qb; const double* dX = dx + NN * DIM; const double* dx1 = dX + NN * DIM;")
        w("        const double* dX1 = dx1 + N1 * DIM; const double* rc = dX1 + N1 * DIM;")
        w("        const double* ps = sPsi2 + q * NN;")
        w("        (void)dx; (void)dX; (void)dx1; (void)dX1; (void)ps;")
        if lowp:
            w(f"        const {lt}* C = reinterpret_cast<const {lt}*>(ebq + NQ * QB) + q * FQB;")
            w(f"        const {lt}* fdx = C + NK; const {lt}* fdX = fdx + NN * DIM; const {lt}* fdx1 = fdX + NN * DIM;")
            w(f"        const {lt}* fdX1 = fdx1 + N1 * DIM; const {lt}* fps = sPsi2f + q * NN; const {lt}* fps1 = sPsi1f + q * N1;")
            w("        (void)fdx; (void)fdX; (void)fdx1; (void)fdX1; (void)fps; (void)fps1;")
        else:
            w("        const double* C = rc + NTC;")
        w("        (void)C;")
        jac_t = {tc - tf * NCT for tc, _ in keys if tc // NCT == tf}
        for c in range(NCT):
            if tci(tf, c) not in used_t:
                continue
            for single in ((False, True) if lowp else (False,)):
                pre = "f" if single else ""
                if c == 0:
                    src_ = (f"{pre}ps[ts]" if tsp == "C2" else
                            ("fps1[ts]" if single else "sPsi1[q * N1 + ts]"))
                elif c <= d:
                    src_ = f"{pre}dx[ts * DIM + {c - 1}]" if tsp == "C2" else f"{pre}dx1[ts * DIM + {c - 1}]"
                else:
                    src_ = f"{pre}dX[ts * DIM + {c - 1 - d}]" if tsp == "C2" else f"{pre}dX1[ts * DIM + {c - 1 - d}]"
                if single and c in jac_t:
                    w(f"        const {lt} fphi{c} = {src_};")
                elif not single and (not lowp or tci(tf, c) in rEn or tci(tf, c) in rLn):
                    w(f"        const double phi{c} = {src_};")
        rterms = [f"rc[{tci(tf, c)}] * phi{c}" for c in range(NCT) if (tci(tf, c) in rEn or tci(tf, c) in rLn)]
        n_rows_tf = sum(1 for r_ in rows_f if r_[0] == tf)
        fl_tr, fl_tj = 2 * len(rterms), 0
        if rterms:
            w(f"        Racc += {' + '.join(rterms)};")
        w("        if (flag == 1) {")
        av: Dict[int, List[str]] = {}
        avp: Dict[int, List[Tuple[str, str]]] = {}
        for kk, (tc, ic) in enumerate(keys):
            if tc // NCT == tf:
                av.setdefault(ic, []).append(f"{'f' if lowp else ''}phi{tc - tf * NCT} * C[{kk}]")
                avp.setdefault(ic, []).append((f"{'f' if lowp else ''}phi{tc - tf * NCT}", f"C[{kk}]"))

        def emit_av(ic, ind):
            # df64: compensated multiply-adds, renormalised once
            if df64:
                w(f"{ind}jreal av{ic} = (jreal)0; " + " ".join(f"fe_mac(av{ic}, {x_}, {y_});" for x_, y_ in avp[ic])
                  + f" av{ic} = fe_norm(av{ic});")
            else:
                w(f"{ind}const jreal av{ic} = {' + '.join(av[ic])};")
        for ic, lst in sorted(av.items()):
            emit_av(ic, "          ")
            fl_tj += 2 * len(lst)
        for g_ in range(nf):
            gsp = fields[g_][1]
            for s_, l in enumerate(_sub_nodes(dc, g_)):
                col = slot[(g_, l)]
                parts = []
                for ic in sorted(av):
                    gf, cc = divmod(ic, NCU)
                    if gf != g_:
                        continue
                    pre = "f" if lowp else ""
                    if gsp == "C2":
                        val, gx, gX = f"{pre}ps[{l}]", f"{pre}dx[{l * d} + {{i}}]", f"{pre}dX[{l * d} + {{i}}]"
                    else:
                        val = f"fps1[{s_}]" if lowp else f"sPsi1[q * N1 + {s_}]"
                        gx, gX = f"{pre}dx1[{s_ * d} + {{i}}]", f"{pre}dX1[{s_ * d} + {{i}}]"
                    if cc == 0:
                        parts.append((f"av{ic}", val))
                    elif cc <= d:
                        parts.append((f"av{ic}", gx.format(i=cc - 1)))
                    elif cc <= 2 * d:
                        parts.append((f"av{ic}", gX.format(i=cc - 1 - d)))
                    else:
                        parts.append((f"av{ic} * w0j", val))
                if parts:
                    if df64:
                        w("          " + " ".join(f"fe_mac(Jr[{col}], {x_}, {y_});" for x_, y_ in parts)
                          + f" Jr[{col}] = fe_norm(Jr[{col}]);")
                    elif f32:
                        w(f"          Jr[{col}] += {' + '.join(f'{x_} * {y_}' for x_, y_ in parts)};")
                    else:
                        # FP64: nested FMAs into the accumulator, one FP64 add
                        # fewer per update (the pipe that bounds the kernel)
                        ch = f"Jr[{col}]"
                        for x_, y_ in parts:
                            ch = f"fe_fma({x_}, {y_}, {ch})"
                        w(f"          Jr[{col}] = {ch};")
                    fl_tj += sum(_ops(f"{x_} * {y_}") for x_, y_ in parts) + len(parts)
        w("        }")
        # mass matrix: the coefficients of the time-derivative components, basis psi
        tics = sorted(ic for ic in av if ic % NCU == 1 + 2 * d)
        if tics:
            w("        if (flag == 2) {")
            for ic in tics:
                emit_av(ic, "          ")
            for g_ in range(nf):
                ic = g_ * NCU + 1 + 2 * d
                if ic not in tics:
                    continue
                for s_, l in enumerate(_sub_nodes(dc, g_)):
                    col = slot[(g_, l)]
                    if fields[g_][1] == "C2":
                        val = f"{'f' if lowp else ''}ps[{l}]"
                    else:
                        val = f"fps1[{s_}]" if lowp else f"sPsi1[q * N1 + {s_}]"
                    if df64:
                        w(f"          fe_mac(Jr[{col}], av{ic}, {val}); Jr[{col}] = fe_norm(Jr[{col}]);")
                    elif f32:
                        w(f"          Jr[{col}] += av{ic} * {val};")
                    else:
                        w(f"          Jr[{col}] = fe_fma(av{ic}, {val}, Jr[{col}]);")
            w("        }")
        w("      }")
        w("      break;")
        w("    }")
        fl_rows_r += n_rows_tf * fl_tr
        fl_rows_j += n_rows_tf * fl_tj
    # operation count per element: phase A per knot, phase B per (row, knot)
    geo = (2 * (2 * nn * d * EDs + 2 * EDs * EDs * d + 2 * EDs * EDs * d + 12) if ed == d else
           (4 * nn + 12 if ed == 1 else 0))
    geo += (nn + n1) * d * EDs * 2 * (2 if lagr else 1) + 4 * nn * d
    dc.flops = float(nq * (geo + interp + fl_point + fl_rows_r + (0 if lowp else fl_rows_j)))
    dc.flops32 = float(nq * fl_rows_j) if f32 else 0.0
    dc.flops_df64 = float(nq * fl_rows_j) if df64 else 0.0
    w("    default: break;")
    w("    }")
    w("    const long long row = (e0 + el) * NLOC + i;")
    w("    a.rbuf[row] = Racc;")
    w("    if (flag == 1 || flag == 2) {")
    w("      jstore* jb = reinterpret_cast<jstore*>(a.jbuf) + row * NLOC;")
    w("      for (int c = 0; c < NLOC; ++c) jb[c] = fe_jstore(Jr[c]);")
    w("    }")
    w("  }")
    w("}")
    w(f"}}  // namespace dom{k}")
    return "\n".join(L)


@dataclass
class FusedKernel:
    source: str
    name: str
    threads: int
    smem_bytes: int
    domains: List[DomainCode]
    params: List[str]
    jac_precision: str


def generate_fused(domains: List[DomainCode], dim: int, params: List[str], nval: int, nh: int,
                   jac_precision: str = "f64", smem_budget: int = 100 * 1024,
                   nthreads_cap: int = 256, rows_per_thread: int = 1) -> FusedKernel:
    """One kernel for all domains: block b runs the domain whose block range
    [block_start[k], block_start[k+1]) of the runtime's FeFusedArgs holds b."""
    if len(domains) > 4:
        raise ValueError("at most 4 fused domains")
    if jac_precision not in ("f64", "f32", "df64"):
        raise ValueError(f"unknown Jacobian precision {jac_precision!r}")
    jreal = {"f64": "double", "f32": "float", "df64": "fe_df64"}[jac_precision]
    jstore = "float" if jac_precision == "f32" else "double"
    bodies = [_domain_source(k, dc, dim, params, nval, nh, smem_budget, nthreads_cap, jac_precision == "f32",
                             jac_precision == "df64", rows_per_thread)
              for k, dc in enumerate(domains)]
    threads = max(32, max(((dc.rows_needed + 31) // 32) * 32 for dc in domains))
    smem = max(dc.smem for dc in domains)
    head = ["// generated fused multi-domain element kernel", '#include "fe_device.cuh"',
            f"typedef {jreal} jreal;", f"typedef {jstore} jstore;", f"#define FE_NT {threads}"]
    src = "\n".join(head + bodies)
    h = hashlib.sha1(src.encode()).hexdigest()[:12]
    name = f"fe_fused_{jac_precision}_{h}"
    # persistent: the grid is sized to the SMs' resident blocks and each block
    # walks the element blocks of every domain (bulk first, then the small
    # interface and contact-line domains) with a static stride
    tail = [f'extern "C" __global__ void __launch_bounds__(FE_NT) {name}(const FeFusedArgs fa) {{',
            "  extern __shared__ __align__(16) unsigned char fe_smem[];",
            "  double* sW = reinterpret_cast<double*>(fe_smem);",
            "  for (int b = blockIdx.x; b < fa.block_start[fa.n_domains]; b += gridDim.x) {"]
    for k in range(len(domains)):
        cond = "if" if k == 0 else "else if"
        tail.append(f"    {cond} (b < fa.block_start[{k + 1}]) dom{k}::run(fa.d[{k}], b - fa.block_start[{k}], sW);")
    tail.append("    __syncthreads();  // the next element block reuses the shared memory")
    tail.append("  }")
    tail.append("}")
    src = src + "\n" + "\n".join(tail) + "\n"
    return FusedKernel(src, name, threads, smem, domains, params, jac_precision)


# ---------------------------------------------------------------------------
# droplet mesh
# ---------------------------------------------------------------------------
def quarter_disk(x: np.ndarray, radius: float = 1.0) -> np.ndarray:
    """Map of the unit square onto the quarter disk of the given radius:
    (x sqrt(1 - y^2/2), y sqrt(1 - x^2/2)); the right and top sides go to
    the arc, the left side to the axis, the bottom to the substrate."""
    X, Y = x[:, 0], x[:, 1]
    return radius * np.stack([X * np.sqrt(1.0 - 0.5 * Y * Y), Y * np.sqrt(1.0 - 0.5 * X * X)], axis=1)


@dataclass
class DropletMesh:
    x: np.ndarray               # [n_nodes, 2] positions (reference configuration)
    conn: np.ndarray            # [n_tri, 6] P2 triangles
    is_vertex: np.ndarray       # [n_nodes]
    boundaries: Dict[str, np.ndarray]
    interface: np.ndarray       # [n_line, 3] counterclockwise line elements on the arc
    contact_line: np.ndarray    # [1, 1]


_TRI_EDGES = ((0, 3, 1), (1, 4, 2), (2, 5, 0))


def droplet_mesh(N: int, radius: float = 1.0) -> DropletMesh:
    """P2 triangles of an N x N split square mapped to the quarter disk.  The
    interface elements are the triangle edges on the arc, created element by
    element in bulk order, each edge oriented like its (counterclockwise)
    triangle, so the outward normal is (tau_1, -tau_0)."""
    md = RectangularQuadMesh(N=N, size=1.0, split_in_tris="left").generate()
    b = md.boundaries
    lines = []
    for e in range(md.conn.shape[0]):
        c = md.conn[e]
        for (i, m, j) in _TRI_EDGES:
            nodes = (c[i], c[m], c[j])
            for side in ("right", "top"):
                if all(b[side][n] for n in nodes):
                    lines.append(nodes)
    inter = np.array(lines, dtype=np.int32).reshape(-1, 3)
    cl = np.nonzero(b["right"] & b["bottom"])[0].astype(np.int32).reshape(1, 1)
    x = quarter_disk(md.x, radius)
    return DropletMesh(x, md.conn.astype(np.int32), md.is_vertex, dict(b), inter, cl)


def bdf_weights(order: int, dt: float, dt_prev: Optional[float] = None) -> Tuple[float, float, float]:
    """d/dt weights of (current, previous, before previous) values: BDF1, or
    BDF2 for variable steps, with the expressions of pyoomph's
    MultiTimeStepper::set_weights (src/timestepper.cpp:32-52, as oomph's
    BDF<2>::set_weights, timesteppers.cc:232-245), so that the weights are
    the reference's to the bit."""
    if order == 1:
        return 1.0 / dt, -1.0 / dt, 0.0
    dtprev = dt_prev if dt_prev else dt
    return (1.0 / dt + 1.0 / (dt + dtprev), -(dt + dtprev) / (dt * dtprev), dt / ((dt + dtprev) * dtprev))


# ---------------------------------------------------------------------------
# the droplet problem
# ---------------------------------------------------------------------------
VALUE_ORDER = ("mesh_x", "mesh_y", "velocity_x", "velocity_y", "pressure", "_kin_bc")

_FUSED_CACHE: Dict[str, "N.Code"] = {}


class DropletProblem:
    """Axisymmetric sessile droplet relaxing to its contact angle: Stokes
    flow (viscosity = Ohnesorge number, surface tension 1) in a drop on a
    pseudo-elastic moving mesh, a free surface with kinematic multiplier,
    and the contact-angle condition at the contact line; BDF2 in time
    (BDF1 on the first step).

    Nodal values per node (``VALUE_ORDER``): positions first, then the
    values -- oomph's numbering of solid nodes (``SolidNode::assign_eqn_numbers``,
    ``nodes.cc:3652-3659``: position data, then nodal data).  Axis: u_r = 0,
    r pinned; substrate: u_z = 0, z pinned (free slip)."""

    def __init__(self, N: int = 8, contact_angle_deg: float = 90.0, ohnesorge: float = 0.1,
                 surface_tension: float = 1.0, radius: float = 1.0, jacobian_precision: str = "fp64"):
        self.N = N
        self.theta = math.radians(contact_angle_deg)
        self.mu = ohnesorge
        self.sigma = surface_tension
        self.radius = radius
        self.jacobian_precision = jacobian_precision
        self.newton_solver_tolerance = 1e-8
        self.max_newton_iterations = 10
        self.max_residuals = 1e10
        self.linear_solver = None
        self.time = 0.0
        self.steps_done = 0
        self.dt_prev: Optional[float] = None
        self._initialised = False
        self.timings: Dict[str, float] = {}
        self.newton_history: List[float] = []
        # launch shape of the fused kernel: thread cap and shared-memory budget
        # per block (both decide elements per block) and local rows per
        # thread of the row phase (threads per element: max(knots, rows /
        # rows_per_thread); the bulk P2 element has 27 rows and 7 knots, so
        # one thread per row leaves three quarters of the block idle in the
        # knot phase).  Defaults: the fastest shapes measured on GB300 for
        # the droplet, side 110 (FP64 J: 4 rows per thread, 512 threads /
        # 200 KB, 0.861 -> 0.732 ms; FP32 J: 2 rows per thread, 128 threads /
        # 64 KB, 0.345 -> 0.307 ms; both give the bits of one thread per row)
        f64 = jacobian_precision in ("fp64", "f64", "df64")
        self.nthreads_cap = 512 if f64 else 128
        self.smem_budget = (200 if f64 else 64) * 1024
        self.rows_per_thread = 4 if f64 else 2
        # compile the element code with device-side bounds checks (status word 2)
        self.bounds_check = False

    # -- lowering (no GPU) ----------------------------------------------
    def lower(self) -> FusedKernel:
        if getattr(self, "kernel", None) is not None:
            return self.kernel
        E.set_dimension(2)
        m = droplet_mesh(self.N, self.radius)
        self.mesh = m
        nval = len(VALUE_ORDER)
        vi = {nm: i for i, nm in enumerate(VALUE_ORDER)}
        bulk_eqs = [AxisymmetricStokesEquations(self.mu), PseudoElasticMesh()]
        surf_eqs = [FreeSurface(self.sigma)]
        pt_eqs = [ContactAngle(self.theta, self.sigma)]
        pvals: Dict[str, float] = {}
        for eqs in (bulk_eqs, surf_eqs, pt_eqs):
            for e in eqs:
                e.define_fields()
        for eqs in (bulk_eqs, surf_eqs, pt_eqs):
            for e in eqs:
                e.define_residuals()
                pvals.update(e.param_values)
        for i in range(3):
            pvals[f"__bdf{i}"] = 0.0
        self.param_names = sorted(pvals, key=E.parameter_order_key)
        self.params = np.array([pvals[p] for p in self.param_names])

        def dom(dtype, eqs, names_spaces):
            flds = [(nm, sp_, vi[nm], nm in E.MESH_FIELDS) for nm, sp_ in names_spaces]
            flds = [f for f in flds if not f[3]] + [f for f in flds if f[3]]
            rE = sum((e.rE for e in eqs), sp.Integer(0))
            rL = sum((e.rL for e in eqs), sp.Integer(0))
            return DomainCode(dtype, flds, rE, rL)

        pos = [("mesh_x", "C2"), ("mesh_y", "C2")]
        vel = [("velocity_x", "C2"), ("velocity_y", "C2")]
        self.domains = [
            dom(TRI6, bulk_eqs, vel + [("pressure", "C1")] + pos),
            dom(LINE3, surf_eqs, vel + [("_kin_bc", "C2")] + pos),
            dom(POINT1, pt_eqs, vel + pos),
        ]
        jp = self.jacobian_precision
        kprec = "df64" if jp == "df64" else ("f64" if jp in ("fp64", "f64") else "f32")
        prec = "f32" if kprec == "f32" else "f64"   # storage of the Jacobian values
        self._prec = prec
        self.kernel = generate_fused(self.domains, 2, self.param_names, nval, 2, kprec,
                                     smem_budget=self.smem_budget, nthreads_cap=self.nthreads_cap,
                                     rows_per_thread=self.rows_per_thread)
        self.conns = [m.conn, m.interface, m.contact_line]
        n = m.x.shape[0]
        present = np.ones((n, nval), dtype=bool)
        present[:, vi["pressure"]] = m.is_vertex
        on_if = np.zeros(n, dtype=bool)
        on_if[m.interface.ravel()] = True
        present[:, vi["_kin_bc"]] = on_if
        pinned = np.zeros((n, nval), dtype=bool)
        axis, sub = m.boundaries["left"], m.boundaries["bottom"]
        pinned[axis, vi["velocity_x"]] = True
        pinned[axis, vi["mesh_x"]] = True
        pinned[sub, vi["velocity_y"]] = True
        pinned[sub, vi["mesh_y"]] = True
        values = np.zeros((n, nval))
        values[:, vi["mesh_x"]] = m.x[:, 0]
        values[:, vi["mesh_y"]] = m.x[:, 1]
        free = present & ~pinned
        eqn = np.full((n, nval), -1, dtype=np.int32)
        self.n_dof = int(free.sum())
        eqn.reshape(-1)[free.reshape(-1)] = np.arange(self.n_dof, dtype=np.int32)
        self.eqn, self.present, self.pinned, self._values0 = eqn, present, pinned, values
        self.n_nodes, self.nval = n, nval
        self.n_elem = sum(c.shape[0] for c in self.conns)
        return self.kernel

    def _descriptors(self, with_code: bool):
        k = self.kernel
        keep = dict(x=np.ascontiguousarray(self.mesh.x, dtype=np.float64),
                    eqn=np.ascontiguousarray(self.eqn),
                    params=np.ascontiguousarray(self.params.copy()))
        dds = []
        for i, (dc, conn) in enumerate(zip(self.domains, self.conns)):
            keep[f"conn{i}"] = np.ascontiguousarray(conn, dtype=np.int32)
            keep[f"ln{i}"] = np.ascontiguousarray(dc.layout_node, dtype=np.int32)
            keep[f"lv{i}"] = np.ascontiguousarray(dc.layout_val, dtype=np.int32)
            keep[f"tab{i}"] = np.ascontiguousarray(dc.dtype.tables(), dtype=np.float64)
            dds.append(N.DomainDesc(self.code.handle if with_code else None, dc.dtype.nnode, dc.nloc,
                                    conn.shape[0], keep[f"conn{i}"].ctypes.data, keep[f"ln{i}"].ctypes.data,
                                    keep[f"lv{i}"].ctypes.data, keep[f"tab{i}"].ctypes.data,
                                    keep[f"tab{i}"].size, dc.epb, k.threads, k.smem_bytes, 0))
        doms = (N.DomainDesc * len(dds))(*dds)
        desc = N.ProblemDesc(2, self.n_nodes, self.nval, keep["x"].ctypes.data, keep["eqn"].ctypes.data,
                             self.n_dof, len(dds), doms, len(self.params), keep["params"].ctypes.data,
                             N.FE_JAC_F64 if self._prec == "f64" else N.FE_JAC_F32, 0, 2,
                             keep["x"].ctypes.data, 1)
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

    # -- device ----------------------------------------------------------
    def initialise(self) -> None:
        if self._initialised:
            return
        import torch
        if not torch.cuda.is_available():
            raise N.FeError(N.FE_ERR_NOGPU, "pyoomph_gb300 needs a CUDA GPU (none visible)")
        self.lower()
        t0 = time.perf_counter()
        ckey = self.kernel.name + ("+bounds" if self.bounds_check else "")
        self.code = _FUSED_CACHE.get(ckey)
        if self.code is None:
            src = ("#define FE_BOUNDS_CHECK 1\n" if self.bounds_check else "") + self.kernel.source
            self.code = N.Code(src, self.kernel.name)
            _FUSED_CACHE[ckey] = self.code
        t1 = time.perf_counter()
        L = N.load()
        desc, self._doms, self._keep = self._descriptors(with_code=True)
        h = ctypes.c_void_p()
        N.check(L.fe_problem_create(ctypes.byref(desc), ctypes.byref(h)))
        self._h = h
        v = np.ascontiguousarray(self._values0)
        N.check(L.fe_problem_set_values(h, v.ctypes.data))
        for lev in range(2):
            N.check(L.fe_problem_set_history(h, lev, v.ctypes.data))
        nd, nnz = ctypes.c_int64(), ctypes.c_int64()
        N.check(L.fe_problem_sizes(h, ctypes.byref(nd), ctypes.byref(nnz)))
        self.nnz = nnz.value
        dev = torch.device("cuda")
        jd = torch.float64 if self._prec == "f64" else torch.float32
        self.x_dev = torch.zeros(max(self.n_dof, 1), dtype=torch.float64, device=dev)
        self.R_dev = torch.zeros(max(self.n_dof, 1), dtype=torch.float64, device=dev)
        self.J_dev = torch.zeros(max(self.nnz, 1), dtype=jd, device=dev)
        self.x_dev[:self.n_dof].copy_(torch.from_numpy(self._dofs_from_values(self._values0)))
        self._initialised = True
        self._pattern_cache = self.pattern()
        self.timings.update(jit_s=t1 - t0, device_setup_s=time.perf_counter() - t1)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.load().fe_problem_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def _dofs_from_values(self, values: np.ndarray) -> np.ndarray:
        x = np.zeros(self.n_dof)
        msk = self.eqn >= 0
        x[self.eqn[msk]] = values[msk]
        return x

    def pattern(self) -> Tuple[np.ndarray, np.ndarray]:
        rp = np.zeros(self.n_dof + 1, dtype=np.int32)
        ci = np.zeros(max(self.nnz, 1), dtype=np.int32)
        N.check(N.load().fe_problem_pattern(self._h, rp.ctypes.data, ci.ctypes.data))
        return rp, ci[:self.nnz]

    def set_params(self, **kw) -> None:
        for k_, v in kw.items():
            self.params[self.param_names.index(k_)] = float(v)
        if self._initialised:
            self._keep["params"][:] = self.params
            N.check(N.load().fe_problem_set_params(self._h, self._keep["params"].ctypes.data))

    def set_state(self, values: np.ndarray, history: Optional[List[np.ndarray]] = None) -> None:
        """Nodal values (and previous time levels), each [n_nodes, nval]."""
        import torch
        self.initialise()
        L = N.load()
        v = np.ascontiguousarray(values, dtype=np.float64)
        N.check(L.fe_problem_set_values(self._h, v.ctypes.data))
        for lev, hv in enumerate(history or []):
            hv = np.ascontiguousarray(hv, dtype=np.float64)
            N.check(L.fe_problem_set_history(self._h, lev, hv.ctypes.data))
        self.x_dev[:self.n_dof].copy_(torch.from_numpy(self._dofs_from_values(v)))

    def get_values(self) -> np.ndarray:
        v = np.zeros((self.n_nodes, self.nval))
        N.check(N.load().fe_problem_get_values(self._h, v.ctypes.data))
        return v

    def assemble_device(self, with_jacobian: bool = True, stream=None) -> None:
        import torch
        flags = N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_VALUES_FROM_DOFS
        if with_jacobian:
            flags |= N.FE_ASSEMBLE_JACOBIAN
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(),
                                     self.J_dev.data_ptr(), flags, ctypes.c_void_p(st)))

    def check(self) -> None:
        N.check(N.load().fe_problem_check(self._h))

    def set_persistent(self, enable: bool) -> None:
        """Persistent fused launch (grid of resident blocks) or one block per
        element block (default)."""
        self.initialise()
        N.check(N.load().fe_problem_set_persistent(self._h, int(enable)))

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

    def launch_count(self, with_jacobian: bool = True) -> int:
        flags = N.FE_ASSEMBLE_RESIDUAL | N.FE_ASSEMBLE_VALUES_FROM_DOFS
        if with_jacobian:
            flags |= N.FE_ASSEMBLE_JACOBIAN
        return N.load().fe_problem_launch_count(self._h, flags)

    def set_stage_timing(self, enable: bool) -> None:
        N.check(N.load().fe_problem_set_timing(self._h, int(enable)))

    def stage_times(self):
        ms = np.zeros(5)
        calls = ctypes.c_int64()
        N.check(N.load().fe_problem_stage_times(self._h, ms.ctypes.data, ctypes.byref(calls)))
        return ms, calls.value

    def element_buffers(self, domain: int):
        """(R_e, J_e) of one domain from the last assembly."""
        dc = self.domains[domain]
        ne = self.conns[domain].shape[0]
        R = np.zeros((ne, dc.nloc))
        J = np.zeros((ne, dc.nloc, dc.nloc), dtype=np.float64 if self._prec == "f64" else np.float32)
        N.check(N.load().fe_problem_element_buffers(self._h, domain, R.ctypes.data, J.ctypes.data))
        return R, J

    def get_residuals(self) -> np.ndarray:
        self.initialise()
        self.assemble_device(with_jacobian=False)
        self.check()
        return self.R_dev[:self.n_dof].cpu().numpy()

    def get_jacobian(self):
        import scipy.sparse as sps
        self.initialise()
        self.assemble_device(with_jacobian=True)
        self.check()
        R = self.R_dev[:self.n_dof].cpu().numpy()
        rp, ci = self._pattern_cache
        vals = self.J_dev[:self.nnz].cpu().numpy().astype(np.float64)
        return R, sps.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))

    def get_mass_matrix(self):
        """The mass matrix dR/d(du/dt) at the current dofs in the Jacobian's
        CSR pattern (pyoomph's mass-matrix assembly, flag 2 of the generated
        element code).  Leaves J_dev holding M."""
        import scipy.sparse as sps
        import torch
        self.initialise()
        st = torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(), self.J_dev.data_ptr(),
                                     N.FE_ASSEMBLE_MASS | N.FE_ASSEMBLE_VALUES_FROM_DOFS, ctypes.c_void_p(st)))
        self.check()
        rp, ci = self._pattern_cache
        vals = self.J_dev[:self.nnz].cpu().numpy().astype(np.float64)
        return sps.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))

    def get_parameter_derivative(self, name: str) -> np.ndarray:
        """dR/dp of one global parameter at the current dofs
        (dResidual{i}dParameter_{k} of pyoomph's generated code)."""
        import torch
        self.initialise()
        N.check(N.load().fe_problem_set_dparam(self._h, self.param_names.index(name)))
        st = torch.cuda.current_stream().cuda_stream
        N.check(N.load().fe_assemble(self._h, self.x_dev.data_ptr(), self.R_dev.data_ptr(), self.J_dev.data_ptr(),
                                     N.FE_ASSEMBLE_DPARAM | N.FE_ASSEMBLE_VALUES_FROM_DOFS, ctypes.c_void_p(st)))
        self.check()
        return self.R_dev[:self.n_dof].cpu().numpy()

    def residual_max(self) -> float:
        import torch
        out = ctypes.c_double()
        N.check(N.load().fe_residual_max(self._h, self.R_dev.data_ptr(), self.n_dof, ctypes.byref(out),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return out.value

    # -- Newton and time stepping ------------------------------------------
    def newton(self) -> List[float]:
        import scipy.sparse as sps
        import scipy.sparse.linalg as spla
        import torch
        self.initialise()
        rp, ci = self._pattern_cache
        hist = []
        t_asm = t_lin = 0.0
        self.assemble_device(with_jacobian=False)
        hist.append(self.residual_max())
        it = 0
        while hist[-1] >= self.newton_solver_tolerance:
            if it >= self.max_newton_iterations or hist[-1] > self.max_residuals:
                raise RuntimeError(f"Newton failed: residuals {hist}")
            ta = time.perf_counter()
            with nvtx_range("fused assembly R+J"):
                self.assemble_device(with_jacobian=True)
                self.check()
                R = self.R_dev[:self.n_dof].cpu().numpy()
                vals = self.J_dev[:self.nnz].cpu().numpy().astype(np.float64)
            tb = time.perf_counter()
            with nvtx_range("linear solve"):
                A = sps.csr_matrix((vals, ci, rp), shape=(self.n_dof, self.n_dof))
                dx = self.linear_solver(A, R) if self.linear_solver else spla.splu(A.tocsc()).solve(R)
            tc = time.perf_counter()
            dxd = torch.as_tensor(dx, device=self.x_dev.device)
            N.check(N.load().fe_dof_update(self._h, self.x_dev.data_ptr(), dxd.data_ptr(), self.n_dof,
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
            self.assemble_device(with_jacobian=False)
            hist.append(self.residual_max())
            t_asm += tb - ta
            t_lin += tc - tb
            it += 1
        self.check()
        self.newton_history = hist
        self.timings.update(newton_assembly_s=t_asm, newton_linear_solve_s=t_lin, newton_iterations=it)
        return hist

    def step(self, dt: float) -> List[float]:
        """One implicit time step (pyoomph's unsteady_newton_solve): shift the
        time levels, set the BDF weights (BDF1 on the first step), Newton."""
        self.initialise()
        N.check(N.load().fe_problem_shift_history(self._h))
        order = 1 if self.steps_done == 0 else 2
        w = bdf_weights(order, dt, self.dt_prev)
        self.set_params(__bdf0=w[0], __bdf1=w[1], __bdf2=w[2])
        hist = self.newton()
        self.steps_done += 1
        self.dt_prev = dt
        self.time += dt
        return hist
