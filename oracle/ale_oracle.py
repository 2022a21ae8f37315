"""CPU oracle for the moving-mesh (ALE) droplet assembly.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py`` as the checker; never by the
package ``pyoomph_gb300``.

An independent restatement, in numpy, of the element residuals of an
axisymmetric sessile droplet in pyoomph:

* bulk (P2 triangles, TGauss<2,3>): axisymmetric Stokes
  (``pyoomph/equations/navier_stokes.py:303-345``) on the Eulerian
  configuration plus the pseudo-elastic mesh (``equations/ALE.py:128-147``)
  on the Lagrangian one;
* interface (3-node lines, TGauss<1,3>): kinematic condition with the
  multiplier ``_kin_bc``, its reaction on the mesh, and surface tension
  (``navier_stokes.py:605-676``);
* contact line (one node): ``sigma m . v`` (``navier_stokes.py:1054-1088``);

written directly from the geometry (determinants, inverse Jacobians, the
tangent of the line) rather than through the weak-form compiler.  Element
Jacobians come from complex-step differentiation of these residuals
(``J[:, k] = Im R(x + i h e_k) / h``, h = 1e-30), which is exact to
rounding and so checks every position (shape-derivative) term of the
generated Jacobian without finite-difference error.  The sparse assembly
restates oomph's vectors-of-pairs assembler (``problem.cc:5332-5666``;
structural pattern, entries in first-insertion order, contributions summed
in element order).

Parity: the shape tables of the bulk come from ``fe_oracle.c`` (pinned
against oomph-lib's own tables); the droplet weak forms themselves are not
pinned by a run of the reference (pyoomph's GiNaC code generator cannot be
built here), only restated from its source.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np

import oracle as O

VALUES = ("mesh_x", "mesh_y", "velocity_x", "velocity_y", "pressure", "_kin_bc")
VI = {n: i for i, n in enumerate(VALUES)}
H_CS = 1e-30

# TGauss<1,3> (integral.cc:311-316)
_K = 0.774596669241483
LINE_S = np.array([0.5 * (1.0 - _K), 0.5, 0.5 * (1.0 + _K)])
LINE_W = np.array([5.0, 8.0, 5.0]) / 18.0


def line_shapes(s):
    """TElement<1,3> (Telements.h:347-366): nodes at s = 0, 1/2, 1."""
    psi = np.array([2.0 * (s - 1.0) * (s - 0.5), 4.0 * (1.0 - s) * s, 2.0 * (s - 0.5) * s])
    dpsi = np.array([4.0 * s - 3.0, 4.0 - 8.0 * s, 4.0 * s - 1.0])
    return psi, dpsi


def tri_tables():
    L = O.lib()
    nq = L.ofe_n_intpt(O.P2_TRI)
    w = np.zeros(nq)
    psi, dpsi = np.zeros((nq, 6)), np.zeros((nq, 6, 2))
    psi1, dpsi1 = np.zeros((nq, 3)), np.zeros((nq, 3, 2))
    for q in range(nq):
        s = np.zeros(3)
        wq = np.zeros(1)
        L.ofe_intpt(O.P2_TRI, q, O._ptr(s), O._ptr(wq))
        w[q] = wq[0]
        p, d = np.zeros(6), np.zeros((6, 2))
        L.ofe_shape_c2(O.P2_TRI, O._ptr(s), O._ptr(p), O._ptr(d))
        psi[q], dpsi[q] = p, d
        p1, d1 = np.zeros(3), np.zeros((3, 2))
        L.ofe_shape_c1(O.P2_TRI, O._ptr(s), O._ptr(p1), O._ptr(d1))
        psi1[q], dpsi1[q] = p1, d1
    return w, psi, dpsi, psi1, dpsi1


# ---------------------------------------------------------------------------
# mesh, pins and numbering
# ---------------------------------------------------------------------------
@dataclass
class Droplet:
    x0: np.ndarray            # [n, 2] reference positions
    tri: np.ndarray           # [E, 6]
    line: np.ndarray          # [Ei, 3]
    point: np.ndarray         # [1, 1]
    present: np.ndarray       # [n, 6] bool
    pinned: np.ndarray        # [n, 6] bool
    eqn: np.ndarray           # [n, 6] int
    n_dof: int


def droplet(N: int, radius: float = 1.0) -> Droplet:
    """Split-square P2 mesh (oracle mesh generator, pyoomph order) mapped to
    the quarter disk; arc edges as counterclockwise line elements in bulk
    element order; the contact-line node; pins (axis: u_r and r, substrate:
    u_z and z) and equation numbers (positions first at each node)."""
    m = O.mesh(O.P2_TRI, N, N, split=0)
    X, Y = m.x[:, 0], m.x[:, 1]
    x0 = radius * np.stack([X * np.sqrt(1 - 0.5 * Y * Y), Y * np.sqrt(1 - 0.5 * X * X)], axis=1)
    bm = m.bmask
    lines = []
    for c in m.conn:
        for (a, mid, b) in ((0, 3, 1), (1, 4, 2), (2, 5, 0)):
            for bit in (O.B_RIGHT, O.B_TOP):
                if all(bm[c[k]] & bit for k in (a, mid, b)):
                    lines.append((c[a], c[mid], c[b]))
    line = np.array(lines, dtype=np.int32)
    cl = [i for i in range(len(bm)) if (bm[i] & O.B_RIGHT) and (bm[i] & O.B_BOTTOM)]
    n = x0.shape[0]
    present = np.ones((n, 6), dtype=bool)
    present[:, VI["pressure"]] = m.is_vertex.astype(bool)
    onif = np.zeros(n, dtype=bool)
    onif[line.ravel()] = True
    present[:, VI["_kin_bc"]] = onif
    pinned = np.zeros((n, 6), dtype=bool)
    axis = (bm & O.B_LEFT) != 0
    sub = (bm & O.B_BOTTOM) != 0
    pinned[axis, VI["velocity_x"]] = pinned[axis, VI["mesh_x"]] = True
    pinned[sub, VI["velocity_y"]] = pinned[sub, VI["mesh_y"]] = True
    eqn = np.full((n, 6), -1, dtype=np.int64)
    k = 0
    for i in range(n):
        for v in range(6):
            if present[i, v] and not pinned[i, v]:
                eqn[i, v] = k
                k += 1
    return Droplet(x0, m.conn.astype(np.int32), line, np.array([cl], dtype=np.int32), present, pinned, eqn, k)


def initial_values(D: Droplet) -> np.ndarray:
    v = np.zeros((D.x0.shape[0], 6))
    v[:, 0:2] = D.x0
    return v


# local layouts: nodal values node by node, then positions node by node
def bulk_layout():
    lay = []
    for l in range(6):
        lay += [(l, VI["velocity_x"]), (l, VI["velocity_y"])]
        if l < 3:
            lay.append((l, VI["pressure"]))
    for l in range(6):
        lay += [(l, 0), (l, 1)]
    return lay


def line_layout():
    lay = []
    for l in range(3):
        lay += [(l, VI["velocity_x"]), (l, VI["velocity_y"]), (l, VI["_kin_bc"])]
    for l in range(3):
        lay += [(l, 0), (l, 1)]
    return lay


def point_layout():
    return [(0, VI["velocity_x"]), (0, VI["velocity_y"]), (0, 0), (0, 1)]


# ---------------------------------------------------------------------------
# element residuals (vectorised over elements; complex-safe)
# ---------------------------------------------------------------------------
def _gather(vals: np.ndarray, conn: np.ndarray, layout) -> np.ndarray:
    return np.stack([vals[conn[:, l], v] for (l, v) in layout], axis=1)


def bulk_residual(loc: np.ndarray, X0e: np.ndarray, p: Dict[str, float]) -> np.ndarray:
    """loc [E, 27] local values in bulk_layout order; X0e [E, 6, 2]."""
    w, psi, dpsi, psi1, dpsi1 = tri_tables()
    E = loc.shape[0]
    ux = loc[:, [0, 3, 6, 9, 11, 13]]
    uy = loc[:, [1, 4, 7, 10, 12, 14]]
    pr = loc[:, [2, 5, 8]]
    xs = loc[:, 15::2]
    ys = loc[:, 16::2]
    mu, Em, nu = p["dynamic_viscosity"], p.get("E", 1.0), p.get("nu", 0.3)
    mum = Em / 2 / (1 + nu)
    lam = Em * nu / (1 + nu) / (1 - 2 * nu)
    lam = 2 * mum * lam / (lam + 2 * mum)
    R = np.zeros((E, 27), dtype=loc.dtype)
    for q in range(len(w)):
        # Eulerian geometry: t[a][i] = dx_i/ds_a
        t00 = xs @ dpsi[q, :, 0]
        t01 = ys @ dpsi[q, :, 0]
        t10 = xs @ dpsi[q, :, 1]
        t11 = ys @ dpsi[q, :, 1]
        det = t00 * t11 - t01 * t10
        # weight: sqrt of the metric determinant (fill_shape_info_at_s), |det t|
        Jw = np.sqrt((t00 * t00 + t01 * t01) * (t10 * t10 + t11 * t11) - (t00 * t10 + t01 * t11) ** 2)
        # dpsi/dx_i = sum_a inv(t)[i][a] dpsi/ds_a, inv(t) = [[t11, -t01], [-t10, t00]] / det
        dpx = (t11[:, None] * dpsi[q, :, 0] - t01[:, None] * dpsi[q, :, 1]) / det[:, None]
        dpy = (-t10[:, None] * dpsi[q, :, 0] + t00[:, None] * dpsi[q, :, 1]) / det[:, None]
        d1x = (t11[:, None] * dpsi1[q, :, 0] - t01[:, None] * dpsi1[q, :, 1]) / det[:, None]
        d1y = (-t10[:, None] * dpsi1[q, :, 0] + t00[:, None] * dpsi1[q, :, 1]) / det[:, None]
        r = xs @ psi[q]
        W = w[q] * Jw * 2 * math.pi * r
        u0, u1 = ux @ psi[q], uy @ psi[q]
        du0dx, du0dy = (ux * dpx).sum(1), (ux * dpy).sum(1)
        du1dx, du1dy = (uy * dpx).sum(1), (uy * dpy).sum(1)
        P = pr @ psi1[q]
        s_xx = 2 * mu * du0dx - P
        s_yy = 2 * mu * du1dy - P
        s_xy = mu * (du0dy + du1dx)
        s_tt = 2 * mu * u0 / r - P
        # velocity tests
        for l, (ix, iy) in enumerate(zip([0, 3, 6, 9, 11, 13], [1, 4, 7, 10, 12, 14])):
            R[:, ix] += W * (s_xx * dpx[:, l] + s_xy * dpy[:, l] + s_tt * psi[q, l] / r)
            R[:, iy] += W * (s_xy * dpx[:, l] + s_yy * dpy[:, l])
        divu = du0dx + du1dy + u0 / r
        for l, ip in enumerate([2, 5, 8]):
            R[:, ip] += W * divu * psi1[q, l]
        # Lagrangian geometry and the pseudo-elastic mesh
        T00 = X0e[:, :, 0] @ dpsi[q, :, 0]
        T01 = X0e[:, :, 1] @ dpsi[q, :, 0]
        T10 = X0e[:, :, 0] @ dpsi[q, :, 1]
        T11 = X0e[:, :, 1] @ dpsi[q, :, 1]
        detL = T00 * T11 - T01 * T10
        JL = np.sqrt((T00 * T00 + T01 * T01) * (T10 * T10 + T11 * T11) - (T00 * T10 + T01 * T11) ** 2)
        dPx = (T11[:, None] * dpsi[q, :, 0] - T01[:, None] * dpsi[q, :, 1]) / detL[:, None]
        dPy = (-T10[:, None] * dpsi[q, :, 0] + T00[:, None] * dpsi[q, :, 1]) / detL[:, None]
        Dx = xs - X0e[:, :, 0]
        Dy = ys - X0e[:, :, 1]
        e_xx = (Dx * dPx).sum(1)
        e_yy = (Dy * dPy).sum(1)
        e_xy = 0.5 * ((Dx * dPy).sum(1) + (Dy * dPx).sum(1))
        tr = e_xx + e_yy
        S_xx = lam * tr + 2 * mum * e_xx
        S_yy = lam * tr + 2 * mum * e_yy
        S_xy = 2 * mum * e_xy
        WL = w[q] * JL
        for l in range(6):
            R[:, 15 + 2 * l] += WL * (S_xx * dPx[:, l] + S_xy * dPy[:, l])
            R[:, 16 + 2 * l] += WL * (S_xy * dPx[:, l] + S_yy * dPy[:, l])
    return R


def line_residual(loc: np.ndarray, hist_x: List[np.ndarray], p: Dict[str, float]) -> np.ndarray:
    """loc [Ei, 15] in line_layout order; hist_x: previous positions [Ei, 3, 2] per level."""
    Ei = loc.shape[0]
    ux, uy, lm = loc[:, 0:9:3], loc[:, 1:9:3], loc[:, 2:9:3]
    xs, ys = loc[:, 9::2], loc[:, 10::2]
    b0, b1, b2 = p["__bdf0"], p["__bdf1"], p["__bdf2"]
    vx = b0 * xs + b1 * hist_x[0][:, :, 0] + b2 * hist_x[1][:, :, 0]
    vy = b0 * ys + b1 * hist_x[0][:, :, 1] + b2 * hist_x[1][:, :, 1]
    sig = p["surface_tension"]
    R = np.zeros((Ei, 15), dtype=loc.dtype)
    for q in range(3):
        psi, dps = line_shapes(LINE_S[q])
        t0, t1 = xs @ dps, ys @ dps
        J = np.sqrt(t0 * t0 + t1 * t1)
        tau0, tau1 = t0 / J, t1 / J
        n0, n1 = tau1, -tau0
        r = xs @ psi
        W = LINE_W[q] * J * 2 * math.pi * r
        kin = ((vx @ psi) - (ux @ psi)) * n0 + ((vy @ psi) - (uy @ psi)) * n1
        lam = lm @ psi
        for l in range(3):
            R[:, 3 * l + 2] += W * kin * psi[l]
            R[:, 9 + 2 * l] += -W * lam * n0 * psi[l]
            R[:, 10 + 2 * l] += -W * lam * n1 * psi[l]
            R[:, 3 * l] += W * sig * (tau0 * dps[l] / J + psi[l] / r)
            R[:, 3 * l + 1] += W * sig * (tau1 * dps[l] / J)
    return R


def point_residual(loc: np.ndarray, p: Dict[str, float]) -> np.ndarray:
    th, sig = p["contact_angle"], p["surface_tension"]
    r = loc[:, 2]
    R = np.zeros((loc.shape[0], 4), dtype=loc.dtype)
    R[:, 0] = sig * (-np.cos(th)) * 2 * math.pi * r
    R[:, 1] = sig * np.sin(th) * 2 * math.pi * r
    return R


def _complex_step(fun, loc: np.ndarray):
    R = fun(loc.astype(np.float64)).real
    n = loc.shape[1]
    J = np.zeros((loc.shape[0], R.shape[1], n))
    for k in range(n):
        z = loc.astype(np.complex128)
        z[:, k] += 1j * H_CS
        J[:, :, k] = fun(z).imag / H_CS
    return R, J


def element_res_jac(D: Droplet, vals: np.ndarray, hist: List[np.ndarray], p: Dict[str, float]):
    """[(R_e, J_e)] for the bulk, interface and contact-line domains."""
    out = []
    lb = bulk_layout()
    X0e = D.x0[D.tri]
    out.append(_complex_step(lambda z: bulk_residual(z, X0e, p), _gather(vals, D.tri, lb)))
    hx = [h[D.line][:, :, 0:2] for h in hist]
    out.append(_complex_step(lambda z: line_residual(z, hx, p), _gather(vals, D.line, line_layout())))
    out.append(_complex_step(lambda z: point_residual(z, p), _gather(vals, D.point, point_layout())))
    return out


def element_mass(D: Droplet, vals: np.ndarray, hist: List[np.ndarray], p: Dict[str, float]):
    """Element mass matrices dR_e/d(du/dt): only the interface's kinematic
    condition has a time derivative (of the positions).  Since
    du/dt = b0 u + b1 u_prev + b2 u_prev2, dR/d(du/dt) = (dR/du_prev) / b1,
    taken by complex steps in the previous positions."""
    lay = line_layout()
    loc = _gather(vals, D.line, lay)
    h0 = hist[0][D.line][:, :, 0:2]
    h1 = hist[1][D.line][:, :, 0:2]
    M = np.zeros((D.line.shape[0], 15, 15))
    for l in range(3):
        for c in range(2):
            z = h0.astype(np.complex128)
            z[:, l, c] += 1j * H_CS
            M[:, :, 9 + 2 * l + c] = line_residual(loc.astype(np.complex128), [z, h1], p).imag / H_CS / p["__bdf1"]
    nb = D.tri.shape[0]
    return [np.zeros((nb, 27, 27)), M, np.zeros((1, 4, 4))]


def element_dparam(D: Droplet, vals: np.ndarray, hist: List[np.ndarray], p: Dict[str, float], name: str):
    """Element residual derivatives dR_e/dp by a complex step in p."""
    q = dict(p)
    q[name] = p[name] + 1j * H_CS
    hx = [h[D.line][:, :, 0:2] for h in hist]
    out = [bulk_residual(_gather(vals, D.tri, bulk_layout()).astype(np.complex128), D.x0[D.tri], q),
           line_residual(_gather(vals, D.line, line_layout()).astype(np.complex128), hx, q),
           point_residual(_gather(vals, D.point, point_layout()).astype(np.complex128), q)]
    return [o.imag / H_CS for o in out]


def assemble_blocks(D: Droplet, blocks_R, blocks_J):
    """Vectors-of-pairs assembly of given element vectors/matrices."""
    conns = [D.tri, D.line, D.point]
    lays = [bulk_layout(), line_layout(), point_layout()]
    R = np.zeros(D.n_dof)
    rows: List[Dict[int, float]] = [dict() for _ in range(D.n_dof)]
    for Re, Je, conn, lay in zip(blocks_R, blocks_J, conns, lays):
        for e in range(conn.shape[0]):
            eq = [int(D.eqn[conn[e, l], v]) for (l, v) in lay]
            for i, gi in enumerate(eq):
                if gi < 0:
                    continue
                if Re is not None:
                    R[gi] += Re[e, i]
                if Je is None:
                    continue
                row = rows[gi]
                for j, gj in enumerate(eq):
                    if gj >= 0:
                        row[gj] = row.get(gj, 0.0) + Je[e, i, j]
    vals = np.fromiter((v for row in rows for v in row.values()), dtype=np.float64)
    return R, vals


def assemble(D: Droplet, vals: np.ndarray, hist: List[np.ndarray], p: Dict[str, float]):
    """Vectors-of-pairs assembly (structural): R, CSR (rowptr, colidx, values)."""
    blocks = element_res_jac(D, vals, hist, p)
    conns = [D.tri, D.line, D.point]
    lays = [bulk_layout(), line_layout(), point_layout()]
    R = np.zeros(D.n_dof)
    rows: List[Dict[int, float]] = [dict() for _ in range(D.n_dof)]
    for (Re, Je), conn, lay in zip(blocks, conns, lays):
        for e in range(conn.shape[0]):
            eq = [int(D.eqn[conn[e, l], v]) for (l, v) in lay]
            for i, gi in enumerate(eq):
                if gi < 0:
                    continue
                R[gi] += Re[e, i]
                row = rows[gi]
                for j, gj in enumerate(eq):
                    if gj < 0:
                        continue
                    row[gj] = row.get(gj, 0.0) + Je[e, i, j]
    rowptr = np.zeros(D.n_dof + 1, dtype=np.int64)
    for i, row in enumerate(rows):
        rowptr[i + 1] = rowptr[i] + len(row)
    colidx = np.fromiter((c for row in rows for c in row.keys()), dtype=np.int64, count=int(rowptr[-1]))
    values = np.fromiter((v for row in rows for v in row.values()), dtype=np.float64, count=int(rowptr[-1]))
    return R, rowptr, colidx, values


def bdf_weights(order: int, dt: float, dt_prev: Optional[float] = None) -> Tuple[float, float, float]:
    """BDF1, or BDF2 for variable steps, with the expressions of pyoomph's
    MultiTimeStepper::set_weights (src/timestepper.cpp:32-52)."""
    if order == 1:
        return 1.0 / dt, -1.0 / dt, 0.0
    dtprev = dt_prev if dt_prev else dt
    return 1.0 / dt + 1.0 / (dt + dtprev), -(dt + dtprev) / (dt * dtprev), dt / ((dt + dtprev) * dtprev)


def newton(D: Droplet, vals: np.ndarray, hist: List[np.ndarray], p: Dict[str, float], tol: float = 1e-10,
           max_iter: int = 12):
    """Newton on the oracle assembly; returns the converged nodal values."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    vals = vals.copy()
    m = D.eqn >= 0
    for _ in range(max_iter):
        R, rp, ci, v = assemble(D, vals, hist, p)
        if np.max(np.abs(R)) < tol:
            return vals
        A = sps.csr_matrix((v, ci, rp), shape=(D.n_dof, D.n_dof))
        dx = spla.splu(A.tocsc()).solve(R)
        vals[m] -= dx[D.eqn[m]]
    raise RuntimeError("oracle Newton did not converge")


def run_steps(N: int, theta_deg: float, mu: float, sigma: float, dt: float, nsteps: int):
    """Time steps of the droplet from the hemisphere; returns the values after each step."""
    D = droplet(N)
    vals = initial_values(D)
    h0, h1 = vals.copy(), vals.copy()
    p = {"dynamic_viscosity": mu, "surface_tension": sigma, "contact_angle": math.radians(theta_deg)}
    out = []
    for k in range(nsteps):
        h1, h0 = h0, vals.copy()
        w = bdf_weights(1 if k == 0 else 2, dt, dt)
        p.update(__bdf0=w[0], __bdf1=w[1], __bdf2=w[2])
        vals = newton(D, vals, [h0, h1], p)
        out.append(vals.copy())
    return D, out
