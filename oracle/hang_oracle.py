"""CPU oracle for assembly on refined meshes with hanging nodes.

TEST INFRASTRUCTURE ONLY.  Imported by tests/ as the checker; never by the
package ``pyoomph_gb300``.

Restates, independently of the package's lattice-based generator:

* quadtree refinement of a Q2 quad mesh (oracle mesh of ``fe_oracle.c`` in
  pyoomph's order) to one or several levels: each chosen element is replaced
  by its four sons (SW, SE, NW, NE) whose nodes are placed by the parent's
  isoparametric map; the leaves in tree order; the nodes numbered by first
  encounter over the leaves (oomph's ``Mesh::reorder_nodes`` after adapt);
* hanging nodes found geometrically: a node strictly inside an edge of a
  coarser leaf takes the values interpolated along that edge by the 1D
  quadratic shapes (oomph's ``RefineableQElement<2>::setup_hang_for_value``),
  completed through hanging masters (``complete_hanging_nodes``), and its
  values are constrained (no equation; ``Node::assign_eqn_numbers``,
  ``nodes.cc:534-561``);
* the element residuals/Jacobians of ``fe_oracle.c`` with the hanging values
  interpolated, assembled with oomph's hanging-node rule (each local equation
  of a hanging value adds, weighted, to its masters' equations, rows and
  columns alike; ``jitbridge_hang.h`` master loops) into the element matrix
  over oomph's local equations (own values, then outside masters), inserted
  in the vectors-of-pairs order (element, local equation i, local equation j).
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, List, Tuple

import numpy as np

import oracle as O


def _shape(s0: float, s1: float) -> np.ndarray:
    psi = np.zeros(9)
    dps = np.zeros((9, 2))
    O.lib().ofe_shape_c2(O.Q2_QUAD, O._ptr(np.array([s0, s1, 0.0])), O._ptr(psi), O._ptr(dps))
    return psi


def _complete(hang: Dict[int, List[Tuple[int, float]]], min_weight: float = 1e-8, rank=None):
    """oomph-lib's complete_hanging_nodes (refineable_mesh.cc:2214-2320) as
    written there: nodes in order; for each hanging node the recursive list
    of (master, weight) -- a hanging master contributes its own masters'
    list, each weight then multiplied by the master's weight -- built on
    the hang infos as completed so far, merged in a map (|w| <= min_weight
    dropped, repeats summed) that replaces the node's hang info.  The map's
    order is the node's address in oomph: ``rank`` gives the nodes' order of
    creation, which the addresses follow in a fresh allocation (default:
    the node number)."""
    hang = {k: list(v) for k, v in hang.items()}

    def rec(node, masters, weights):
        if node in hang:
            for m, w in hang[node]:
                first = len(masters)
                rec(m, masters, weights)
                for k in range(first, len(masters)):
                    weights[k] = w * weights[k]
        else:
            masters.append(node)
            weights.append(1.0)

    for node in sorted(hang):
        masters: List[int] = []
        weights: List[float] = []
        rec(node, masters, weights)
        merged: Dict[int, float] = {}
        for m, w in zip(masters, weights):
            if abs(w) > min_weight:
                merged[m] = merged.get(m, 0.0) + w
        hang[node] = [(m, merged[m]) for m in sorted(merged, key=(lambda q: rank[q]) if rank else None)]
    return hang


def refine_levels(m: O.Mesh, chosen, max_level: int, with_c1: bool = False):
    """(x, conn, hang, on_boundary) of a quadtree refinement to several
    levels: an element (a map X(s) of the reference square) is split into
    its sons SW, SE, NW, NE -- son maps composed with the parent's -- while
    ``chosen(cx, cy, level)`` holds at its centre node and level <
    max_level; leaves in tree order; nodes found by position and numbered
    by first encounter over the leaves' local nodes (oomph-lib's
    Mesh::reorder_nodes, mesh.cc:541-640, called after every adapt);
    hanging nodes found geometrically on the leaves' edges and completed
    recursively (``_complete``)."""
    leaves = []   # per leaf: its 9 node positions
    sons_at = []  # (level, [4 x 9 positions]) of every split, in tree order

    def split(nodes9: np.ndarray, level: int):
        c = nodes9[4]
        if level < max_level and chosen(c[0], c[1], level):
            sons = [np.array([_shape(sx0 + 0.5 * i, sy0 + 0.5 * j) @ nodes9 for j in range(3) for i in range(3)])
                    for (sx0, sy0) in ((-1.0, -1.0), (0.0, -1.0), (-1.0, 0.0), (0.0, 0.0))]
            sons_at.append((level, sons))
            for son in sons:
                split(son, level + 1)
        else:
            leaves.append(nodes9)

    for e in range(m.conn.shape[0]):
        split(m.x[m.conn[e]].copy(), 0)
    ids: Dict[Tuple[float, float], int] = {}
    x: List[np.ndarray] = []
    conn = []
    for nodes9 in leaves:
        row = []
        for p in nodes9:
            k = (round(float(p[0]), 12), round(float(p[1]), 12))
            if k not in ids:
                ids[k] = len(x)
                x.append(p)
            row.append(ids[k])
        conn.append(row)
    x = np.array(x)
    conn = np.array(conn, dtype=np.int32)
    hang: Dict[int, List[Tuple[int, float]]] = {}
    edges = [(c[a], c[mid], c[b]) for c in conn for a, mid, b in ((0, 1, 2), (6, 7, 8), (0, 3, 6), (2, 5, 8))]
    for k in range(x.shape[0]):
        for a, mid, b in edges:
            if k in (a, mid, b):
                continue
            pa, pb = x[a], x[b]
            t = pb - pa
            u = np.dot(x[k] - pa, t) / np.dot(t, t)
            if 0.0 < u < 1.0 and np.linalg.norm(pa + u * t - x[k]) < 1e-12:
                s = np.round((2.0 * u - 1.0) * 2.0 ** 20) / 2.0 ** 20   # dyadic, as the tree's coordinates
                w = (0.5 * s * (s - 1.0), 1.0 - s * s, 0.5 * s * (s + 1.0))
                hang[k] = [(a, w[0]), (mid, w[1]), (b, w[2])]
                break
    # order of creation in oomph: the base mesh's nodes in its own order,
    # then one adapt per level, each building the new sons in tree order,
    # nodes in local order (a node already there is shared)
    key = lambda p: (round(float(p[0]), 12), round(float(p[1]), 12))
    rank = {ids[key(p)]: g for g, p in enumerate(m.x)}
    for level in range(max_level):
        for lv, sons in sons_at:
            if lv == level:
                for son in sons:
                    for p in son:
                        rank.setdefault(ids[key(p)], len(rank))
    hang = _complete(hang, rank=rank)
    lo, hi = x.min(axis=0), x.max(axis=0)
    on_b = (np.abs(x[:, 0] - lo[0]) < 1e-12) | (np.abs(x[:, 0] - hi[0]) < 1e-12) | \
           (np.abs(x[:, 1] - lo[1]) < 1e-12) | (np.abs(x[:, 1] - hi[1]) < 1e-12)
    if not with_c1:
        return x, conn, hang, on_b
    # C1 values live on the leaves' vertices and interpolate bilinearly: a
    # vertex strictly inside a leaf edge -- its middle node included --
    # takes the value interpolated linearly between the edge's two end
    # vertices (setup_hang_for_value with the vertices as the interpolating
    # nodes, pyoomph's BulkElementQuad2dC2::interpolating_node_pt,
    # elements.cpp:9162-9250), completed through hanging masters
    vertices = sorted(set(int(c[s_]) for c in conn for s_ in (0, 2, 6, 8)))
    hang_c1: Dict[int, List[Tuple[int, float]]] = {}
    for k in vertices:
        for a, mid, b in edges:
            if k in (a, b):
                continue
            pa, pb = x[a], x[b]
            t = pb - pa
            u = np.dot(x[k] - pa, t) / np.dot(t, t)
            if 0.0 < u < 1.0 and np.linalg.norm(pa + u * t - x[k]) < 1e-12:
                u = np.round(u * 2.0 ** 20) / 2.0 ** 20              # dyadic, as the tree's coordinates
                hang_c1[k] = [(a, 1.0 - u), (b, u)]
                break
    hang_c1 = _complete(hang_c1, rank=rank)
    return x, conn, hang, hang_c1, on_b


def refinement_plan(m: O.Mesh, chosen, max_level: int):
    """(level, centre x, centre y) of every element that ``refine_levels``
    splits, in tree order."""
    plan = []

    def split(nodes9: np.ndarray, level: int):
        c = nodes9[4]
        if level < max_level and chosen(c[0], c[1], level):
            plan.append((level, float(c[0]), float(c[1])))
            for (sx0, sy0) in ((-1.0, -1.0), (0.0, -1.0), (-1.0, 0.0), (0.0, 0.0)):
                split(np.array([_shape(sx0 + 0.5 * i, sy0 + 0.5 * j) @ nodes9 for j in range(3) for i in range(3)]),
                      level + 1)

    for e in range(m.conn.shape[0]):
        split(m.x[m.conn[e]].copy(), 0)
    return plan


REF_HANG_DRIVER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "oomph_hang_driver")


def ref_hang_available() -> bool:
    return os.path.exists(REF_HANG_DRIVER)


def ref_hang_run(N: int, chosen, max_level: int, gaussians: np.ndarray, dofs=None) -> dict:
    """oomph-lib's own refinement, hanging nodes, numbering and
    Problem::get_jacobian on the refined oracle mesh (oracle/ref/
    oomph_hang_driver.cc, compiled from the reference tree).  ``dofs``:
    the free values in oomph's equation order (default 0)."""
    import subprocess
    import tempfile
    m = O.mesh(O.Q2_QUAD, N, N)
    plan = np.array(refinement_plan(m, chosen, max_level), dtype=np.float64).reshape(-1, 3)
    g = np.asarray(gaussians, dtype=np.float64)
    params = np.concatenate([[g.shape[0]], g.reshape(-1)])
    with tempfile.TemporaryDirectory() as td:
        fin, fd, fout = (os.path.join(td, n) for n in ("in.bin", "dofs.bin", "out.bin"))
        with open(fin, "wb") as f:
            np.array([m.x.shape[0], m.conn.shape[0], plan.shape[0], params.size], dtype=np.int32).tofile(f)
            np.ascontiguousarray(m.x, dtype=np.float64).tofile(f)
            np.ascontiguousarray(m.conn, dtype=np.int32).tofile(f)
            np.ascontiguousarray(m.bmask, dtype=np.uint32).tofile(f)
            plan.tofile(f)
            params.tofile(f)
        if dofs is not None:
            np.ascontiguousarray(dofs, dtype=np.float64).tofile(fd)
        subprocess.run([REF_HANG_DRIVER, fin, fd if dofs is not None else "", fout], check=True)
        b = open(fout, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(b, dtype=dt, count=n, offset=off)
        off += a.nbytes
        return a.copy()

    nn, ne, nd, nnz = (int(v) for v in take(np.int32, 4))
    x = take(np.float64, 2 * nn).reshape(nn, 2)
    conn = take(np.int32, 9 * ne).reshape(ne, 9)
    eqn = take(np.int32, nn)
    hang = {}
    for i in range(nn):
        k = int(take(np.int32, 1)[0])
        ms = []
        for _ in range(k):
            mm = int(take(np.int32, 1)[0])
            ms.append((mm, float(take(np.float64, 1)[0])))
        if k:
            hang[i] = ms
    rp = take(np.int32, nd + 1)
    ci = take(np.int32, nnz)
    v = take(np.float64, nnz)
    R = take(np.float64, nd)
    return dict(x=x, conn=conn, eqn=eqn, hang=hang, rowptr=rp, colidx=ci, vals=v, R=R)


class HangProblem:
    """Scalar Q2 problem (Poisson / nonlinear diffusion) on a refined mesh,
    u = 0 on the outer boundary (``refine_levels``; without max_level one
    level, ``chosen(cx, cy)``)."""

    def __init__(self, N: int, chosen, gaussians: np.ndarray, eq: int = O.EQ_POISSON, max_level=None):
        if max_level is None:   # one level, chosen(cx, cy)
            self.x, self.conn, self.hang, on_b = refine_levels(O.mesh(O.Q2_QUAD, N, N),
                                                               lambda x, y, level: chosen(x, y), 1)
        else:
            self.x, self.conn, self.hang, on_b = refine_levels(O.mesh(O.Q2_QUAD, N, N), chosen, max_level)
        n = self.x.shape[0]
        self.eq = eq
        self.params = O.gaussian_params(gaussians)
        self.values = np.zeros(n)
        self.eqn = np.full(n, -1, dtype=np.int64)
        k = 0
        for i in range(n):
            if not on_b[i] and i not in self.hang:
                self.eqn[i] = k
                k += 1
        self.n_dof = k

    def dofs(self) -> np.ndarray:
        m = self.eqn >= 0
        out = np.zeros(self.n_dof)
        out[self.eqn[m]] = self.values[m]
        return out

    def set_dofs(self, d: np.ndarray) -> None:
        m = self.eqn >= 0
        self.values[m] = d[self.eqn[m]]
        for h, ms in self.hang.items():
            self.values[h] = sum(w * self.values[mm] for mm, w in ms)

    def expand(self, node: int) -> List[Tuple[int, float]]:
        if node in self.hang:
            return [(int(self.eqn[mm]), w) for mm, w in self.hang[node] if self.eqn[mm] >= 0]
        return [(int(self.eqn[node]), 1.0)] if self.eqn[node] >= 0 else []

    def assemble(self):
        L = O.lib()
        R = np.zeros(self.n_dof)
        rows: List[Dict[int, float]] = [dict() for _ in range(self.n_dof)]
        isv = np.zeros(self.x.shape[0], dtype=np.uint8)
        vals = np.ascontiguousarray(self.values.reshape(-1, 1))
        Re = np.zeros(9)
        Je = np.zeros(81)
        xx = np.ascontiguousarray(self.x)
        for e in range(self.conn.shape[0]):
            c = np.ascontiguousarray(self.conn[e])
            L.ofe_element_res_jac(O.Q2_QUAD, self.eq, 2, O._ptr(xx), O._ptr(c), 1, O._ptr(vals), O._ptr(isv),
                                  O._ptr(self.params), len(self.params), O._ptr(Re), O._ptr(Je))
            J = Je.reshape(9, 9)
            exp = [self.expand(int(n)) for n in c]
            # oomph's local equations of the element: its own non-hanging
            # values in local order, then the masters of its hanging values
            # that are not its own nodes, by first appearance
            # (RefineableElement::assign_hanging_local_eqn_numbers)
            dofs = [int(self.eqn[n]) for n in c if int(n) not in self.hang and self.eqn[n] >= 0]
            own = set(int(n) for n in c)
            for n in c:
                for mm, _ in self.hang.get(int(n), []):
                    q = int(self.eqn[mm])
                    if mm not in own and q >= 0 and q not in dofs:
                        dofs.append(q)
            pos = {q: a for a, q in enumerate(dofs)}
            Jl = np.zeros((len(dofs), len(dofs)))
            Rl = np.zeros(len(dofs))
            for i in range(9):
                for (r, wr) in exp[i]:
                    Rl[pos[r]] += wr * Re[i]
                    for j in range(9):
                        for (cc, wc) in exp[j]:
                            Jl[pos[r], pos[cc]] += wr * wc * J[i, j]
            # the vectors-of-pairs insertion: (local equation i, local equation j)
            for a, r in enumerate(dofs):
                R[r] += Rl[a]
                row = rows[r]
                for b, cc in enumerate(dofs):
                    row[cc] = row.get(cc, 0.0) + Jl[a, b]
        rp = np.zeros(self.n_dof + 1, dtype=np.int64)
        for i, row in enumerate(rows):
            rp[i + 1] = rp[i] + len(row)
        ci = np.fromiter((k for row in rows for k in row), dtype=np.int64, count=int(rp[-1]))
        v = np.fromiter((val for row in rows for val in row.values()), dtype=np.float64, count=int(rp[-1]))
        return R, rp, ci, v

    def newton(self, tol: float = 1e-11, max_iter: int = 20) -> np.ndarray:
        import scipy.sparse as sps
        import scipy.sparse.linalg as spla
        for _ in range(max_iter):
            R, rp, ci, v = self.assemble()
            if np.max(np.abs(R)) < tol:
                return self.dofs()
            A = sps.csr_matrix((v, ci, rp), shape=(self.n_dof, self.n_dof))
            self.set_dofs(self.dofs() - spla.splu(A.tocsc()).solve(R))
        raise RuntimeError("oracle Newton did not converge")


class HangNSProblem:
    """Taylor-Hood Navier-Stokes (Q2 velocity, Q1 pressure) on a refined
    mesh: the lid-driven cavity of ``O.navier_stokes_problem`` (velocity
    pinned on the boundary, u_x = 16x^2(1-x)^2 on top; the pressure pinned
    at the first node of the first element).  Velocity values hang by the C2
    hang infos, pressure values (vertices only) by the C1 ones.  oomph's
    local equations of an element: its own free values in local order (node
    by node, velocity then pressure: fe_oracle.c's layout), then the
    (master node, value) pairs of its hanging values that are not values of
    its own, by first appearance (RefineableElement::
    assign_hanging_local_eqn_numbers); equations numbered node by node,
    value by value (Node::assign_eqn_numbers)."""

    def __init__(self, N: int, chosen, max_level: int, rho: float = 1.0, mu: float = 0.01):
        self.x, self.conn, hang, hang_c1, on_b = refine_levels(O.mesh(O.Q2_QUAD, N, N), chosen, max_level,
                                                                with_c1=True)
        self.hang, self.hang_c1 = hang, hang_c1
        n = self.x.shape[0]
        self.isv = np.zeros(n, dtype=np.uint8)
        self.isv[np.unique(self.conn[:, [0, 2, 6, 8]])] = 1
        present = np.ones((n, 3), dtype=bool)
        present[:, 2] = self.isv != 0
        pinned = np.zeros((n, 3), dtype=bool)
        pinned[on_b, 0] = pinned[on_b, 1] = True
        pinned[int(self.conn[0, 0]), 2] = True
        self.values = np.zeros((n, 3))
        top = np.abs(self.x[:, 1] - self.x[:, 1].max()) < 1e-12
        self.values[top, 0] = O.lid_velocity(self.x[top, 0])
        # hang infos per (node, value)
        self.hv: Dict[Tuple[int, int], List[Tuple[int, float]]] = {}
        for h, ms in hang.items():
            for f in (0, 1):
                self.hv[(h, f)] = ms
        for h, ms in hang_c1.items():
            if present[h, 2]:
                self.hv[(h, 2)] = ms
        self.present = present
        self.eqn = np.full((n, 3), -1, dtype=np.int64)
        k = 0
        for i in range(n):
            for f in range(3):
                if present[i, f] and not pinned[i, f] and (i, f) not in self.hv:
                    self.eqn[i, f] = k
                    k += 1
        self.n_dof = k
        self.params = np.array([rho, mu])
        self._interpolate_hanging()

    def _interpolate_hanging(self) -> None:
        for (h, f), ms in self.hv.items():
            self.values[h, f] = sum(w * self.values[m, f] for m, w in ms)

    def dofs(self) -> np.ndarray:
        m = self.eqn >= 0
        out = np.zeros(self.n_dof)
        out[self.eqn[m]] = self.values[m]
        return out

    def set_dofs(self, d: np.ndarray) -> None:
        m = self.eqn >= 0
        self.values[m] = d[self.eqn[m]]
        self._interpolate_hanging()

    def expand(self, node: int, f: int) -> List[Tuple[int, float]]:
        if (node, f) in self.hv:
            return [(int(self.eqn[mm, f]), w) for mm, w in self.hv[(node, f)] if self.eqn[mm, f] >= 0]
        return [(int(self.eqn[node, f]), 1.0)] if self.eqn[node, f] >= 0 else []

    def assemble(self):
        L = O.lib()
        R = np.zeros(self.n_dof)
        rows: List[Dict[int, float]] = [dict() for _ in range(self.n_dof)]
        vals = np.ascontiguousarray(self.values)
        xx = np.ascontiguousarray(self.x)
        isv = np.ascontiguousarray(self.isv)
        layout = [(l, f) for l in range(9) for f in range(3) if f < 2 or l in (0, 2, 6, 8)]
        nl = len(layout)
        Re = np.zeros(nl)
        Je = np.zeros(nl * nl)
        for e in range(self.conn.shape[0]):
            c = np.ascontiguousarray(self.conn[e])
            rc = L.ofe_element_res_jac(O.Q2_QUAD, O.EQ_NAVIER_STOKES_TH, 2, O._ptr(xx), O._ptr(c), 3, O._ptr(vals),
                                       O._ptr(isv), O._ptr(self.params), len(self.params), O._ptr(Re), O._ptr(Je))
            if rc != nl:                      # the local size on success
                raise RuntimeError("oracle element failed")
            J = Je.reshape(nl, nl)
            slots = [(int(c[l]), f) for l, f in layout]
            exp = [self.expand(nd, f) for nd, f in slots]
            dofs = [int(self.eqn[nd, f]) for nd, f in slots if (nd, f) not in self.hv and self.eqn[nd, f] >= 0]
            own = set(slots)
            for nd, f in slots:
                for mm, _ in self.hv.get((nd, f), []):
                    q = int(self.eqn[mm, f])
                    if (mm, f) not in own and q >= 0 and q not in dofs:
                        dofs.append(q)
            pos = {q: a for a, q in enumerate(dofs)}
            Jl = np.zeros((len(dofs), len(dofs)))
            Rl = np.zeros(len(dofs))
            for i in range(nl):
                for (r, wr) in exp[i]:
                    Rl[pos[r]] += wr * Re[i]
                    for j in range(nl):
                        for (cc, wc) in exp[j]:
                            Jl[pos[r], pos[cc]] += wr * wc * J[i, j]
            for a, r in enumerate(dofs):
                R[r] += Rl[a]
                row = rows[r]
                for b, cc in enumerate(dofs):
                    row[cc] = row.get(cc, 0.0) + Jl[a, b]
        rp = np.zeros(self.n_dof + 1, dtype=np.int64)
        for i, row in enumerate(rows):
            rp[i + 1] = rp[i] + len(row)
        ci = np.fromiter((k for row in rows for k in row), dtype=np.int64, count=int(rp[-1]))
        v = np.fromiter((val for row in rows for val in row.values()), dtype=np.float64, count=int(rp[-1]))
        return R, rp, ci, v

    def newton(self, tol: float = 1e-11, max_iter: int = 20) -> np.ndarray:
        import scipy.sparse as sps
        import scipy.sparse.linalg as spla
        for _ in range(max_iter):
            R, rp, ci, v = self.assemble()
            if np.max(np.abs(R)) < tol:
                return self.dofs()
            A = sps.csr_matrix((v, ci, rp), shape=(self.n_dof, self.n_dof))
            self.set_dofs(self.dofs() - spla.splu(A.tocsc()).solve(R))
        raise RuntimeError("oracle Newton did not converge")
