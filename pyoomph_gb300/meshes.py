"""Structured mesh templates in pyoomph's node and element order.

The order of nodes fixes the equation numbering and therefore the CSR
pattern, so it must match the reference exactly:

* ``RectangularQuadMesh.define_geometry`` (``pyoomph/meshes/simplemeshes.py:225-305``)
  visits cells with ``ix`` outer and ``iy`` inner and adds the corner nodes
  n00, n10, n01, n11 through ``add_node_unique`` (deduplication by position,
  ``src/meshtemplate.cpp:1378``); split cells give the triangles
  ``(n00,n10,n11),(n00,n11,n01)`` ("left") or ``(n01,n10,n11),(n00,n10,n01)``
  ("right");
* ``CuboidBrickMesh`` (``simplemeshes.py:515-545``) visits ``ix, iy, iz`` and
  adds the corners in the order 000,100,010,110,001,101,011,111;
* the conversion to the quadratic space then appends, element by element,
  the midside/face/centre nodes in the call order of
  ``convert_for_C2_space`` (``meshtemplate.cpp:401-409`` quad,
  ``:494-499`` triangle, ``:579-621`` brick);
* the mesh keeps template-index order (``src/mesh2d.hpp:265-300``).

Every node sits on a half-cell lattice, so the generator computes the
sequence of lattice keys in the reference's insertion order and numbers
each key at its first occurrence, all in vectorised numpy.  A node's
position is the one computed at its first insertion, with the reference's
arithmetic (``0.5*(a+b)``, ``0.25*(a+b+c+d)``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple, Union

import numpy as np

from .spaces import ELEMENT_TYPES, ElementType


@dataclass
class MeshData:
    etype: ElementType
    x: np.ndarray                # [n_nodes, dim]
    conn: np.ndarray             # [n_elem, nnode] int32
    is_vertex: np.ndarray        # [n_nodes] bool (C1 nodes)
    boundaries: Dict[str, np.ndarray] = field(default_factory=dict)  # name -> bool mask over nodes
    lattice: Optional[np.ndarray] = None  # [n_nodes, dim] int64 half-cell coordinates
    hang: Optional[Dict[int, list]] = None  # hanging node -> [(master node, weight)] (refined meshes)
    hang_c1: Optional[Dict[int, list]] = None  # the same for C1 (vertex) values

    @property
    def n_nodes(self) -> int:
        return self.x.shape[0]

    @property
    def n_elem(self) -> int:
        return self.conn.shape[0]

    @property
    def dim(self) -> int:
        return self.etype.dim


def _number_first_touch(keys: np.ndarray):
    """Node ids by order of first occurrence of each key."""
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    return rank[inv], first[order], len(uniq)


class MeshTemplate:
    domain_name = "domain"
    transform = None  # optional callable x[n, dim] -> x[n, dim] applied to all nodes

    def generate(self) -> MeshData:
        md = self._generate()
        if self.transform is not None:
            md.x = np.ascontiguousarray(self.transform(md.x.copy()), dtype=np.float64)
        return md

    def _generate(self) -> MeshData:  # pragma: no cover - abstract
        raise NotImplementedError


class RectangularQuadMesh(MeshTemplate):
    """Unit-square-style rectangle of Q2 quads, or of P2 triangles with
    ``split_in_tris="left"|"right"``."""

    def __init__(self, *, N: Union[int, List[int]] = 10, size: Union[float, List[float]] = 1.0,
                 lower_left: Union[float, List[float]] = 0.0, split_in_tris: Union[bool, str] = False,
                 name: str = "domain", transform=None):
        self.transform = transform
        self.N = [N, N] if isinstance(N, int) else list(N)
        self.size = [size, size] if isinstance(size, (int, float)) else list(size)
        self.lower_left = [lower_left, lower_left] if isinstance(lower_left, (int, float)) else list(lower_left)
        if split_in_tris not in (False, "left", "right"):
            raise ValueError("split_in_tris must be False, 'left' or 'right'")
        self.split = split_in_tris
        self.domain_name = name

    def _generate(self) -> MeshData:
        nx, ny = self.N
        lx, ly = self.size
        x0, y0 = self.lower_left
        LX = 2 * nx + 1
        ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        ix = ix.ravel().astype(np.int64)
        iy = iy.ravel().astype(np.int64)  # cells in (ix outer, iy inner) order
        corners = [(0, 0), (2, 0), (0, 2), (2, 2)]  # n00, n10, n01, n11
        lat_c = np.stack([np.stack([2 * ix + a, 2 * iy + b], axis=1) for a, b in corners], axis=1)  # [cells,4,2]

        def pos_vertex(lat):
            # (ix * size) / N + lower_left, as the template computes it
            return np.stack([(lat[..., 0] // 2) * lx / nx + x0, (lat[..., 1] // 2) * ly / ny + y0], axis=-1)

        pc = pos_vertex(lat_c)
        if not self.split:
            et = ELEMENT_TYPES["Q2_QUAD"]
            # C2 additions per element: n1=mid(0,1), n3=mid(0,2), n4=centre, n5=mid(1,3), n7=mid(2,3)
            mids = [(0, 1), (0, 2), None, (1, 3), (2, 3)]
            lat_m, pos_m = [], []
            for m in mids:
                if m is None:
                    lat_m.append((lat_c[:, 0] + lat_c[:, 3]) // 2)
                    pos_m.append(0.25 * (pc[:, 0] + pc[:, 1] + pc[:, 2] + pc[:, 3]))
                else:
                    a, b = m
                    lat_m.append((lat_c[:, a] + lat_c[:, b]) // 2)
                    pos_m.append(0.5 * (pc[:, a] + pc[:, b]))
            lat_m = np.stack(lat_m, axis=1)
            pos_m = np.stack(pos_m, axis=1)
            # element slots: (n00, n1, n10, n3, n4, n5, n01, n7, n11)
            slot_lat = np.stack([lat_c[:, 0], lat_m[:, 0], lat_c[:, 1], lat_m[:, 1], lat_m[:, 2], lat_m[:, 3],
                                 lat_c[:, 2], lat_m[:, 4], lat_c[:, 3]], axis=1)
            touch_lat = np.concatenate([lat_c.reshape(-1, 2), lat_m.reshape(-1, 2)])
            touch_pos = np.concatenate([pc.reshape(-1, 2), pos_m.reshape(-1, 2)])
        else:
            et = ELEMENT_TYPES["P2_TRI"]
            if self.split == "left":
                tris = [(0, 1, 3), (0, 3, 2)]
            else:
                tris = [(2, 1, 3), (0, 1, 2)]
            vlat = np.stack([np.stack([lat_c[:, a], lat_c[:, b], lat_c[:, c]], axis=1) for a, b, c in tris],
                            axis=1).reshape(-1, 3, 2)  # [2*cells, 3, 2], element order
            vpos = np.stack([np.stack([pc[:, a], pc[:, b], pc[:, c]], axis=1) for a, b, c in tris],
                            axis=1).reshape(-1, 3, 2)
            pairs = [(0, 1), (1, 2), (0, 2)]
            lat_m = np.stack([(vlat[:, a] + vlat[:, b]) // 2 for a, b in pairs], axis=1)
            pos_m = np.stack([0.5 * (vpos[:, a] + vpos[:, b]) for a, b in pairs], axis=1)
            slot_lat = np.concatenate([vlat, lat_m], axis=1)
            touch_lat = np.concatenate([lat_c.reshape(-1, 2), lat_m.reshape(-1, 2)])
            touch_pos = np.concatenate([pc.reshape(-1, 2), pos_m.reshape(-1, 2)])
        key = lambda lat: lat[..., 0] + LX * lat[..., 1]
        ids, first, n_nodes = _number_first_touch(key(touch_lat))
        x = touch_pos[first]
        lat = touch_lat[first]
        # element connectivity through the same numbering
        uniq_keys = key(lat)
        lut = np.full(LX * (2 * ny + 1), -1, dtype=np.int64)
        lut[uniq_keys] = np.arange(n_nodes)
        conn = lut[key(slot_lat)].astype(np.int32)
        is_vertex = (lat[:, 0] % 2 == 0) & (lat[:, 1] % 2 == 0)
        b = {"left": lat[:, 0] == 0, "right": lat[:, 0] == 2 * nx,
             "bottom": lat[:, 1] == 0, "top": lat[:, 1] == 2 * ny}
        return MeshData(et, x, conn, is_vertex, b, lat)


_HEX_C2_ORDER = [1, 3, 4, 5, 7, 9, 11, 15, 17, 19, 21, 22, 23, 25, 10, 12, 14, 16, 13]


class CuboidBrickMesh(MeshTemplate):
    """Box of Q2 hexahedra (27 nodes each)."""

    def __init__(self, *, N: Union[int, List[int]] = 10, size: Union[float, List[float]] = 1.0,
                 lower_left: Union[float, List[float]] = 0.0, domain_name: str = "domain", transform=None):
        self.transform = transform
        self.N = [N, N, N] if isinstance(N, int) else list(N)
        self.size = [size] * 3 if isinstance(size, (int, float)) else list(size)
        self.lower_left = [lower_left] * 3 if isinstance(lower_left, (int, float)) else list(lower_left)
        self.domain_name = domain_name

    def _generate(self) -> MeshData:
        nx, ny, nz = self.N
        L = self.size
        ll = self.lower_left
        LX, LY = 2 * nx + 1, 2 * ny + 1
        g = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        cell = [a.ravel().astype(np.int64) for a in g]  # (ix, iy, iz) with iz fastest
        ncell = cell[0].size
        # corner c = px + 2 py + 4 pz at element slot (2px, 2py, 2pz)
        slot_ijk = np.array([[s % 3, (s // 3) % 3, s // 9] for s in range(27)])
        corner_slots = [0, 2, 6, 8, 18, 20, 24, 26]
        lat = np.zeros((ncell, 27, 3), dtype=np.int64)
        for d in range(3):
            lat[:, :, d] = 2 * cell[d][:, None] + slot_ijk[None, :, d]
        P = np.zeros((ncell, 27, 3))
        nn = [nx, ny, nz]
        for s in corner_slots:
            for d in range(3):
                P[:, s, d] = (lat[:, s, d] // 2) * L[d] / nn[d] + ll[d]
        # positions of the C2 nodes, in the reference's arithmetic
        two = {1: (0, 2), 3: (0, 6), 5: (2, 8), 7: (6, 8), 9: (0, 18), 11: (2, 20), 15: (6, 24), 17: (8, 26),
               19: (18, 20), 21: (18, 24), 23: (20, 26), 25: (24, 26), 10: (9, 11), 12: (9, 15), 14: (11, 17),
               16: (15, 17)}
        four = {4: (0, 2, 6, 8), 22: (18, 20, 24, 26), 13: (0, 8, 20, 24)}
        for s in _HEX_C2_ORDER:
            if s in two:
                a, b = two[s]
                P[:, s] = 0.5 * (P[:, a] + P[:, b])
            else:
                a, b, c, d = four[s]
                P[:, s] = 0.25 * (P[:, a] + P[:, b] + P[:, c] + P[:, d])
        touch_slots = corner_slots + _HEX_C2_ORDER
        # vertex touches come first (all cells), then the C2 additions (all elements)
        v_lat = lat[:, corner_slots].reshape(-1, 3)
        v_pos = P[:, corner_slots].reshape(-1, 3)
        m_lat = lat[:, _HEX_C2_ORDER].reshape(-1, 3)
        m_pos = P[:, _HEX_C2_ORDER].reshape(-1, 3)
        touch_lat = np.concatenate([v_lat, m_lat])
        touch_pos = np.concatenate([v_pos, m_pos])
        key = lambda q: q[..., 0] + LX * (q[..., 1] + LY * q[..., 2])
        ids, first, n_nodes = _number_first_touch(key(touch_lat))
        x = touch_pos[first]
        nlat = touch_lat[first]
        lut = np.full(LX * LY * (2 * nz + 1), -1, dtype=np.int64)
        lut[key(nlat)] = np.arange(n_nodes)
        conn = lut[key(lat)].astype(np.int32)
        is_vertex = np.all(nlat % 2 == 0, axis=1)
        b = {"left": nlat[:, 0] == 0, "right": nlat[:, 0] == 2 * nx, "bottom": nlat[:, 1] == 0,
             "top": nlat[:, 1] == 2 * ny, "back": nlat[:, 2] == 0, "front": nlat[:, 2] == 2 * nz}
        del touch_slots
        return MeshData(ELEMENT_TYPES["Q2_HEX"], x, conn, is_vertex, b, nlat)


# 1D quadratic shapes at the quarter points of an edge (nodes at s = -1, 0, 1):
# psi(-1/2) = (3/8, 3/4, -1/8), psi(1/2) = (-1/8, 3/4, 3/8)
def complete_hanging(hang: Dict[int, List[Tuple[int, float]]], min_weight: float = 1e-8,
                     rank: Optional[Dict[int, int]] = None) -> Dict[int, List[Tuple[int, float]]]:
    """Hang infos whose masters do not hang (oomph-lib's
    TreeBasedRefineableMeshBase::complete_hanging_nodes, refineable_mesh.cc:
    2214-2320): a master that hangs is replaced by its own masters, weights
    multiplied, recursively; then the list is merged -- entries with
    |weight| <= min_weight dropped, repeated masters summed.  oomph merges in
    a map keyed by the node's address, i.e. in the order the nodes were
    created; ``rank`` gives that order (default: the node number)."""
    def expand(n: int, w: float, out: List[Tuple[int, float]], depth: int = 0) -> None:
        if depth > 64:
            raise ValueError("cyclic hanging-node dependencies")
        if n in hang:
            for m, wm in hang[n]:
                expand(m, w * wm, out, depth + 1)
        else:
            out.append((n, w))

    done: Dict[int, List[Tuple[int, float]]] = {}
    for h in sorted(hang):
        lst: List[Tuple[int, float]] = []
        for m, w in hang[h]:
            expand(m, w, lst)
        merged: Dict[int, float] = {}
        for m, w in lst:
            if abs(w) > min_weight:
                merged[m] = merged.get(m, 0.0) + w
        key = (lambda m: rank[m]) if rank is not None else None
        done[h] = [(m, merged[m]) for m in sorted(merged, key=key)]
    return done


class AdaptiveQuadMesh(MeshTemplate):
    """A RectangularQuadMesh of Q2 quads refined by quadtrees to several
    levels: an element at level l (the base elements at 0) is split into its
    four sons SW, SE, NW, NE while ``refine(centre_x, centre_y, l)`` holds
    and l < max_level.  No 2:1 balance is imposed.

    As oomph-lib's refineable meshes after ``adapt``: the elements are the
    leaves of the forest in tree order (base elements in order, sons in
    order, depth first); the nodes are numbered by first encounter over the
    elements' local nodes (``Mesh::reorder_nodes``, mesh.cc:517-640); a node
    strictly inside an edge of a coarser neighbour (and not one of its
    nodes) hangs on that edge's three nodes with the 1D quadratic Lagrange
    weights at its position (``RefineableQElement<2>::setup_hang_for_value``);
    masters that hang themselves are resolved recursively
    (``complete_hanging``).  Positions are the base element's isoparametric
    map at the node's local coordinate.  The masters of a hang info are
    ordered as oomph creates the nodes: the base mesh's in template order,
    then, adapt by adapt (one level each), the new sons' in tree order and
    local node order, a node shared with an existing one created once."""

    def __init__(self, *, N: int = 8, refine=None, max_level: int = 2, size: float = 1.0, name: str = "domain",
                 transform=None):
        self.N = int(N)
        self.refine = refine or (lambda x, y, level: x < 0.5 ** (level + 1))
        self.max_level = int(max_level)
        if self.max_level < 0 or self.max_level > 12:
            raise ValueError("max_level must be in 0..12")
        self.size = float(size)
        self.domain_name = name
        self.transform = None
        self._post = transform

    def generate(self) -> MeshData:
        md = self._generate()
        if self._post is not None:
            md.x = np.ascontiguousarray(self._post(md.x.copy()), dtype=np.float64)
        return md

    def _generate(self) -> MeshData:
        from .spaces import Q2_QUAD
        N, L = self.N, self.max_level
        S = 2 ** (L + 1)                     # fine-lattice units per base cell (node spacing at level L)
        base = RectangularQuadMesh(N=N, size=self.size).generate()
        conn0, x0, lat0 = base.conn, base.x, base.lattice
        hcell = self.size / N
        leaves: List[Tuple[int, int, int, int]] = []   # (base element, qx0, qy0, span)
        splits: List[Tuple[int, int, int, int]] = []   # (level, qx0, qy0, span) of split elements, tree order

        def split(e: int, qx: int, qy: int, span: int, level: int) -> None:
            cx = (qx + 0.5 * span) * hcell / S
            cy = (qy + 0.5 * span) * hcell / S
            if level < L and bool(self.refine(cx, cy, level)):
                splits.append((level, qx, qy, span))
                h = span // 2
                for dy, dx in ((0, 0), (0, 1), (1, 0), (1, 1)):          # SW, SE, NW, NE
                    split(e, qx + dx * h, qy + dy * h, h, level + 1)
            else:
                leaves.append((e, qx, qy, span))

        for e in range(conn0.shape[0]):
            ix, iy = int(lat0[conn0[e, 0]][0]) // 2, int(lat0[conn0[e, 0]][1]) // 2
            split(e, ix * S, iy * S, S, 0)
        Q = N * S + 1
        key = lambda qx, qy: int(qx) + Q * int(qy)
        node_of: Dict[int, int] = {}
        xs: List[np.ndarray] = []
        qlat: List[Tuple[int, int]] = []
        conn: List[List[int]] = []
        for e, qx0, qy0, span in leaves:
            Xe = x0[conn0[e]]
            bx, by = (qx0 // S) * S, (qy0 // S) * S
            h = span // 2
            child = []
            for j in range(3):
                for i in range(3):
                    qx, qy = qx0 + i * h, qy0 + j * h
                    k = key(qx, qy)
                    if k not in node_of:
                        s = np.array([2.0 * (qx - bx) / S - 1.0, 2.0 * (qy - by) / S - 1.0])
                        psi, _ = Q2_QUAD.shape_c2(s)
                        node_of[k] = len(xs)
                        xs.append(psi @ Xe)
                        qlat.append((qx, qy))
                    child.append(node_of[k])
            conn.append(child)
        x = np.array(xs)
        ql = np.array(qlat, dtype=np.int64)
        n = x.shape[0]
        # leaf edges by line: horizontal (y, x_start, x_end), vertical (x, y_start, y_end)
        hor: Dict[int, List[Tuple[int, int]]] = {}
        ver: Dict[int, List[Tuple[int, int]]] = {}
        for _, qx0, qy0, span in leaves:
            for y in (qy0, qy0 + span):
                hor.setdefault(y, []).append((qx0, qx0 + span))
            for xq in (qx0, qx0 + span):
                ver.setdefault(xq, []).append((qy0, qy0 + span))
        hang: Dict[int, List[Tuple[int, float]]] = {}
        for k in range(n):
            qx, qy = int(ql[k, 0]), int(ql[k, 1])
            found = None
            for a, b in hor.get(qy, ()):
                if a < qx < b and 2 * qx != a + b:
                    found = ((a, qy), ((a + b) // 2, qy), (b, qy), 2.0 * (qx - a) / (b - a) - 1.0)
                    break
            if found is None:
                for a, b in ver.get(qx, ()):
                    if a < qy < b and 2 * qy != a + b:
                        found = ((qx, a), (qx, (a + b) // 2), (qx, b), 2.0 * (qy - a) / (b - a) - 1.0)
                        break
            if found is not None:
                pa, pm, pb, s = found
                w = (0.5 * s * (s - 1.0), 1.0 - s * s, 0.5 * s * (s + 1.0))
                hang[k] = [(node_of[key(*pa)], w[0]), (node_of[key(*pm)], w[1]), (node_of[key(*pb)], w[2])]
        # creation order: base nodes (template order), then adapt by adapt
        # the new sons' nodes in tree order and local node order
        rank: Dict[int, int] = {}
        for g in range(x0.shape[0]):
            rank[node_of[key(int(lat0[g][0]) * S // 2, int(lat0[g][1]) * S // 2)]] = g
        nxt = x0.shape[0]
        for level in range(L):
            for lv, qx0, qy0, span in splits:
                if lv != level:
                    continue
                h = span // 2
                for dy, dx in ((0, 0), (0, 1), (1, 0), (1, 1)):
                    for j in range(3):
                        for i in range(3):
                            k = node_of[key(qx0 + dx * h + i * (h // 2), qy0 + dy * h + j * (h // 2))]
                            if k not in rank:
                                rank[k] = nxt
                                nxt += 1
        hang = complete_hanging(hang, rank=rank)
        is_vertex = np.zeros(n, dtype=bool)
        for c in conn:
            for s_ in (0, 2, 6, 8):
                is_vertex[c[s_]] = True
        # C1 values (element vertices, bilinear): a vertex strictly inside an
        # edge of a coarser leaf -- the edge's midpoint too, which the C2
        # values share with that leaf -- hangs on the edge's two end
        # vertices with the 1D linear weights at its position (the vertices
        # are the C1 space's interpolating nodes in setup_hang_for_value:
        # BulkElementQuad2dC2::interpolating_node_pt, elements.cpp:9162-9250)
        hang_c1: Dict[int, List[Tuple[int, float]]] = {}
        for k in np.flatnonzero(is_vertex):
            qx, qy = int(ql[k, 0]), int(ql[k, 1])
            found = None
            for a, b in hor.get(qy, ()):
                if a < qx < b:
                    found = ((a, qy), (b, qy), (qx - a) / (b - a))
                    break
            if found is None:
                for a, b in ver.get(qx, ()):
                    if a < qy < b:
                        found = ((qx, a), (qx, b), (qy - a) / (b - a))
                        break
            if found is not None:
                pa, pb, t = found
                hang_c1[int(k)] = [(node_of[key(*pa)], 1.0 - t), (node_of[key(*pb)], t)]
        hang_c1 = complete_hanging(hang_c1, rank=rank)
        top = N * S
        b = {"left": ql[:, 0] == 0, "right": ql[:, 0] == top, "bottom": ql[:, 1] == 0, "top": ql[:, 1] == top}
        md = MeshData(ELEMENT_TYPES["Q2_QUAD"], x, np.array(conn, dtype=np.int32), is_vertex, b, ql)
        md.hang = hang
        md.hang_c1 = hang_c1
        return md


class RefinedQuadMesh(AdaptiveQuadMesh):
    """One level of quadtree refinement: the elements chosen by
    ``refine(centre_x, centre_y)`` are split once into their four sons (an
    AdaptiveQuadMesh with max_level 1: oomph's leaf order, node numbering
    and hang infos)."""

    def __init__(self, *, N: int = 8, refine=None, size: float = 1.0, name: str = "domain", transform=None):
        chosen = refine or (lambda x, y: x < 0.5)
        super().__init__(N=N, refine=lambda x, y, level: bool(chosen(x, y)), max_level=1, size=size, name=name,
                         transform=transform)
