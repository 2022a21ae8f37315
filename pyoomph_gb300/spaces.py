"""Element types of the engine: reference shape functions, integration
rules and the element-local value layout.

The tables are evaluated on the host in float64 and staged by every element
kernel into shared memory.  Their constants are the reference's own:

* Gauss<2,3> knots/weights, oomph ``integral.cc:84-102`` -- including the
  transposed digits (``0.774596662941483``) of some knots, which shift
  results at the 1e-9 level and so must be kept for 1e-12 parity;
* TGauss<2,3>, ``integral.cc:355-369`` (13-digit knots);
* Gauss<3,3>, ``integral.cc:169-206`` (14-digit knots and weights);
* one-dimensional Lagrange shapes ``shape.h:607-650``, the six-node
  triangle ``Telements.h:627-680`` and pyoomph's C1 sub-spaces
  (``elements.cpp:9274-9300, 10097-10130, 11163``).

Node order inside an element is oomph's: lexicographic with s0 fastest for
Q elements; vertices (1,0),(0,1),(0,0) then edge midpoints 01, 12, 20 for
the quadratic triangle.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List

import numpy as np

_K = 0.774596669241483
_K_TYPO = 0.774596662941483
# Gauss<2,3>::Knot (integral.cc:84-93)
GAUSS_Q2_KNOTS = np.array([
    [-_K, -_K], [-_K, 0.0], [-_K, _K_TYPO],
    [0.0, -_K], [0.0, 0.0], [0.0, _K_TYPO],
    [_K_TYPO, -_K], [_K_TYPO, 0.0], [_K_TYPO, _K_TYPO]])
GAUSS_Q2_WEIGHTS = np.array([25.0 / 81.0, 40.0 / 81.0, 25.0 / 81.0, 40.0 / 81.0, 64.0 / 81.0,
                             40.0 / 81.0, 25.0 / 81.0, 40.0 / 81.0, 25.0 / 81.0])
# TGauss<2,3> (integral.cc:355-369)
GAUSS_T2_KNOTS = np.array([
    [0.1012865073235, 0.1012865073235], [0.7974269853531, 0.1012865073235],
    [0.1012865073235, 0.7974269853531], [0.4701420641051, 0.0597158717898],
    [0.4701420641051, 0.4701420641051], [0.0597158717898, 0.4701420641051],
    [0.3333333333333, 0.3333333333333]])
GAUSS_T2_WEIGHTS = np.array([0.5 * 0.1259391805448] * 3 + [0.5 * 0.1323941527885] * 3 + [0.5 * 0.225])
# Gauss<3,3> (integral.cc:169-206): 14-digit knots, first coordinate slowest
_K3 = 0.77459666924148
_G3_1D = np.array([-_K3, 0.0, _K3])
GAUSS_H3_KNOTS = np.array([[_G3_1D[i // 9], _G3_1D[(i // 3) % 3], _G3_1D[i % 3]] for i in range(27)])
GAUSS_H3_WEIGHTS = np.array([
    0.17146776406035, 0.27434842249657, 0.17146776406035, 0.27434842249657,
    0.43895747599451, 0.27434842249657, 0.17146776406035, 0.27434842249657,
    0.17146776406035, 0.27434842249657, 0.43895747599451, 0.27434842249657,
    0.43895747599451, 0.70233196159122, 0.43895747599451, 0.27434842249657,
    0.43895747599451, 0.27434842249657, 0.17146776406035, 0.27434842249657,
    0.17146776406035, 0.27434842249657, 0.43895747599451, 0.27434842249657,
    0.17146776406035, 0.27434842249657, 0.17146776406035])


def _lag3(s):
    p = np.array([0.5 * s * (s - 1.0), 1.0 - s * s, 0.5 * s * (s + 1.0)])
    d = np.array([s - 0.5, -2.0 * s, s + 0.5])
    return p, d


def _lag2(s):
    return np.array([0.5 * (1.0 - s), 0.5 * (1.0 + s)]), np.array([-0.5, 0.5])


def _tensor(s, dim, lag):
    """Tensor-product shapes, node index lexicographic with s0 fastest."""
    pd = [lag(s[k]) for k in range(dim)]
    n1 = len(pd[0][0])
    nn = n1 ** dim
    psi = np.zeros(nn)
    dps = np.zeros((nn, dim))
    for n in range(nn):
        idx = [(n // n1 ** k) % n1 for k in range(dim)]  # idx[0] = s0 index
        # psi = psi_{d-1}[i_{d-1}] * ... * psi_0[i_0] (oomph's product order)
        val = 1.0
        for k in reversed(range(dim)):
            val = val * pd[k][0][idx[k]] if k != dim - 1 else pd[k][0][idx[k]]
        psi[n] = val
        for a in range(dim):
            v = 1.0
            first = True
            for k in reversed(range(dim)):
                f = pd[k][1][idx[k]] if k == a else pd[k][0][idx[k]]
                v = f if first else v * f
                first = False
            dps[n, a] = v
    return psi, dps


def _tri6(s):
    s2 = 1.0 - s[0] - s[1]
    psi = np.array([2.0 * s[0] * (s[0] - 0.5), 2.0 * s[1] * (s[1] - 0.5), 2.0 * s2 * (s2 - 0.5),
                    4.0 * s[0] * s[1], 4.0 * s[1] * s2, 4.0 * s2 * s[0]])
    dps = np.array([
        [4.0 * s[0] - 1.0, 0.0],
        [0.0, 4.0 * s[1] - 1.0],
        [2.0 * (2.0 * s[0] - 1.5 + 2.0 * s[1]), 2.0 * (2.0 * s[0] - 1.5 + 2.0 * s[1])],
        [4.0 * s[1], 4.0 * s[0]],
        [-4.0 * s[1], 4.0 * (1.0 - s[0] - 2.0 * s[1])],
        [4.0 * (1.0 - 2.0 * s[0] - s[1]), -4.0 * s[0]]])
    return psi, dps


def _tri3(s):
    return np.array([s[0], s[1], 1.0 - s[0] - s[1]]), np.array([[1.0, 0.0], [0.0, 1.0], [-1.0, -1.0]])


@dataclass(frozen=True)
class ElementType:
    name: str
    dim: int
    nnode: int           # C2 (position) nodes
    nnode_c1: int
    c1_index: tuple      # element-local indices of the C1 nodes
    knots: np.ndarray
    weights: np.ndarray

    @property
    def nq(self) -> int:
        return len(self.weights)

    def shape_c2(self, s):
        if self.name == "Q2_QUAD":
            return _tensor(s, 2, _lag3)
        if self.name == "P2_TRI":
            return _tri6(s)
        return _tensor(s, 3, _lag3)

    def shape_c1(self, s):
        if self.name == "Q2_QUAD":
            return _tensor(s, 2, _lag2)
        if self.name == "P2_TRI":
            return _tri3(s)
        return _tensor(s, 3, _lag2)

    def tables(self):
        """Reference tables at the knots, in the layout the kernels stage:
        W[NQ], PSI2[NQ][NN], DPS2[NQ][NN][DIM], PSI1[NQ][NN1], DPS1[NQ][NN1][DIM]."""
        nq, nn, n1, dim = self.nq, self.nnode, self.nnode_c1, self.dim
        psi2 = np.zeros((nq, nn))
        dps2 = np.zeros((nq, nn, dim))
        psi1 = np.zeros((nq, n1))
        dps1 = np.zeros((nq, n1, dim))
        for q in range(nq):
            psi2[q], dps2[q] = self.shape_c2(self.knots[q])
            psi1[q], dps1[q] = self.shape_c1(self.knots[q])
        return dict(W=self.weights.copy(), PSI2=psi2, DPS2=dps2, PSI1=psi1, DPS1=dps1)

    def packed_tables(self) -> np.ndarray:
        t = self.tables()
        return np.concatenate([t["W"].ravel(), t["PSI2"].ravel(), t["DPS2"].ravel(),
                               t["PSI1"].ravel(), t["DPS1"].ravel()]).astype(np.float64)


Q2_QUAD = ElementType("Q2_QUAD", 2, 9, 4, (0, 2, 6, 8), GAUSS_Q2_KNOTS, GAUSS_Q2_WEIGHTS)
P2_TRI = ElementType("P2_TRI", 2, 6, 3, (0, 1, 2), GAUSS_T2_KNOTS, GAUSS_T2_WEIGHTS)
Q2_HEX = ElementType("Q2_HEX", 3, 27, 8, (0, 2, 6, 8, 18, 20, 24, 26), GAUSS_H3_KNOTS, GAUSS_H3_WEIGHTS)
ELEMENT_TYPES = {e.name: e for e in (Q2_QUAD, P2_TRI, Q2_HEX)}


@dataclass
class Layout:
    """Element-local values, node-major (the order oomph numbers an element's
    nodal values, ``elements.cc:694``): for each node in element order, the
    fields present there in nodal-value order (C2 fields at every node, C1
    fields at C1 nodes)."""
    node: List[int]      # element node slot of local value k
    val: List[int]       # nodal value index (= field index) of local value k
    field: List[int]
    sub: List[int]       # index of the node inside its field's space
    loc_of: List[List[int]]  # loc_of[field][sub] -> local index

    @property
    def n(self) -> int:
        return len(self.node)


def make_layout(et: ElementType, field_spaces: List[str]) -> Layout:
    nf = len(field_spaces)
    node, val, field, sub = [], [], [], []
    loc_of = [[-1] * (et.nnode if sp == "C2" else et.nnode_c1) for sp in field_spaces]
    for l in range(et.nnode):
        for f, sp in enumerate(field_spaces):
            if sp == "C2":
                k = l
            else:
                if l not in et.c1_index:
                    continue
                k = et.c1_index.index(l)
            loc_of[f][k] = len(node)
            node.append(l)
            val.append(f)
            field.append(f)
            sub.append(k)
    return Layout(node, val, field, sub, loc_of)
