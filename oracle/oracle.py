"""CPU oracle for the pyoomph residual/Jacobian assembly path.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py`` as the checker; never by the
package ``pyoomph_gb300``.

Wraps ``oracle/fe_oracle.c`` (restated mesh order, shape/geometry, element
residuals and the vectors-of-pairs sparse assembler of oomph-lib
``problem.cc:5332-5666``) and adds, in numpy/scipy:

* global equation numbering (oomph ``mesh.cc:686-708``: nodes in mesh order,
  values in node order, pinned values get no number);
* the Newton loop of ``Problem::newton_solve`` (``problem.cc:8986-9300``):
  residual max-norm with NaN -> inf (``double_vector.cc:611-629``), linear
  solve with SuperLU (``scipy.sparse.linalg.splu``, the reference's default
  serial solver, ``pyoomph/solvers/scipy.py``), update ``x -= dx``.

When the reference tree is present, ``ref_driver_assemble`` runs the
reference's own oomph-lib core (built by ``oracle/ref/Makefile`` into
``oracle/_ref/``) on the same input, which pins this restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfe_oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "oomph_ref_driver")

Q2_QUAD, P2_TRI, Q2_HEX = 0, 1, 2
EQ_POISSON, EQ_NAVIER_STOKES_TH, EQ_NONLINEAR_DIFFUSION = 0, 1, 2
B_LEFT, B_RIGHT, B_BOTTOM, B_TOP, B_BACK, B_FRONT = 1, 2, 4, 8, 16, 32

_lib = None


def build() -> str:
    """Compile the C oracle (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class _CSR(ctypes.Structure):
    _fields_ = [
        ("n_dof", ctypes.c_int64),
        ("nnz", ctypes.c_int64),
        ("rowptr", ctypes.POINTER(ctypes.c_int32)),
        ("colidx", ctypes.POINTER(ctypes.c_int32)),
        ("vals", ctypes.POINTER(ctypes.c_double)),
        ("residual", ctypes.POINTER(ctypes.c_double)),
    ]


JIT_LIB_PATH = os.path.join(HERE, "_build", "libfe_oracle_jit.so")


def use_jit_flags_build() -> str:
    """Switch this process to the oracle built with pyoomph's JIT flags
    (-O3 -march=native, the timed CPU baseline); returns the flags used."""
    global _lib, LIB_PATH
    if not os.path.exists(JIT_LIB_PATH):
        build()
    LIB_PATH, _lib = JIT_LIB_PATH, None
    lib()
    with open(os.path.join(HERE, "_build", "jit_flags.txt")) as f:
        return f.read().strip()


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        p = ctypes.c_void_p
        L.ofe_mesh_sizes.argtypes = [ctypes.c_int] * 4 + [p, p, p]
        L.ofe_mesh_fill.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double] * 3 + [ctypes.c_int, p, p, p, p]
        L.ofe_assemble.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int, p,
                                   ctypes.c_int64, p, ctypes.c_int, p, p, ctypes.c_int64, p,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ofe_assemble.restype = ctypes.POINTER(_CSR)
        L.ofe_csr_free.argtypes = [ctypes.POINTER(_CSR)]
        L.ofe_pairs_from_elements.argtypes = [ctypes.c_int64, ctypes.c_int, p, p, ctypes.c_int64, ctypes.c_double]
        L.ofe_pairs_from_elements.restype = ctypes.POINTER(_CSR)
        L.ofe_element_res_jac.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, p, p, ctypes.c_int,
                                          p, p, p, ctypes.c_int, p, p]
        L.ofe_element_mass.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, p, p, ctypes.c_double, p]
        L.ofe_n_intpt.argtypes = [ctypes.c_int]
        L.ofe_intpt.argtypes = [ctypes.c_int, ctypes.c_int, p, p]
        L.ofe_shape_c2.argtypes = [ctypes.c_int, p, p, p]
        L.ofe_shape_c1.argtypes = [ctypes.c_int, p, p, p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Mesh:
    etype: int
    dim: int
    x: np.ndarray          # [n_nodes, dim]
    conn: np.ndarray       # [n_elem, nne] int32
    bmask: np.ndarray      # [n_nodes] uint32
    is_vertex: np.ndarray  # [n_nodes] uint8


def mesh(etype: int, nx: int, ny: int, nz: int = 0, lx: float = 1.0, ly: float = 1.0,
         lz: float = 1.0, split: int = 0) -> Mesh:
    """Structured mesh in pyoomph's node and element order
    (simplemeshes.py:225-305 / :515-545, meshtemplate.cpp C2 conversion)."""
    L = lib()
    nn = ctypes.c_int64()
    ne = ctypes.c_int64()
    nne = ctypes.c_int()
    if L.ofe_mesh_sizes(etype, nx, ny, nz, ctypes.byref(nn), ctypes.byref(ne), ctypes.byref(nne)):
        raise ValueError("bad mesh size")
    dim = 3 if etype == Q2_HEX else 2
    x = np.zeros((nn.value, dim))
    conn = np.zeros((ne.value, nne.value), dtype=np.int32)
    bmask = np.zeros(nn.value, dtype=np.uint32)
    isv = np.zeros(nn.value, dtype=np.uint8)
    rc = L.ofe_mesh_fill(etype, nx, ny, nz, lx, ly, lz, split, _ptr(x), _ptr(conn), _ptr(bmask), _ptr(isv))
    if rc:
        raise RuntimeError(f"ofe_mesh_fill failed: {rc}")
    return Mesh(etype, dim, x, conn, bmask, isv)


def number_equations(nvalue: np.ndarray, pinned: np.ndarray) -> tuple[np.ndarray, int]:
    """Mesh::assign_global_eqn_numbers (mesh.cc:686-708) restated:
    nodes in order, values in order, pinned or absent values -> -1."""
    n_nodes, nval = pinned.shape
    present = np.arange(nval)[None, :] < nvalue[:, None]
    free = present & (pinned == 0)
    eqn = np.full((n_nodes, nval), -1, dtype=np.int32)
    flat = free.reshape(-1)
    eqn.reshape(-1)[flat] = np.arange(int(flat.sum()), dtype=np.int32)
    return eqn, int(flat.sum())


@dataclass
class Problem:
    """One oracle problem: mesh, equation, nodal values and pins."""
    mesh: Mesh
    eq: int
    nval: int
    nvalue: np.ndarray        # [n_nodes] values present per node
    pinned: np.ndarray        # [n_nodes, nval] int32
    values: np.ndarray        # [n_nodes, nval] float64
    params: np.ndarray        # float64
    eqn: np.ndarray = field(default=None)
    n_dof: int = 0

    def __post_init__(self):
        self.eqn, self.n_dof = number_equations(self.nvalue, self.pinned)

    def dofs(self) -> np.ndarray:
        m = self.eqn >= 0
        x = np.zeros(self.n_dof)
        x[self.eqn[m]] = self.values[m]
        return x

    def set_dofs(self, x: np.ndarray) -> None:
        m = self.eqn >= 0
        self.values[m] = x[self.eqn[m]]


def assemble(P: Problem, with_jac: bool = True, zero_threshold: float = 0.0):
    """R (and CSR J) by the restated vectors-of-pairs assembler."""
    L = lib()
    m = P.mesh
    x = np.ascontiguousarray(m.x, dtype=np.float64)
    conn = np.ascontiguousarray(m.conn, dtype=np.int32)
    vals = np.ascontiguousarray(P.values, dtype=np.float64)
    eqn = np.ascontiguousarray(P.eqn, dtype=np.int32)
    params = np.ascontiguousarray(P.params, dtype=np.float64)
    c = L.ofe_assemble(m.etype, P.eq, x.shape[0], m.dim, _ptr(x), conn.shape[0], _ptr(conn), P.nval,
                       _ptr(vals), _ptr(eqn), P.n_dof, _ptr(params), len(params), int(with_jac),
                       float(zero_threshold))
    if not c:
        raise RuntimeError("ofe_assemble failed")
    try:
        cc = c.contents
        n = cc.n_dof
        R = np.ctypeslib.as_array(cc.residual, shape=(max(n, 1),))[:n].copy()
        if not with_jac:
            return R
        nnz = cc.nnz
        rowptr = np.ctypeslib.as_array(cc.rowptr, shape=(n + 1,)).copy()
        colidx = np.ctypeslib.as_array(cc.colidx, shape=(max(nnz, 1),))[:nnz].copy()
        v = np.ctypeslib.as_array(cc.vals, shape=(max(nnz, 1),))[:nnz].copy()
        return R, rowptr, colidx, v
    finally:
        L.ofe_csr_free(c)


def vectors_of_pairs(elem_eqns, Je, n_dof: int, threshold: float = 0.0):
    """CSR of Problem::sparse_assemble_row_or_column_compressed_with_vectors_
    of_pairs (problem.cc:5459-5660) over GIVEN element matrices, restated in
    pure Python for small cases: elements in order, local i then local j;
    an entry with |J_e(i,j)| <= threshold is skipped (problem.cc:5520-5524,
    NaN included); otherwise row eqn_i is searched for column eqn_j
    (problem.cc:5530-5545) and the value added, or the pair appended.  A
    negative threshold keeps every structural coupling.  elem_eqns[e][k]:
    global equation of local value k of element e (-1: none); Je[e]: its
    element matrix.  Returns (rowptr, colidx, values)."""
    rows = [[] for _ in range(n_dof)]
    where = [dict() for _ in range(n_dof)]        # the linear search's answer, found faster
    for e in range(len(elem_eqns)):
        eq = [int(q) for q in elem_eqns[e]]
        Jm = Je[e]
        for i, ei in enumerate(eq):
            if ei < 0:
                continue
            for j, ej in enumerate(eq):
                if ej < 0:
                    continue
                v = float(Jm[i][j])
                if abs(v) > threshold:
                    k = where[ei].get(ej)
                    if k is None:
                        where[ei][ej] = len(rows[ei])
                        rows[ei].append([ej, v])
                    else:
                        rows[ei][k][1] += v
    rowptr = np.zeros(n_dof + 1, dtype=np.int32)
    for r in range(n_dof):
        rowptr[r + 1] = rowptr[r] + len(rows[r])
    colidx = np.array([c for row in rows for c, _ in row], dtype=np.int32)
    vals = np.array([v for row in rows for _, v in row], dtype=np.float64)
    return rowptr, colidx, vals


def pairs_from_elements(elem_eqns: np.ndarray, Je: np.ndarray, n_dof: int, threshold: float = 0.0):
    """vectors_of_pairs in C (ofe_pairs_from_elements), for full-size meshes:
    (rowptr, colidx, values)."""
    L = lib()
    eq = np.ascontiguousarray(elem_eqns, dtype=np.int32)
    J = np.ascontiguousarray(Je, dtype=np.float64)
    E, n = eq.shape
    c = L.ofe_pairs_from_elements(E, n, _ptr(eq), _ptr(J), n_dof, float(threshold))
    if not c:
        raise RuntimeError("ofe_pairs_from_elements failed")
    try:
        cc = c.contents
        nnz = cc.nnz
        rowptr = np.ctypeslib.as_array(cc.rowptr, shape=(n_dof + 1,)).copy()
        colidx = np.ctypeslib.as_array(cc.colidx, shape=(max(nnz, 1),))[:nnz].copy()
        v = np.ctypeslib.as_array(cc.vals, shape=(max(nnz, 1),))[:nnz].copy()
        return rowptr, colidx, v
    finally:
        L.ofe_csr_free(c)


def max_norm(R: np.ndarray) -> float:
    """DoubleVector::max (double_vector.cc:611-629): max |r|, NaN -> inf."""
    if R.size == 0:
        return 0.0
    if np.isnan(R).any():
        return float("inf")
    return float(np.max(np.abs(R)))


def newton(P: Problem, tol: float = 1e-10, max_iter: int = 20, max_residual: float = 1e10):
    """Problem::newton_solve (problem.cc:8986-9300) with SuperLU solves.
    Returns the list of residual max-norms (first = initial)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    hist = []
    R = assemble(P, with_jac=False)
    hist.append(max_norm(R))
    it = 0
    while hist[-1] > tol:
        if it >= max_iter or hist[-1] > max_residual:
            raise RuntimeError(f"Newton failed: residuals {hist}")
        R, rp, ci, v = assemble(P, with_jac=True)
        A = sp.csr_matrix((v, ci, rp), shape=(P.n_dof, P.n_dof))
        dx = spla.splu(A.tocsc()).solve(R)
        x = P.dofs() - dx
        P.set_dofs(x)
        R = assemble(P, with_jac=False)
        hist.append(max_norm(R))
        it += 1
    return hist


def ref_driver_available() -> bool:
    return os.path.exists(REF_DRIVER)


def ref_driver_assemble(P: Problem, with_jac: bool = True, zero_threshold: float = 0.0):
    """Run the reference's own oomph-lib Problem::get_jacobian on P.
    Returns (eqn, R, rowptr, colidx, vals)."""
    m = P.mesh
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.bin")
        fout = os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([m.etype, P.eq, m.dim, P.nval], dtype=np.int32).tofile(f)
            np.array([m.x.shape[0], m.conn.shape[0]], dtype=np.int64).tofile(f)
            np.array([m.conn.shape[1], len(P.params), int(with_jac)], dtype=np.int32).tofile(f)
            np.array([zero_threshold], dtype=np.float64).tofile(f)
            np.ascontiguousarray(m.x, dtype=np.float64).tofile(f)
            np.ascontiguousarray(m.conn, dtype=np.int32).tofile(f)
            np.ascontiguousarray(P.nvalue, dtype=np.int32).tofile(f)
            np.ascontiguousarray(P.pinned, dtype=np.int32).tofile(f)
            np.ascontiguousarray(P.values, dtype=np.float64).tofile(f)
            np.ascontiguousarray(P.params, dtype=np.float64).tofile(f)
        subprocess.run([REF_DRIVER, "assemble", fin, fout], check=True)
        with open(fout, "rb") as f:
            n_dof, nnz = np.fromfile(f, dtype=np.int64, count=2)
            eqn = np.fromfile(f, dtype=np.int32, count=P.eqn.size).reshape(P.eqn.shape)
            R = np.fromfile(f, dtype=np.float64, count=n_dof)
            if not with_jac:
                return eqn, R
            rp = np.fromfile(f, dtype=np.int32, count=n_dof + 1)
            ci = np.fromfile(f, dtype=np.int32, count=nnz)
            v = np.fromfile(f, dtype=np.float64, count=nnz)
    return eqn, R, rp, ci, v


def ref_driver_tables():
    """oomph's integration knots/weights and C2 shape tables, per element type."""
    with tempfile.TemporaryDirectory() as td:
        fout = os.path.join(td, "t.bin")
        subprocess.run([REF_DRIVER, "tables", fout], check=True)
        raw = open(fout, "rb").read()
    out = {}
    off = 0
    for et in (Q2_QUAD, P2_TRI, Q2_HEX):
        nq, dim, nn = np.frombuffer(raw, dtype=np.int32, count=3, offset=off)
        off += 12
        per = dim + 1 + nn + nn * dim
        arr = np.frombuffer(raw, dtype=np.float64, count=nq * per, offset=off).reshape(nq, per)
        off += nq * per * 8
        out[et] = dict(s=arr[:, :dim], w=arr[:, dim], psi=arr[:, dim + 1:dim + 1 + nn],
                       dpsi=arr[:, dim + 1 + nn:].reshape(nq, nn, dim))
    return out


def oracle_tables(etype: int):
    """The restated tables, in the same layout as ref_driver_tables."""
    L = lib()
    nq = L.ofe_n_intpt(etype)
    dim = 3 if etype == Q2_HEX else 2
    nn = {Q2_QUAD: 9, P2_TRI: 6, Q2_HEX: 27}[etype]
    s = np.zeros((nq, 3))
    w = np.zeros(nq)
    psi = np.zeros((nq, nn))
    dpsi = np.zeros((nq, nn, dim))
    for q in range(nq):
        sq = np.zeros(3)
        wq = np.zeros(1)
        L.ofe_intpt(etype, q, _ptr(sq), _ptr(wq))
        s[q] = sq
        w[q] = wq[0]
        p = np.zeros(nn)
        d = np.zeros((nn, dim))
        L.ofe_shape_c2(etype, _ptr(sq), _ptr(p), _ptr(d))
        psi[q] = p
        dpsi[q] = d
    return dict(s=s[:, :dim], w=w, psi=psi, dpsi=dpsi)


# --------------------------------------------------------------------------
# The workloads, restated: boundary pins, initial values and parameters.
# --------------------------------------------------------------------------

def gaussian_params(gaussians: np.ndarray) -> np.ndarray:
    """Pack [n, dim+2] rows (centre..., width, amplitude) into oracle params."""
    g = np.asarray(gaussians, dtype=np.float64)
    return np.concatenate([[float(g.shape[0])], g.reshape(-1)])


def poisson_problem(m: Mesh, gaussians: np.ndarray, eq: int = EQ_POISSON) -> Problem:
    """u = 0 on every boundary node, one value per node (poisson.py:66-69)."""
    n = m.x.shape[0]
    pinned = (m.bmask != 0).astype(np.int32)[:, None]
    return Problem(mesh=m, eq=eq, nval=1, nvalue=np.ones(n, dtype=np.int32), pinned=pinned,
                   values=np.zeros((n, 1)), params=gaussian_params(gaussians))


def lid_velocity(x: np.ndarray) -> np.ndarray:
    return 16.0 * x * x * (1.0 - x) * (1.0 - x)


def navier_stokes_problem(m: Mesh, rho: float = 1.0, mu: float = 0.01,
                          perturb: Optional[np.ndarray] = None) -> Problem:
    """Lid-driven cavity, Taylor-Hood: velocity pinned on the boundary
    (u_x = 16x^2(1-x)^2 on top, no-slip elsewhere), pressure pinned at the
    first node of the first element (PressureFixationTaylorHood,
    navier_stokes.py:55-85)."""
    n = m.x.shape[0]
    nvalue = np.where(m.is_vertex != 0, 3, 2).astype(np.int32)
    pinned = np.zeros((n, 3), dtype=np.int32)
    onb = m.bmask != 0
    pinned[onb, 0] = 1
    pinned[onb, 1] = 1
    pinned[int(m.conn[0, 0]), 2] = 1
    values = np.zeros((n, 3))
    top = (m.bmask & B_TOP) != 0
    values[top, 0] = lid_velocity(m.x[top, 0])
    P = Problem(mesh=m, eq=EQ_NAVIER_STOKES_TH, nval=3, nvalue=nvalue, pinned=pinned,
                values=values, params=np.array([rho, mu]))
    if perturb is not None:
        P.set_dofs(P.dofs() + perturb)
    return P
