"""Device solve of saddle-point Newton systems (Taylor-Hood Navier-Stokes).

The reference solves every Newton system J dx = R on the host with SuperLU
(``pyoomph/solvers/scipy.py``, ``src/pybind/solver.cpp:105-133``).  For a
Jacobian with a zero diagonal block -- velocity u and pressure p,

    J = [[A, Bt],
         [B,  0]],

Jacobi- or ILU-preconditioned Krylov methods need iteration counts that grow
with the mesh.  This solver keeps everything on the device and converges in
a mesh-independent number of iterations:

* flexible right-preconditioned GMRES (restarted, classical Gram-Schmidt
  applied twice; the preconditioned vectors kept for the update; the
  Hessenberg matrix stays on the device and the host reads it every few
  iterations for the Givens rotations) on the resident CSR Jacobian
  (``fe_csr_spmv``), to the relative tolerance of an inexact Newton step
  (``newton_forcing``);
* the block upper-triangular preconditioner P = [[A, Bt], [0, S_hat]]:
  p = S_hat^-1 r_p, u = A_hat^-1 (r_u - Bt p), which would need two GMRES
  iterations with exact blocks;
* S_hat = sigma M_p / mu: the lumped mass matrix of the pressure space
  divided by the viscosity, spectrally equivalent to the Schur complement
  -B A^-1 Bt of Stokes-dominated flow; the sign sigma is measured on the
  matrix itself;
* A_hat^-1 = one V-cycle of smoothed-aggregation multigrid on the velocity
  block (aggregates of strongly coupled unknowns of the same component,
  ``fe_sa_aggregate``; prolongators smoothed by one damped-Jacobi step;
  Galerkin coarse operators; damped-Jacobi smoothing; a dense inverse on
  the coarsest level), every level applied with the library's CSR kernel;
* the preconditioner in FP32 by default (``fe_csr_update_f32``): on GB300
  the FP64 pipe bounds an FP64 SpMV, and flexible GMRES takes an inexact
  preconditioner at no cost in accuracy.

The hierarchy is built on the host once, from the first Jacobian, and kept
for the following Newton steps (only the finest velocity block is refreshed
from each new Jacobian): the preconditioner changes slowly along a Newton
solve, and GMRES stays exact whatever the preconditioner.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional

import numpy as np

from . import _native as N
from .linsolve import DeviceCSR, LinearSolverError


class _DevCSR:
    """A CSR matrix on the device in the layout of fe_csr_spmv (int32
    indices, FP64 or FP32 values -- with vectors of the same type);
    rectangular matrices too."""

    def __init__(self, torch, A, dev, dtype=None):
        A = A.tocsr()
        A.sort_indices()
        self.n, self.m = A.shape
        self.nnz = int(A.nnz)
        self.f32 = dtype is not None and dtype == torch.float32
        npd = np.float32 if self.f32 else np.float64
        self.rp = torch.as_tensor(A.indptr.astype(np.int32), device=dev)
        self.ci = torch.as_tensor(A.indices.astype(np.int32) if A.nnz else np.zeros(1, np.int32), device=dev)
        self.v = torch.as_tensor(A.data.astype(npd) if A.nnz else np.zeros(1, npd), device=dev)

    def update(self, x, b, z, w, sc: float, y, stream) -> None:
        """y = z + sc * w o (b - A x) (fe_csr_update / _f32; None: 0, 0, 1)."""
        if self.n == 0:
            return
        ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        f = N.load().fe_csr_update_f32 if self.f32 else N.load().fe_csr_update
        N.check(f(ctypes.c_void_p(self.rp.data_ptr()), ctypes.c_void_p(self.ci.data_ptr()),
                  ctypes.c_void_p(self.v.data_ptr()), ptr(x), ptr(b), ptr(z), ptr(w),
                  float(sc), ctypes.c_void_p(y.data_ptr()), self.n, self.nnz, ctypes.c_void_p(stream)))

    def mv(self, x, y, stream) -> None:
        """y = A x."""
        if self.n == 0:
            return
        if self.f32:
            self.update(x, None, None, None, -1.0, y, stream)
            return
        N.check(N.load().fe_csr_spmv(ctypes.c_void_p(self.rp.data_ptr()), ctypes.c_void_p(self.ci.data_ptr()),
                                     ctypes.c_void_p(self.v.data_ptr()), N.FE_JAC_F64,
                                     ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), self.n,
                                     self.nnz, ctypes.c_void_p(stream)))


def aggregate(A, comp: np.ndarray, theta: float):
    """Aggregates of A's unknowns (fe_sa_aggregate): (agg [n], n_agg)."""
    A = A.tocsr()
    n = A.shape[0]
    agg = np.zeros(max(n, 1), dtype=np.int32)
    na = ctypes.c_int64()
    rp = np.ascontiguousarray(A.indptr, dtype=np.int32)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    v = np.ascontiguousarray(A.data, dtype=np.float64)
    c = np.ascontiguousarray(comp, dtype=np.int32)
    N.check(N.load().fe_sa_aggregate(n, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, c.ctypes.data,
                                     float(theta), agg.ctypes.data, ctypes.byref(na)))
    return agg[:n], int(na.value)


class _Block:
    """The pattern of one block of a CSR matrix (fe_csr_block): indptr,
    indices (columns ascending), shape, and each entry's slot in the
    matrix."""

    def __init__(self, indptr, indices, slots, shape):
        self.indptr, self.indices, self.slots, self.shape = indptr, indices, slots, shape


def csr_block(rp, ci, label: np.ndarray, rl: int, cl: int) -> _Block:
    """Rows labelled rl and columns labelled cl of the CSR pattern (rp, ci),
    renumbered within their label."""
    rp = np.ascontiguousarray(rp, dtype=np.int32)
    ci = np.ascontiguousarray(ci, dtype=np.int32)
    n = rp.size - 1
    L = N.load()
    nnz = ctypes.c_int64()
    N.check(L.fe_csr_block(n, rp.ctypes.data, ci.ctypes.data, label.ctypes.data, rl, cl, ctypes.byref(nnz),
                           None, None, None))
    nr, nc = int(np.count_nonzero(label == rl)), int(np.count_nonzero(label == cl))
    indptr = np.zeros(nr + 1, np.int32)
    indices = np.zeros(max(nnz.value, 1), np.int32)
    slots = np.zeros(max(nnz.value, 1), np.int64)
    N.check(L.fe_csr_block(n, rp.ctypes.data, ci.ctypes.data, label.ctypes.data, rl, cl, ctypes.byref(nnz),
                           indptr.ctypes.data, indices.ctypes.data, slots.ctypes.data))
    return _Block(indptr, indices[:nnz.value], slots[:nnz.value], (nr, nc))


def sa_level(A, agg: np.ndarray, n_agg: int):
    """One smoothed-aggregation level of A from its aggregates
    (fe_sa_level_build, host threads): (P, Ac, lam) with lam = 1.1 x the
    largest eigenvalue of D^-1 A, P = P0 - (4/3)/lam D^-1 A P0 (P0 the
    aggregation) and Ac = P^T A P, as scipy CSR matrices."""
    import scipy.sparse as sps
    A = A.tocsr()
    n = A.shape[0]
    rp = np.ascontiguousarray(A.indptr, dtype=np.int32)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    v = np.ascontiguousarray(A.data, dtype=np.float64)
    a = np.ascontiguousarray(agg, dtype=np.int32)
    L = N.load()
    h = ctypes.c_void_p()
    N.check(L.fe_sa_level_build(n, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, a.ctypes.data, int(n_agg),
                                ctypes.byref(h)))
    try:
        nnz_p, nnz_a, lam = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        N.check(L.fe_sa_level_info(h, ctypes.byref(nnz_p), ctypes.byref(nnz_a), ctypes.byref(lam)))
        prp, arp = np.empty(n + 1, np.int32), np.empty(n_agg + 1, np.int32)
        pci, pv = np.empty(max(nnz_p.value, 1), np.int32), np.empty(max(nnz_p.value, 1))
        aci, av = np.empty(max(nnz_a.value, 1), np.int32), np.empty(max(nnz_a.value, 1))
        N.check(L.fe_sa_level_copy(h, prp.ctypes.data, pci.ctypes.data, pv.ctypes.data, arp.ctypes.data,
                                   aci.ctypes.data, av.ctypes.data))
    finally:
        L.fe_sa_level_destroy(h)
    P = sps.csr_matrix((pv[:nnz_p.value], pci[:nnz_p.value], prp), shape=(n, n_agg))
    Ac = sps.csr_matrix((av[:nnz_a.value], aci[:nnz_a.value], arp), shape=(n_agg, n_agg))
    return P, Ac, float(lam.value)


def lumped_field_mass(P, field: str) -> np.ndarray:
    """Row sums of the mass matrix of one field (lumped mass), per dof of
    that field: sum over elements and knots of w |det J| psi_k."""
    mesh, et = P.mesh, P.mesh.etype
    t = et.tables()
    names = [n_ for n_, _ in P.fields]
    f = names.index(field)
    space = P.fields[f][1]
    W = np.asarray(t["W"]).reshape(et.nq)
    dps2 = np.asarray(t["DPS2"]).reshape(et.nq, et.nnode, et.dim)
    if space == "C1":
        psi = np.asarray(t["PSI1"]).reshape(et.nq, et.nnode_c1)
        slots = np.asarray(et.c1_index)
    else:
        psi = np.asarray(t["PSI2"]).reshape(et.nq, et.nnode)
        slots = np.arange(et.nnode)
    X = mesh.x[mesh.conn]                              # [E, nnode, dim]
    G = np.tensordot(X, dps2, axes=([1], [1]))         # dx_d/ds_b: [E, dim, nq, dim]
    if et.dim == 2:
        det = G[:, 0, :, 0] * G[:, 1, :, 1] - G[:, 0, :, 1] * G[:, 1, :, 0]
    elif et.dim == 3:
        det = (G[:, 0, :, 0] * (G[:, 1, :, 1] * G[:, 2, :, 2] - G[:, 1, :, 2] * G[:, 2, :, 1])
               - G[:, 0, :, 1] * (G[:, 1, :, 0] * G[:, 2, :, 2] - G[:, 1, :, 2] * G[:, 2, :, 0])
               + G[:, 0, :, 2] * (G[:, 1, :, 0] * G[:, 2, :, 1] - G[:, 1, :, 1] * G[:, 2, :, 0]))
    else:
        det = G[:, 0, :, 0]
    contrib = (np.abs(det) * W) @ psi                  # [E, nslots]
    eqn = np.asarray(P.eqn).reshape(mesh.n_nodes, len(P.fields))[:, f]
    rows = eqn[mesh.conn[:, slots]]
    ok = rows >= 0
    out = np.zeros(P.n_dof)
    np.add.at(out, rows[ok], contrib[ok])
    return out


class BlockView:
    """One diagonal block (replica s) of a problem stacking independent
    replicas, seen as a problem of its own by SaddlePointSolver: replica
    0's pattern, numbering and mesh (every replica has them), replica s's
    Jacobian values (a view of `vals`, the stacked values or a snapshot of
    them)."""

    def __init__(self, P, s: int, vals, rp_host, ci_host, rp_dev, ci_dev):
        from types import SimpleNamespace
        n0, e0 = P.base_n_nodes, P.base_n_elem
        self.n_dof = int(rp_host.shape[0] - 1)
        self.nnz = int(ci_host.shape[0])
        self.J_dev = vals[s * self.nnz:(s + 1) * self.nnz]
        self.fields = P.fields
        self.eqn = np.asarray(P.eqn).reshape(P.mesh.n_nodes, len(P.fields))[:n0]
        self.mesh = SimpleNamespace(n_nodes=n0, n_elem=e0, x=P.mesh.x[:n0], conn=P.mesh.conn[:e0],
                                    etype=P.mesh.etype)
        self._rp, self._ci = rp_host, ci_host
        self._rpd, self._cid = rp_dev, ci_dev

    def pattern(self):
        return self._rp, self._ci

    def device_csr(self) -> DeviceCSR:
        return DeviceCSR(self._rpd.data_ptr(), self._cid.data_ptr(), self.J_dev, self.n_dof, self.nnz)


def newton_forcing(eta: float = 1e-5, eta_min: float = 1e-11) -> float:
    """Relative tolerance of the linear solve of a Newton step: the forcing
    term eta, not below eta_min (the 2-norm residual of a Krylov solve of
    these systems stalls near cond x eps).  The step's linear error enters
    the next residual as about eta |R| (inexact Newton: Dembo, Eisenstat and
    Steihaug, SIAM J. Numer. Anal. 19, 1982), far below the quadratic term of
    the steps a Newton solve takes from a perturbed state, so the residual
    history is that of exact steps.  Restarted GMRES with the block
    preconditioner reaches 1e-5 within its first restart cycle on these
    systems and then gains about 1.5x per cycle, so a tighter target would
    spend most iterations on accuracy the next residual cannot show."""
    return max(float(eta_min), float(eta))


class SaddlePointSolver:
    """GMRES with the block-triangular multigrid preconditioner for the
    Jacobian of a problem with one constrained field (the pressure):
    ``solve(R)`` returns dx with J dx = R, J the problem's current device
    Jacobian (J_dev).  schur_scale is the viscosity (the Schur complement is
    approximated by the pressure mass over it)."""

    def __init__(self, P, schur_field: str, schur_scale: float, restart: int = 60, smooth_steps: int = 2,
                 theta: float = 0.08, coarse_size: int = 800, max_levels: int = 12, precond_precision: str = "fp32"):
        import scipy.sparse as sps
        import torch
        self.torch = torch
        if precond_precision not in ("fp32", "fp64"):
            raise ValueError("precond_precision: 'fp32' or 'fp64'")
        # the preconditioner's arithmetic: the multigrid cycle, Bt and the
        # Schur scaling in FP32 (flexible GMRES keeps every preconditioned
        # vector, so its rounding does not enter the solution's accuracy)
        self.pdt = torch.float32 if precond_precision == "fp32" else torch.float64
        self.P = P
        self.dev = P.J_dev.device
        self.restart = int(restart)
        self.nu = max(1, int(smooth_steps))
        self.theta = float(theta)
        self.coarse_size = int(coarse_size)
        self.max_levels = int(max_levels)
        n = P.n_dof
        eqn = np.asarray(P.eqn).reshape(P.mesh.n_nodes, len(P.fields))
        f = [n_ for n_, _ in P.fields].index(schur_field)
        comp = np.full(n, -1, dtype=np.int32)
        for k in range(len(P.fields)):
            col = eqn[:, k]
            comp[col[col >= 0]] = k
        is_p = comp == f
        self.vel = np.nonzero(~is_p)[0]
        self.pre = np.nonzero(is_p)[0]
        self.comp_v = comp[self.vel]
        rp, ci = P.pattern()
        # patterns and slot maps of the velocity block A, the coupling Bt and
        # the constraint block B inside the CSR (native split)
        label = np.ascontiguousarray(is_p, dtype=np.int8)
        A_pat = csr_block(rp, ci, label, 0, 0)
        B_pat = csr_block(rp, ci, label, 0, 1)
        C_pat = csr_block(rp, ci, label, 1, 0)
        self.A_shape, self.B_shape, self.C_shape = A_pat, B_pat, C_pat
        self.map_a = torch.as_tensor(A_pat.slots, device=self.dev)
        self.map_b = torch.as_tensor(B_pat.slots, device=self.dev)
        self.map_c = torch.as_tensor(C_pat.slots, device=self.dev)
        self.vel_t = torch.as_tensor(self.vel, device=self.dev)
        self.pre_t = torch.as_tensor(self.pre, device=self.dev)
        mass = lumped_field_mass(P, schur_field)[self.pre]
        if np.any(mass <= 0):
            raise LinearSolverError("pressure lumped mass is not positive")
        self.mass = mass
        self.schur_scale = float(schur_scale)
        self.levels: Optional[List[dict]] = None
        self.iterations = 0
        self.stagnated = False
        self.use_graph = True
        self._graph = None
        self.check_every = 4          # Arnoldi steps between host looks at the residual estimate
        self.J = P.device_csr() if hasattr(P, "device_csr") else DeviceCSR.of_problem(P)

    def renew_if_changed(self, key, schur_scale: float) -> None:
        """Forget the hierarchy (rebuilt at the next solve) when `key` (the
        problem's parameters) differs from the one it was built for."""
        if key != getattr(self, "_key", None):
            self._key = key
            self.schur_scale = float(schur_scale)
            self.levels = None

    # -- set-up ------------------------------------------------------------
    def _host_blocks(self):
        """(A, Bt, B) of the current Jacobian on the host (gathered on the
        device)."""
        import scipy.sparse as sps
        vals = self.P.J_dev[:self.P.nnz].to(self.torch.float64)

        def take(pat, m):
            return sps.csr_matrix((vals.index_select(0, m).cpu().numpy(), pat.indices, pat.indptr), shape=pat.shape)
        return (take(self.A_shape, self.map_a), take(self.B_shape, self.map_b),
                take(self.C_shape, self.map_c))

    def setup(self) -> None:
        """The multigrid hierarchy of the current velocity block and the
        sign of the Schur approximation (host, once)."""
        import scipy.sparse as sps
        torch = self.torch
        A, Bt, B = self._host_blocks()
        D = A.diagonal()
        if np.any(D == 0) or not np.all(np.isfinite(A.data)):
            raise LinearSolverError("velocity block has a zero diagonal entry or non-finite values")
        # the Schur complement S = -B A^-1 Bt ~ sigma M_p / mu: its sign from
        # q^T B D^-1 Bt q for a random q (the weak form fixes the signs of B, Bt)
        q = np.random.default_rng(1).normal(size=self.pre.size)
        s = float(q @ (B @ ((Bt @ q) / D)))
        self.sigma = -1.0 if s > 0 else 1.0
        pdt = self.pdt
        npdt = np.float32 if pdt == torch.float32 else np.float64
        # host-side casts and uninitialised buffers: no torch FP32 kernel runs
        # (their first use in a process costs seconds on this machine)
        dv = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=npdt), device=self.dev)
        buf = lambda m: torch.empty(m, dtype=pdt, device=self.dev)
        self.sinv = dv(self.sigma * self.schur_scale / self.mass)
        levels = []
        comp = self.comp_v
        while A.shape[0] > self.coarse_size and len(levels) < self.max_levels:
            agg, na = aggregate(A, comp, self.theta)
            if na >= 0.9 * A.shape[0]:
                break
            n = A.shape[0]
            Dl = A.diagonal()
            Pm, Ac, lam = sa_level(A, agg, na)
            cc = np.zeros(na, dtype=np.int32)
            cc[agg] = comp
            levels.append({"A": _DevCSR(torch, A, self.dev, pdt), "P": _DevCSR(torch, Pm, self.dev, pdt),
                           "R": _DevCSR(torch, Pm.T.tocsr(), self.dev, pdt),
                           "dinv": dv(1.0 / Dl), "om": 1.0 / lam, "n": n, "nc": na,
                           "dinv_om": dv((1.0 / lam) / Dl),
                           "x": buf(n), "x2": buf(n), "t": buf(n), "bc": buf(na)})
            A, comp = Ac, cc
        # the coarsest operator's inverse on the host (<= coarse_size unknowns;
        # numpy), applied on the device as a dense matrix in CSR form by the
        # library's kernel: its summation order is fixed, so a solve does not
        # depend on the stream or the library workspace it runs with
        inv = np.linalg.inv(A.toarray())
        self.coarse_inv = _DevCSR(torch, sps.csr_matrix(inv), self.dev, pdt)
        self.coarse_out = buf(inv.shape[0])
        self.levels = levels
        self._graph = None                          # recaptured for the new hierarchy
        self.Bt = _DevCSR(torch, Bt, self.dev, pdt)
        # the FP32 preconditioner's vectors
        nv, npre = self.vel.size, self.pre.size
        self._rv, self._p, self._tv, self._b0 = buf(nv), buf(npre), buf(nv), buf(nv)
        self._x0 = buf(nv)
        self._ones = dv(np.ones(nv))
        self._z = torch.zeros(self.P.n_dof, dtype=torch.float64, device=self.dev)
        self.sizes = [lv["n"] for lv in levels] + [A.shape[0]]

    # -- application -------------------------------------------------------
    def _vcycle(self, lvl: int, b, first_done: bool = False):
        """One V-cycle on level lvl for right-hand side b: nu damped-Jacobi
        steps from zero, the coarse-grid correction, nu steps; every update
        one fused pass over its matrix (fe_csr_update).  Returns one of the
        level's iterate buffers (valid until the next cycle on this level).
        first_done: the first step from zero is already in the level's x."""
        torch = self.torch
        st = torch.cuda.current_stream().cuda_stream
        if lvl == len(self.levels):
            self.coarse_inv.mv(b, self.coarse_out, st)
            return self.coarse_out
        L = self.levels[lvl]
        A, dinv, om = L["A"], L["dinv"], L["om"]
        x, y = L["x"], L["x2"]
        if first_done:
            pass
        elif self.pdt == torch.float32:                       # the first step from zero
            vp = ctypes.c_void_p
            N.check(N.load().fe_sub_mul_f32(vp(b.data_ptr()), None, vp(L["dinv_om"].data_ptr()), None,
                                            vp(x.data_ptr()), L["n"], vp(st)))
        else:
            torch.mul(b, L["dinv_om"], out=x)
        for _ in range(self.nu - 1):
            A.update(x, b, x, dinv, om, y, st)
            x, y = y, x
        A.update(x, b, None, None, 1.0, L["t"], st)            # residual
        L["R"].mv(L["t"], L["bc"], st)                         # restriction
        L["P"].update(self._vcycle(lvl + 1, L["bc"]), None, x, None, -1.0, y, st)   # x + P xc
        x, y = y, x
        for _ in range(self.nu):
            A.update(x, b, x, dinv, om, y, st)
            x, y = y, x
        return x

    def precondition(self, r):
        """z = P^-1 r (the captured CUDA graph where there is one)."""
        if self._graph is None and self.use_graph:
            self._capture()
        if self._graph is None:
            return self._precondition(r)
        self._gin.copy_(r)
        self._graph.replay()
        return self._gout

    def _capture(self) -> None:
        """Record one preconditioner application (every level's SpMVs, the
        smoothing and transfer updates, the coarse solve: about a hundred
        launches) as a CUDA graph on fixed buffers; the matrices it reads are
        refreshed in place between Newton steps."""
        torch = self.torch
        self._gin = torch.zeros(self.P.n_dof, dtype=torch.float64, device=self.dev)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self._precondition(self._gin)           # warm-up: kernels loaded, buffers cached
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        # thread-local: other threads' work (another request's assembly, a
        # synchronous copy) must not abort this capture, nor be refused
        # while it runs
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self._gout = self._precondition(self._gin)
        self._graph = g

    def _precondition(self, r):
        """z = P^-1 r: p = S_hat^-1 r_p, u = A_hat^-1 (r_u - Bt p), in the
        preconditioner's precision; z in FP64."""
        torch = self.torch
        st = torch.cuda.current_stream().cuda_stream
        if self.pdt == torch.float32:
            # the library's kernels only (gather-cast, subtract-scale,
            # scatter-cast): fixed buffers, no torch FP32 kernel
            L, vp = N.load(), ctypes.c_void_p
            nv, npre = self.vel.size, self.pre.size
            r = r.contiguous()
            N.check(L.fe_gather_cast_f32(vp(r.data_ptr()), vp(self.vel_t.data_ptr()), nv, None,
                                         vp(self._rv.data_ptr()), vp(st)))
            N.check(L.fe_gather_cast_f32(vp(r.data_ptr()), vp(self.pre_t.data_ptr()), npre,
                                         vp(self.sinv.data_ptr()), vp(self._p.data_ptr()), vp(st)))
            self.Bt.mv(self._p, self._tv, st)
            if self.levels:
                L0 = self.levels[0]
                N.check(L.fe_sub_mul_f32(vp(self._rv.data_ptr()), vp(self._tv.data_ptr()),
                                         vp(L0["dinv_om"].data_ptr()), vp(self._b0.data_ptr()),
                                         vp(L0["x"].data_ptr()), nv, vp(st)))
                u = self._vcycle(0, self._b0, first_done=True)
            else:
                N.check(L.fe_sub_mul_f32(vp(self._rv.data_ptr()), vp(self._tv.data_ptr()),
                                         vp(self._ones.data_ptr()), vp(self._b0.data_ptr()),
                                         vp(self._x0.data_ptr()), nv, vp(st)))
                u = self._vcycle(0, self._b0)
            N.check(L.fe_scatter_cast_f64(vp(u.data_ptr()), vp(self.vel_t.data_ptr()), nv,
                                          vp(self._z.data_ptr()), vp(st)))
            N.check(L.fe_scatter_cast_f64(vp(self._p.data_ptr()), vp(self.pre_t.data_ptr()), npre,
                                          vp(self._z.data_ptr()), vp(st)))
            return self._z
        rp_ = r.to(self.pdt)
        p = self.sinv * rp_.index_select(0, self.pre_t)
        tv = torch.empty(self.vel.size, dtype=self.pdt, device=self.dev)
        self.Bt.mv(p, tv, st)
        u = self._vcycle(0, rp_.index_select(0, self.vel_t) - tv)
        z = torch.empty(r.shape, dtype=self.pdt, device=self.dev)
        z.index_copy_(0, self.vel_t, u)
        z.index_copy_(0, self.pre_t, p)
        z = z.to(torch.float64)
        return z

    def refresh(self) -> None:
        """Take the finest velocity block (and Bt) from the current Jacobian;
        the coarse levels stay."""
        torch = self.torch
        vals = self.P.J_dev[:self.P.nnz].to(torch.float64)
        if self.pdt == torch.float32:
            L, vp = N.load(), ctypes.c_void_p
            st = torch.cuda.current_stream().cuda_stream
            vals = vals.contiguous()
            pairs = ([(self.levels[0]["A"], self.map_a)] if self.levels else []) + [(self.Bt, self.map_b)]
            for M, m in pairs:
                N.check(L.fe_gather_cast_f32(vp(vals.data_ptr()), vp(m.data_ptr()), int(m.numel()), None,
                                             vp(M.v.data_ptr()), vp(st)))
            return
        if self.levels:
            self.levels[0]["A"].v.copy_(vals.index_select(0, self.map_a))
        self.Bt.v.copy_(vals.index_select(0, self.map_b))

    def solve(self, b, tol: float = 1e-10, atol: float = 0.0, maxiter: int = 2000):
        """x with J x = b (device vectors), stopping at ||b - J x||_2 <=
        max(tol ||b||_2, atol).  Returns (x, iterations)."""
        torch = self.torch
        if self.levels is None:
            self.setup()
        else:
            self.refresh()
        st = torch.cuda.current_stream().cuda_stream
        n = self.P.n_dof
        # a private copy: b may be a slice of a stacked vector at any offset,
        # and a reduction's vector width (so its summation order) follows
        # the alignment of the memory it reads
        b = b.reshape(-1)[:n].to(torch.float64).clone()
        if not bool(torch.isfinite(b).all()):
            raise LinearSolverError("non-finite right-hand side")
        bnorm = float(torch.linalg.vector_norm(b))
        target = max(tol * bnorm, atol)
        x = torch.zeros(n, dtype=torch.float64, device=self.dev)
        if bnorm == 0.0:
            return x, 0
        m = self.restart
        V = torch.zeros((m + 1, n), dtype=torch.float64, device=self.dev)
        # flexible GMRES: the preconditioned vectors are kept, and the
        # update is built from them (x += Z y), so a preconditioner that is
        # not exactly linear (FP32 rounding) costs no accuracy
        Z = torch.zeros((m, n), dtype=torch.float64, device=self.dev)
        Az = torch.empty(n, dtype=torch.float64, device=self.dev)
        L = N.load()
        work = torch.empty(int(L.fe_gmres_cgs2_scratch(n, m)), dtype=torch.float64, device=self.dev)
        vp = ctypes.c_void_p
        its = 0
        r = b.clone()
        beta = bnorm
        stalled = 0
        self.stagnated = False
        self.restart_residuals = [bnorm]     # ||b - J x||_2 at every restart
        while its < maxiter:
            beta_start = beta
            V[0] = r / beta
            H = np.zeros((m + 1, m))
            g = np.zeros(m + 1)
            g[0] = beta
            cs, sn = np.zeros(m), np.zeros(m)
            HdT = torch.zeros((m, m + 1), dtype=torch.float64, device=self.dev)   # row k: column k of H
            k = 0
            done = False
            for k in range(m):
                Z[k].copy_(self.precondition(V[k]))
                self.J.matvec(Z[k], Az, st)
                # classical Gram-Schmidt twice, Az overwritten (fe_gmres_cgs2)
                N.check(L.fe_gmres_cgs2(vp(V.data_ptr()), n, n, k, vp(Az.data_ptr()), vp(HdT[k].data_ptr()),
                                        vp(work.data_ptr()), vp(st)))
                its += 1
                if (k + 1) % self.check_every and k + 1 < m and its < maxiter:
                    continue                     # the host looks every check_every steps only
                # Givens rotations of the columns since the last look (one synchronisation)
                k0 = (k // self.check_every) * self.check_every if (k + 1) % self.check_every else k + 1 - self.check_every
                k0 = max(0, min(k0, k))
                H[:, k0:k + 1] = HdT[k0:k + 1].cpu().numpy().T
                for j in range(k0, k + 1):
                    for i in range(j):
                        t_ = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                        H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                        H[i, j] = t_
                    den = np.hypot(H[j, j], H[j + 1, j])
                    cs[j], sn[j] = (1.0, 0.0) if den == 0 else (H[j, j] / den, H[j + 1, j] / den)
                    H[j, j] = den
                    H[j + 1, j] = 0.0
                    g[j + 1] = -sn[j] * g[j]
                    g[j] = cs[j] * g[j]
                    if not np.isfinite(g[j + 1]):
                        raise LinearSolverError("GMRES broke down (non-finite residual)")
                    if abs(g[j + 1]) <= target or H[j, j] == 0.0:
                        k = j                    # the least-squares problem up to column j
                        done = True
                        break
                if done or its >= maxiter:
                    break
            kk = k + 1
            y = np.linalg.solve(np.triu(H[:kk, :kk]), g[:kk]) if kk else np.zeros(0)
            yt = torch.as_tensor(y, device=self.dev)
            x += Z[:kk].T @ yt
            self.J.matvec(x, Az, st)
            r = b - Az
            beta = float(torch.linalg.vector_norm(r))
            self.restart_residuals.append(beta)
            if beta <= target:
                self.iterations = its
                return x, its
            # a restart cycle that gains less than 1% twice in a row: stagnation
            # at the attainable accuracy; the Newton step is taken as it is
            # (the Newton loop's residual check decides), unless nothing was
            # gained at all
            stalled = stalled + 1 if beta > 0.99 * beta_start else 0
            if stalled >= 2:
                break
        self.iterations = its
        if np.isfinite(beta) and beta <= 1e-3 * bnorm:
            self.stagnated = True
            return x, its
        raise LinearSolverError(f"GMRES did not converge in {its} iterations (residual {beta:.3e}, "
                                f"target {target:.3e})")


def _main(argv=None) -> None:
    """One device Newton solve of the Navier-Stokes workload with this
    solver (a small driver for profiling): ``python -m
    pyoomph_gb300.fieldsplit 128 fp64`` = side 128, FP64 Jacobian."""
    import argparse
    import time
    import torch
    from . import workloads as W
    ap = argparse.ArgumentParser(prog="python -m pyoomph_gb300.fieldsplit")
    ap.add_argument("side", type=int)
    ap.add_argument("precision", choices=["fp64", "fp32"], nargs="?", default="fp64")
    a = ap.parse_args(argv)
    P = W.navier_stokes_problem(N=a.side, jacobian_precision=a.precision)
    P.initialise()
    W.perturb_dofs(P, seed=0, sigma=1e-3)
    P.linear_solver = "fieldsplit"
    P.newton_solver_tolerance = 1e-10
    P.max_newton_iterations = 30
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = P.solve()
    torch.cuda.synchronize()
    print(f"ns side {a.side} {a.precision}: {P.n_dof} dofs, {len(hist) - 1} Newton steps, "
          f"{P.timings.get('krylov_iterations')} GMRES iterations, {time.perf_counter() - t0:.3f} s, "
          f"max |R| {hist[-1]:.2e}, levels {P._fieldsplit.sizes}")


if __name__ == "__main__":
    _main()
