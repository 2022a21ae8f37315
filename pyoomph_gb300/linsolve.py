"""Device Newton linear solve: Jacobi-preconditioned BiCGStab on the
resident CSR Jacobian.

The reference solves J dx = R on the host with SuperLU
(``pyoomph/solvers/scipy.py``, ``src/pybind/solver.cpp:105``), which needs
the Jacobian copied to the host every Newton step and dominates the solve
time at large sizes.  Here the Jacobian never leaves the device: the native
solver (``fe_krylov_*`` in the C-ABI) runs the matrix-vector products in the
library's CSR kernel (``fe_csr_spmv``: 4..32 lanes per row by the mean row
length) on the assembled values and the vector algebra in its own fused
kernels, replays blocks of iterations as one CUDA graph on its own stream,
and synchronises with the host only at the convergence checks between
blocks.

BiCGStab (van der Vorst 1992) with the diagonal as right preconditioner
suits the diffusion-type Jacobians of Poisson and nonlinear diffusion (also
the non-symmetric ones); saddle-point systems with a zero diagonal block
(Taylor-Hood Navier-Stokes) are rejected -- they keep the host SuperLU path.

``BatchedBiCGStab`` iterates S independent diagonal blocks of one stacked
matrix together (the replicas of a problem: block s owns rows s*n..(s+1)*n
and couples only to them).  Every scalar is per block, every reduction runs
over fixed chunks of one block's rows in a fixed order, and a block stops
(its iterate frozen) at the iteration its own residual reaches the target,
so a block's solution is bit-identical whatever slot it occupies and
whatever the other blocks hold.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N


class LinearSolverError(RuntimeError):
    pass


@dataclass
class DeviceCSR:
    """The resident CSR pattern of a problem with a values tensor (f64 or f32)."""
    rowptr: int          # device pointers (int32)
    colidx: int
    vals: "object"       # torch tensor on the device
    n: int
    nnz: int

    @classmethod
    def of_problem(cls, P, vals=None) -> "DeviceCSR":
        rp = ctypes.c_void_p()
        ci = ctypes.c_void_p()
        N.check(N.load().fe_problem_pattern_device(P._h, ctypes.byref(rp), ctypes.byref(ci)))
        return cls(rp.value, ci.value, P.J_dev if vals is None else vals, P.n_dof, P.nnz)

    @property
    def precision(self) -> int:
        import torch
        return N.FE_JAC_F64 if self.vals.dtype == torch.float64 else N.FE_JAC_F32

    def matvec(self, x, y, stream) -> None:
        N.check(N.load().fe_csr_spmv(ctypes.c_void_p(self.rowptr), ctypes.c_void_p(self.colidx),
                                     ctypes.c_void_p(self.vals.data_ptr()), self.precision,
                                     ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), self.n,
                                     self.nnz, ctypes.c_void_p(stream)))

    def diagonal(self, out, stream) -> None:
        N.check(N.load().fe_csr_diagonal(ctypes.c_void_p(self.rowptr), ctypes.c_void_p(self.colidx),
                                         ctypes.c_void_p(self.vals.data_ptr()), self.precision,
                                         ctypes.c_void_p(out.data_ptr()), self.n, ctypes.c_void_p(stream)))


class BatchedBiCGStab:
    """The native batched solver (``fe_krylov_create`` / ``fe_krylov_solve``)
    bound to a DeviceCSR whose values buffer stays in place (the values may
    change between solves: the next Newton step's Jacobian)."""

    def __init__(self, A: DeviceCSR, blocks: int = 1, check_every: int = 8, graph: bool = True):
        import torch
        if blocks < 1 or A.n % blocks:
            raise ValueError(f"{A.n} rows do not split into {blocks} equal blocks")
        self.torch = torch
        self.A = A
        self.S = blocks
        self.n = A.n // blocks
        self.check_every = int(check_every)
        h = ctypes.c_void_p()
        N.check(N.load().fe_krylov_create(ctypes.c_void_p(A.rowptr), ctypes.c_void_p(A.colidx),
                                          ctypes.c_void_p(A.vals.data_ptr()), A.precision, A.n, A.nnz, blocks,
                                          self.check_every, int(bool(graph)), ctypes.byref(h)))
        self._h = h
        self.x = torch.zeros((self.S, self.n), dtype=torch.float64, device=A.vals.device)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.load().fe_krylov_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def info(self) -> dict:
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        N.check(N.load().fe_krylov_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"launches": a.value, "graph_replays": b.value, "restarts": c.value}

    def matvec(self, x, y) -> None:
        """y = A x with the solver's matrix and SpMV kernel, on the current stream."""
        N.check(N.load().fe_krylov_matvec(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                          ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)))

    @property
    def graph_replays(self) -> int:
        return self.info()["graph_replays"]

    def solve(self, b, active=None, tol: float = 1e-13, maxiter: int = 20000, max_restarts: int = 20,
              stream=None, atol: float = 0.0):
        """Solve A_s x_s = b_s for the active blocks s (all by default); b is
        the stacked right-hand side (S*n,) or (S, n) on the device.  Stops a
        block when ||r_s||_inf <= max(tol * ||b_s||_inf, atol).  Returns (x, iterations):
        x the (S, n) result (inactive blocks hold 0), iterations per block
        (multiples of check_every).  `stream` (a CUDA stream handle, default
        the current stream) orders the solve after the work that produced b
        and the work that reads x after it; the call releases the GIL while
        it iterates, so other threads keep running."""
        torch = self.torch
        b = b.reshape(-1)
        if b.numel() != self.S * self.n or b.dtype != torch.float64 or not b.is_contiguous():
            raise ValueError("b must be a contiguous float64 vector of the matrix's size")
        act = None
        if active is not None:
            act = np.ascontiguousarray(np.asarray(active, dtype=bool).astype(np.uint8))
            if act.shape != (self.S,):
                raise ValueError(f"active must have {self.S} entries")
        its = np.zeros(self.S, dtype=np.int64)
        rc = N.load().fe_krylov_solve(self._h, ctypes.c_void_p(b.data_ptr()),
                                      None if act is None else act.ctypes.data_as(ctypes.c_void_p),
                                      float(tol), float(atol), int(maxiter), int(max_restarts),
                                      ctypes.c_void_p(self.x.data_ptr()), its.ctypes.data_as(ctypes.c_void_p),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream
                                                      if stream is None else stream))
        if rc == N.FE_ERR_SOLVER:
            raise LinearSolverError(N.load().fe_last_error().decode(errors="replace"))
        N.check(rc)
        return self.x, its


def bicgstab(A: DeviceCSR, b, tol: float = 1e-13, maxiter: int = 20000, check_every: int = 8,
             graph: bool = True):
    """Solve A x = b on the device (one block); stop when ||b - A x||_inf <=
    tol * ||b||_inf.  Returns (x, iterations)."""
    solver = BatchedBiCGStab(A, 1, check_every=check_every, graph=graph)
    x, its = solver.solve(b, tol=tol, maxiter=maxiter)
    return x.view(-1).clone(), int(its[0])


def _main(argv=None) -> None:
    """SpMV micro-benchmark on an assembled Jacobian:
    ``python -m pyoomph_gb300.linsolve [hex|poisson|ns] [side] [fp64|fp32]``.
    Prints the kernel time (CUDA events, 20 repeats after 3) and the
    algorithmic bandwidth (values + column indices + row pointers + x + y)."""
    import argparse
    import torch
    from . import workloads as W
    ap = argparse.ArgumentParser(prog="python -m pyoomph_gb300.linsolve")
    ap.add_argument("workload", nargs="?", default="hex", choices=["hex", "poisson", "ns"])
    ap.add_argument("side", nargs="?", type=int, default=32)
    ap.add_argument("precision", nargs="?", default="fp64", choices=["fp64", "fp32"])
    a = ap.parse_args(argv)
    make = {"hex": lambda: W.nonlinear_diffusion_problem(N=a.side, seed=2, jacobian_precision=a.precision),
            "poisson": lambda: W.poisson_problem(N=a.side, seed=2, jacobian_precision=a.precision),
            "ns": lambda: W.navier_stokes_problem(N=a.side, jacobian_precision=a.precision)}
    P = make[a.workload]()
    P.initialise()
    P.assemble_device(with_jacobian=True)
    A = DeviceCSR.of_problem(P)
    x = torch.ones(P.n_dof, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(3):
        A.matvec(x, y, st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        A.matvec(x, y, st)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 20
    jb = 8 if a.precision == "fp64" else 4
    nbytes = P.nnz * (jb + 4) + (P.n_dof + 1) * 4 + 16 * P.n_dof
    print(f"{a.workload} side {a.side} {a.precision}: n={P.n_dof} nnz={P.nnz} spmv {ms:.4f} ms, "
          f"{nbytes / ms / 1e6:.0f} GB/s algorithmic")


if __name__ == "__main__":
    _main()
