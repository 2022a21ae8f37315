"""Device Newton linear solve: Jacobi-preconditioned BiCGStab on the
resident CSR Jacobian.

The reference solves J dx = R on the host with SuperLU
(``pyoomph/solvers/scipy.py``, ``src/pybind/solver.cpp:105``), which needs
the Jacobian copied to the host every Newton step and dominates the solve
time at large sizes.  Here the Jacobian never leaves the device: the
matrix-vector products run in the library's CSR kernel (``fe_csr_spmv``, one
warp per row) on the assembled values, the vector algebra in torch, and the
only host synchronisation is the convergence check every few iterations.

BiCGStab (van der Vorst 1992) with the diagonal as right preconditioner
suits the diffusion-type Jacobians of Poisson and nonlinear diffusion (also
the non-symmetric ones); saddle-point systems with a zero diagonal block
(Taylor-Hood Navier-Stokes) are rejected -- they keep the host SuperLU path.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

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

    @classmethod
    def of_problem(cls, P, vals=None) -> "DeviceCSR":
        rp = ctypes.c_void_p()
        ci = ctypes.c_void_p()
        N.check(N.load().fe_problem_pattern_device(P._h, ctypes.byref(rp), ctypes.byref(ci)))
        return cls(rp.value, ci.value, P.J_dev if vals is None else vals, P.n_dof)

    @property
    def precision(self) -> int:
        import torch
        return N.FE_JAC_F64 if self.vals.dtype == torch.float64 else N.FE_JAC_F32

    def matvec(self, x, y, stream) -> None:
        N.check(N.load().fe_csr_spmv(ctypes.c_void_p(self.rowptr), ctypes.c_void_p(self.colidx),
                                     ctypes.c_void_p(self.vals.data_ptr()), self.precision,
                                     ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), self.n,
                                     ctypes.c_void_p(stream)))

    def diagonal(self, out, stream) -> None:
        N.check(N.load().fe_csr_diagonal(ctypes.c_void_p(self.rowptr), ctypes.c_void_p(self.colidx),
                                         ctypes.c_void_p(self.vals.data_ptr()), self.precision,
                                         ctypes.c_void_p(out.data_ptr()), self.n, ctypes.c_void_p(stream)))


def bicgstab(A: DeviceCSR, b, tol: float = 1e-13, maxiter: int = 20000, check_every: int = 8,
             x0=None):
    """Solve A x = b on the device; stop when ||b - A x||_inf <= tol *
    ||b||_inf (checked every `check_every` iterations with the recursively
    updated residual, confirmed with a true residual).  Returns (x,
    iterations)."""
    import torch
    st = torch.cuda.current_stream().cuda_stream
    n = A.n
    dev = b.device
    diag = torch.empty(n, dtype=torch.float64, device=dev)
    A.diagonal(diag, st)
    if bool((diag == 0).any()):
        raise LinearSolverError("zero diagonal entry: Jacobi-preconditioned BiCGStab does not apply "
                                "(saddle-point system); use the host solver")
    minv = 1.0 / diag
    x = torch.zeros(n, dtype=torch.float64, device=dev) if x0 is None else x0.clone()
    r = b.clone()
    if x0 is not None:
        t = torch.empty_like(b)
        A.matvec(x, t, st)
        r -= t
    bnorm = float(b.abs().max())
    if bnorm == 0.0:
        return x, 0
    target = tol * bnorm
    rhat = r.clone()
    p = torch.zeros_like(r)
    v = torch.zeros_like(r)
    s = torch.empty_like(r)
    t = torch.empty_like(r)
    rho_old = torch.ones((), dtype=torch.float64, device=dev)
    alpha = torch.ones((), dtype=torch.float64, device=dev)
    omega = torch.ones((), dtype=torch.float64, device=dev)
    x_good = x.clone()
    restarts = 0

    def restart():
        # from the last checked iterate, with the true residual as shadow vector
        nonlocal r, rhat, rho_old, alpha, omega
        A.matvec(x, t, st)
        r = b - t
        rhat = r.clone()
        p.zero_()
        v.zero_()
        rho_old = torch.ones((), dtype=torch.float64, device=dev)
        alpha = torch.ones((), dtype=torch.float64, device=dev)
        omega = torch.ones((), dtype=torch.float64, device=dev)

    for it in range(1, maxiter + 1):
        rho = torch.dot(rhat, r)
        beta = (rho / rho_old) * (alpha / omega)
        p.sub_(omega * v).mul_(beta).add_(r)
        phat = p * minv
        A.matvec(phat, v, st)
        alpha = rho / torch.dot(rhat, v)
        torch.sub(r, alpha * v, out=s)
        shat = s * minv
        A.matvec(shat, t, st)
        omega = torch.dot(t, s) / torch.dot(t, t)
        x.add_(alpha * phat).add_(omega * shat)
        torch.sub(s, omega * t, out=r)
        rho_old = rho
        if it % check_every == 0:
            rn = float(r.abs().max())
            if not (rn == rn) or not bool(torch.isfinite(x).all()):
                # breakdown (rho or omega ~ 0): back to the last good iterate and restart
                restarts += 1
                if restarts > 20:
                    raise LinearSolverError(f"BiCGStab broke down repeatedly ({it} iterations)")
                x.copy_(x_good)
                restart()
                continue
            x_good.copy_(x)
            if rn <= target:
                A.matvec(x, t, st)
                true = float((b - t).abs().max())
                if true <= target * 10:
                    return x, it
                restart()
    raise LinearSolverError(f"BiCGStab did not reach {tol} in {maxiter} iterations")
