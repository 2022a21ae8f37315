"""Serving: a continuous-batching loop of assemble + Newton-solve requests.

Requests (a Poisson or a Navier-Stokes problem of some mesh side, with its
own source or Reynolds number) arrive over time.  The server keeps, per mesh
class (equation, side, Jacobian precision), one *batch*: a resident
problem that stacks S independent replicas of the mesh (``Problem.replicas``),
each replica reading its own parameters.  A request is admitted into a free
replica slot of its class as soon as one is free and the device has the
memory for the class (``fe_device_info`` free bytes, minus a reserve);
otherwise it waits.  Admission happens at Newton-step boundaries, so
requests join and leave a running batch continuously.

Each request advances on its own: assembly, residual check, the linear
solve J dx = R of its diagonal block in a worker process (SuperLU through
scipy, the reference's default solver; processes because SuperLU holds the
GIL; the class's CSR pattern is published once in shared memory), update,
next assembly.  The pending assemblies of a class are served by one launch
sequence for all its replicas (dof scatter, element kernel, residual and
Jacobian scatter) on the class's own CUDA stream, with the per-replica
residual max-norms reduced on the device -- so the solves of all active
requests run in parallel on the host cores while the GPU assembles.  With
``device_solver=True`` every request is solved on the device instead: the
Poisson requests of a class by one batched Jacobi-BiCGStab over the class's
replicas (``linsolve.BatchedBiCGStab``, CUDA-graph blocks of iterations),
each Navier-Stokes request of side >= ``device_saddle_min_side`` by its
own saddle-point solver over its replica's diagonal block
(``fieldsplit.SaddlePointSolver``: GMRES with a block-triangular multigrid
preconditioner built from that request's own Jacobian); smaller
Navier-Stokes systems stay with SuperLU in the workers, which solves many
of them in parallel faster.

Results do not depend on the mix: every element, CSR slot and residual
entry of a replica is computed from that replica's values only, in a fixed
order, so a request gives bit-identical dofs alone or among others.

Per-request latency = completion - arrival; the summary reports p50/p99 and
solves/s.  ``serve_sequential`` is the plain path: one request at a time,
one problem per request, FP64 Jacobian.
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import _native as N
from . import workloads as W


@dataclass
class Request:
    rid: int
    kind: str                   # "poisson" | "ns"
    side: int
    arrival: float              # seconds after the start of the stream
    seed: int = 0
    Re: float = 100.0
    # results
    dofs: Optional[np.ndarray] = None
    t_admit: float = float("nan")
    t_done: float = float("nan")
    newton_iterations: int = 0
    residuals: List[float] = field(default_factory=list)
    error: Optional[str] = None

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def make_stream(n: int, rate: float, seed: int = 0, side_range: Tuple[int, int] = (16, 512),
                kinds=("poisson", "ns"), ns_side_max: Optional[int] = None) -> List[Request]:
    """Poisson-process arrivals at `rate` per second; side log-uniform in
    side_range; kind uniform over kinds; source seed / Re from the seed."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    out = []
    for i in range(n):
        kind = kinds[int(rng.integers(len(kinds)))]
        side = int(round(np.exp(rng.uniform(np.log(side_range[0]), np.log(side_range[1])))))
        if kind == "ns" and ns_side_max:
            side = min(side, ns_side_max)
        out.append(Request(i, kind, side, float(t[i]), seed=int(rng.integers(1 << 30)),
                           Re=float(rng.uniform(10.0, 100.0))))
    return out


def _class_problem(kind: str, side: int, precision: str, replicas: int):
    if kind == "poisson":
        P = W.poisson_problem(N=side, seed=0, jacobian_precision=precision)
    else:
        P = W.navier_stokes_problem(N=side, Re=100.0, jacobian_precision=precision)
    P.replicas = replicas
    return P


def _request_params(req: Request, P) -> np.ndarray:
    """The parameter vector of one replica, in P.param_names order."""
    names = P.param_names
    v = np.zeros(len(names))
    if req.kind == "poisson":
        g = W.draw_gaussians(req.seed, 8, 2)
        d = {}
        for k in range(g.shape[0]):
            d[f"g{k}_c0"], d[f"g{k}_c1"], d[f"g{k}_w"], d[f"g{k}_A"] = g[k]
    else:
        d = {"mass_density": 1.0, "dynamic_viscosity": 1.0 / req.Re}
    for j, nm in enumerate(names):
        v[j] = d[nm]
    return v


def estimate_bytes(P) -> int:
    """Device memory of a lowered problem (element buffers, CSR values,
    pattern and scatter lists, nodal arrays), before creating it."""
    E = P.mesh.n_elem
    nl = P.kernel.layout.n
    jb = 8 if P._prec == "f64" else 4
    nnz_est = E * nl * nl  # upper bound of the number of CSR slots
    return int(E * nl * nl * (jb + 4) + nnz_est * (jb + 8 + 4) + E * nl * 12 + P.mesh.n_nodes * 64)


_PATTERNS: Dict[str, tuple] = {}


def _attach_pattern(name: str, n: int, nnz: int):
    """The CSR pattern of a mesh class, published once in shared memory by
    the server and attached (and cached) by each worker process."""
    got = _PATTERNS.get(name)
    if got is None:
        from multiprocessing import shared_memory
        shm = shared_memory.SharedMemory(name=name)
        rp = np.ndarray((n + 1,), dtype=np.int32, buffer=shm.buf)
        ci = np.ndarray((nnz,), dtype=np.int32, buffer=shm.buf, offset=4 * (n + 1))
        got = _PATTERNS[name] = (shm, rp, ci)
    return got[1], got[2]


def _splu_solve(pattern: str, vals: np.ndarray, R: np.ndarray) -> np.ndarray:
    """J dx = R with SuperLU in a worker process (SuperLU holds the GIL, so
    parallel solves need processes); the pattern comes from shared memory."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = R.shape[0]
    rp, ci = _attach_pattern(pattern, n, vals.shape[0])
    A = sp.csr_matrix((vals.astype(np.float64), ci, rp), shape=(n, n))
    return spla.splu(A.tocsc()).solve(R)


class _Batch:
    def __init__(self, key, P, slots: int, stream):
        from multiprocessing import shared_memory
        self.key = key
        self.P = P
        self.slots = slots
        self.stream = stream
        self.req: List[Optional[Request]] = [None] * slots
        self.state: List[str] = ["free"] * slots        # free | assemble | solving
        self.n_dof = P.n_dof // slots
        self.nnz = P.nnz // slots
        rp, ci = P.pattern()
        self.shm = shared_memory.SharedMemory(create=True, size=4 * (self.n_dof + 1 + self.nnz))
        np.ndarray((self.n_dof + 1,), dtype=np.int32, buffer=self.shm.buf)[:] = rp[:self.n_dof + 1]
        np.ndarray((self.nnz,), dtype=np.int32, buffer=self.shm.buf, offset=4 * (self.n_dof + 1))[:] = ci[:self.nnz]
        self.x0 = P.get_dofs()[:self.n_dof].copy()
        self.last_used = time.perf_counter()
        self.krylov = None      # device solver of the class (device_solver=True)
        self.fs = {}            # Navier-Stokes: the device saddle-point solver of each slot's request
        self.pat_dev = None     # replica 0's pattern on the device (for those solvers)
        self.jsnap = None       # the J values and residual the in-flight device solve reads
        self.rsnap = None
        self.inflight = False   # a device solve of this class is running

    def free_slot(self) -> int:
        for s, r in enumerate(self.req):
            if r is None:
                return s
        return -1

    def active(self) -> bool:
        return any(r is not None for r in self.req)

    def release(self) -> None:
        try:
            self.shm.close()
            self.shm.unlink()
        except Exception:
            pass


class Server:
    """Continuous batching: each request advances on its own (assemble ->
    solve in a worker -> update -> assemble ...); a class's pending
    assemblies are served by one launch sequence for all its replicas."""

    @staticmethod
    def default_saddle_min_side() -> int:
        return 96

    def __init__(self, slots: int = 4, jacobian_precision: str = "fp32", tol: float = 1e-10,
                 max_newton: int = 20, workers: int = 8, hbm_reserve: float = 0.1, device_solver: bool = False):
        import torch
        self.torch = torch
        self.slots = slots
        self.precision = jacobian_precision
        self.tol = tol
        self.max_newton = max_newton
        import multiprocessing as mp
        # linear solves in worker processes (spawned: safe after CUDA init)
        self.pool = cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"))
        self.hbm_reserve = hbm_reserve
        # device_solver: Newton systems solved on the device instead of by
        # SuperLU in the workers -- Poisson requests by one batched BiCGStab
        # per class and round (a block per replica, so a request's iterates
        # never depend on its neighbours), Navier-Stokes requests by their
        # own saddle-point solvers
        self.device_solver = device_solver
        # Navier-Stokes requests of at least this side are solved on the
        # device (saddle-point GMRES), smaller ones by SuperLU in the worker
        # processes.  Alone, a request's Newton solve is faster on the device
        # from side 32 (0.16 s against SuperLU's 0.30 s); in a stream of
        # sides 16..64 the workers' 14 parallel SuperLU solves still serve
        # more requests per second below side 96 (16.4/s against 11.0/s
        # with the threshold at 32)
        self.device_saddle_min_side = self.default_saddle_min_side()
        # device solves run in threads (the native solve releases the GIL),
        # so a long solve of one class does not stall the others
        self.tpool = cf.ThreadPoolExecutor(max_workers=4) if device_solver else None
        self.device_solves = 0
        self.solver_launches = 0      # kernel launches of the device solver
        self.batches: Dict[tuple, _Batch] = {}
        self.launches = 0
        self.assemblies = 0
        self.t_solve = 0.0

    # -- memory ------------------------------------------------------------
    def _free_bytes(self) -> int:
        f = ctypes.c_size_t()
        t = ctypes.c_size_t()
        N.check(N.load().fe_device_info(None, None, None, ctypes.byref(f), ctypes.byref(t)))
        return int(f.value - self.hbm_reserve * t.value)

    def _get_batch(self, req: Request) -> Optional[_Batch]:
        key = (req.kind, req.side, self.precision)
        b = self.batches.get(key)
        if b is not None:
            return b
        P = _class_problem(req.kind, req.side, self.precision, self.slots)
        P.lower()
        need = estimate_bytes(P)
        while need > self._free_bytes():
            idle = [k for k, bb in self.batches.items() if not bb.active()]
            if not idle:
                return None  # admission refused for now: not enough HBM
            victim = min(idle, key=lambda k: self.batches[k].last_used)
            self.batches.pop(victim).release()
            self.torch.cuda.synchronize()
        P.initialise()
        b = _Batch(key, P, self.slots, self.torch.cuda.Stream())
        self.batches[key] = b
        return b

    def _admit(self, req: Request, now: float) -> bool:
        b = self._get_batch(req)
        if b is None:
            return False
        s = b.free_slot()
        if s < 0:
            return False
        P = b.P
        P.set_parameter_vector(_request_params(req, P), replica=s)
        with self.torch.cuda.stream(b.stream):
            P.x_dev[s * b.n_dof:(s + 1) * b.n_dof].copy_(self.torch.as_tensor(b.x0, device="cuda"))
        b.req[s] = req
        b.state[s] = "assemble"
        req.t_admit = now
        return True

    def _assemble(self, b: _Batch, t0: float, futs: dict) -> List[Request]:
        """One launch sequence for every replica of the class; then, per
        replica waiting for an assembly, the convergence check and either
        completion or a solve submitted to the workers."""
        torch = self.torch
        P = b.P
        done = []
        dev_solve: List[int] = []
        on_device = self.device_solver and (b.key[0] == "poisson" or b.key[1] >= self.device_saddle_min_side)
        with torch.cuda.stream(b.stream):
            P.assemble_device(with_jacobian=True, stream=b.stream.cuda_stream)
            self.launches += P.launch_count(True)
            self.assemblies += 1
            Rv = P.R_dev[:P.n_dof].view(b.slots, b.n_dof)
            norms = torch.nan_to_num(Rv.abs().amax(dim=1), nan=float("inf")).cpu().numpy()
        R = J = None
        for s, req in enumerate(b.req):
            if req is None or b.state[s] != "assemble":
                continue
            req.residuals.append(float(norms[s]))
            if norms[s] < self.tol or req.newton_iterations >= self.max_newton or not np.isfinite(norms[s]):
                if norms[s] >= self.tol:
                    req.error = f"Newton did not converge: {req.residuals}"
                req.dofs = P.x_dev[s * b.n_dof:(s + 1) * b.n_dof].cpu().numpy()
                req.t_done = time.perf_counter() - t0
                b.req[s] = None
                b.state[s] = "free"
                b.fs.pop(s, None)
                done.append(req)
                continue
            if on_device:
                dev_solve.append(s)
                continue
            if J is None:
                with torch.cuda.stream(b.stream):
                    R = Rv.cpu().numpy()
                    J = P.J_dev[:P.nnz].view(b.slots, b.nnz).cpu().numpy()
            b.state[s] = "solving"
            futs[self.pool.submit(_splu_solve, b.shm.name, J[s], R[s])] = (b, s, time.perf_counter())
        if dev_solve and b.inflight:
            for s in dev_solve:            # solved after the class's running solve
                b.state[s] = "wait"
        elif dev_solve:
            # one batched BiCGStab for every replica that needs a step (a
            # block per replica, each with its own scalars and stopping
            # point), in a worker thread on snapshots of J and R so that the
            # class can be re-assembled meanwhile
            from .linsolve import BatchedBiCGStab, DeviceCSR
            with torch.cuda.stream(b.stream):
                if b.jsnap is None:
                    b.jsnap = torch.empty_like(P.J_dev[:P.nnz])
                    b.rsnap = torch.empty_like(P.R_dev[:P.n_dof])
                if b.krylov is None and b.key[0] == "poisson":
                    b.krylov = BatchedBiCGStab(DeviceCSR.of_problem(P, vals=b.jsnap), blocks=b.slots)
                b.jsnap.copy_(P.J_dev[:P.nnz])
                b.rsnap.copy_(P.R_dev[:P.n_dof])
            mask = np.zeros(b.slots, dtype=bool)
            mask[dev_solve] = True
            for s in dev_solve:
                b.state[s] = "solving"
            b.inflight = True
            # inexact Newton: the step need only bring max|R| an order below
            # the request's tolerance, so each block stops at |r_s| <=
            # max(1e-13 |R_s|, 0.1 tol) -- a pure 1e-13 relative target is
            # below the attainable accuracy of large meshes (cond x eps) --
            # and the target depends on the block's own residual only
            solve = self._device_solve if b.key[0] == "poisson" else self._device_solve_saddle
            fut = self.tpool.submit(solve, b, mask, 0.1 * self.tol)
            futs[fut] = (b, tuple(dev_solve), time.perf_counter())
        b.last_used = time.perf_counter()
        return done

    def _device_solve(self, b: _Batch, mask: np.ndarray, atol: float):
        """Worker thread: the batched solve of one class (native, GIL released)."""
        l0 = b.krylov.info()["launches"]
        dx, _ = b.krylov.solve(b.rsnap, active=mask, tol=1e-13, atol=atol, stream=b.stream.cuda_stream)
        return dx, b.krylov.info()["launches"] - l0

    def _device_solve_saddle(self, b: _Batch, mask: np.ndarray, atol: float):
        """Worker thread: the Navier-Stokes Newton steps of one class on the
        device, one request after the other, each with its own saddle-point
        solver (fieldsplit.py) over its replica's diagonal block of the J
        snapshot.  A request's solver is built from its own first Jacobian
        and kept for its later steps, so nothing it computes depends on the
        other requests of the class."""
        from .fieldsplit import BlockView, SaddlePointSolver, newton_forcing
        torch = self.torch
        P = b.P
        with torch.cuda.stream(b.stream):
            if b.pat_dev is None:
                rp, ci = P.pattern()
                rp0, ci0 = rp[:b.n_dof + 1].copy(), ci[:b.nnz].copy()
                b.pat_dev = (rp0, ci0, torch.as_tensor(rp0, device="cuda"), torch.as_tensor(ci0, device="cuda"))
            rp0, ci0, rpd, cid = b.pat_dev
            dx = torch.zeros((b.slots, b.n_dof), dtype=torch.float64, device="cuda")
            rv = b.rsnap.view(b.slots, b.n_dof)
            for s in np.nonzero(mask)[0]:
                sol = b.fs.get(int(s))
                if sol is None:
                    view = BlockView(P, int(s), b.jsnap, rp0, ci0, rpd, cid)
                    sol = b.fs[int(s)] = SaddlePointSolver(view, "pressure", 1.0 / b.req[s].Re)
                x, _ = sol.solve(rv[s], tol=newton_forcing(), atol=atol)
                dx[s] = x
        return dx, 0

    def _apply_device(self, b: _Batch, slots, result) -> None:
        dx, launches = result
        self.solver_launches += launches
        self.device_solves += len(slots)
        with self.torch.cuda.stream(b.stream):
            xv = b.P.x_dev[:b.P.n_dof].view(b.slots, b.n_dof)
            for s in slots:
                xv[s] -= dx[s]
                b.req[s].newton_iterations += 1
                b.state[s] = "assemble"
        b.inflight = False
        for s, st_ in enumerate(b.state):
            if st_ == "wait":
                b.state[s] = "assemble"

    def _apply(self, b: _Batch, s: int, dx: np.ndarray) -> None:
        with self.torch.cuda.stream(b.stream):
            sl = b.P.x_dev[s * b.n_dof:(s + 1) * b.n_dof]
            sl -= self.torch.as_tensor(dx, device="cuda")
        b.req[s].newton_iterations += 1
        b.state[s] = "assemble"

    def _fail(self, b: _Batch, slots, exc: BaseException, t0: float, device: bool) -> List[Request]:
        """End the requests of `slots` with the solve's error; free their slots."""
        out = []
        for s in slots:
            req = b.req[s]
            req.error = f"linear solve failed: {exc}"
            req.dofs = b.P.x_dev[s * b.n_dof:(s + 1) * b.n_dof].cpu().numpy()
            req.t_done = time.perf_counter() - t0
            b.req[s] = None
            b.state[s] = "free"
            b.fs.pop(s, None)
            out.append(req)
        if device:
            b.inflight = False
            for k, st_ in enumerate(b.state):
                if st_ == "wait":
                    b.state[k] = "assemble"
        return out

    def close(self) -> None:
        self.pool.shutdown(wait=True)
        if self.tpool is not None:
            self.tpool.shutdown(wait=True)
        for b in self.batches.values():
            b.release()
        self.batches.clear()

    def run(self, requests: List[Request], realtime: bool = True) -> List[Request]:
        """Serve a stream; arrivals are honoured in real time."""
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting: List[Request] = []
        finished: List[Request] = []
        futs: Dict[cf.Future, tuple] = {}
        t0 = time.perf_counter()
        i = 0
        while len(finished) < len(requests):
            now = time.perf_counter() - t0
            while i < len(pending) and (pending[i].arrival <= now or not realtime):
                waiting.append(pending[i])
                i += 1
            waiting = [r for r in waiting if not self._admit(r, time.perf_counter() - t0)]
            ready = [b for b in self.batches.values() if "assemble" in b.state]
            for b in ready:
                finished += self._assemble(b, t0, futs)
            if len(finished) >= len(requests):
                break
            if not futs and not ready:
                if i < len(pending) and realtime:
                    time.sleep(max(0.0, min(0.01, pending[i].arrival - now)))
                    continue
                if waiting:
                    raise RuntimeError("requests cannot be admitted (device memory)")
                continue
            if futs:
                nxt = pending[i].arrival - (time.perf_counter() - t0) if (i < len(pending) and realtime) else None
                timeout = None if nxt is None else max(0.0, nxt)
                dn, _ = cf.wait(list(futs), timeout=timeout, return_when=cf.FIRST_COMPLETED)
                for f in dn:
                    b, s, ts = futs.pop(f)
                    self.t_solve += time.perf_counter() - ts
                    exc = f.exception()
                    if exc is not None:
                        # a failed solve ends its requests with the error; the server goes on
                        finished += self._fail(b, s if isinstance(s, tuple) else (s,), exc, t0,
                                               device=isinstance(s, tuple))
                    elif isinstance(s, tuple):
                        self._apply_device(b, s, f.result())
                    else:
                        self._apply(b, s, f.result())
        self.torch.cuda.synchronize()
        return finished


def serve_sequential(requests: List[Request], precision: str = "fp64", tol: float = 1e-10,
                     realtime: bool = True, device_solver: bool = False,
                     device_saddle_min_side: int = 32) -> List[Request]:
    """The plain path: requests one at a time in arrival order, one problem
    per request (resident meshes cached per class), Newton with SuperLU
    (with device_solver: Poisson requests with the device BiCGStab, as the
    batched server then does)."""
    cache: Dict[tuple, tuple] = {}
    t0 = time.perf_counter()
    for req in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if realtime and req.arrival > now:
            time.sleep(req.arrival - now)
        key = (req.kind, req.side)
        if key not in cache:
            P = _class_problem(req.kind, req.side, precision, 1)
            if device_solver and (req.kind == "poisson" or req.side >= device_saddle_min_side):
                P.linear_solver = "bicgstab" if req.kind == "poisson" else "fieldsplit"
                P.linear_solver_atol = 0.1 * tol     # the batched server's inexact step
            P.initialise()
            cache[key] = (P, P.get_dofs().copy())
        P, x0 = cache[key]
        req.t_admit = time.perf_counter() - t0
        P.set_parameter_vector(_request_params(req, P))
        P.set_dofs(x0)
        P.newton_solver_tolerance = tol
        P.max_newton_iterations = 20
        try:
            req.residuals = P.solve()
            req.newton_iterations = len(req.residuals) - 1
        except Exception as e:  # recorded per request
            req.error = str(e)
        req.dofs = P.get_dofs()
        req.t_done = time.perf_counter() - t0
    return requests


def summary(reqs: List[Request], wall: float) -> dict:
    lat = np.array([r.latency for r in reqs if r.error is None])
    return {"requests": len(reqs), "errors": sum(r.error is not None for r in reqs),
            "p50_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_s": float(np.percentile(lat, 99)) if lat.size else None,
            "solves_per_s": len(reqs) / wall if wall > 0 else None,
            "mean_newton_iterations": float(np.mean([r.newton_iterations for r in reqs]))}
