"""Serving: continuous batching of assemble + Newton requests.

A request's result is the same alone and in a mix (bit-identical dofs);
every request converges to the FP64 oracle's solution within 1e-10; the
stream summary reports p50/p99 latency."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _oracle_solution(req, tol: float = 1e-10):
    from pyoomph_gb300 import workloads as W
    if req.kind == "poisson":
        OP = O.poisson_problem(O.mesh(O.Q2_QUAD, req.side, req.side), W.draw_gaussians(req.seed, 8, 2))
    else:
        OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, req.side, req.side), rho=1.0, mu=1.0 / req.Re)
    O.newton(OP, tol=tol)
    return OP.dofs()


def test_request_alone_equals_request_in_mix_and_matches_oracle():
    from pyoomph_gb300 import serving as S
    probe = S.Request(0, "ns", 8, 0.0, seed=5, Re=70.0)
    alone = S.Server(slots=3).run([probe], realtime=False)[0]
    assert alone.error is None, alone.error
    mix = [S.Request(1, "poisson", 8, 0.0, seed=1), S.Request(2, "ns", 8, 0.0, seed=2, Re=30.0),
           S.Request(3, "poisson", 12, 0.0, seed=3), S.Request(4, "ns", 8, 0.0, seed=4, Re=90.0),
           S.Request(0, "ns", 8, 0.0, seed=5, Re=70.0), S.Request(5, "poisson", 8, 0.0, seed=6)]
    out = {r.rid: r for r in S.Server(slots=3).run(mix, realtime=False)}
    assert all(r.error is None for r in out.values())
    assert np.array_equal(out[0].dofs, alone.dofs)
    for r in out.values():
        x = _oracle_solution(r)
        assert np.max(np.abs(r.dofs - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))


def test_stream_summary_and_sequential_path_agree():
    from pyoomph_gb300 import serving as S
    reqs = S.make_stream(12, rate=200.0, seed=3, side_range=(8, 20))
    import copy
    # both paths converge to 1e-12 so that their solutions agree to 1e-10
    seq = S.serve_sequential(copy.deepcopy(reqs), realtime=True, tol=1e-12)
    bat = S.Server(slots=4, tol=1e-12).run(copy.deepcopy(reqs), realtime=True)
    sb = {r.rid: r for r in bat}
    for r in seq:
        assert r.error is None and sb[r.rid].error is None
        assert np.max(np.abs(r.dofs - sb[r.rid].dofs)) <= 1e-10 * max(1.0, np.max(np.abs(r.dofs)))
    s = S.summary(bat, max(r.t_done for r in bat))
    assert s["p50_s"] is not None and s["p99_s"] >= s["p50_s"] and s["errors"] == 0


def test_device_solver_alone_equals_mix_and_matches_oracle():
    """Poisson requests solved on the device (one batched BiCGStab per class
    round): a request's dofs are bit-identical alone or in a mix, and every
    request converges to the oracle's solution within 1e-10."""
    from pyoomph_gb300 import serving as S
    srv = S.Server(slots=3, tol=1e-12, device_solver=True)
    alone = srv.run([S.Request(0, "poisson", 10, 0.0, seed=7)], realtime=False)[0]
    srv.close()
    assert alone.error is None, alone.error
    mix = [S.Request(1, "poisson", 10, 0.0, seed=1), S.Request(2, "ns", 8, 0.0, seed=2, Re=30.0),
           S.Request(0, "poisson", 10, 0.0, seed=7), S.Request(3, "poisson", 10, 0.0, seed=3)]
    srv = S.Server(slots=3, tol=1e-12, device_solver=True)
    out = {r.rid: r for r in srv.run(mix, realtime=False)}
    srv.close()
    assert srv.device_solves > 0
    assert np.array_equal(out[0].dofs, alone.dofs)
    for r in out.values():
        assert r.error is None
        x = _oracle_solution(r)
        assert np.max(np.abs(r.dofs - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))


def test_failed_device_solve_ends_only_its_requests(monkeypatch):
    """A device solve that raises (a fake of the failing call, on the host)
    ends the requests of that solve with the error; the other requests of
    the stream still complete and match the oracle."""
    from pyoomph_gb300 import serving as S
    from pyoomph_gb300.linsolve import LinearSolverError
    real = S.Server._device_solve
    calls = {"n": 0}

    def flaky(self, b, mask, atol):
        calls["n"] += 1
        if calls["n"] == 1:
            raise LinearSolverError("injected failure")
        return real(self, b, mask, atol)
    monkeypatch.setattr(S.Server, "_device_solve", flaky)
    srv = S.Server(slots=2, tol=1e-12, device_solver=True)
    reqs = [S.Request(1, "poisson", 10, 0.0, seed=1), S.Request(2, "ns", 8, 0.0, seed=2, Re=30.0),
            S.Request(3, "poisson", 12, 0.0, seed=3)]
    out = {r.rid: r for r in srv.run(reqs, realtime=False)}
    srv.close()
    failed = [r for r in out.values() if r.error]
    assert len(out) == 3 and failed and all("injected failure" in r.error for r in failed)
    for r in out.values():
        if r.error is None:
            x = _oracle_solution(r)
            assert np.max(np.abs(r.dofs - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))


def test_navier_stokes_requests_on_the_device_alone_equal_mix():
    """Navier-Stokes requests solved on the device (each by its own
    saddle-point solver over its replica's block): bit-identical alone or
    in a mix with other requests of the class, and within 1e-10 of the
    oracle's solution."""
    from pyoomph_gb300 import serving as S
    srv = S.Server(slots=3, tol=1e-12, device_solver=True)
    srv.device_saddle_min_side = 8
    alone = srv.run([S.Request(0, "ns", 10, 0.0, seed=5, Re=70.0)], realtime=False)[0]
    srv.close()
    assert alone.error is None, alone.error
    mix = [S.Request(1, "ns", 10, 0.0, seed=1, Re=40.0), S.Request(2, "poisson", 8, 0.0, seed=2),
           S.Request(0, "ns", 10, 0.0, seed=5, Re=70.0), S.Request(3, "ns", 10, 0.0, seed=3, Re=100.0)]
    srv = S.Server(slots=3, tol=1e-12, device_solver=True)
    srv.device_saddle_min_side = 8
    out = {r.rid: r for r in srv.run(mix, realtime=False)}
    assert srv.device_solves > 0
    srv.close()
    assert np.array_equal(out[0].dofs, alone.dofs)
    for r in out.values():
        assert r.error is None, r.error
        # the device solves take inexact Newton steps, so the requests follow
        # other iterates than the oracle's exact ones: both are compared
        # converged well below the tolerance (the oracle to 1e-13)
        x = _oracle_solution(r, tol=1e-13)
        assert np.max(np.abs(r.dofs - x)) <= 1e-10 * max(1.0, np.max(np.abs(x)))
