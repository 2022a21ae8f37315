"""Parity at the benchmark's own sizes: the CUDA assembly of the bench
workloads (same meshes, seeds and perturbed states as bench.py) against
the oracle's restated vectors-of-pairs assembly (problem.cc:4038-4165,
5332-5666) on identical dof vectors.

* Navier-Stokes Taylor-Hood P2/P1, 256x256 split mesh (131,072 elements,
  588,290 dofs, 17.4 M CSR entries);
* Poisson Q2, 64x64 (4,096 elements);
* nonlinear diffusion Q2 hex, 24^3 and 48^3 (110,592 elements, 52.7 M
  entries).

Contract: CSR rowptr/colidx bit-exact (structural pattern, oomph's
threshold -1); FP64 and df64 residual and Jacobian within 1e-12 of the
oracle's max norm; FP32 Jacobian within 1e-5 (residual still 1e-12).
Precisions "J:R" select a residual precision too: "fp32:df64" is the FP32
Jacobian with the residual path in double-float (same 1e-12 contract).
"""
import gc

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-12
JTOL32 = 1e-5


def _relmax(a, b):
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - b)) / max(np.max(np.abs(b)), 1e-300))


def _problems(workload, side):
    """(oracle problem in the bench's state, factory of the product problem
    in the same state by precision)."""
    from pyoomph_gb300 import workloads as W
    if workload == "ns":
        OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, side, side), rho=1.0, mu=0.01)

        def make(prec):
            jp, _, rp = prec.partition(":")
            P = W.navier_stokes_problem(N=side, jacobian_precision=jp)
            P.residual_precision = rp or "fp64"
            P.initialise()
            W.perturb_dofs(P, seed=0, sigma=1e-3)
            return P
    elif workload == "poisson":
        OP = O.poisson_problem(O.mesh(O.Q2_QUAD, side, side), W.draw_gaussians(0, 8, 2))

        def make(prec):
            jp, _, rp = prec.partition(":")
            P = W.poisson_problem(N=side, seed=0, jacobian_precision=jp)
            P.residual_precision = rp or "fp64"
            P.initialise()
            P.set_dofs(np.random.default_rng(1).normal(0.0, 0.3, P.n_dof))
            return P
    else:
        OP = O.poisson_problem(O.mesh(O.Q2_HEX, side, side, side), W.draw_gaussians(0, 16, 3),
                               eq=O.EQ_NONLINEAR_DIFFUSION)

        def make(prec):
            jp, _, rp = prec.partition(":")
            P = W.nonlinear_diffusion_problem(N=side, seed=0, jacobian_precision=jp)
            P.residual_precision = rp or "fp64"
            P.initialise()
            P.set_dofs(np.random.default_rng(0).normal(0.0, 0.1, P.n_dof))
            return P
    return OP, make


CASES = [("ns", 256, ("fp64", "df64", "fp32", "fp32:df64", "df64:df64")),
         ("poisson", 64, ("fp64", "df64", "fp32", "fp32:df64")),
         ("hex", 24, ("fp64", "df64", "fp32", "df64:df64")),
         ("hex", 48, ("fp64", "fp32", "fp32:df64"))]


@pytest.mark.parametrize("workload,side,precs", CASES, ids=[f"{w}{s}" for w, s, _ in CASES])
def test_full_size_assembly_matches_oracle(workload, side, precs):
    OP, make = _problems(workload, side)
    ref = None
    for prec in precs:
        P = make(prec)
        if ref is None:
            assert P.n_dof == OP.n_dof and np.array_equal(P.eqn, OP.eqn)
            OP.set_dofs(P.get_dofs())
            ref = O.assemble(OP, True, -1.0)
        else:
            x = P.get_dofs()
            assert np.array_equal(x, OP.dofs())
        R0, rp, ci, v = ref
        R, J = P.get_jacobian()
        assert np.array_equal(J.indptr, rp), prec
        assert np.array_equal(J.indices, ci), prec
        assert _relmax(R, R0) <= RTOL, (prec, _relmax(R, R0))
        err = _relmax(J.data, v)
        assert err <= (JTOL32 if prec.startswith("fp32") else RTOL), (prec, err)
        del P, R, J
        gc.collect()
