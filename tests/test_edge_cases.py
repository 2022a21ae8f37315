"""Edge cases of the assembly: a problem without unknowns, a single element,
a strongly ragged mesh, an empty element range."""
import ctypes

import numpy as np
import pytest

import oracle as O
from pyoomph_gb300 import _native as N
from pyoomph_gb300 import workloads as W


def _all_pinned():
    P = W.poisson_problem(N=3, seed=1)
    P.lower()
    P.eqn = np.full_like(P.eqn, -1)
    P.n_dof = 0
    return P


def test_pattern_of_a_problem_without_unknowns_is_empty():
    rp, ci = _all_pinned().host_pattern()
    assert rp.tolist() == [0] and ci.size == 0


@pytest.mark.parametrize("shape", [[1, 1], [7, 2], [2, 9]])
def test_host_pattern_single_element_and_ragged_meshes(shape):
    P = W.poisson_problem(N=shape, seed=2)
    rp, ci = P.host_pattern()
    OP = O.poisson_problem(O.mesh(O.Q2_QUAD, shape[0], shape[1]), W.draw_gaussians(2, 8, 2))
    _, orp, oci, _ = O.assemble(OP, True, -1.0)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


def test_empty_element_range_is_accepted_on_the_host():
    P = W.poisson_problem(N=2, seed=1)
    P.lower()
    desc, doms, keep = P._descriptors(with_code=False)
    doms[0].n_elem = 0
    nnz = ctypes.c_int64()
    assert N.load().fe_pattern_host(ctypes.byref(desc), ctypes.byref(nnz), None, None) == 0
    assert nnz.value == 0


@pytest.mark.gpu
def test_assembly_without_unknowns_runs():
    P = _all_pinned()
    P.initialise()
    P.assemble_device(with_jacobian=True)
    P.check()
    assert P.nnz == 0 and P.residual_max() == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [[1, 1], [7, 2]])
def test_single_element_and_ragged_meshes_match_the_oracle(shape):
    P = W.poisson_problem(N=shape, seed=2)
    P.initialise()
    x = np.random.default_rng(0).normal(size=P.n_dof)
    P.set_dofs(x)
    R, J = P.get_jacobian()
    OP = O.poisson_problem(O.mesh(O.Q2_QUAD, shape[0], shape[1]), W.draw_gaussians(2, 8, 2))
    OP.set_dofs(x)
    Ro, orp, oci, ov = O.assemble(OP, True, -1.0)
    assert np.max(np.abs(R - Ro)) <= 1e-12 * max(1.0, np.max(np.abs(Ro)))
    assert np.max(np.abs(J.data - ov)) <= 1e-12 * np.max(np.abs(ov))
