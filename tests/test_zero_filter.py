"""The reference's default sparse assembly on the device: oomph's zero
filter (Problem::Numerical_zero_for_sparse_assembly = 0.0, problem.cc:110),
which leaves out every element entry with |J_e(i,j)| <= threshold, so that
the CSR pattern depends on the values (problem.cc:5520-5560).

* Poisson and nonlinear-diffusion fixtures of the reference's own oomph-lib
  (tests/golden): rowptr/colidx bit-exact, values within 1e-12.
* Every element type, also Taylor-Hood, whose pattern depends on which
  analytically-zero entries round to exactly 0.0 (GiNaC's operation order,
  unpinnable here): bit-exact against the restated insertion loop
  (oracle.vectors_of_pairs) run on the product's own element matrices, and
  the matrix within 1e-12 of the reference's.
* Full size (NS 256^2, Poisson 64^2, hex 24^3): the matrix within 1e-12 of
  the C oracle's filtered assembly (its pattern too, where no entry rounds
  to zero), and bit-exact against the insertion loop in C
  (oracle.pairs_from_elements) on the product's own element matrices.
"""
import glob
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = [c for c in sorted(glob.glob(os.path.join(GOLD, "*_*.npz"))) if not c.endswith("oomph_tables.npz")]


def _relmax(a, b):
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - b)) / max(np.max(np.abs(b)), 1e-300))


def _elem_eqns(P):
    lay = P.kernel.layout
    eqn = np.asarray(P.eqn).reshape(P.mesh.n_nodes, len(P.fields))
    return eqn[P.mesh.conn[:, lay.node], lay.val]


def _sparse_maxdiff(rp_a, ci_a, va, rp_b, ci_b, vb, n):
    A = sp.csr_matrix((np.asarray(va, dtype=np.float64), ci_a, rp_a), shape=(n, n))
    B = sp.csr_matrix((np.asarray(vb, dtype=np.float64), ci_b, rp_b), shape=(n, n))
    d = (A - B).tocsr()
    return (float(np.max(np.abs(d.data))) if d.nnz else 0.0) / float(np.max(np.abs(B.data)))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_golden_zero_filtered_pattern(path):
    from test_gpu_parity import _product_for
    g = np.load(path)
    P = _product_for(g)
    P.set_values(g["values"])
    P.numerical_zero_for_sparse_assembly = 0.0
    R, J = P.get_jacobian()
    Re, Je = P.element_buffers()
    rp, ci, v = O.vectors_of_pairs(_elem_eqns(P), Je, P.n_dof, 0.0)
    # the device compaction is the reference's insertion loop on these element matrices
    assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
    assert np.array_equal(J.data, v)
    n = P.n_dof
    if int(g["eq"]) != O.EQ_NAVIER_STOKES_TH:
        # no analytically-zero entries: the reference's own pattern, bit for bit
        assert np.array_equal(J.indptr, g["rowptr_zf"]) and np.array_equal(J.indices, g["colidx_zf"])
        assert _relmax(J.data, g["vals_zf"]) <= 1e-12
    assert _sparse_maxdiff(J.indptr, J.indices, J.data, g["rowptr_zf"], g["colidx_zf"], g["vals_zf"], n) <= 1e-12
    assert _relmax(R, g["R"]) <= 1e-12
    # the structural assembly is unchanged by a filtered one, and the filtered
    # values are the structural ones on the surviving slots
    P.numerical_zero_for_sparse_assembly = None
    R2, J2 = P.get_jacobian()
    assert np.array_equal(J2.indptr, g["rowptr_st"]) and np.array_equal(R, R2)
    assert _sparse_maxdiff(J.indptr, J.indices, J.data, J2.indptr, J2.indices, J2.data, n) == 0.0


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("threshold", [0.0, 1e-3])
def test_thresholds_and_precisions_match_the_insertion_loop(prec, threshold):
    """A positive threshold also drops small entries from the sums; FP32
    Jacobians filter their own values."""
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=[5, 4], jacobian_precision=prec)
    P.initialise()
    W.perturb_dofs(P, seed=2, sigma=0.05)
    P.numerical_zero_for_sparse_assembly = threshold
    R, J = P.get_jacobian()
    Re, Je = P.element_buffers()
    rp, ci, v = O.vectors_of_pairs(_elem_eqns(P), Je.astype(np.float64), P.n_dof, threshold)
    assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
    if prec == "fp64":
        assert np.array_equal(J.data, v)
    else:   # FP32 sums in FP32 on the device
        assert _relmax(J.data, v) <= 1e-6
    if threshold > 0:
        assert J.nnz < P.nnz


FULL = [("ns", 256), ("poisson", 64), ("hex", 24)]


@pytest.mark.parametrize("workload,side", FULL, ids=[f"{w}{s}" for w, s in FULL])
def test_full_size_zero_filter_vs_oracle(workload, side):
    from test_fullsize_parity import _problems
    OP, make = _problems(workload, side)
    P = make("fp64")
    OP.set_dofs(P.get_dofs())
    R0, rp, ci, v = O.assemble(OP, True, 0.0)
    P.numerical_zero_for_sparse_assembly = 0.0
    R, J = P.get_jacobian()
    assert _relmax(R, R0) <= 1e-12
    assert _sparse_maxdiff(J.indptr, J.indices, J.data, rp, ci, v, P.n_dof) <= 1e-12
    if workload != "ns":
        assert np.array_equal(J.indptr, rp) and np.array_equal(J.indices, ci)
        assert _relmax(J.data, v) <= 1e-12
    # the compaction is the reference's insertion loop on the product's own
    # element matrices (rounding decides which Taylor-Hood entries are 0.0,
    # and so where a column is first inserted)
    Re, Je = P.element_buffers()
    rp2, ci2, v2 = O.pairs_from_elements(_elem_eqns(P), Je.reshape(Je.shape[0], -1), P.n_dof, 0.0)
    assert np.array_equal(J.indptr, rp2) and np.array_equal(J.indices, ci2) and np.array_equal(J.data, v2)
