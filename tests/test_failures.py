"""Failure detection without a GPU fault: errors become status codes.

Host-side injected failures (a compile error, a bad mesh, an element that
collapses, NaN dofs, an admission the HBM budget refuses) must come back as
clean error codes / exceptions, and the bounds-checked device build must turn
an out-of-range connectivity entry into a status word instead of an
out-of-bounds read.  Nothing here faults, traps or hangs a GPU: the planted
bad index runs only in the CPU emulator of the generated code."""
import numpy as np
import pytest

import ale_oracle as A
import kernel_emulator as KE
from pyoomph_gb300 import _native as N


def test_compile_error_is_reported_with_the_log(tmp_path):
    with pytest.raises(N.FeError) as ei:
        N.code_build('extern "C" __global__ void broken_kernel() { this is not C++; }', "broken_kernel",
                     str(tmp_path))
    assert ei.value.code == N.FE_ERR_COMPILE
    assert "error" in str(ei.value).lower()


def test_connectivity_out_of_range_is_rejected_on_the_host():
    from pyoomph_gb300 import ale
    P = ale.DropletProblem(N=3)
    P.lower()
    P.conns[0] = P.conns[0].copy()
    P.conns[0][2, 4] = P.n_nodes + 5
    with pytest.raises(N.FeError) as ei:
        P.host_pattern()
    assert ei.value.code == N.FE_ERR_ARG and "out of range" in str(ei.value)


def test_bounds_checked_build_records_a_bad_node_instead_of_reading_it():
    """The generated fused kernel, emulated on the CPU with FE_BOUNDS_CHECK:
    a connectivity entry far outside the node arrays sets status 2 and the
    element index; the kernel reads node 0 in its place."""
    from pyoomph_gb300 import ale
    P = ale.DropletProblem(N=3)
    fk = P.lower()
    D = A.droplet(3)
    v = A.initial_values(D)
    conns = [c.copy() for c in P.conns]
    conns[0][5, 2] = 10 ** 8
    params = np.array([{"__bdf0": 1e3, "__bdf1": -1e3, "__bdf2": 0.0, "contact_angle": 1.2,
                        "dynamic_viscosity": 0.1, "surface_tension": 1.0}[n] for n in P.param_names])
    outs, status = KE.run_fused(fk, conns, v, [v, v], D.x0, params, defines=("FE_BOUNDS_CHECK",))
    assert status[0] == 2 and status[1] == 5
    outs_ok, status_ok = KE.run_fused(fk, P.conns, v, [v, v], D.x0, params, defines=("FE_BOUNDS_CHECK",))
    assert not status_ok.any()
    # elements other than the corrupted one are unaffected
    keep = np.arange(conns[0].shape[0]) != 5
    assert np.array_equal(outs[0][0][keep], outs_ok[0][0][keep])


@pytest.mark.gpu
def test_nan_dofs_give_an_infinite_residual_and_a_newton_error():
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.problem import NewtonSolverError
    P = W.poisson_problem(N=8)
    P.initialise()
    x = P.get_dofs()
    x[3] = np.nan
    P.set_dofs(x)
    P.assemble_device(with_jacobian=False)
    assert P.residual_max() == float("inf")
    with pytest.raises(NewtonSolverError):
        P.solve()


@pytest.mark.gpu
def test_collapsed_elements_set_the_status_word():
    from pyoomph_gb300 import workloads as W

    def squash(x):
        x = x.copy()
        x[:, 0] = np.maximum(x[:, 0], 0.5)     # the left half collapses onto x = 0.5
        return x
    P = W.poisson_problem(N=8, transform=squash)
    P.geometry = "general"
    P.initialise()
    P.assemble_device(with_jacobian=True)
    with pytest.raises(N.FeError) as ei:
        P.check()
    assert ei.value.code == N.FE_ERR_DEVICE


@pytest.mark.gpu
def test_bounds_checked_build_gives_identical_results_on_valid_meshes():
    import torch
    from pyoomph_gb300 import ale
    out = []
    for bc in (False, True):
        P = ale.DropletProblem(N=6, contact_angle_deg=70.0)
        P.bounds_check = bc
        P.initialise()
        P.set_params(__bdf0=1e3, __bdf1=-1e3, __bdf2=0.0)
        R, J = P.get_jacobian()
        out.append((R, J.data))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.gpu
def test_admission_is_refused_when_the_hbm_budget_is_exhausted():
    from pyoomph_gb300 import serving as S
    srv = S.Server(slots=2, hbm_reserve=1.0, workers=1)   # reserve all device memory
    try:
        with pytest.raises(RuntimeError, match="cannot be admitted"):
            srv.run([S.Request(0, "poisson", 8, 0.0, seed=1)], realtime=False)
    finally:
        srv.close()
