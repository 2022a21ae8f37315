"""CUDA-graph replay of an assembly and the launch-shape autotuner."""
import numpy as np
import pytest


def test_autotune_cache_roundtrip(tmp_path):
    from pyoomph_gb300 import autotune as AT
    path = str(tmp_path / "tune.json")
    assert AT.cached("k", path) is None
    AT.store("k", {"best": 8, "ms": {"8": 1.0, "16": 2.0}}, path)
    assert AT.cached("k", path)["best"] == 8
    # a cached result is returned without building anything
    best, table = AT.tune("k", lambda c: (_ for _ in ()).throw(AssertionError("no build")), [1, 2], path=path)
    assert best == 8 and table["16"] == 2.0


def test_epb_candidates_fit_a_block():
    from pyoomph_gb300 import autotune as AT
    for nq, nloc in ((9, 9), (7, 15), (27, 27), (7, 27)):
        c = AT.epb_candidates(nq, nloc)
        assert c and all(max(e * nq, e * nloc) <= 1024 for e in c)


def test_oversized_launch_shape_is_rejected():
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=4)
    P.elems_per_block = 128
    with pytest.raises(ValueError):
        P.lower()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_graph_replay_equals_direct_assembly(prec):
    import torch
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=12, jacobian_precision=prec)
    P.initialise()
    W.perturb_dofs(P, seed=2, sigma=1e-2)
    P.assemble_device(True)
    R0, J0 = P.R_dev.clone(), P.J_dev.clone()
    P.capture_assembly(True)
    P.R_dev.zero_()
    P.J_dev.zero_()
    P.assemble_graph()
    torch.cuda.synchronize()
    P.check()
    assert torch.equal(P.R_dev, R0) and torch.equal(P.J_dev, J0)
    # the graph reads the dof vector at replay time
    W.perturb_dofs(P, seed=3, sigma=1e-2)
    P.assemble_graph()
    R1 = P.R_dev.clone()
    P.assemble_device(True)
    assert torch.equal(P.R_dev, R1) and not torch.equal(R1, R0)


@pytest.mark.gpu
def test_graph_replay_of_the_fused_droplet_assembly():
    import torch
    from pyoomph_gb300 import ale
    P = ale.DropletProblem(N=6, contact_angle_deg=80.0)
    P.initialise()
    P.set_params(__bdf0=1000.0, __bdf1=-1000.0, __bdf2=0.0)
    P.assemble_device(True)
    R0, J0 = P.R_dev.clone(), P.J_dev.clone()
    P.capture_assembly(True)
    P.R_dev.zero_()
    P.J_dev.zero_()
    P.assemble_graph()
    torch.cuda.synchronize()
    assert torch.equal(P.R_dev, R0) and torch.equal(P.J_dev, J0)


@pytest.mark.gpu
def test_autotune_picks_a_measured_candidate(tmp_path):
    from pyoomph_gb300 import autotune as AT
    from pyoomph_gb300 import workloads as W

    def make(e):
        P = W.poisson_problem(N=16, seed=0)
        P.elems_per_block = e
        P.initialise()
        return P
    best, table = AT.tune("poisson16", make, [2, 4, 8], steps=3, warmup=1, path=str(tmp_path / "t.json"))
    assert best in (2, 4, 8) and set(table) == {"2", "4", "8"}
    P = make(best)
    assert P.kernel.epb == best


@pytest.mark.gpu
@pytest.mark.parametrize("kind,prec,chunks", [("ns", "fp64", 1), ("ns", "fp64", 5), ("ns", "fp32", 8),
                                               ("poisson", "fp64", 3)])
def test_pipelined_host_assembly_equals_device_assembly(kind, prec, chunks):
    import torch
    from pyoomph_gb300 import workloads as W
    P = (W.navier_stokes_problem(N=20, jacobian_precision=prec) if kind == "ns"
         else W.poisson_problem(N=20, jacobian_precision=prec))
    P.initialise()
    W.perturb_dofs(P, seed=4, sigma=1e-2)
    P.assemble_device(True)
    R0 = P.R_dev[:P.n_dof].cpu()
    J0 = P.J_dev[:P.nnz].cpu()
    xh = P.x_dev[:P.n_dof].cpu().pin_memory()
    Rh = torch.full((P.n_dof,), float("nan"), dtype=torch.float64).pin_memory()
    Jh = torch.full((P.nnz,), float("nan"), dtype=P.J_dev.dtype).pin_memory()
    for _ in range(2):                          # a second call reuses the plan and buffers
        P.assemble_host(xh, Rh, Jh, chunks=chunks)
        torch.cuda.current_stream().synchronize()
        P.check()
        assert torch.equal(Rh, R0) and torch.equal(Jh, J0)
    # with stage timing: the call's timeline, per chunk element kernel <=
    # gathers <= copies, and the same bits
    assert P.pipeline_times().size == 0
    P.set_stage_timing(True)
    P.assemble_host(xh, Rh, Jh, chunks=chunks)
    T = P.pipeline_times()
    P.set_stage_timing(False)
    P.stage_times()
    assert T.shape[1] == 3 and 1 <= T.shape[0] <= chunks
    assert (T[:, 0] <= T[:, 1]).all() and (T[:, 1] <= T[:, 2] + 1e-3).all() and (np.diff(T[:, 0]) >= 0).all()
    torch.cuda.current_stream().synchronize()
    assert torch.equal(Rh, R0) and torch.equal(Jh, J0)
    # element chunks on two alternating streams: the same bits
    P.set_pipeline_streams(2)
    Rh.fill_(float("nan"))
    Jh.fill_(float("nan"))
    for _ in range(2):
        P.assemble_host(xh, Rh, Jh, chunks=chunks)
        torch.cuda.current_stream().synchronize()
        P.check()
        assert torch.equal(Rh, R0) and torch.equal(Jh, J0)
    P.set_pipeline_streams(0)
