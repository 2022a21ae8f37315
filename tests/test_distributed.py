"""Element-partitioned assembly: each rank assembles its contiguous element
range, the plan maps its local CSR into the global pattern, one halo
exchange (an all-to-all to the rows' owners) completes the owned rows; the
result equals the single-rank assembly.  On 2 and 3 host ranks (gloo, CPU)
with the oracle as each rank's assembler, and on 2 gloo ranks sharing the
GPU with the engine (-m gpu).  A rank that fails before the exchange makes
the others raise instead of hanging."""
import os
import socket

import numpy as np
import pytest

import oracle as O


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, kind, fail_rank, q):
    import sys
    import datetime
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    import oracle as O
    from pyoomph_gb300 import distributed as D
    from pyoomph_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        if kind == "ns":
            P = W.navier_stokes_problem(N=[5, 4])
            m = O.mesh(O.P2_TRI, 5, 4)
            OP = O.navier_stokes_problem(m, rho=1.0, mu=0.01)
            x = OP.dofs() + np.random.default_rng(0).normal(0, 0.1, OP.n_dof)
        else:
            gauss = W.draw_gaussians(0, 8, 2)
            P = W.poisson_problem(N=[6, 5], gaussians=gauss)
            m = O.mesh(O.Q2_QUAD, 6, 5)
            OP = O.poisson_problem(m, gauss)
            x = np.random.default_rng(0).normal(0, 0.5, OP.n_dof)
        OP.set_dofs(x)
        rowptr, colidx = P.host_pattern()          # global pattern, identical on every rank
        lo, hi = D.element_ranges(m.conn.shape[0], world)[rank]
        sub = O.Mesh(m.etype, m.dim, m.x, np.ascontiguousarray(m.conn[lo:hi]), m.bmask, m.is_vertex)
        LP = O.Problem(mesh=sub, eq=OP.eq, nval=OP.nval, nvalue=OP.nvalue, pinned=OP.pinned,
                       values=OP.values.copy(), params=OP.params)
        R_loc, lrp, lci, lv = O.assemble(LP, True, -1.0)   # this rank's element block
        plan = D.make_plan(rank, world, rowptr, colidx, lrp, lci)
        if rank == fail_rank:
            raise RuntimeError("injected failure before the exchange")
        full, R = D.reduce_owned(plan, torch.as_tensor(lv), torch.as_tensor(R_loc))
        vals, Rown = D.owned_view(plan, rowptr, full, R)
        R0, rp0, ci0, v0 = O.assemble(OP, True, -1.0)
        a, b = plan.rows
        ok = (np.array_equal(rowptr, rp0) and np.array_equal(colidx, ci0) and
              np.max(np.abs(vals.numpy() - v0[rp0[a]:rp0[b]])) <= 1e-13 * np.max(np.abs(v0)) and
              np.max(np.abs(Rown.numpy() - R0[a:b])) <= 1e-13 * np.max(np.abs(R0)) and
              plan.halo_slots.size < plan.nnz)
        q.put((rank, "ok" if ok else "mismatch"))
    except Exception as e:  # reported to the parent
        q.put((rank, f"error: {type(e).__name__}: {e}"))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, kind, fail_rank=-1):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, kind, fail_rank, q)) for r in range(world)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
    out = {}
    while not q.empty():
        r, s = q.get()
        out[r] = s
    for p in ps:
        if p.is_alive():
            p.kill()
    return out


@pytest.mark.parametrize("world,kind", [(2, "poisson"), (3, "poisson"), (2, "ns")])
def test_partitioned_assembly_equals_single_rank(world, kind):
    out = _run(world, kind)
    assert out == {r: "ok" for r in range(world)}, out


def test_failed_rank_is_detected_not_hung():
    out = _run(2, "poisson", fail_rank=1)
    assert out[1].startswith("error: RuntimeError: injected")
    assert out[0].startswith("error:"), out


def _engine_worker(rank, world, port, kind, prec, q):
    import sys
    import datetime
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from pyoomph_gb300 import distributed as D
    from pyoomph_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        torch.cuda.set_device(0)

        def make():
            if kind == "ns":
                P = W.navier_stokes_problem(N=[24, 20], jacobian_precision=prec)
            else:
                P = W.nonlinear_diffusion_problem(N=[6, 5, 4], jacobian_precision=prec)
            return P
        full = make()
        full.initialise()
        x = full.get_dofs() + np.random.default_rng(3).normal(0.0, 0.05, full.n_dof)
        full.set_dofs(x)
        R0, J0 = full.get_jacobian()                          # the single-rank engine assembly
        local = make()
        local.element_range = D.element_ranges(full.mesh.n_elem, world)[rank]
        local.initialise()
        local.set_dofs(x)
        Rl, Jl = local.get_jacobian()                          # this rank's elements only, on the GPU
        plan = D.make_plan(rank, world, J0.indptr, J0.indices, Jl.indptr, Jl.indices)
        vals, R = D.reduce_owned(plan, torch.as_tensor(Jl.data.astype(np.float64)), torch.as_tensor(Rl))
        v, Ro = D.owned_view(plan, J0.indptr, vals, R)
        a, b = plan.rows
        tol = 1e-12 if prec == "fp64" else 1e-6
        v0 = J0.data.astype(np.float64)
        errJ = np.max(np.abs(v.numpy() - v0[J0.indptr[a]:J0.indptr[b]])) / np.max(np.abs(v0))
        errR = np.max(np.abs(Ro.numpy() - R0[a:b])) / np.max(np.abs(R0))
        ok = errJ <= tol and errR <= 1e-12 and 0 < plan.halo_slots.size < plan.nnz and Jl.nnz < J0.nnz
        q.put((rank, "ok" if ok else f"mismatch J {errJ:.2e} R {errR:.2e}"))
    except Exception as e:
        q.put((rank, f"error: {type(e).__name__}: {e}"))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


@pytest.mark.gpu
@pytest.mark.parametrize("kind,prec", [("ns", "fp64"), ("hex", "fp32")])
def test_engine_ranks_assemble_their_elements_and_match_single_rank(kind, prec):
    """Two gloo ranks sharing the one GPU: each rank's engine assembles its
    contiguous element range (Problem.element_range, the reference's
    First_el_for_assembly split) with the global numbering, the halo
    exchange (host tensors, gloo) completes its owned rows, and they equal
    the single-rank engine assembly (values 1e-12; FP32 Jacobians 1e-6, their
    partial sums round differently).  No kernel waits on another rank."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_engine_worker, args=(r, 2, port, kind, prec, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=600)
    out = {}
    while not q.empty():
        r, s = q.get()
        out[r] = s
    for p in ps:
        if p.is_alive():
            p.kill()
    assert out == {0: "ok", 1: "ok"}, out


def test_element_range_patterns_cover_the_global_pattern():
    """Host only: the CSR patterns of the element ranges (Problem.element_range,
    global numbering, fe_pattern_host) lie inside the global pattern and
    together cover it."""
    from pyoomph_gb300 import distributed as D
    from pyoomph_gb300 import workloads as W
    G = W.navier_stokes_problem(N=[7, 5])
    rp, ci = G.host_pattern()
    keys = set(zip(np.repeat(np.arange(len(rp) - 1), np.diff(rp)).tolist(), ci.tolist()))
    seen = set()
    for lo, hi in D.element_ranges(G.mesh.n_elem, 3):
        P = W.navier_stokes_problem(N=[7, 5])
        P.element_range = (lo, hi)
        lrp, lci = P.host_pattern()
        assert lrp.shape == rp.shape
        lk = set(zip(np.repeat(np.arange(len(lrp) - 1), np.diff(lrp)).tolist(), lci.tolist()))
        assert lk <= keys and len(lk) < len(keys)
        seen |= lk
    assert seen == keys
    P = W.navier_stokes_problem(N=[7, 5])
    P.element_range = (0, 10 ** 6)
    with pytest.raises(ValueError):
        P.host_pattern()
