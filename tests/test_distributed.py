"""Element-partitioned assembly on 2 and 3 host ranks (gloo, CPU): each rank
assembles its contiguous element range (here with the oracle standing in for
the rank's GPU), the plan maps its local CSR into the global pattern, one
halo exchange completes the owned rows; the result equals the single-rank
assembly.  A rank that fails before the exchange makes the others raise
instead of hanging."""
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
