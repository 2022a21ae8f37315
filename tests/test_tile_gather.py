"""The tile gather (k_gather_tiles) against the per-slot gather
(k_gather_slots / k_gather_rows): both sum every CSR slot and residual entry
from its element contributions in element order, the order of the
reference's scatter loop (problem.cc:5500-5560), so they must give the same
bits -- R and J, FP64 and FP32 Jacobians, for every width of element row the
tile gather has a kernel for (4, 8, 16, 32 lanes per incidence), for the
fused multi-domain (moving-mesh) assembly, and for the residual alone; the
pipelined host assembly (per-slot sums) agrees with it bit for bit.
Problems it does not apply to (more than 32 local values per element) keep
the per-slot gather."""
import numpy as np
import pytest


def _fields_problem(names, dim, N, prec, space="C2"):
    """Independent Poisson fields on Q2 quads / hexahedra: len(names) x
    (9 or 27) local values (4 or 8 for C1)."""
    from pyoomph_gb300.equations import DirichletBC, PoissonEquation
    from pyoomph_gb300.meshes import CuboidBrickMesh, RectangularQuadMesh
    from pyoomph_gb300.problem import Problem
    P = Problem()
    P.jacobian_precision = prec
    if dim == 3:
        P += CuboidBrickMesh(N=N)
        walls = ["left", "right", "top", "bottom", "back", "front"]
    else:
        P += RectangularQuadMesh(N=N)
        walls = ["left", "right", "top", "bottom"]
    eq = None
    for k, nm in enumerate(names):
        e = PoissonEquation(nm, space=space, source=float(k + 1))
        eq = e if eq is None else eq + e
    P += (eq + DirichletBC(**{names[0]: 0.0}) @ walls) @ "domain"
    return P


def _make(case, prec):
    from pyoomph_gb300 import workloads as W
    if case == "c1_quad":          # 4 local values
        return _fields_problem(["u"], 2, 9, prec, space="C1")
    if case == "p2_tri":           # 6
        return W.poisson_problem(N=9, split="left", jacobian_precision=prec)
    if case == "ns_p2p1_tri":      # 15
        return W.navier_stokes_problem(N=11, jacobian_precision=prec)
    if case == "q2_hex":           # 27
        return W.nonlinear_diffusion_problem(N=4, jacobian_precision=prec)
    if case == "two_q2_hex":       # 54: per-slot gather
        return _fields_problem(["u", "w"], 3, 3, prec)
    raise KeyError(case)


LANES = {"c1_quad": 4, "p2_tri": 8, "ns_p2p1_tri": 16, "q2_hex": 32, "two_q2_hex": 0}


def _bits(t):
    import torch
    return t.view(torch.int64) if t.dtype == torch.float64 else t.view(torch.int32)


def _same_bits(a, b) -> bool:
    import torch
    return bool(torch.equal(_bits(a), _bits(b)))


def _assemble_both(P):
    """(R, J) with the tile gather, then with the per-slot gather."""
    import torch
    from pyoomph_gb300 import _native as N
    out = []
    for mode in (N.FE_GATHER_TILES, N.FE_GATHER_SLOTS):
        N.check(N.load().fe_problem_set_gather(P._h, mode))
        P.R_dev.fill_(float("nan"))
        P.J_dev.fill_(float("nan"))
        P.assemble_device(True)
        torch.cuda.synchronize()
        P.check()
        out.append((P.R_dev[:P.n_dof].clone(), P.J_dev[:P.nnz].clone()))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("case", list(LANES))
def test_tile_gather_gives_the_bits_of_the_slot_gather(case, prec):
    from pyoomph_gb300 import _native as N
    from pyoomph_gb300 import workloads as W
    P = _make(case, prec)
    P.initialise()
    W.perturb_dofs(P, seed=7, sigma=0.05)
    L = N.load()
    assert L.fe_problem_gather_lanes(P._h) == 0
    n_slots = P.launch_count(True)
    N.check(L.fe_problem_set_gather(P._h, N.FE_GATHER_TILES))
    assert L.fe_problem_gather_lanes(P._h) == LANES[case]
    n_tiles = P.launch_count(True)
    (R0, J0), (R1, J1) = _assemble_both(P)
    assert _same_bits(R0, R1) and _same_bits(J0, J1)
    assert bool(np.isfinite(J0.double().cpu().numpy()).all())
    # the residual rides in the Jacobian's launch either way
    assert n_tiles == n_slots
    # a residual-only assembly keeps its own gather and the same bits
    P.R_dev.fill_(float("nan"))
    P.assemble_device(False)
    assert _same_bits(P.R_dev[:P.n_dof], R0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,chunks", [("fp64", 1), ("fp64", 5), ("fp32", 3)])
def test_pipelined_host_assembly_equals_the_tile_gather(prec, chunks):
    import torch
    from pyoomph_gb300 import _native as N
    from pyoomph_gb300 import workloads as W
    P = W.navier_stokes_problem(N=17, jacobian_precision=prec)
    P.initialise()
    W.perturb_dofs(P, seed=5, sigma=0.02)
    (R0, J0), _ = _assemble_both(P)
    xh = P.x_dev[:P.n_dof].cpu().pin_memory()
    Rh = torch.full((P.n_dof,), float("nan"), dtype=torch.float64).pin_memory()
    Jh = torch.full((P.nnz,), float("nan"), dtype=P.J_dev.dtype).pin_memory()
    P.assemble_host(xh, Rh, Jh, chunks=chunks)
    torch.cuda.current_stream().synchronize()
    P.check()
    assert _same_bits(Rh, R0.cpu()) and _same_bits(Jh, J0.cpu())


@pytest.mark.gpu
def test_fused_moving_mesh_assembly_with_the_tile_gather():
    from pyoomph_gb300 import _native as N
    from pyoomph_gb300 import ale
    P = ale.DropletProblem(N=6, contact_angle_deg=80.0)
    P.initialise()
    P.set_params(__bdf0=1000.0, __bdf1=-1000.0, __bdf2=0.0)
    N.check(N.load().fe_problem_set_gather(P._h, N.FE_GATHER_TILES))
    assert N.load().fe_problem_gather_lanes(P._h) > 0
    (R0, J0), (R1, J1) = _assemble_both(P)
    assert _same_bits(R0, R1) and _same_bits(J0, J1)
