"""The synthetic workloads of the benchmark, built through the public API.

* Poisson -Laplace(u) = f on the unit square, Q2 quads, u = 0 on the
  boundary, f a sum of 8 Gaussians drawn from a seed;
* steady incompressible Navier-Stokes, Taylor-Hood P2/P1 on a split
  structured mesh, Re = 100 (rho = 1, mu = 1/100), lid u_x = 16x^2(1-x)^2
  on top, no-slip elsewhere, one pressure pinned, dofs perturbed by
  N(0, 1e-3) from a seed;
* 3D nonlinear diffusion -div((1+u^2) grad u) = f on the unit cube, Q2
  hexahedra, f a sum of 16 Gaussians from a seed.

Gaussians: centres U[0,1]^dim, widths U[0.05, 0.2], amplitudes N(0,1),
f(x) = sum_k A_k exp(-|x - c_k|^2 / (2 w_k^2)), numpy default_rng(seed).
"""
from __future__ import annotations

import numpy as np

from .equations import (DiffusionEquation, DirichletBC, NavierStokesEquations, NonlinearDiffusionEquation,
                        PoissonEquation, PressureFixation)
from .meshes import CuboidBrickMesh, RectangularQuadMesh
from .problem import Problem


def draw_gaussians(seed: int, n: int, dim: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, (n, dim))
    w = rng.uniform(0.05, 0.2, (n, 1))
    A = rng.normal(0.0, 1.0, (n, 1))
    return np.hstack([c, w, A])


def lid_velocity(x, y):
    return 16.0 * x * x * (1.0 - x) * (1.0 - x)


def poisson_problem(N=64, seed: int = 0, gaussians: np.ndarray = None, split: str = None,
                    jacobian_precision: str = "fp64", transform=None, transient: bool = False) -> Problem:
    """transient: the diffusion equation du/dt - Laplace(u) = f instead."""
    g = draw_gaussians(seed, 8, 2) if gaussians is None else gaussians
    P = Problem()
    P.jacobian_precision = jacobian_precision
    P.transient = transient
    P += RectangularQuadMesh(N=N, split_in_tris=split or False, transform=transform)
    eq = DiffusionEquation(source=g) if transient else PoissonEquation(source=g)
    P += (eq + DirichletBC(u=0.0) @ ["left", "right", "top", "bottom"]) @ "domain"
    return P


def nonlinear_diffusion_problem(N=48, seed: int = 0, gaussians: np.ndarray = None,
                                jacobian_precision: str = "fp64", dim: int = 3, transform=None,
                                transient: bool = False) -> Problem:
    """transient: du/dt - div((1+u^2) grad u) = f instead."""
    g = draw_gaussians(seed, 16, dim) if gaussians is None else gaussians
    P = Problem()
    P.jacobian_precision = jacobian_precision
    P.transient = transient
    if dim == 3:
        P += CuboidBrickMesh(N=N, transform=transform)
        walls = ["left", "right", "top", "bottom", "back", "front"]
    else:
        P += RectangularQuadMesh(N=N, transform=transform)
        walls = ["left", "right", "top", "bottom"]
    P += (NonlinearDiffusionEquation(source=g, temporal_factor=1 if transient else 0) + DirichletBC(u=0.0) @ walls) @ "domain"
    return P


def navier_stokes_problem(N=256, Re: float = 100.0, split: str = "left",
                          jacobian_precision: str = "fp64", transform=None, transient: bool = False) -> Problem:
    P = Problem()
    P.jacobian_precision = jacobian_precision
    P.transient = transient
    P += RectangularQuadMesh(N=N, split_in_tris=split, transform=transform)
    eqs = NavierStokesEquations(mass_density=1.0, dynamic_viscosity=1.0 / Re)
    eqs += DirichletBC(velocity_x=lid_velocity, velocity_y=0.0) @ "top"
    eqs += DirichletBC(velocity_x=0.0, velocity_y=0.0) @ ["left", "right", "bottom"]
    eqs += PressureFixation("pressure", 0.0)
    P += eqs @ "domain"
    return P


def wavy(amplitude: float = 0.02):
    """A smooth non-affine deformation of the unit square/cube that keeps the
    boundary in place: x_i += a sin(pi x_i) sin(2 pi x_j) for j != i."""
    def f(x):
        y = x.copy()
        d = x.shape[1]
        for i in range(d):
            y[:, i] = x[:, i] + amplitude * np.sin(np.pi * x[:, i]) * np.sin(2 * np.pi * x[:, (i + 1) % d])
        return y
    return f


def perturb_dofs(P: Problem, seed: int, sigma: float = 1e-3) -> None:
    """Add N(0, sigma) to every dof (from a seed)."""
    x = P.get_dofs()
    x = x + np.random.default_rng(seed).normal(0.0, sigma, x.size)
    P.set_dofs(x)


def _main(argv=None) -> None:
    """Repeated R+J assemblies of one workload (a small driver for profiling
    the element kernel): ``python -m pyoomph_gb300.workloads ns 128 df64 5``
    = Navier-Stokes side 128, double-float Jacobian, 5 assemblies after one
    warm-up."""
    import argparse
    import torch
    ap = argparse.ArgumentParser(prog="python -m pyoomph_gb300.workloads")
    ap.add_argument("workload", choices=["ns", "poisson", "hex"])
    ap.add_argument("side", type=int)
    ap.add_argument("precision", choices=["fp64", "fp32", "df64"])
    ap.add_argument("repeat", type=int, nargs="?", default=3)
    ap.add_argument("--epb", type=int, default=None, help="elements per block (default: the generator's)")
    ap.add_argument("--jref", type=int, choices=[0, 1], default=None,
                    help="1: contract the Jacobian in reference coordinates, 0: physical (default: the generator's)")
    ap.add_argument("--tc", type=int, choices=[0, 1], default=None,
                    help="1: FP32 Jacobian contracted on the tensor cores, 0: on the FP32 pipes "
                         "(default: the generator's)")
    ap.add_argument("--zero-filter", action="store_true",
                    help="assemble J in the reference's zero-filtered pattern (threshold 0.0)")
    ap.add_argument("--transient", action="store_true",
                    help="the transient form (BDF2 weights of dt = 1e-3, both previous levels = the current values)")
    ap.add_argument("--min-blocks", type=int, default=None,
                    help="resident blocks per SM to bound the element kernel's registers for")
    ap.add_argument("--threads", type=int, default=None,
                    help="threads per block of the element kernel (default: one per local row)")
    ap.add_argument("--residual", choices=["fp64", "df64"], default="fp64",
                    help="df64: the residual path in double-float on the FP32 pipes (fp32/df64 Jacobians)")
    ap.add_argument("--tile-gather", action="store_true",
                    help="sum the CSR values with a warp per tile of rows instead of a thread per slot")
    a = ap.parse_args(argv)
    if a.workload == "ns":
        P = navier_stokes_problem(N=a.side, jacobian_precision=a.precision, transient=a.transient)
    elif a.workload == "poisson":
        P = poisson_problem(N=a.side, seed=0, jacobian_precision=a.precision, transient=a.transient)
    else:
        P = nonlinear_diffusion_problem(N=a.side, seed=0, jacobian_precision=a.precision, transient=a.transient)
    P.elems_per_block = a.epb
    P.min_blocks_per_sm = a.min_blocks
    P.residual_precision = a.residual
    P.threads_per_block = a.threads
    if a.jref is not None:
        P.jacobian_reference = bool(a.jref)
    if a.tc is not None:
        P.tensor_cores = bool(a.tc)
    P.initialise()
    if a.tile_gather:
        from . import _native as N
        N.check(N.load().fe_problem_set_gather(P._h, N.FE_GATHER_TILES))
    perturb_dofs(P, seed=0, sigma=1e-3)
    if a.transient:
        from .ale import bdf_weights
        P.assemble_device(with_jacobian=False)
        P.set_history_values(0, P.get_values())
        P.set_history_values(1, P.get_values())
        P.set_parameters(**dict(zip(("_bdf_w0", "_bdf_w1", "_bdf_w2"), bdf_weights(2, 1e-3, 1e-3))))
    zt = 0.0 if a.zero_filter else None
    P.assemble_device(with_jacobian=True, zero_threshold=zt)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.repeat):
        P.assemble_device(with_jacobian=True, zero_threshold=zt)
    e1.record()
    torch.cuda.synchronize()
    P.check()
    # the same assemblies once more with events around the stages
    P.set_stage_timing(True)
    P.stage_times()
    for _ in range(a.repeat):
        P.assemble_device(with_jacobian=True, zero_threshold=zt)
    torch.cuda.synchronize()
    ms, calls = P.stage_times()
    P.set_stage_timing(False)
    stages = ", ".join(f"{k} {v / max(calls, 1):.4f}" for k, v in
                       zip(("dof scatter", "element kernels", "residual gather", "jacobian gather", "tensor cores"), ms))
    print(f"{a.workload} side {a.side} {a.precision}: {P.mesh.n_elem} elements, kernel {P.kernel.name}, "
          f"{e0.elapsed_time(e1) / a.repeat:.4f} ms per assembly ({stages} ms)")


if __name__ == "__main__":
    _main()
