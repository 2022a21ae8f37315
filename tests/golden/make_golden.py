"""Generate the golden fixtures in this folder from the reference's own
oomph-lib core (oracle/_ref/oomph_ref_driver, built by oracle/ref/Makefile
from the reference tree).  Run in the build container, where the reference
tree exists:

    make -C oracle/ref REFERENCE=/root/reference -j8
    python tests/golden/make_golden.py

Each case stores the mesh, pins, nodal values, parameters and the
reference's equation numbers, residual and CSR Jacobian (rowptr, colidx,
vals) from Problem::get_jacobian with the vectors-of-pairs assembler, for
both the default zero filter (threshold 0.0) and the structural pattern
(threshold -1, every coupling kept).  It also stores oomph's integration
knots, weights and shape tables per element type.

The hang/*.npz cases come from oracle/_ref/oomph_hang_driver: Q2 meshes refined
by oomph's own quadtrees (several levels, no 2:1 balance), with the
refinement plan (level and centre of every split element), oomph's node
positions, elements, equation numbers, completed hang infos (masters in
oomph's order), and the structural CSR Jacobian and residual of the Poisson
form with Gaussian sources at given dofs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

CASES = [
    # name, etype, eq, nx, ny, nz, split
    ("poisson_q2_4x3", O.Q2_QUAD, O.EQ_POISSON, 4, 3, 0, 0),
    ("poisson_p2_3x4_left", O.P2_TRI, O.EQ_POISSON, 3, 4, 0, 0),
    ("nldiff_q2hex_2x2x3", O.Q2_HEX, O.EQ_NONLINEAR_DIFFUSION, 2, 2, 3, 0),
    ("nldiff_q2_3x3", O.Q2_QUAD, O.EQ_NONLINEAR_DIFFUSION, 3, 3, 0, 0),
    ("ns_th_4x3_left", O.P2_TRI, O.EQ_NAVIER_STOKES_TH, 4, 3, 0, 0),
    ("ns_th_3x3_right", O.P2_TRI, O.EQ_NAVIER_STOKES_TH, 3, 3, 0, 1),
]


def _around(px, py, n):
    return lambda x, y, level: abs(x - px) < 0.5 / n / 2 ** level and abs(y - py) < 0.5 / n / 2 ** level


HANG_CASES = [
    # name, N, max level, refinement predicate (centre x, centre y, level)
    ("hang_point_4_L4", 4, 4, _around(0.26, 0.26, 4)),
    ("hang_ring_4_L3", 4, 3, lambda x, y, l: abs(np.hypot(x - 0.5, y - 0.5) - 0.3) < 0.2 / 2 ** l),
    ("hang_two_points_6_L3", 6, 3, lambda x, y, l: _around(0.2, 0.7, 6)(x, y, l) or _around(0.55, 0.3, 6)(x, y, l)),
]


def hang_cases():
    import hang_oracle as H
    if not H.ref_hang_available():
        raise SystemExit("oracle/_ref/oomph_hang_driver missing: build it with make -C oracle/ref")
    for k, (name, N, L, chosen) in enumerate(HANG_CASES):
        rng = np.random.default_rng(2000 + k)
        g = gaussians(rng, 2)
        plan = np.array(H.refinement_plan(O.mesh(O.Q2_QUAD, N, N), chosen, L)).reshape(-1, 3)
        r0 = H.ref_hang_run(N, chosen, L, g)
        dofs = rng.normal(0.0, 0.3, r0["R"].size)
        r = H.ref_hang_run(N, chosen, L, g, dofs=dofs)
        hn = np.array(sorted(r["hang"]), dtype=np.int64)
        hp = np.cumsum([0] + [len(r["hang"][h]) for h in hn]).astype(np.int64)
        hm = np.array([m for h in hn for m, _ in r["hang"][h]], dtype=np.int64)
        hw = np.array([w for h in hn for _, w in r["hang"][h]])
        os.makedirs(os.path.join(HERE, "hang"), exist_ok=True)
        np.savez_compressed(os.path.join(HERE, "hang", name + ".npz"), N=N, L=L, plan=plan, gaussians=g, dofs=dofs,
                            x=r["x"], conn=r["conn"], eqn=r["eqn"], hang_node=hn, hang_ptr=hp, hang_master=hm,
                            hang_weight=hw, rowptr=r["rowptr"], colidx=r["colidx"], vals=r["vals"], R=r["R"])
        print(name, r["R"].size, r["colidx"].size, len(hn))


def gaussians(rng, dim, n=8):
    c = rng.uniform(0.0, 1.0, (n, dim))
    w = rng.uniform(0.05, 0.2, (n, 1))
    A = rng.normal(0.0, 1.0, (n, 1))
    return np.hstack([c, w, A])


def main():
    if not O.ref_driver_available():
        raise SystemExit("oracle/_ref/oomph_ref_driver missing: build it with make -C oracle/ref")
    for k, (name, et, eq, nx, ny, nz, split) in enumerate(CASES):
        rng = np.random.default_rng(1000 + k)
        m = O.mesh(et, nx, ny, nz, split=split)
        if eq == O.EQ_NAVIER_STOKES_TH:
            P = O.navier_stokes_problem(m, rho=1.0, mu=0.01)
            P.set_dofs(P.dofs() + rng.normal(0.0, 1e-3, P.n_dof))
        else:
            P = O.poisson_problem(m, gaussians(rng, m.dim), eq=eq)
            P.set_dofs(rng.normal(0.0, 0.3, P.n_dof))
        out = dict(etype=et, eq=eq, nx=nx, ny=ny, nz=nz, split=split, x=m.x, conn=m.conn,
                   bmask=m.bmask, is_vertex=m.is_vertex, nvalue=P.nvalue, pinned=P.pinned,
                   values=P.values, params=P.params)
        for tag, thr in (("zf", 0.0), ("st", -1.0)):
            eqn, R, rp, ci, v = O.ref_driver_assemble(P, True, thr)
            out[f"eqn"] = eqn
            out[f"R"] = R
            out[f"rowptr_{tag}"] = rp
            out[f"colidx_{tag}"] = ci
            out[f"vals_{tag}"] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, P.n_dof, len(out["colidx_st"]), len(out["colidx_zf"]))
    T = O.ref_driver_tables()
    tabs = {}
    for et, t in T.items():
        for key, val in t.items():
            tabs[f"{et}_{key}"] = val
    np.savez_compressed(os.path.join(HERE, "oomph_tables.npz"), **tabs)
    hang_cases()


if __name__ == "__main__":
    main()
