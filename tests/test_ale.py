"""Moving-mesh droplet (pyoomph_gb300.ale): fused bulk + interface +
contact-line kernel against the ALE oracle (independent numpy restatement
with complex-step Jacobians)."""
import math

import numpy as np
import pytest

import ale_oracle as A
import kernel_emulator as KE
from pyoomph_gb300 import ale

PAR = {"dynamic_viscosity": 0.1, "surface_tension": 1.0}


def _state(D, seed, amp=0.3, move=None):
    """Random nodal values and previous positions; positions moved by
    less than the element size allows (no inverted elements)."""
    rng = np.random.default_rng(seed)
    n1d = int(round(np.sqrt(D.tri.shape[0] / 2)))
    move = 0.04 / n1d ** 2 if move is None else move
    v = A.initial_values(D)
    v[:, 2:] = rng.normal(size=(v.shape[0], 4)) * amp
    v[:, 0:2] += rng.normal(size=(v.shape[0], 2)) * move
    h0 = v.copy()
    h0[:, 0:2] += rng.normal(size=(v.shape[0], 2)) * move
    h1 = h0.copy()
    h1[:, 0:2] += rng.normal(size=(v.shape[0], 2)) * move
    v[D.pinned] = A.initial_values(D)[D.pinned]
    return v, h0, h1


def _params(theta_deg, bdf=(1500.0, -2000.0, 500.0)):
    p = dict(PAR, contact_angle=math.radians(theta_deg))
    p.update(__bdf0=bdf[0], __bdf1=bdf[1], __bdf2=bdf[2])
    return p


def _pvec(P, p):
    return np.array([p[n] for n in P.param_names])


# ---------------------------------------------------------------------------
# CPU: the oracle itself, the mesh, the generated code (emulated), the pattern
# ---------------------------------------------------------------------------
def test_oracle_complex_step_matches_central_differences():
    D = A.droplet(3)
    v, h0, h1 = _state(D, 1)
    p = _params(70)
    blocks = A.element_res_jac(D, v, [h0, h1], p)
    funs = [lambda z: A.bulk_residual(z, D.x0[D.tri], p),
            lambda z: A.line_residual(z, [h0[D.line][:, :, 0:2], h1[D.line][:, :, 0:2]], p),
            lambda z: A.point_residual(z, p)]
    lays = [A.bulk_layout(), A.line_layout(), A.point_layout()]
    conns = [D.tri, D.line, D.point]
    for (R, J), f, lay, c in zip(blocks, funs, lays, conns):
        loc = A._gather(v, c, lay)
        eps = 1e-6
        for k in range(loc.shape[1]):
            zp, zm = loc.copy(), loc.copy()
            zp[:, k] += eps
            zm[:, k] -= eps
            fd = (f(zp) - f(zm)) / (2 * eps)
            assert np.max(np.abs(fd - J[:, :, k])) < 1e-6 * (1 + np.max(np.abs(J)))


def test_droplet_mesh_matches_oracle():
    for N in (3, 5):
        P = ale.DropletProblem(N=N)
        P.lower()
        D = A.droplet(N)
        assert np.array_equal(P.mesh.x, D.x0)
        assert np.array_equal(P.mesh.conn, D.tri)
        assert np.array_equal(P.mesh.interface, D.line)
        assert np.array_equal(P.mesh.contact_line, D.point)
        assert np.array_equal(P.eqn, D.eqn)
        assert P.n_dof == D.n_dof
        # interface: 2N lines, counterclockwise with the outward normal (tau_1, -tau_0)
        assert D.line.shape[0] == 2 * N
        for e in range(D.line.shape[0]):
            xs = D.x0[D.line[e]]
            t = xs[2] - xs[0]
            assert np.dot([t[1], -t[0]], xs[1]) > 0
        assert np.allclose(np.hypot(*D.x0[D.line.ravel()].T), 1.0)


@pytest.mark.parametrize("N,theta,prec", [(3, 60.0, "fp64"), (4, 120.0, "fp64"), (6, 110.0, "fp64"),
                                          (4, 90.0, "fp32"), (4, 90.0, "df64"), (6, 110.0, "df64")])
def test_emulated_fused_kernel_matches_oracle(N, theta, prec):
    P = ale.DropletProblem(N=N, contact_angle_deg=theta, jacobian_precision=prec)
    fk = P.lower()
    D = A.droplet(N)
    p = _params(theta)
    for seed in (0, 1):
        v, h0, h1 = _state(D, seed)
        outs, status = KE.run_fused(fk, P.conns, v, [h0, h1], D.x0, _pvec(P, p))
        assert not status.any()
        ref = A.element_res_jac(D, v, [h0, h1], p)
        for (Re, Je), (Ro, Jo) in zip(outs, ref):
            assert np.max(np.abs(Re - Ro)) <= 1e-12 * np.max(np.abs(Ro))
            tol = 1e-6 if prec == "fp32" else 1e-12
            assert np.max(np.abs(Je.astype(np.float64) - Jo)) <= tol * np.max(np.abs(Jo))


def test_emulated_inverted_elements_use_the_metric_weight():
    """An inverted element (negative det dx/ds) is integrated with the weight
    sqrt(det(t t^T)) = |det| of the metric formulation, in the kernel and in
    the oracle alike."""
    P = ale.DropletProblem(N=6, contact_angle_deg=110.0)
    fk = P.lower()
    D = A.droplet(6)
    p = _params(110.0)
    v, h0, h1 = _state(D, 7, move=0.01)
    w, psi, dpsi, _, _ = A.tri_tables()
    t = np.einsum("eli,la->eai", v[:, :2][D.tri], dpsi[0])
    assert (t[:, 0, 0] * t[:, 1, 1] - t[:, 0, 1] * t[:, 1, 0]).min() < 0
    outs, _ = KE.run_fused(fk, P.conns, v, [h0, h1], D.x0, _pvec(P, p))
    ref = A.element_res_jac(D, v, [h0, h1], p)
    # the folded elements are badly conditioned: rounding grows ~100x
    for (Re, Je), (Ro, Jo) in zip(outs, ref):
        assert np.max(np.abs(Re - Ro)) <= 1e-10 * np.max(np.abs(Ro))
        assert np.max(np.abs(Je - Jo)) <= 1e-10 * np.max(np.abs(Jo))


def test_emulated_residual_only_flag_leaves_jacobian_untouched():
    P = ale.DropletProblem(N=3)
    fk = P.lower()
    D = A.droplet(3)
    v, h0, h1 = _state(D, 3)
    p = _params(80)
    outs, _ = KE.run_fused(fk, P.conns, v, [h0, h1], D.x0, _pvec(P, p), flag=0)
    ref = A.element_res_jac(D, v, [h0, h1], p)
    for (Re, Je), (Ro, _) in zip(outs, ref):
        assert np.max(np.abs(Re - Ro)) <= 1e-12 * np.max(np.abs(Ro))
        assert not Je.any()


@pytest.mark.parametrize("N", [3, 6])
def test_host_pattern_matches_oracle(N):
    P = ale.DropletProblem(N=N)
    rp, ci = P.host_pattern()
    D = A.droplet(N)
    v = A.initial_values(D)
    _, orp, oci, _ = A.assemble(D, v, [v, v], _params(90))
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


def test_bdf_weights():
    for order in (1, 2):
        for dt, dtp in ((1e-3, 1e-3), (2e-3, 1e-3)):
            w = ale.bdf_weights(order, dt, dtp)
            assert np.allclose(w, A.bdf_weights(order, dt, dtp))
            # exact for polynomials of degree <= order: t, t^2 with t_n = 0
            ts = np.array([0.0, -dt, -dt - dtp])
            assert abs(np.dot(w, ts) - 1.0) < 1e-9
            if order == 2:
                assert abs(np.dot(w, ts ** 2)) < 1e-9
    assert ale.bdf_weights(2, 1e-3) == pytest.approx((1500.0, -2000.0, 500.0))


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _gpu_problem(N, theta, prec="fp64"):
    P = ale.DropletProblem(N=N, contact_angle_deg=theta, jacobian_precision=prec)
    P.initialise()
    return P


@pytest.mark.gpu
def test_gpu_element_buffers_match_oracle():
    P = _gpu_problem(4, 75.0)
    D = A.droplet(4)
    p = _params(75.0)
    P.set_params(**{k: p[k] for k in ("__bdf0", "__bdf1", "__bdf2")})
    v, h0, h1 = _state(D, 5)
    P.set_state(v, [h0, h1])
    P.assemble_device(with_jacobian=True)
    P.check()
    ref = A.element_res_jac(D, v, [h0, h1], p)
    for dom, (Ro, Jo) in enumerate(ref):
        Re, Je = P.element_buffers(dom)
        assert np.max(np.abs(Re - Ro)) <= 1e-12 * np.max(np.abs(Ro))
        assert np.max(np.abs(Je - Jo)) <= 1e-12 * np.max(np.abs(Jo))


@pytest.mark.gpu
@pytest.mark.parametrize("N,theta", [(3, 60.0), (6, 110.0)])
def test_gpu_assembly_matches_oracle(N, theta):
    P = _gpu_problem(N, theta)
    D = A.droplet(N)
    p = _params(theta)
    P.set_params(**{k: p[k] for k in ("__bdf0", "__bdf1", "__bdf2")})
    v, h0, h1 = _state(D, 7)
    P.set_state(v, [h0, h1])
    R, J = P.get_jacobian()
    Ro, orp, oci, ov = A.assemble(D, v, [h0, h1], p)
    rp, ci = P.pattern()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.max(np.abs(R - Ro)) <= 1e-12 * np.max(np.abs(Ro))
    assert np.max(np.abs(J.data - ov)) <= 1e-12 * np.max(np.abs(ov))
    # dof scatter, ONE fused element launch, R and J summed in one gather launch
    assert P.launch_count(True) == 3


@pytest.mark.gpu
def test_gpu_time_steps_match_oracle():
    N, theta, dt = 4, 70.0, 1e-3
    P = _gpu_problem(N, theta)
    P.newton_solver_tolerance = 1e-11
    D, ref = A.run_steps(N, theta, PAR["dynamic_viscosity"], PAR["surface_tension"], dt, 3)
    for k in range(3):
        P.step(dt)
        v = P.get_values()
        scale = np.max(np.abs(ref[k]), axis=0) + 1e-300
        err = np.max(np.abs(v - ref[k]) * D.present, axis=0) / scale
        assert np.all(err < 1e-10), (k, err)


@pytest.mark.gpu
@pytest.mark.parametrize("N,theta", [(3, 60.0), (6, 110.0)])
def test_gpu_df64_assembly_matches_oracle(N, theta):
    """The double-float Jacobian of the fused moving-mesh kernel: pattern
    bit-exact, R and J within the FP64 contract."""
    P = _gpu_problem(N, theta, "df64")
    D = A.droplet(N)
    p = _params(theta)
    P.set_params(**{k: p[k] for k in ("__bdf0", "__bdf1", "__bdf2")})
    v, h0, h1 = _state(D, 7)
    P.set_state(v, [h0, h1])
    R, J = P.get_jacobian()
    Ro, orp, oci, ov = A.assemble(D, v, [h0, h1], p)
    rp, ci = P.pattern()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.max(np.abs(R - Ro)) <= 1e-12 * np.max(np.abs(Ro))
    assert np.max(np.abs(J.data - ov)) <= 1e-12 * np.max(np.abs(ov))


@pytest.mark.gpu
def test_gpu_fp32_jacobian_converges_to_fp64_solution():
    N, theta, dt = 6, 110.0, 1e-3
    P64 = _gpu_problem(N, theta, "fp64")
    P32 = _gpu_problem(N, theta, "fp32")
    for P in (P64, P32):
        P.newton_solver_tolerance = 1e-11
        P.max_newton_iterations = 20
        for _ in range(2):
            P.step(dt)
    a, b = P64.get_values(), P32.get_values()
    assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(a))


@pytest.mark.gpu
def test_gpu_assembly_is_deterministic():
    P = _gpu_problem(8, 95.0)
    D = A.droplet(8)
    v, h0, h1 = _state(D, 11)
    P.set_params(__bdf0=1500.0, __bdf1=-2000.0, __bdf2=500.0)
    P.set_state(v, [h0, h1])
    R1, J1 = P.get_jacobian()
    R2, J2 = P.get_jacobian()
    assert np.array_equal(R1, R2) and np.array_equal(J1.data, J2.data)


@pytest.mark.gpu
def test_gpu_full_size_jacobian_is_the_derivative_of_the_residual():
    """At the full droplet size (~200k dofs) no oracle assembly runs; the
    Jacobian must still be the derivative of the residual along a random
    direction (central differences, second order)."""
    import torch
    P = _gpu_problem(110, 75.0)
    assert P.n_dof > 190_000
    P.set_params(__bdf0=1500.0, __bdf1=-2000.0, __bdf2=500.0)
    rng = np.random.default_rng(3)
    v0 = P._values0
    v = v0.copy()
    v[:, 2:] = rng.normal(size=(v.shape[0], 4)) * 0.1
    v[:, 0:2] += rng.normal(size=(v.shape[0], 2)) * 0.04 / 110 ** 2
    v[P.pinned] = v0[P.pinned]
    P.set_state(v, [v0, v0])
    x = P.x_dev[:P.n_dof].cpu().numpy().copy()
    d = rng.normal(size=x.shape)
    pos = np.zeros(x.shape, dtype=bool)
    for c in (0, 1):
        e = P.eqn[:, c]
        pos[e[e >= 0]] = True
    d[pos] *= 1.0 / 110 ** 2          # positions move by a fraction of the element size
    R, J = P.get_jacobian()
    Jd = J @ d
    h = 1e-4
    P.x_dev[:P.n_dof].copy_(torch.from_numpy(x + h * d))
    Rp = P.get_residuals()
    P.x_dev[:P.n_dof].copy_(torch.from_numpy(x - h * d))
    Rm = P.get_residuals()
    fd = (Rp - Rm) / (2 * h)
    assert np.max(np.abs(fd - Jd)) <= 1e-6 * np.max(np.abs(Jd))


# ---------------------------------------------------------------------------
# mass matrices and parameter derivatives
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["fp64", "fp32", "df64"])
def test_emulated_mass_matrix_and_parameter_derivatives(prec):
    P = ale.DropletProblem(N=4, contact_angle_deg=75.0, jacobian_precision=prec)
    fk = P.lower()
    D = A.droplet(4)
    p = _params(75.0)
    v, h0, h1 = _state(D, 2)
    outs, status = KE.run_fused(fk, P.conns, v, [h0, h1], D.x0, _pvec(P, p), flag=2)
    assert not status.any()
    tol = 1e-6 if prec == "fp32" else 1e-12
    for (_, Me), Mo in zip(outs, A.element_mass(D, v, [h0, h1], p)):
        assert np.max(np.abs(Me.astype(np.float64) - Mo)) <= tol * max(1.0, np.max(np.abs(Mo)))
    for name in ("dynamic_viscosity", "surface_tension", "contact_angle"):
        outs, _ = KE.run_fused(fk, P.conns, v, [h0, h1], D.x0, _pvec(P, p), flag=3,
                               aux=P.param_names.index(name))
        for (Re, Je), Ro in zip(outs, A.element_dparam(D, v, [h0, h1], p, name)):
            assert np.max(np.abs(Re - Ro)) <= 1e-12 * max(1.0, np.max(np.abs(Ro)))
            assert not Je.any()


@pytest.mark.gpu
def test_gpu_mass_matrix_and_parameter_derivatives_match_oracle():
    P = _gpu_problem(5, 65.0)
    D = A.droplet(5)
    p = _params(65.0)
    P.set_params(**{k: p[k] for k in ("__bdf0", "__bdf1", "__bdf2")})
    v, h0, h1 = _state(D, 9)
    P.set_state(v, [h0, h1])
    M = P.get_mass_matrix()
    _, Mo = A.assemble_blocks(D, [None] * 3, A.element_mass(D, v, [h0, h1], p))
    assert np.max(np.abs(M.data - Mo)) <= 1e-12 * np.max(np.abs(Mo))
    for name in ("dynamic_viscosity", "surface_tension", "contact_angle"):
        dR = P.get_parameter_derivative(name)
        Ro, _ = A.assemble_blocks(D, A.element_dparam(D, v, [h0, h1], p, name), [None] * 3)
        assert np.max(np.abs(dR - Ro)) <= 1e-12 * np.max(np.abs(Ro))
    # the Jacobian path is unaffected afterwards
    R, J = P.get_jacobian()
    Ro, orp, oci, ov = A.assemble(D, v, [h0, h1], p)
    assert np.max(np.abs(J.data - ov)) <= 1e-12 * np.max(np.abs(ov))


@pytest.mark.gpu
def test_gpu_persistent_fused_launch_gives_identical_results():
    P = _gpu_problem(9, 100.0)
    D = A.droplet(9)
    v, h0, h1 = _state(D, 13)
    P.set_params(__bdf0=1500.0, __bdf1=-2000.0, __bdf2=500.0)
    P.set_state(v, [h0, h1])
    R1, J1 = P.get_jacobian()
    P.set_persistent(True)
    R2, J2 = P.get_jacobian()
    P.set_persistent(False)
    assert np.array_equal(R1, R2) and np.array_equal(J1.data, J2.data)
