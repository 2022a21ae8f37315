"""Parameter derivatives dR/dp of the fixed-mesh kernels (pyoomph's
dResidual{i}dParameter_{k}, codegen.cpp:4743-4760, used by arclength
continuation and bifurcation tracking).  The generated kernel differentiates
the weak form's pointwise flux by the parameter symbolically (through the
Gaussian source terms by the chain rule); the reference here is a central
difference of the residual in that parameter: exact up to rounding where R
is linear in p (viscosity, density, amplitude), within the truncation error
of the difference for the Gaussian centres and widths."""
import numpy as np
import pytest

import element_cases as C


def _fd(run, params, j, h):
    pp, pm = params.copy(), params.copy()
    pp[j] += h
    pm[j] -= h
    return (run(pp) - run(pm)) / (2.0 * h)


@pytest.mark.parametrize("geometry", ["affine", "general"])
@pytest.mark.parametrize("kind,prec", [(k, "fp64") for k in C.KINDS] + [("ns_th", "df64"), ("poisson_q2", "fp32")])
def test_emulated_dparam_matches_central_differences(kind, geometry, prec):
    import kernel_emulator as KE
    P, ks, values, _, _ = C.build(kind, geometry, prec)
    m = P.mesh

    def residual(params):
        rb, _, st = KE.run(ks, m.x, m.conn, values, params, flag=0)
        assert not st.any()
        return rb

    R0 = residual(P.params)
    rscale = max(np.max(np.abs(R0)), 1e-300)
    for j, name in enumerate(P.param_names):
        D, _, st = KE.run(ks, m.x, m.conn, values, P.params, flag=3, aux=j)
        assert not st.any()
        h = 1e-5 * max(1.0, abs(P.params[j]))
        fd = _fd(residual, P.params, j, h)
        err = np.max(np.abs(D - fd))
        # rounding of the difference ~ eps |R| / h, truncation ~ h^2 |R'''|
        assert err <= 1e-7 * max(np.max(np.abs(fd)), 1e-3 * rscale), (name, err, np.max(np.abs(fd)))
    # the residual path afterwards is the plain residual
    assert np.array_equal(residual(P.params), R0)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ns", "poisson", "hex"])
def test_gpu_parameter_derivative_matches_central_differences(kind):
    from pyoomph_gb300 import workloads as W
    make = {"ns": lambda: W.navier_stokes_problem(N=8, Re=50.0),
            "poisson": lambda: W.poisson_problem(N=8, seed=2),
            "hex": lambda: W.nonlinear_diffusion_problem(N=4, seed=2)}
    P = make[kind]()
    P.initialise()
    rng = np.random.default_rng(5)
    x = rng.normal(0.0, 0.3, P.n_dof)
    P.set_dofs(x)
    R0 = P.get_residuals()
    p0 = P.params[:len(P.param_names)].copy()
    rscale = max(np.max(np.abs(R0)), 1e-300)
    names = P.param_names if kind == "ns" else P.param_names[:8]
    for j, name in enumerate(names):
        D = P.get_parameter_derivative(name)
        h = 1e-5 * max(1.0, abs(p0[j]))

        def res(p):
            P.set_parameter_vector(p)
            P.set_dofs(x)
            return P.get_residuals()

        fd = _fd(res, p0, j, h)
        P.set_parameter_vector(p0)
        P.set_dofs(x)
        assert np.max(np.abs(D - fd)) <= 1e-7 * max(np.max(np.abs(fd)), 1e-3 * rscale), name
    assert np.array_equal(P.get_residuals(), R0)
    with pytest.raises(KeyError):
        P.get_parameter_derivative("no_such_parameter")
