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


class _Param:
    def __init__(self, v):
        self.value = v


class _HostProblem:
    """Stands for a pyoomph Problem: current dofs and named global parameters."""

    def __init__(self, x, params):
        self.x = x
        self.params = {k: _Param(v) for k, v in params.items()}

    def get_current_dofs(self):
        return self.x, None

    def get_global_parameter_names(self):
        return list(self.params)

    def get_global_parameter(self, name):
        return self.params[name]


def test_assembler_copies_changed_host_parameters_into_the_engine():
    """Host logic of the drop-in assembler: parameters the weak form reads
    follow the host problem (arclength continuation changes them between
    solves); others are ignored; nothing is uploaded when nothing changed;
    a Jacobian derived by a parameter is refused as pyoomph refuses it."""
    from pyoomph_gb300 import GB300Assembler

    class Engine:
        param_names = ["dynamic_viscosity", "mass_density"]
        params = np.array([0.01, 1.0])
        n_dof = 3
        uploads = []

        def initialise(self):
            pass

        def set_parameters(self, **kw):
            self.uploads.append(dict(kw))
            for k, v in kw.items():
                self.params[self.param_names.index(k)] = v

        def set_dofs(self, x):
            self.x = x

        def get_parameter_derivative(self, name):
            return np.full(self.n_dof, float(self.param_names.index(name)))

    eng = Engine()
    asm = GB300Assembler(eng)
    host = _HostProblem(np.zeros(3), {"dynamic_viscosity": 0.01, "mass_density": 1.0, "unrelated": 7.0})
    asm._set_problem(host)
    assert np.array_equal(asm.get_residuals_and_jacobian(False, "mass_density"), np.ones(3))
    assert eng.uploads == []
    host.params["dynamic_viscosity"].value = 0.02
    asm.get_residuals_and_jacobian(False, "dynamic_viscosity")
    assert eng.uploads == [{"dynamic_viscosity": 0.02}] and eng.params[0] == 0.02
    with pytest.raises(RuntimeError):
        asm.get_residuals_and_jacobian(True, "dynamic_viscosity")


@pytest.mark.gpu
def test_gpu_assembler_parameter_derivative_and_sync():
    """Through pyoomph's CustomAssemblyBase contract: dR/dp from
    get_residuals_and_jacobian(False, name) equals the engine's, and a
    parameter changed on the host reaches the next residual."""
    from pyoomph_gb300 import GB300Assembler, workloads as W
    eng = W.navier_stokes_problem(N=6, Re=50.0)
    asm = GB300Assembler(eng)
    asm.initialize()
    x = np.random.default_rng(2).normal(0.0, 0.3, eng.n_dof)
    host = _HostProblem(x, {"dynamic_viscosity": 0.02, "mass_density": 1.0})
    asm._set_problem(host)
    R1 = asm.get_residuals_and_jacobian(False)
    D = asm.get_residuals_and_jacobian(False, "dynamic_viscosity")
    assert D.dtype == np.float64 and D.shape == (eng.n_dof,)
    host.params["dynamic_viscosity"].value = 0.03
    R2 = asm.get_residuals_and_jacobian(False)
    # R is linear in the viscosity
    assert np.max(np.abs(R2 - R1 - 0.01 * D)) <= 1e-12 * max(1.0, np.max(np.abs(R1)))


def test_assembler_custom_solve_routine_host_logic():
    """pyoomph's hook for the Newton linear solve: off by default (pyoomph
    keeps its own solver); with device_linear_solve the engine's device
    solve answers, and its refusal propagates instead of a silent
    fallback."""
    from pyoomph_gb300 import GB300Assembler
    from pyoomph_gb300.linsolve import LinearSolverError

    class Engine:
        refuse = False

        def solve_linear_device(self, b):
            if self.refuse:
                raise LinearSolverError("zero diagonal")
            return 2.0 * b

    eng = Engine()
    assert not GB300Assembler(eng).has_custom_solve_routine()
    asm = GB300Assembler(eng, device_linear_solve=True)
    assert asm.has_custom_solve_routine()
    never = lambda b: (_ for _ in ()).throw(AssertionError("host solve called"))
    assert np.array_equal(asm.custom_solve_routine(never, np.arange(3.0)), 2.0 * np.arange(3.0))
    eng.refuse = True
    with pytest.raises(LinearSolverError):
        asm.custom_solve_routine(never, np.arange(3.0))
