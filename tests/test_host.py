"""Host-side checks (no GPU): the C-ABI library loads and exports every
symbol include/fe_gb300.h declares, generated kernels compile with nvrtc for
sm_103a, the product's mesh generator and reference tables match the oracle
and the reference's oomph-lib tables, and the generated pointwise
derivatives match finite differences of the weak form."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def _header_symbols():
    src = open(os.path.join(ROOT, "include", "fe_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fe_[a-z_0-9]+)\s*\(", src)))


def test_library_loads_and_exports_header_symbols():
    from pyoomph_gb300 import _native as N
    L = N.load()
    syms = _header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(N.EXPORTS) == syms
    assert b"sm_103a" in L.fe_version()


def test_device_calls_fail_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from pyoomph_gb300 import _native as N
    L = N.load()
    n = ctypes.c_int()
    rc = L.fe_device_info(ctypes.byref(n), None, None, None, None)
    assert rc == N.FE_ERR_NOGPU
    assert L.fe_last_error()


def test_null_arguments_are_rejected():
    from pyoomph_gb300 import _native as N
    L = N.load()
    assert L.fe_problem_create(None, None) == N.FE_ERR_ARG
    assert L.fe_problem_sizes(None, None, None) == N.FE_ERR_ARG
    assert L.fe_assemble(None, None, None, None, 3, None) == N.FE_ERR_ARG
    assert L.fe_problem_set_pipeline_streams(None, 1) == N.FE_ERR_ARG
    assert L.fe_problem_pipeline_times(None, None, 0) == N.FE_ERR_ARG


def test_krylov_solver_arguments_are_checked_before_any_device_call():
    """fe_krylov_* reject bad arguments with FE_ERR_ARG (no GPU needed):
    null handles and buffers, an empty matrix, rows that do not split into
    the blocks, an unknown value precision, a check interval out of range."""
    from pyoomph_gb300 import _native as N
    L = N.load()
    out = ctypes.c_void_p()
    fake = ctypes.c_void_p(16)   # never dereferenced: the checks fail first
    assert L.fe_krylov_create(None, None, None, N.FE_JAC_F64, 10, 10, 1, 8, 1, ctypes.byref(out)) == N.FE_ERR_ARG
    assert L.fe_krylov_create(fake, fake, fake, N.FE_JAC_F64, 0, 10, 1, 8, 1, ctypes.byref(out)) == N.FE_ERR_ARG
    assert L.fe_krylov_create(fake, fake, fake, N.FE_JAC_F64, 10, 10, 3, 8, 1, ctypes.byref(out)) == N.FE_ERR_ARG
    assert "equal blocks" in L.fe_last_error().decode()
    assert L.fe_krylov_create(fake, fake, fake, 7, 10, 10, 1, 8, 1, ctypes.byref(out)) == N.FE_ERR_ARG
    assert L.fe_krylov_create(fake, fake, fake, N.FE_JAC_F64, 10, 10, 1, 0, 1, ctypes.byref(out)) == N.FE_ERR_ARG
    assert L.fe_krylov_create(fake, fake, fake, N.FE_JAC_F64, 10, 10, 1, 8, 1, None) == N.FE_ERR_ARG
    assert L.fe_krylov_solve(None, None, None, 1e-12, 0.0, 10, 1, None, None, None) == N.FE_ERR_ARG
    assert L.fe_krylov_matvec(None, None, None, None) == N.FE_ERR_ARG
    assert L.fe_krylov_info(None, None, None, None) == N.FE_ERR_ARG
    L.fe_krylov_destroy(None)
    assert L.fe_csr_spmv(None, None, None, N.FE_JAC_F64, None, None, 10, 10, None) == N.FE_ERR_ARG


@pytest.mark.parametrize("kind", ["poisson", "poisson_p2", "ns", "ns32", "nsdf", "hex", "hex32", "hexdf",
                                  "ns_t", "ns32_t", "hexdf_t", "ns32_rdf", "nsdf_rdf", "hex32_rdf", "hexdf_rdf",
                                  "poisson32_rdf"])
def test_generated_kernels_compile_for_sm103a(kind, tmp_path):
    from pyoomph_gb300 import _native as N
    from pyoomph_gb300 import workloads as W
    P = {"poisson": lambda: W.poisson_problem(N=4), "poisson_p2": lambda: W.poisson_problem(N=4, split="left"),
         "ns": lambda: W.navier_stokes_problem(N=4), "ns32": lambda: W.navier_stokes_problem(N=4, jacobian_precision="fp32"),
         "hex": lambda: W.nonlinear_diffusion_problem(N=2),
         "hex32": lambda: W.nonlinear_diffusion_problem(N=2, jacobian_precision="fp32"),
         "nsdf": lambda: W.navier_stokes_problem(N=4, jacobian_precision="df64"),
         "hexdf": lambda: W.nonlinear_diffusion_problem(N=2, jacobian_precision="df64"),
         "ns_t": lambda: W.navier_stokes_problem(N=4, transient=True),
         "ns32_t": lambda: W.navier_stokes_problem(N=4, jacobian_precision="fp32", transient=True),
         "hexdf_t": lambda: W.nonlinear_diffusion_problem(N=2, jacobian_precision="df64", transient=True),
         "ns32_rdf": lambda: W.navier_stokes_problem(N=4, jacobian_precision="fp32"),
         "nsdf_rdf": lambda: W.navier_stokes_problem(N=4, jacobian_precision="df64"),
         "hex32_rdf": lambda: W.nonlinear_diffusion_problem(N=2, jacobian_precision="fp32"),
         "hexdf_rdf": lambda: W.nonlinear_diffusion_problem(N=2, jacobian_precision="df64"),
         "poisson32_rdf": lambda: W.poisson_problem(N=4, jacobian_precision="fp32")}[kind]()
    if kind.endswith("_rdf"):
        P.residual_precision = "df64"
    ks = P.lower()
    assert ks.smem_bytes <= 227 * 1024 and ks.threads % 32 == 0 and ks.threads <= 1024
    assert N.code_build(ks.source, ks.name, str(tmp_path)) > 0


@pytest.mark.parametrize("case", [("Q2_QUAD", 0, (7, 5, 0), False), ("P2_TRI", 1, (6, 4, 0), "left"),
                                  ("P2_TRI", 1, (3, 5, 0), "right"), ("Q2_HEX", 2, (3, 4, 2), None)])
def test_mesh_order_matches_oracle(case):
    from pyoomph_gb300.meshes import CuboidBrickMesh, RectangularQuadMesh
    name, et, (nx, ny, nz), split = case
    m = O.mesh(et, nx, ny, nz, split=0 if split in (False, None, "left") else 1)
    g = (CuboidBrickMesh(N=[nx, ny, nz]) if et == O.Q2_HEX else
         RectangularQuadMesh(N=[nx, ny], split_in_tris=split)).generate()
    assert np.array_equal(g.conn, m.conn)
    assert np.array_equal(g.x, m.x)
    assert np.array_equal(g.is_vertex, m.is_vertex.astype(bool))
    bm = np.zeros(g.n_nodes, dtype=np.uint32)
    for i, nm in enumerate(["left", "right", "bottom", "top", "back", "front"]):
        if nm in g.boundaries:
            bm |= g.boundaries[nm].astype(np.uint32) << i
    assert np.array_equal(bm, m.bmask)


def test_reference_tables_match_oomph():
    from pyoomph_gb300.spaces import ELEMENT_TYPES
    T = np.load(os.path.join(GOLD, "oomph_tables.npz"))
    for et, name in ((O.Q2_QUAD, "Q2_QUAD"), (O.P2_TRI, "P2_TRI"), (O.Q2_HEX, "Q2_HEX")):
        e = ELEMENT_TYPES[name]
        t = e.tables()
        assert np.array_equal(e.knots, T[f"{et}_s"])
        assert np.array_equal(t["W"], T[f"{et}_w"])
        assert np.array_equal(t["PSI2"], T[f"{et}_psi"])
        assert np.array_equal(t["DPS2"], T[f"{et}_dpsi"])


def test_pointwise_derivatives_match_finite_differences():
    """D = dr/du from the code generator against central differences of r."""
    import sympy as sp
    from pyoomph_gb300 import expressions as E
    from pyoomph_gb300.codegen import differentiate, time_derivative_symbols
    from pyoomph_gb300.equations import NavierStokesEquations
    E.set_dimension(2)
    eq = NavierStokesEquations(mass_density=1.3, dynamic_viscosity=0.07)
    eq._fields, eq._residual = [], 0
    eq.define_fields()
    eq.define_residuals()
    fields = sorted(eq._fields, key=lambda f: {"C2": 0, "C1": 1}[f[1]])
    params = sorted(eq.parameter_values())
    # the steady form (partial_t terms vanish)
    steady = eq._residual.subs({s_: 0 for s_ in time_derivative_symbols(fields)})
    pw = differentiate(fields, 2, steady, params)
    usyms = []
    for name, _ in fields:
        usyms += [E.REG.value[name]] + list(E.REG.grad[name][:2])
    rng = np.random.default_rng(0)
    vals = dict(zip(usyms, rng.normal(size=len(usyms))))
    vals.update({E.parameter(p): eq.parameter_values()[p] for p in params})
    r = [sp.lambdify(list(vals), e) for e in pw.r_exprs]
    base = list(vals.values())
    for tc, ic, d in pw.d_entries:
        h = 1e-6
        xp = list(base); xp[ic] += h
        xm = list(base); xm[ic] -= h
        fd = (r[tc](*xp) - r[tc](*xm)) / (2 * h)
        exact = float(d.subs(vals))
        assert abs(fd - exact) <= 1e-6 * max(1.0, abs(exact))
    # Taylor-Hood: 2 velocity comps x 3 + pressure x 3 test components
    assert pw.ntc == 9 and len(pw.d_entries) > 0


def _product_for_golden(g):
    from pyoomph_gb300 import workloads as W
    et, eq = int(g["etype"]), int(g["eq"])
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    if eq == O.EQ_NAVIER_STOKES_TH:
        return W.navier_stokes_problem(N=[nx, ny], Re=1.0 / float(g["params"][1]),
                                       split="left" if int(g["split"]) == 0 else "right")
    dim = 3 if et == O.Q2_HEX else 2
    gauss = g["params"][1:].reshape(int(g["params"][0]), dim + 2)
    if eq == O.EQ_POISSON:
        return W.poisson_problem(N=[nx, ny], gaussians=gauss, split=None if et == O.Q2_QUAD else "left")
    return W.nonlinear_diffusion_problem(N=[nx, ny, nz] if dim == 3 else [nx, ny], gaussians=gauss, dim=dim)


GOLD_CASES = [c for c in sorted(__import__("glob").glob(os.path.join(GOLD, "*_*.npz")))
              if not c.endswith("oomph_tables.npz")]


@pytest.mark.parametrize("path", GOLD_CASES, ids=[os.path.basename(c)[:-4] for c in GOLD_CASES])
def test_host_pattern_and_numbering_bit_exact_vs_reference(path):
    """The engine's CSR pattern (built by the C-ABI on the host) and equation
    numbering against the reference's own oomph-lib (structural pattern)."""
    g = np.load(path)
    P = _product_for_golden(g)
    P.lower()
    assert np.array_equal(P.eqn, g["eqn"])
    assert np.array_equal(P._values0[P.pinned], g["values"][P.pinned])
    rp, ci = P.host_pattern()
    assert np.array_equal(rp, g["rowptr_st"])
    assert np.array_equal(ci, g["colidx_st"])


@pytest.mark.parametrize("kind", ["ns", "hex"])
def test_host_pattern_vs_oracle_larger(kind):
    from pyoomph_gb300 import workloads as W
    if kind == "ns":
        P = W.navier_stokes_problem(N=[13, 11])
        OP = O.navier_stokes_problem(O.mesh(O.P2_TRI, 13, 11))
    else:
        P = W.nonlinear_diffusion_problem(N=[4, 3, 5])
        OP = O.poisson_problem(O.mesh(O.Q2_HEX, 4, 3, 5), np.array([[0.5, 0.5, 0.5, 0.1, 1.0]]),
                               eq=O.EQ_NONLINEAR_DIFFUSION)
    rp, ci = P.host_pattern()
    assert np.array_equal(P.eqn, OP.eqn)
    R, rp0, ci0, v0 = O.assemble(OP, True, -1.0)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0)


@pytest.mark.parametrize("jref", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("geometry", ["affine", "general"])
@pytest.mark.parametrize("kind", ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex", "nldiff_q2"])
def test_generated_kernel_emulated_on_cpu_matches_oracle_elements(kind, geometry, prec, jref):
    """Every generated kernel variant (Jacobian contracted in physical or in
    reference coordinates), run on the CPU by the sequential emulator,
    reproduces the oracle's element residuals and matrices."""
    import element_cases as C
    import kernel_emulator as KE
    P, ks, values, Rr, Jr = C.build(kind, geometry, prec, jref=jref)
    assert P.affine == (geometry == "affine")
    rb, jb, st = KE.run(ks, P.mesh.x, P.mesh.conn, values, P.params)
    assert st[0] == 0
    assert C.relmax(rb, Rr) <= 1e-12
    assert C.relmax(jb, Jr) <= (1e-12 if prec == "fp64" else 1e-5)


@pytest.mark.parametrize("geometry", ["affine", "general"])
@pytest.mark.parametrize("kind", ["poisson_q2", "poisson_p2", "ns_th", "nldiff_hex", "nldiff_q2"])
def test_df64_jacobian_emulated_on_cpu_matches_oracle_elements(kind, geometry):
    """The double-float Jacobian (FP64 D, contraction in pairs of FP32 on the
    FP32 pipes, FP64 storage) reproduces the oracle's element matrices
    within the FP64 contract; its error sits near 2^-48, far below the
    FP32 Jacobian's."""
    import element_cases as C
    import kernel_emulator as KE
    P, ks, values, Rr, Jr = C.build(kind, geometry, "df64")
    assert ks.jac_precision == "df64" and "fe_df64" in ks.source
    rb, jb, st = KE.run(ks, P.mesh.x, P.mesh.conn, values, P.params)
    assert st[0] == 0
    assert C.relmax(rb, Rr) <= 1e-12
    err = C.relmax(jb, Jr)
    print(kind, geometry, "df64 J rel err", err)
    assert err <= 1e-12


@pytest.mark.parametrize("kind", ["ns_th", "poisson_q2", "poisson_p2", "nldiff_hex", "nldiff_q2"])
@pytest.mark.parametrize("jac", ["fp32", "df64"])
@pytest.mark.parametrize("geometry", ["affine", "general"])
def test_df64_residual_emulated_on_cpu_matches_oracle_elements(geometry, jac, kind):
    """The double-float residual path (values staged as differences from
    node 0 in FP64, interpolation -- sum-factorised for the Q2 hex --,
    pointwise residual with the Gaussian source evaluated in FP64, pull-back
    and test-function contraction in pairs of FP32) reproduces the oracle's
    element residuals within the FP64 contract."""
    import element_cases as C
    import kernel_emulator as KE
    P, ks, values, Rr, Jr = C.build(kind, geometry, jac, residual="df64")
    assert "_rdf" in ks.name and "fe_df64 U[FE_NTC]" in ks.source
    rb, jb, st = KE.run(ks, P.mesh.x, P.mesh.conn, values, P.params)
    assert st[0] == 0
    err = C.relmax(rb, Rr)
    print(kind, geometry, jac, "df64 residual rel err", err)
    assert err <= 1e-13
    assert C.relmax(jb, Jr) <= (1e-12 if jac == "df64" else 1e-5)


def test_df64_residual_is_refused_where_it_does_not_apply():
    """FP64 Jacobians, transient forms and pointwise terms with libm calls
    other than the Gaussian source keep the FP64 residual: asking for
    double-float is an error, not a silent fallback."""
    import types
    import sympy as sp
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.codegen import df64_residual_supported
    for make in (lambda: W.navier_stokes_problem(N=4),
                 lambda: W.navier_stokes_problem(N=4, jacobian_precision="fp32", transient=True)):
        P = make()
        P.residual_precision = "df64"
        with pytest.raises(ValueError):
            P.lower()
    x = sp.Symbol("x")
    assert not df64_residual_supported(types.SimpleNamespace(r_exprs=[sp.exp(x)], d_entries=[]))
    assert not df64_residual_supported(types.SimpleNamespace(r_exprs=[sp.sqrt(x)], d_entries=[]))
    assert df64_residual_supported(types.SimpleNamespace(r_exprs=[x ** 2 / (1 + x)], d_entries=[(0, 0, 2 * x)]))


def test_launch_shapes_balance_the_waves():
    """Elements per block follow EPB' = ceil(E / (SMs x W)), W the waves of
    the generator's shape on 152 SMs: a small mesh fills one wave (Poisson
    Q2 64^2: 4,096 elements -> 27 per block = 152 blocks), a large one keeps
    its shape, replicated problems (serving classes of many sizes) keep the
    generator's shape so that they share one kernel."""
    from pyoomph_gb300 import problem as PR
    from pyoomph_gb300 import workloads as W
    PR._SMS = 152
    ks = W.poisson_problem(N=64).lower()
    assert ks.epb == 27 and -(-4096 // ks.epb) == 152
    assert W.navier_stokes_problem(N=256).lower().epb == 32
    P = W.poisson_problem(N=16)
    P.replicas = 4
    assert P.lower().epb == 32            # the generator's shape for the Poisson Q2 kernel
    P = W.poisson_problem(N=64)
    P.elems_per_block = 32                # an explicit shape is kept
    assert P.lower().epb == 32


def test_assembler_refuses_a_differently_numbered_host_problem():
    """GB300Assembler.check_numbering against a host problem that exposes
    pyoomph's ndof() and get_mesh(name).nodes() with Node.eqn_number: equal
    numbering passes; another dof count or a swapped pair of equations is an
    error (the CSR would otherwise belong to a different system)."""
    from pyoomph_gb300 import GB300Assembler, workloads as W
    eng = W.navier_stokes_problem(N=3)
    eng.lower()
    eqn = np.asarray(eng.eqn).reshape(eng.mesh.n_nodes, 3).copy()

    class Node:
        def __init__(self, row):
            self.row = row

        def nvalue(self):
            return 3 if self.row[2] != -2 else 2

        def eqn_number(self, vi):
            return int(self.row[vi])

    class Mesh:
        def __init__(self, table):
            self.table = table

        def nodes(self):
            return [Node(r) for r in self.table]

    class Host:
        def __init__(self, table, ndof):
            self.table, self.n = table, ndof

        def ndof(self):
            return self.n

        def get_mesh(self, name):
            return Mesh(self.table)

    asm = GB300Assembler(eng)
    asm._set_problem(Host(eqn, eng.n_dof))
    asm.check_numbering()
    assert asm._numbering_checked
    asm._set_problem(Host(eqn, eng.n_dof + 1))
    with pytest.raises(RuntimeError):
        asm.check_numbering()
    swapped = eqn.copy()
    a, b = np.argwhere(swapped >= 0)[:2]
    swapped[tuple(a)], swapped[tuple(b)] = swapped[tuple(b)], swapped[tuple(a)]
    asm._set_problem(Host(swapped, eng.n_dof))
    with pytest.raises(RuntimeError, match="numbering differs"):
        asm.check_numbering()


def test_thread_layout_rule():
    """Threads per block: max(knots, ceil(rows/2)) per element in whole
    warps.  The Taylor-Hood element (15 rows, 7 knots) runs 8 per element;
    elements with no more rows than knots keep one thread per row; an
    explicit count overrides, and only a changed count renames a kernel."""
    from pyoomph_gb300 import workloads as W
    from pyoomph_gb300.codegen import _threads_for
    assert _threads_for(32, 7, 15) == 256 and _threads_for(24, 7, 15) == 192
    assert _threads_for(27, 9, 9) == 256 and _threads_for(13, 27, 27) == 352
    P = W.navier_stokes_problem(N=256)
    ks = P.lower()
    assert (ks.epb, ks.threads) == (32, 256)
    P = W.poisson_problem(N=64)
    ks = P.lower()
    assert ks.threads == ((ks.epb * 9 + 31) // 32) * 32
    P = W.navier_stokes_problem(N=256, jacobian_precision="fp32")
    P.threads_per_block = 480
    ks480 = P.lower()
    assert ks480.threads == 480 and "#define FE_NT 480" in ks480.source
    P2 = W.navier_stokes_problem(N=256, jacobian_precision="fp32")
    assert P2.lower().name != ks480.name


def test_fused_rows_per_thread_shapes():
    """The fused moving-mesh kernel: threads per element max(knots, rows /
    rows_per_thread); the bulk P2 element (27 rows, 7 knots) at 4 rows per
    thread runs 7 threads per element; one row per thread keeps 27."""
    from pyoomph_gb300.ale import DropletProblem
    D = DropletProblem(N=20, jacobian_precision="fp64")
    assert D.rows_per_thread == 4
    bulk = D.lower().domains[0]
    assert bulk.rows_needed == bulk.epb * 7
    D1 = DropletProblem(N=20, jacobian_precision="fp64")
    D1.rows_per_thread = 1
    bulk1 = D1.lower().domains[0]
    assert bulk1.rows_needed == bulk1.epb * 27
    assert DropletProblem(N=20, jacobian_precision="fp32").rows_per_thread == 2


def test_df64_printer_splits_literals_exactly_and_refuses_libm():
    """Double-float literals are the binary64 value split into its binary32
    pair at generation time (hi + lo recovers the double to 48 bits);
    exp, non-integer powers and Gaussian sums are refused."""
    import re
    import numpy as np
    import sympy as sp
    from pyoomph_gb300.codegen import _DF64Printer
    pr = _DF64Printer({})
    for v in (2.0, 0.1, 1.0 / 3.0, -1.0e-5, 123456.789):
        m = re.fullmatch(r"fe_df64\((\S+)f, (\S+)f\)", pr._lit(v))
        hi, lo = float(m.group(1)), float(m.group(2))
        assert np.float32(hi) == hi and np.float32(lo) == lo
        assert abs((hi + lo) - v) <= abs(v) * 2.0 ** -47
    x = sp.Symbol("x")
    assert "fe_df64(1.0f, 0.0f)" in pr.doprint(1 / x)
    for bad in (sp.exp(x), x ** sp.Rational(1, 3)):
        with pytest.raises(NotImplementedError):
            pr.doprint(bad)
