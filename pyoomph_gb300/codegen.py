"""CUDA code generator: lowers a weak form to a fused element kernel.

The reference's ``FiniteElementCode::write_code`` (``src/codegen.cpp:4684``,
``write_generic_RJM`` :3912-4110) emits, per domain, a C function that loops
over integration points, asks the host for the shape buffer
(``fill_shape_buffer_for_point``), interpolates the fields, and adds
``R[l_test] += ...`` and ``J[l_test][l_shape] += ...``.

Here the same weak form is split into

* a *pointwise* function of the field values and gradients at one
  integration point that returns the test-component coefficients ``r`` and
  their derivatives ``D = dr/d(field components)`` (sympy differentiates and
  eliminates common subexpressions, the job GiNaC does in the reference),
* a fixed kernel skeleton that stages reference tables and nodal data in
  shared memory, computes the metric-tensor geometry of
  ``fill_shape_info_at_s`` (``elements.cpp:3593-3990``) per (element,
  integration point) thread, and contracts ``J_e = sum_q B^T D B`` per
  (element, row) thread.

The residual is accumulated in FP64 with the coefficients pulled back to
reference coordinates (``rhat_b = w sum_i g^{bi} r_i``), so it never needs
per-element physical shape gradients; the Jacobian uses physical gradients
and ``D`` in FP64 or FP32 (``jac_precision``).
"""
from __future__ import annotations

import hashlib
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import sympy as sp
from sympy.printing.c import C99CodePrinter

from . import expressions as E
from .spaces import ElementType, Layout, make_layout


class _Printer(C99CodePrinter):
    """C printer: small integer powers as products, libm calls; with
    ``fp32`` every literal and call is single precision."""

    def __init__(self, names: Dict[sp.Symbol, str], fp32: bool = False):
        super().__init__()
        self._names = names
        self._fp32 = fp32

    def _lit(self, v: float) -> str:
        return f"{v!r}f" if self._fp32 else repr(v)

    def _fn(self, name: str) -> str:
        return name + "f" if self._fp32 else name

    def _print_Symbol(self, s):
        if s in self._names:
            return self._names[s]
        return super()._print_Symbol(s)

    def _print_Pow(self, e):
        b, x = e.args
        one = self._lit(1.0)
        if x.is_Integer:
            n = int(x)
            if n == 2:
                bs = self._print(b)
                return f"(({bs})*({bs}))"
            if n == -1:
                return f"({one}/({self._print(b)}))"
            if n == -2:
                bs = self._print(b)
                return f"({one}/(({bs})*({bs})))"
            if 2 < n <= 4:
                bs = self._print(b)
                return "(" + "*".join([f"({bs})"] * n) + ")"
        if x == sp.Rational(1, 2):
            return f"{self._fn('sqrt')}({self._print(b)})"
        return f"{self._fn('pow')}({self._print(b)}, {self._print(x)})"

    def _print_GaussianSum(self, e):
        k0 = next(i for i, a in enumerate(e.args) if a.is_Integer)
        n, dim = int(e.args[k0]), int(e.args[k0 + 1])
        refs = [self._names.get(a, "") for a in e.args[k0 + 2:]]
        idx = [int(r[r.index("[") + 1:-1]) if r.endswith("]") else -1 for r in refs]
        if self._fp32 or len(idx) != n * (dim + 2) or idx != list(range(idx[0], idx[0] + len(idx))):
            raise NotImplementedError("GaussianSum needs its parameters contiguous in the FP64 array")
        base = refs[0][:refs[0].index("[")]
        xq = self._names[E.X[0]][:self._names[E.X[0]].index("[")]
        return f"FE_GAUSS({dim}, {xq}, {base} + {idx[0]}, {n})"

    def _print_exp(self, e):
        return f"{self._fn('exp')}({self._print(e.args[0])})"

    def _print_Rational(self, e):
        return f"({self._lit(float(e.p))}/{self._lit(float(e.q))})"

    def _print_Float(self, e):
        return self._lit(float(e))

    def _print_Integer(self, e):
        return self._lit(float(int(e)))

    def _print_Pi(self, e):
        return self._lit(3.141592653589793)


class _DF64Printer(_Printer):
    """C printer for double-float (``fe_df64``) arithmetic: every literal is
    split into its binary32 pair at generation time (the binary64 value of
    the FP64 code, to 48 bits), operations are + - * / and small integer
    powers.  A Gaussian source term is evaluated in FP64 (the device helper
    of the FP64 code, under the FP64 names of the coordinates and
    parameters) and converted once.  Anything else (libm calls) is refused:
    see ``df64_residual_supported``."""

    def __init__(self, names: Dict[sp.Symbol, str], fp64_names: Optional[Dict[sp.Symbol, str]] = None):
        super().__init__(names)
        self._fp64_names = fp64_names

    def _lit(self, v: float) -> str:
        hi = float(np.float32(v))
        lo = float(np.float32(v - hi))
        return f"fe_df64({hi!r}f, {lo!r}f)"

    def _print_Rational(self, e):
        return self._lit(float(e.p) / float(e.q))

    def _print_Pow(self, e):
        x = e.args[1]
        if x.is_Integer and int(x) in (2, 3, 4, -1, -2):
            return super()._print_Pow(e)
        raise NotImplementedError(f"no double-float form of {e}")

    def _print_exp(self, e):
        raise NotImplementedError("no double-float exp")

    def _print_GaussianSum(self, e):
        if self._fp64_names is None:
            raise NotImplementedError("a double-float Gaussian sum needs the FP64 names")
        return f"fe_df64({_Printer(self._fp64_names)._print_GaussianSum(e)})"

    def _print_Function(self, e):
        raise NotImplementedError(f"no double-float {e.func}")


def df64_residual_supported(pw: "Pointwise") -> bool:
    """Whether the pointwise residual and derivatives are rational in the
    fields, coordinates and parameters (+ - * / and integer powers between
    -2 and 4), Gaussian source terms aside (evaluated in FP64): the forms a
    double-float residual can be generated for."""
    ok = (sp.Add, sp.Mul, sp.Symbol, sp.Number, sp.Pow)
    for e in list(pw.r_exprs) + [d for (_, _, d) in pw.d_entries]:
        it = sp.preorder_traversal(sp.sympify(e))
        for s in it:
            if isinstance(s, E.GaussianSum):
                it.skip()          # evaluated in FP64, converted once
                continue
            if not isinstance(s, ok):
                return False
            if isinstance(s, sp.Pow) and not (s.args[1].is_Integer and int(s.args[1]) in (2, 3, 4, -1, -2)):
                return False
    return True


# the BDF weights of the current step (time derivative at a node:
# du/dt = w0 u + w1 u_{n-1} + w2 u_{n-2}), appended to the parameter array
# of a transient problem (the timestepper weights of pyoomph's shape buffer,
# elements.cpp:4577-4656)
BDF_PARAMS = ("_bdf_w0", "_bdf_w1", "_bdf_w2")


def time_derivative_symbols(fields: List[Tuple[str, str]]) -> List[sp.Symbol]:
    return [E.REG.dt[name] for name, _ in fields]


@dataclass
class Pointwise:
    """Result of differentiating a weak form at one integration point."""
    fields: List[Tuple[str, str]]          # (name, space) in nodal value order
    dim: int
    params: List[str]                      # parameter names in array order
    r_exprs: List[sp.Expr]                 # [NTC]
    d_entries: List[Tuple[int, int, sp.Expr]]  # (tc, ic, expr), nonzero only
    uses_x: bool
    dt_fields: List[int] = None            # fields whose time derivative the form reads
    m_entries: List[Tuple[int, sp.Expr]] = None  # (index into d_entries, dr/d(du/dt))

    @property
    def ntc(self) -> int:
        return len(self.fields) * (1 + self.dim)

    @property
    def transient(self) -> bool:
        return bool(self.dt_fields)


def differentiate(fields: List[Tuple[str, str]], dim: int, integrand: sp.Expr,
                  params: List[str]) -> Pointwise:
    """r_tc = d(integrand)/d(test component tc); D[tc, ic] = d r_tc / d(field
    component ic).  Components per field: value, d/dx_0 .. d/dx_{dim-1}.

    A time derivative du/dt of a field (partial_t) is one more pointwise
    input; since du/dt = w0 u + (history), its derivative enters the value
    column as w0 dr/d(du/dt) (w0 the first BDF weight, a parameter), and
    dr/d(du/dt) alone is the mass matrix's coefficient (flag 2 of the
    generated ResidualAndJacobian, jitbridge.h:285)."""
    integrand = sp.expand(integrand) if integrand.has(sp.Symbol) else integrand
    nc = 1 + dim
    tsyms, usyms = [], []
    for name, _ in fields:
        E.REG.field(name)
        tsyms += [E.REG.test[name]] + list(E.REG.test_grad[name][:dim])
        usyms += [E.REG.value[name]] + list(E.REG.grad[name][:dim])
    dsyms = time_derivative_symbols(fields)
    dt_fields = [f for f, s_ in enumerate(dsyms) if sp.sympify(integrand).has(s_)]
    if dt_fields and BDF_PARAMS[0] not in params:
        raise ValueError("a transient form needs the BDF weights among its parameters")
    w0 = E.parameter(BDF_PARAMS[0]) if dt_fields else None
    r_exprs = []
    for t in tsyms:
        r = sp.diff(integrand, t)
        if any(r.has(tt) for tt in tsyms):
            raise ValueError("residual is not linear in the test functions")
        r_exprs.append(sp.simplify(r) if r.count_ops() < 40 else r)
    d_entries, m_entries = [], []
    for tc, r in enumerate(r_exprs):
        for ic, u in enumerate(usyms):
            d = sp.diff(r, u)
            m = sp.diff(r, dsyms[ic // nc]) if (ic % nc == 0 and ic // nc in dt_fields) else sp.Integer(0)
            if m != 0:
                d = d + w0 * m
            if d != 0:
                if m != 0:
                    m_entries.append((len(d_entries), m))
                d_entries.append((tc, ic, d))
    uses_x = any(any(e.has(x) for x in E.X) for e in r_exprs)
    return Pointwise(fields, dim, params, r_exprs, d_entries, uses_x, dt_fields, m_entries)


def _symbol_names(pw: Pointwise, prefix: str = "") -> Dict[sp.Symbol, str]:
    names = {}
    nc = 1 + pw.dim
    for f, (name, _) in enumerate(pw.fields):
        names[E.REG.value[name]] = f"{prefix}U[{f * nc}]"
        for i in range(pw.dim):
            names[E.REG.grad[name][i]] = f"{prefix}U[{f * nc + 1 + i}]"
        if pw.dt_fields and f in pw.dt_fields:
            names[E.REG.dt[name]] = f"{prefix}U[{pw.ntc + f}]"
    for i in range(3):
        names[E.X[i]] = f"{prefix}Xq[{i}]"
    for k, p in enumerate(pw.params):
        names[E.parameter(p)] = f"{prefix}P[{k}]"
    return names


def _emit(exprs, names, fp32: bool, outs, indent="  ", df64: bool = False, fp64_names=None):
    real = "fe_df64" if df64 else "float" if fp32 else "double"
    pr = _DF64Printer(dict(names), fp64_names) if df64 else _Printer(dict(names), fp32=fp32)
    repl, reduced = sp.cse(exprs, symbols=sp.numbered_symbols("t_"), optimizations="basic")
    lines = []
    for s_, e in repl:
        pr._names[s_] = s_.name
    for s_, e in repl:
        lines.append(f"{indent}const {real} {s_.name} = {pr.doprint(e)};")
    for o, e in zip(outs, reduced):
        lines.append(f"{indent}{o} = {pr.doprint(e)};")
    return lines


def dparam_source(pw: Pointwise) -> str:
    """``fe_pointwise_dparam(U, Xq, P, r, dparam)``: the residual
    coefficients differentiated by the global parameter P[dparam]
    (dResidual{i}dParameter_{k} of pyoomph's generated code,
    codegen.cpp:4743-4760).  Parameters inside a Gaussian source enter by
    the chain rule through the sum's closed-form derivatives
    (fe_gauss_dparam)."""
    names = _symbol_names(pw)
    nr = len(pw.r_exprs)
    atoms = sorted({g for e in pw.r_exprs for g in e.atoms(E.GaussianSum)}, key=str)
    gsyms = [sp.Symbol(f"FE_GS{a}", real=True) for a in range(len(atoms))]
    ginfo = []
    for a, ga in enumerate(atoms):
        k0 = next(i for i, x_ in enumerate(ga.args) if x_.is_Integer)
        n, dim = int(ga.args[k0]), int(ga.args[k0 + 1])
        pars = list(ga.args[k0 + 2:])
        ref0 = names[pars[0]]
        base = int(ref0[ref0.index("[") + 1:-1])
        names[gsyms[a]] = f"fe_gauss_sum<{dim}>(Xq, P + {base}, {n})"
        ginfo.append((dim, base, pars))
    subs = dict(zip(atoms, gsyms))
    rs = [e.subs(subs) for e in pw.r_exprs]
    lines = ["__device__ __forceinline__ void fe_pointwise_dparam(const double* __restrict__ U, "
             "const double* __restrict__ Xq, const double* __restrict__ P, double* __restrict__ r, int dparam) {",
             "  (void)U; (void)Xq; (void)P;",
             f"  for (int k = 0; k < {nr}; ++k) r[k] = 0.0;",
             "  switch (dparam) {"]
    for j, pname in enumerate(pw.params):
        if pname in BDF_PARAMS:
            continue
        psym = E.parameter(pname)
        exprs = []
        for e in rs:
            d = sp.diff(e, psym)
            for a, (dim, base, pars) in enumerate(ginfo):
                if psym in pars:
                    dg = sp.Symbol(f"FE_DG{a}_{j}", real=True)
                    names[dg] = f"fe_gauss_dparam<{dim}>(Xq, P + {base}, {j - base})"
                    d = d + sp.diff(e, gsyms[a]) * dg
            exprs.append(sp.simplify(d) if d != 0 else d)
        if all(d == 0 for d in exprs):
            continue
        lines.append(f"    case {j}: {{")
        keep = [(k, d) for k, d in enumerate(exprs) if d != 0]
        lines += _emit([d for _, d in keep], names, False, [f"r[{k}]" for k, _ in keep], "      ")
        lines.append("      break; }")
    lines += ["    default: break;", "  }", "}"]
    return "\n".join(lines)


def pointwise_source(pw: Pointwise, jreal: str = "double", rdf: bool = False) -> str:
    """The generated device functions.

    ``fe_pointwise(U, Xq, P, r, D, flag)`` computes the residual coefficients
    r in FP64 and, when jreal is double, the derivatives D too (sharing the
    common subexpressions).  With jreal float, D comes from the separate
    single-precision ``fe_pointwise_jac(U, Xq, P, D)``: the Jacobian then
    costs no FP64 instructions.  With ``rdf`` (double-float residual) U and
    r are ``fe_df64`` and the arithmetic runs on the FP32 pipes; D too when
    jreal is double (the double-float Jacobian)."""
    names = _symbol_names(pw)
    fp64_names = dict(names)
    nr = len(pw.r_exprs)
    nd = len(pw.d_entries)
    if rdf:
        # parameters and coordinates converted once per call
        names = {k_: v_.replace("P[", "Pd[").replace("Xq[", "Xd[") for k_, v_ in names.items()}
        dt = "fe_df64" if jreal == "double" else "jreal"
        hdr = ("__device__ __forceinline__ void fe_pointwise(const fe_df64* __restrict__ U, "
               "const double* __restrict__ Xq, const double* __restrict__ P, fe_df64* __restrict__ r, "
               f"{dt}* __restrict__ D, int flag, const double* __restrict__ gsT, const int* __restrict__ gsI) {{")
        lines = [hdr, "  (void)gsT; (void)gsI; (void)Xq; (void)P; (void)D; (void)flag;",
                 f"  fe_df64 Pd[{max(1, len(pw.params))}];",
                 "  #pragma unroll",
                 f"  for (int k = 0; k < {len(pw.params)}; ++k) Pd[k] = fe_df64(P[k]);",
                 "  fe_df64 Xd[3];",
                 "  #pragma unroll",
                 "  for (int k = 0; k < 3; ++k) Xd[k] = fe_df64(Xq[k]);",
                 "  (void)Pd; (void)Xd;"]
    else:
        hdr = ("__device__ __forceinline__ void fe_pointwise(const double* __restrict__ U, "
               "const double* __restrict__ Xq, const double* __restrict__ P, double* __restrict__ r, "
               "jreal* __restrict__ D, int flag, const double* __restrict__ gsT, const int* __restrict__ gsI) {")
        lines = [hdr, "  (void)gsT; (void)gsI;"]
    mass = _mass_lines(pw, names, False) if pw.transient else []
    if jreal == "double" and nd:
        exprs = list(pw.r_exprs) + [d for (_, _, d) in pw.d_entries]
        outs = [f"r[{k}]" for k in range(nr)] + [f"D[{k}]" for k in range(nd)]
        body = _emit(exprs, names, False, outs, "  ", df64=rdf, fp64_names=fp64_names)
        # D assignments only when flag: move them under the branch
        rl = [l for l in body if not l.strip().startswith("D[")]
        dl = [l for l in body if l.strip().startswith("D[")]
        lines += rl
        if mass:
            lines += ["  if (flag == 2) {"] + mass + ["  } else if (flag) {"] + ["  " + l for l in dl] + ["  }"]
        else:
            lines += ["  if (flag) {"] + ["  " + l for l in dl] + ["  }"]
    else:
        lines += _emit(list(pw.r_exprs), names, False, [f"r[{k}]" for k in range(nr)], "  ", df64=rdf,
                       fp64_names=fp64_names)
    lines.append("}")
    names = _symbol_names(pw)
    # Hessian-vector product: D'(U; V) = sum_c dD/dU_c V_c, V the interpolated direction
    nc = 1 + pw.dim
    usyms, vsyms = [], []
    for f, (name, _) in enumerate(pw.fields):
        usyms += [E.REG.value[name]] + list(E.REG.grad[name][:pw.dim])
        vsyms += [sp.Symbol(f"V_{f}_{c}", real=True) for c in range(nc)]
    hnames = dict(names)
    for k, v in enumerate(vsyms):
        hnames[v] = f"V[{k}]"
    # a transient form: the direction moves du/dt by w0 times its value component
    dsyms = time_derivative_symbols(pw.fields)
    w0 = E.parameter(BDF_PARAMS[0]) if pw.transient else None
    hexprs = [sum((sp.diff(d, u) * v for u, v in zip(usyms, vsyms)), sp.Integer(0)) +
              sum((sp.diff(d, dsyms[f]) * w0 * vsyms[f * nc] for f in (pw.dt_fields or [])), sp.Integer(0))
              for (_, _, d) in pw.d_entries]
    lines.append("__device__ __forceinline__ void fe_pointwise_hvp(const double* __restrict__ U, "
                 "const double* __restrict__ V, const double* __restrict__ Xq, const double* __restrict__ P, "
                 "jreal* __restrict__ D) {")
    lines.append("  (void)U; (void)V; (void)Xq; (void)P;")
    if nd:
        hl = _emit(hexprs, hnames, False, [f"D[{k}]" for k in range(nd)], "  ")
        lines += [l.replace("] = ", "] = (jreal)(", 1) + ")" if l.strip().startswith("D[") else l for l in hl]
        lines = [l[:-2] + ");" if l.strip().startswith("D[") and l.endswith(";)") else l for l in lines]
    lines.append("}")
    if jreal != "double":
        fl = _symbol_names(pw, prefix="f")
        ut = "fe_df64" if rdf else "double"
        lines.append(f"__device__ __forceinline__ void fe_pointwise_jac(const {ut}* __restrict__ U, "
                     "const double* __restrict__ Xq, const double* __restrict__ P, float* __restrict__ D, int flag) {")
        lines.append("  (void)flag;")
        nc = 1 + pw.dim
        nu = len(pw.fields) * nc + (len(pw.fields) if pw.transient else 0)
        lines.append(f"  float fU[{max(1, nu)}]; float fXq[3]; float fP[{max(1, len(pw.params))}];")
        # (a double-float value's high word is its nearest binary32)
        lines.append(f"  #pragma unroll\n  for (int k = 0; k < {nu}; ++k) fU[k] = {'U[k].hi' if rdf else '(float)U[k]'};")
        lines.append("  fXq[0] = (float)Xq[0]; fXq[1] = (float)Xq[1]; fXq[2] = (float)Xq[2];")
        if pw.params:
            lines.append(f"  #pragma unroll\n  for (int k = 0; k < {len(pw.params)}; ++k) fP[k] = (float)P[k];")
        if nd:
            dl = _emit([d for (_, _, d) in pw.d_entries], fl, True, [f"D[{k}]" for k in range(nd)], "  ")
            if pw.transient:
                lines += ["  if (flag == 2) {"] + _mass_lines(pw, fl, True) + ["    return;", "  }"]
            lines += dl
        lines.append("}")
    return "\n".join(lines)


def _mass_lines(pw: Pointwise, names, fp32: bool) -> List[str]:
    """Flag 2: D holds dr/d(du/dt) (the mass matrix's pointwise coefficients)
    at the value columns of the time-differentiated fields, 0 elsewhere."""
    real = "float" if fp32 else "double"
    lines = [f"    #pragma unroll\n    for (int k = 0; k < {max(1, len(pw.d_entries))}; ++k) D[k] = ({real})0;"]
    if pw.m_entries:
        lines += _emit([m for _, m in pw.m_entries], names, fp32, [f"D[{k}]" for k, _ in pw.m_entries], "    ")
    return lines


@dataclass
class KernelSpec:
    name: str
    source: str
    et: ElementType
    layout: Layout
    pointwise: Pointwise
    epb: int
    threads: int
    smem_bytes: int
    jac_precision: str
    tables: np.ndarray = field(repr=False, default=None)
    sumfac_blocks: int = 0       # > 0: sum-factorised Jacobian with this many (a, b) blocks
    # tensor-core contraction (csrc/fe_tc.cuh): the kernel writes the
    # pulled-back derivatives Dhat (per knot, these (test, trial) reference
    # components) and the library contracts them into J_e; None otherwise
    tc_pairs: Optional[List[Tuple[int, int]]] = None
    gauss_sep: int = 0           # > 0: this many Gaussians of the source evaluated separably per element
    sum_fact_interp: bool = False  # interpolation and residual contraction sum-factorised (Q2 hex)
    min_blocks: int = 0          # > 0: registers bounded for this many resident blocks per SM
    residual_precision: str = "f64"  # "df64": the residual path in double-float on the FP32 pipes

    @property
    def key(self) -> str:
        return hashlib.sha1(self.source.encode()).hexdigest()[:16]


def tc_tables(ks: "KernelSpec"):
    """(test components, trial components, phi [nq][1 + dim][n]) of a kernel
    generated for the tensor-core contraction: the reference basis of its
    single field (value and d/ds_b at the knots) in local order, and the
    component pairs of its pulled-back derivatives."""
    et, lay = ks.et, ks.layout
    t = et.tables()
    psi = np.asarray(t["PSI2"]).reshape(et.nq, et.nnode)
    dps = np.asarray(t["DPS2"]).reshape(et.nq, et.nnode, et.dim)
    node = np.asarray(lay.node)
    phi = np.empty((et.nq, et.dim + 1, lay.n))
    phi[:, 0, :] = psi[:, node]
    for b in range(et.dim):
        phi[:, 1 + b, :] = dps[:, node, b]
    pa = np.array([a for a, _ in ks.tc_pairs], dtype=np.int32)
    pb = np.array([b for _, b in ks.tc_pairs], dtype=np.int32)
    return pa, pb, np.ascontiguousarray(phi)


def _launch_shape(et: ElementType, nloc: int, per_elem_bytes: int, table_bytes: int,
                  smem_cap: int = 200 * 1024, max_threads: int = 512,
                  largest: bool = False) -> Tuple[int, int]:
    """Elements per block and threads: keep both thread phases (element x
    integration point, element x row) busy in whole warps, within the
    shared-memory budget (or, with `largest`, the most elements that fit)."""
    best = None
    for epb in range(1, 65):
        smem = table_bytes + epb * per_elem_bytes
        if smem > smem_cap:
            break
        work = max(epb * et.nq, epb * nloc)
        threads = ((work + 31) // 32) * 32
        if threads > max_threads:
            break
        # prefer whole-warp phases and larger blocks
        waste = (threads - epb * et.nq) / threads + (threads - epb * nloc) / threads
        score = (epb,) if largest else (-waste, epb)
        if best is None or score > best[0]:
            best = (score, epb, threads)
    if best is None:
        raise ValueError("element does not fit in shared memory")
    return best[1], best[2]


def _threads_for(epb: int, nq: int, nloc: int) -> int:
    """Threads per block for EPB elements: max(knots, ceil(rows / 2)) per
    element, in whole warps.  Phase A (one thread per element and knot)
    then fills the block, and phase B (one thread per element and row)
    takes two rounds where an element has more rows than knots.  With one
    thread per row the Taylor-Hood P2/P1 element (15 rows, 7 knots) leaves
    8 of 15 warps waiting at phase A's barrier; measured on GB300 (NS
    256^2, 32 elements per block): 480 -> 256 threads, FP64 element kernel
    1.461 -> 1.413 ms, FP32 0.341 -> 0.297 ms, df64 with the double-float
    residual 0.669 -> 0.642 ms."""
    return ((epb * max(nq, -(-nloc // 2)) + 31) // 32) * 32


def generate_kernel(et: ElementType, pw: Pointwise, jac_precision: str = "f64",
                    name: str = None, epb: int = None, affine: bool = False, jref: bool = None,
                    gauss_sep: bool = False, tc: bool = None, min_blocks: int = None,
                    residual_precision: str = "f64", threads: int = None) -> KernelSpec:
    """Fused element kernel for one element type and weak form.

    Thread phases (all in one launch, EPB elements per block):
      0. stage reference tables and the elements' nodal positions/values in
         shared memory;
      G. (affine elements only) geometry once per element;
      A. one thread per (element, integration point): geometry (unless
         affine), interpolation, pointwise residual coefficients (FP64,
         pulled back to reference coordinates) and derivatives D (Jacobian
         precision), physical shape gradients for the Jacobian;
      B. one thread per (element, local row), rows ordered field-major so a
         warp shares its test field: R_i = sum_q rhat . phi_i and
         J_ij = sum_q phi_i^T D psi_j, written to the element buffers.

    With ``tc`` (default: FP32 Jacobians of steady single-field forms on
    elements of 17-32 local values, i.e. the Q2 hex) phase B builds no
    Jacobian: the kernel writes the pulled-back derivatives Dhat of its
    elements to ``a.dhat`` and the library contracts them on the tensor
    cores (csrc/fe_tc.cuh, fe_problem_set_tensor_contraction).

    With ``jref`` (default: FP32 Jacobians, 3D elements, single-field
    forms) the Jacobian is contracted in
    reference coordinates too: phase A pulls D back, Dhat = T^T D T with
    T = diag(1, g) per field (the same route as the residual's rhat), and
    phase B contracts Dhat with the reference shape tables shared by all
    elements.  Nothing of size (knots x nodes x dim) is kept per element, so
    a block holds several times more elements (the Q2 hex element needs 27 x
    27 x 3 physical gradients otherwise).

    With ``residual_precision="df64"`` (FP32 or double-float Jacobians of
    steady forms whose pointwise terms are rational, Gaussian sources
    aside) the residual path runs in double-float on the FP32 pipes:
    interpolation (sum-factorised for the Q2 hex), pointwise residual,
    pull-back and the contraction with the test functions; the geometry
    and the Gaussian source factors stay FP64.  Nodal values are staged as differences from the element's
    node 0, formed in FP64 (u = u_0 + sum_l (u_l - u_0) psi_l, grad u =
    sum_l (u_l - u_0) grad psi_l by the partition of unity), so that the
    48-bit significand rounds only the small differences: the cancellation
    in the reference gradients does not amplify it.
    """
    dim, nn, nn1, nq = et.dim, et.nnode, et.nnode_c1, et.nq
    fields = pw.fields
    nf = len(fields)
    nc = 1 + dim
    ntc = nf * nc
    spaces = [sp_ for _, sp_ in fields]
    layout = make_layout(et, spaces)
    nloc = layout.n
    nval = nf
    has_c1 = any(s_ == "C1" for s_ in spaces)
    ndnz = max(1, len(pw.d_entries))
    if jac_precision not in ("f64", "f32", "df64"):
        raise ValueError(f"unknown Jacobian precision {jac_precision!r}")
    df64 = jac_precision == "df64"
    nt_req = threads     # an explicit thread count (else the launch shape's)
    if residual_precision not in ("f64", "df64"):
        raise ValueError(f"unknown residual precision {residual_precision!r}")
    rdf = residual_precision == "df64"
    if rdf:
        if jac_precision == "f64":
            raise ValueError("a double-float residual goes with an FP32 or double-float Jacobian")
        if pw.transient:
            raise ValueError("the double-float residual is generated for steady forms")
        if not df64_residual_supported(pw):
            raise ValueError("the double-float residual needs pointwise terms rational in the fields "
                             "(+ - * / and integer powers; Gaussian sources are allowed)")
        if not et.c1_index or et.c1_index[0] != 0:
            raise ValueError("the double-float residual stages values relative to node 0, a C1 node")
        if jref is False:
            raise ValueError("the double-float residual goes with the reference-coordinate Jacobian (jref)")
        jref = True
    # jreal: phase A (pointwise D and its pull-back); jacc: phase B (the
    # contraction that builds J) -- for df64 D is formed in FP64 and the
    # contraction runs in double-float on the FP32 pipes (fe_df64.cuh)
    jreal = "float" if jac_precision == "f32" else "double"
    jacc = "fe_df64" if df64 else jreal
    jstore = "float" if jac_precision == "f32" else "double"
    jbytes = 4 if jac_precision == "f32" else 8
    if df64:
        if jref is False:
            raise ValueError("the df64 Jacobian is built in reference coordinates (jref)")
        jref = True
    if jref is None:
        # measured on GB300: faster for every FP32 Jacobian, for 3D elements
        # and for single-field forms; slower for the FP64 Taylor-Hood
        # Jacobian, whose pulled-back D is denser than D
        jref = jac_precision == "f32" or dim == 3 or nf == 1
    tc_ok = bool(jac_precision == "f32" and jref and nf == 1 and spaces[0] == "C2" and not pw.transient
                 and nloc <= 32 and nq <= 32)
    use_tc = bool(tc_ok and nloc > 16) if tc is None else bool(tc)
    if use_tc and not tc_ok:
        raise ValueError("the tensor-core contraction needs an FP32 Jacobian in reference coordinates of a "
                         "steady single-field (C2) form with at most 32 local values and 32 knots")
    # Dhat blocks (test field, trial field) -> rows/cols in reference components
    blocks: Dict[Tuple[int, int], List[Tuple[int, int, int]]] = {}
    for k, (tc, ic, _) in enumerate(pw.d_entries):
        blocks.setdefault((tc // nc, ic // nc), []).append((tc % nc, ic % nc, k))
    hat: List[Tuple[int, int, int, int]] = []
    for (tf_, gf_), ents in sorted(blocks.items()):
        rows_ = ([0] if any(a_ == 0 for a_, _, _ in ents) else []) + \
            (list(range(1, nc)) if any(a_ >= 1 for a_, _, _ in ents) else [])
        cols_ = ([0] if any(b_ == 0 for _, b_, _ in ents) else []) + \
            (list(range(1, nc)) if any(b_ >= 1 for _, b_, _ in ents) else [])
        for ah in rows_:
            for bh in cols_:
                hat.append((tf_, gf_, ah, bh))
    ndnz_hat = max(1, len(hat))
    table_doubles = nq + nq * nn + nq * nn * dim + nq * nn1 + nq * nn1 * dim
    table_bytes = table_doubles * 8
    tab_copy = bool(jref and (jreal == "float" or df64))   # reference tables in the contraction type
    tabt = jacc if tab_copy else "double"
    tabf = (nq * nn * (1 + dim) + nq * nn1 * (1 + dim)) if tab_copy else 0
    table_bytes += ((tabf * (8 if df64 else 4) + 15) // 16) * 16
    # double-float residual with an FP32 Jacobian: double-float tables too
    # (the sum-factorised Q2 hex path uses 1D tables instead: decided below)
    rtab = rdf and not df64
    geo_doubles = (dim * dim + 1) if affine else 0
    # separable Gaussian source (axis-aligned affine Q2 elements, the caller
    # checks the alignment): the element's per-axis factors in shared memory
    gs_atoms = set()
    for e_ in pw.r_exprs:
        gs_atoms |= e_.atoms(E.GaussianSum)
    gsep = bool(gauss_sep and affine and et.name in ("Q2_QUAD", "Q2_HEX") and len(gs_atoms) == 1)
    gs_n = gs_base = 0
    if gsep:
        ga = next(iter(gs_atoms))
        k0 = next(i for i, a_ in enumerate(ga.args) if a_.is_Integer)
        gs_n, gdim = int(ga.args[k0]), int(ga.args[k0 + 1])
        ref0 = _symbol_names(pw)[ga.args[k0 + 2]]
        gs_base = int(ref0[ref0.index("[") + 1:-1])
        gsep = gdim == dim
    gsd = gs_n * dim * 3 if gsep else 0          # doubles per element
    # sum factorisation of the Q2 hex Jacobian (tensor-product shapes and
    # Gauss<3,3> knots): J_ij = sum_ab sum_q prod_d F^d_ab[q_d][i_d][j_d] Dhat_ab(q)
    # contracted one direction at a time (3 x 81 + 3 x 243 + 3 x 729 multiply-adds
    # per (a, b) block instead of 27 x 27 x 27)
    # (FP64 Jacobians only: for FP32 the contraction is cheap on the FP32 pipe
    # and the staged form measured slower on GB300)
    sumfac = bool(jref and et.name == "Q2_HEX" and nf == 1 and spaces[0] == "C2" and jac_precision in ("f64", "df64"))
    if sumfac:
        table_bytes += ((4 * 27 * jbytes + 15) // 16) * 16
    # sum factorisation of the interpolation (value and reference gradient
    # at the 27 knots) and of the residual's test-function contraction of the
    # Q2 hex: one axis at a time, 729 multiply-adds each instead of 27 x 27 x 4
    sfi = bool(jref and et.name == "Q2_HEX" and nf == 1 and spaces[0] == "C2"
               and list(layout.loc_of[0]) == list(range(nn)))
    rtab = rtab and not sfi
    if rtab:
        table_bytes += tabf * 8
    # transient forms: nodal du/dt = w0 u + w1 u_{n-1} + w2 u_{n-2} staged per
    # element beside the values, interpolated as one more input per field
    transient = pw.transient
    nu = ntc + (nf if transient else 0)
    bdf_idx = [pw.params.index(n_) for n_ in BDF_PARAMS] if transient else []
    sfi_own = sfi and not sumfac            # buffers of its own (else the Jacobian's stage buffers)
    if jref:
        per_elem = (nn * dim + 2 * nn * nval + nq * ntc + geo_doubles + gsd) * 8 + nq * ndnz_hat * jbytes
        if sumfac:
            per_elem += (81 + 243 + 729) * jbytes
    else:
        per_elem = ((nn * dim + 2 * nn * nval + nq * ntc + geo_doubles + gsd) * 8
                    + (nq * ndnz + nq * nn * dim + (nq * nn1 * dim if has_c1 else 0)) * jbytes)
    if sfi_own:
        per_elem += (54 + 81 + 108) * 8
    if transient:
        per_elem += nn * nval * 8
    if epb is None:
        # df64: the most elements that fit 720 threads and 224 KB (GB300
        # sweeps: the Q2 hex kernel is fastest at 12 elements per block, the
        # largest that fits the shared memory; the P2 Taylor-Hood kernel at
        # 48, 720 threads)
        # (the sum-factorised Q2 hex kernels are fastest at the largest block
        # that fits too: the steady FP64 one at 13 elements)
        epb, auto_threads = _launch_shape(et, nloc, per_elem, table_bytes,
                                          smem_cap=224 * 1024 if df64 else 216 * 1024,
                                          max_threads=720 if df64 else 512, largest=df64 or sumfac)
        threads = _threads_for(epb, nq, nloc) if nt_req is None else nt_req
    elif threads is None:
        threads = _threads_for(epb, nq, nloc)
    # (every phase is a block-strided loop: fewer threads than rows or knots
    # take several rounds)
    threads = (int(threads) + 31) // 32 * 32
    row_threads = ((max(epb * nq, epb * nloc) + 31) // 32) * 32   # one thread per row
    smem = table_bytes + epb * per_elem
    smem = (smem + 15) // 16 * 16
    if threads > 1024 or smem > 227 * 1024:
        raise ValueError(f"{epb} elements per block do not fit a block ({threads} threads, {smem} B shared)")
    if min_blocks is None:
        # FP64 / double-float Jacobians of 2D elements: bound the registers
        # for two resident blocks where their shared memory allows it.  With
        # one thread per row (480 threads) the Taylor-Hood kernel took 78
        # (FP64) / 101 (df64) registers, so one block per SM; bounded to 64
        # it spilled 88 / 324 bytes and ran 6% / 10% faster on GB300.  At the
        # default 256 threads the bound (128 registers) no longer binds, and
        # two blocks fit as they are
        if jac_precision in ("f64", "df64") and et.dim == 2 and threads <= 512 and 2 * smem <= 227 * 1024:
            min_blocks = 2
    elif min_blocks <= 0:
        min_blocks = None
    if name is None:
        h = hashlib.sha1((et.name + jac_precision + str(affine) + str(epb) + str(jref) + str(sumfac) + str(gsep) +
                          ("tc" if use_tc else "") + (f"mb{int(min_blocks)}" if min_blocks else "") +
                          ("rdf" if rdf else "") + (f"nt{threads}" if threads != row_threads else "") +
                          str(sfi) + (str(pw.m_entries) if transient else "") +
                          str(pw.r_exprs) +
                          str(pw.d_entries)).encode()).hexdigest()[:10]
        name = f"fe_elem_{et.name.lower()}_{jac_precision}{'_rdf' if rdf else ''}{'_aff' if affine else ''}_{h}"

    nsub = [nn if s_ == "C2" else nn1 for s_ in spaces]
    loc_of_flat = [layout.loc_of[f][k] for f in range(nf) for k in range(nsub[f])]
    loc_off = [sum(nsub[:f]) for f in range(nf)]
    used_ic = sorted({ic for (_, ic, _) in pw.d_entries})
    src = []
    w = src.append
    w("// generated element kernel -- do not edit")
    w('#include "fe_device.cuh"')
    w(f"#define FE_DIM {dim}\n#define FE_NN {nn}\n#define FE_NN1 {nn1}\n#define FE_NQ {nq}")
    w(f"#define FE_NVAL {nval}\n#define FE_NLOC {nloc}\n#define FE_EPB {epb}\n#define FE_NT {threads}")
    w(f"#define FE_NF {nf}\n#define FE_NTC {ntc}\n#define FE_NDNZ {ndnz}\n#define FE_AFFINE {1 if affine else 0}")
    w(f"#define FE_NDNZH {ndnz_hat}")
    w(f"typedef {jreal} jreal;")
    w(f"typedef {jacc} jacc;")
    w(f"typedef {jstore} jstore;")
    w(f"__constant__ int c_loc_of[{len(loc_of_flat)}] = {{{', '.join(map(str, loc_of_flat))}}};")
    if sumfac:
        from .spaces import _G3_1D, _lag3
        M_ = [np.array([_lag3(g)[0] for g in _G3_1D]), np.array([_lag3(g)[1] for g in _G3_1D])]
        F_ = [repr(float(M_[c >> 1][q][i] * M_[c & 1][q][j]))
              for c in range(4) for q in range(3) for i in range(3) for j in range(3)]
        w(f"__constant__ double c_F[108] = {{{', '.join(F_)}}};")
    if gsep:
        w("#define FE_GAUSS(d, x, g, n) fe_gauss_sep<d>(gsT, gsI, g, n)")
    else:
        w("#define FE_GAUSS(d, x, g, n) fe_gauss_sum<d>(x, g, n)")
    if sfi:
        from .spaces import _G3_1D, _lag3
        Mv = [repr(float(_lag3(g)[c][i])) for c in range(2) for g in _G3_1D for i in range(3)]
        w(f"__constant__ double c_M[18] = {{{', '.join(Mv)}}};")
    w(pointwise_source(pw, jreal, rdf=rdf))
    w(dparam_source(pw))
    lb = f"FE_NT, {int(min_blocks)}" if min_blocks else "FE_NT"
    w(f'extern "C" __global__ void __launch_bounds__({lb}) {name}(const FeElemArgs a) {{')
    w("  extern __shared__ __align__(16) unsigned char fe_smem[];")
    w("  double* sW = reinterpret_cast<double*>(fe_smem);")
    w("  double* sPsi2 = sW + FE_NQ;")
    w("  double* sDps2 = sPsi2 + FE_NQ * FE_NN;")
    w("  double* sPsi1 = sDps2 + FE_NQ * FE_NN * FE_DIM;")
    w("  double* sDps1 = sPsi1 + FE_NQ * FE_NN1;")
    w("  double* sX = sDps1 + FE_NQ * FE_NN1 * FE_DIM;")
    w("  double* sU = sX + FE_EPB * FE_NN * FE_DIM;")
    w("  double* sY = sU + FE_EPB * FE_NN * FE_NVAL;  // direction of the Hessian-vector product (flag 4)")
    if transient:
        w("  double* sUt = sY + FE_EPB * FE_NN * FE_NVAL;  // nodal du/dt (BDF weights of the step)")
        w("  double* sRh = sUt + FE_EPB * FE_NN * FE_NVAL;")
    else:
        w("  double* sRh = sY + FE_EPB * FE_NN * FE_NVAL;")
    w("  double* sG = sRh + FE_EPB * FE_NQ * FE_NTC;")
    w(f"  double* sGe = sG + FE_EPB * {geo_doubles};  // separable Gaussian factors, {gsd} per element")
    w(f"  jacc* sD = reinterpret_cast<jacc*>(sGe + FE_EPB * {gsd});")
    w("  (void)sGe;")
    if rdf:
        # double-float residual: values staged as differences from node 0
        # (node 0: its value), residual coefficients per knot in double-float
        w("  fe_df64* sUr = reinterpret_cast<fe_df64*>(sU);")
        w("  fe_df64* sRhr = reinterpret_cast<fe_df64*>(sRh);")
    if jref:
        w("  jacc* sEnd = sD + FE_EPB * FE_NQ * FE_NDNZH;")
        if tab_copy:
            # copies of the reference tables in the contraction type (after the element data)
            w("  jacc* sPsi2j = sEnd;")
            w("  jacc* sDps2j = sPsi2j + FE_NQ * FE_NN;")
            w("  jacc* sPsi1j = sDps2j + FE_NQ * FE_NN * FE_DIM;")
            w("  jacc* sDps1j = sPsi1j + FE_NQ * FE_NN1;")
            if rtab:
                off = ((tabf * 4 + 15) // 16 * 16) // 4
                w(f"  fe_df64* sPsi2r = reinterpret_cast<fe_df64*>(sPsi2j + {off});  // double-float tables (residual)")
                w("  fe_df64* sDps2r = sPsi2r + FE_NQ * FE_NN;")
                w("  fe_df64* sPsi1r = sDps2r + FE_NQ * FE_NN * FE_DIM;")
                w("  fe_df64* sDps1r = sPsi1r + FE_NQ * FE_NN1;")
            elif rdf and df64:
                w("  fe_df64* sPsi2r = sPsi2j; fe_df64* sDps2r = sDps2j; fe_df64* sPsi1r = sPsi1j; fe_df64* sDps1r = sDps1j;")
                w("  (void)sPsi2r; (void)sDps2r; (void)sPsi1r; (void)sDps1r;")
        else:
            w("  (void)sEnd;")
            w("  const double* sPsi2j = sPsi2; const double* sDps2j = sDps2;")
            w("  const double* sPsi1j = sPsi1; const double* sDps1j = sDps1;")
        w("  (void)sPsi1j; (void)sDps1j; (void)sG;")
        if sumfac:
            # per element: stage buffers and the element matrix; per block: F tables
            base = "sPsi2j + " + str(tabf) if tab_copy else "sEnd"
            w(f"  jacc* sS1 = {base};")
            w("  jacc* sS2 = sS1 + FE_EPB * 81;")
            w("  jacc* sJe = sS2 + FE_EPB * 243;")
            w("  jacc* sF = sJe + FE_EPB * 729;")
        if sfi:
            if sumfac:
                w("  double* sIa = reinterpret_cast<double*>(sS1);  // interpolation / residual stages")
                w("  double* sIb = reinterpret_cast<double*>(sS2);")
                w("  double* sIc = reinterpret_cast<double*>(sJe);")
                sfs = (81, 243, 729)
            else:
                assert not tab_copy or (tabf * (8 if df64 else 4)) % 8 == 0, "stage buffers must be 8-byte aligned"
                base = f"sPsi2j + {tabf}" if tab_copy else "sEnd"
                w(f"  double* sIa = reinterpret_cast<double*>({base});  // interpolation / residual stages")
                w("  double* sIb = sIa + FE_EPB * 54;")
                w("  double* sIc = sIb + FE_EPB * 81;")
                sfs = (54, 81, 108)
    else:
        w("  jreal* sDx2 = sD + FE_EPB * FE_NQ * FE_NDNZ;")
        w("  jreal* sDx1 = sDx2 + FE_EPB * FE_NQ * FE_NN * FE_DIM;")
        w("  (void)sDx1; (void)sG;")
    w("  const long long e0 = (long long)blockIdx.x * FE_EPB;")
    w("  const long long rem = a.n_elem - e0;")
    w("  const int nel = rem < FE_EPB ? (int)rem : FE_EPB;")
    # flag 3 (dR/dp of global parameter a.aux): the residual path with the
    # differentiated coefficients, no Jacobian
    w("  const int flag = a.flag == 3 ? 0 : a.flag;")
    w("  const bool dpar = a.flag == 3;")
    w(f"  for (int k = threadIdx.x; k < {table_doubles}; k += FE_NT) sW[k] = a.tables[k];")
    if tab_copy:
        w(f"  for (int k = threadIdx.x; k < {tabf}; k += FE_NT) sPsi2j[k] = (jacc)a.tables[FE_NQ + k];")
    if rtab:
        w(f"  for (int k = threadIdx.x; k < {tabf}; k += FE_NT) sPsi2r[k] = fe_df64(a.tables[FE_NQ + k]);")
    if sfi:
        # 1D Lagrange values M0[q][i] and derivatives M1[q][i] at the 1D Gauss points
        w("  __shared__ double sM[18];")
        w("  for (int k = threadIdx.x; k < 18; k += FE_NT) sM[k] = c_M[k];")
        if rdf:
            w("  __shared__ fe_df64 sMr[18];")
            w("  for (int k = threadIdx.x; k < 18; k += FE_NT) sMr[k] = fe_df64(c_M[k]);")
    if sumfac:
        from .spaces import _G3_1D, _lag3
        M = [np.array([_lag3(g)[0] for g in _G3_1D]), np.array([_lag3(g)[1] for g in _G3_1D])]
        Fv = []
        for c in range(4):
            for q in range(3):
                for i in range(3):
                    for j in range(3):
                        Fv.append(M[c >> 1][q][i] * M[c & 1][q][j])
        w(f"  for (int k = threadIdx.x; k < 108; k += FE_NT) sF[k] = (jacc)c_F[k];")

    w("  for (int k = threadIdx.x; k < nel * FE_NN; k += FE_NT) {")
    w("    const int el = k / FE_NN, l = k - el * FE_NN;")
    w("    int node = a.conn[(e0 + el) * FE_NN + l];")
    w("    FE_CHECK_NODE(node, e0 + el, a);")
    w("    #pragma unroll")
    w("    for (int d = 0; d < FE_DIM; ++d) sX[k * FE_DIM + d] = a.x[(long long)node * FE_DIM + d];")
    if rdf:
        w("    { int node0 = a.conn[(e0 + el) * FE_NN];")
        w("      FE_CHECK_NODE(node0, e0 + el, a);")
        w("      #pragma unroll")
        w("      for (int v = 0; v < FE_NVAL; ++v) {")
        w("        const double u = a.values[(long long)node * a.nval + v];")
        w("        sUr[k * FE_NVAL + v] = fe_df64(l == 0 ? u : u - a.values[(long long)node0 * a.nval + v]); } }")
    else:
        w("    #pragma unroll")
        w("    for (int v = 0; v < FE_NVAL; ++v) sU[k * FE_NVAL + v] = a.values[(long long)node * a.nval + v];")
    w("    if (flag == 4)")
    w("      for (int v = 0; v < FE_NVAL; ++v) sY[k * FE_NVAL + v] = a.dir[(long long)node * a.nval + v];")
    if transient:
        w("    { const double* Pe0 = a.params + (a.replica_elems > 0 ? ((e0 + el) / a.replica_elems) * a.params_stride : 0);")
        w(f"      const double w0 = Pe0[{bdf_idx[0]}], w1 = Pe0[{bdf_idx[1]}], w2 = Pe0[{bdf_idx[2]}];")
        w("      #pragma unroll")
        w("      for (int v = 0; v < FE_NVAL; ++v) {")
        w("        double ut = w0 * sU[k * FE_NVAL + v];")
        w("        if (a.n_hist > 0) ut += w1 * a.hist[(long long)node * a.nval + v];")
        w("        if (a.n_hist > 1) ut += w2 * a.hist[a.hist_stride + (long long)node * a.nval + v];")
        w("        sUt[k * FE_NVAL + v] = ut;")
        w("      } }")
    w("  }")
    w("  __syncthreads();")
    if affine:
        # ---------------- phase G: constant geometry of affine elements ----------------
        w("  for (int el = threadIdx.x; el < nel; el += FE_NT) {")
        w("    double g[FE_DIM][FE_DIM]; double J;")
        w("    fe_metric_geometry<FE_DIM, FE_NN>(sX + el * FE_NN * FE_DIM, sDps2, g, J);")
        w("    if (!(J > 0.0)) atomicExch(a.status, 1);")
        w("    double* sg = sG + el * (FE_DIM * FE_DIM + 1);")
        w("    #pragma unroll")
        w("    for (int b = 0; b < FE_DIM; ++b)")
        w("      #pragma unroll")
        w("      for (int i = 0; i < FE_DIM; ++i) sg[b * FE_DIM + i] = g[b][i];")
        w("    sg[FE_DIM * FE_DIM] = J;")
        w("  }")
        w("  __syncthreads();")
    if gsep:
        # ---------------- phase S: the separable Gaussian factors ----------------
        # one thread per (element, Gaussian, axis, knot coordinate): x_d at the
        # knot with index i along axis d and 0 along the others, formed as
        # phase A forms Xq (vertex shapes of the affine map)
        w(f"  for (int p = threadIdx.x; p < nel * {gsd}; p += FE_NT) {{")
        w(f"    const int el = p / {gsd}, o = p - el * {gsd};")
        w("    const int i = o % 3, kd = o / 3, d = kd % FE_DIM, k = kd / FE_DIM;")
        w(f"    const int q = i * (FE_DIM == 3 ? (d == 0 ? 9 : d == 1 ? 3 : 1) : (d == 0 ? 3 : 1));")
        w("    const double* X = sX + el * FE_NN * FE_DIM;")
        w("    double xd = 0.0;")
        for l, node in enumerate(et.c1_index):
            w(f"    xd += X[{node} * FE_DIM + d] * sPsi1[q * FE_NN1 + {l}];")
        w("    const double* Pe = a.params + (a.replica_elems > 0 ? ((e0 + el) / a.replica_elems) * a.params_stride : 0);")
        w(f"    const double* g = Pe + {gs_base} + k * (FE_DIM + 2);")
        w("    const double dd = xd - g[d], w = g[FE_DIM];")
        w("    sGe[el * " + str(gsd) + " + o] = exp(-(dd * dd) / (2.0 * w * w));")
        w("  }")
        w("  __syncthreads();")
    if sfi and rdf:
        SA, SB, SC = sfs
        # ---------------- phase I (double-float): sum-factorised interpolation ----------------
        # of the staged differences d_l = u_l - u_0 (d_0 = 0; node 0 holds u_0,
        # added to the value in phase A), one axis at a time, renormalised
        # after each stage's three multiply-adds
        w("  { fe_df64* Ia = reinterpret_cast<fe_df64*>(sIa); fe_df64* Ib = reinterpret_cast<fe_df64*>(sIb);")
        w("    fe_df64* Ic = reinterpret_cast<fe_df64*>(sIc);")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // axis 0: A, B [i1][i2][q0]")
        w("    const int el = p / 27, o = p - el * 27, i1 = o / 9, i2 = (o / 3) % 3, q0 = o % 3;")
        w("    const fe_df64* u = sUr + el * FE_NN * FE_NVAL + (3 * i1 + 9 * i2) * FE_NVAL;")
        w("    fe_df64 a_ = fe_df64(0.0f, 0.0f), b_ = fe_df64(0.0f, 0.0f);")
        w("    #pragma unroll")
        w("    for (int i0 = 0; i0 < 3; ++i0) {")
        w("      const fe_df64 uu = (i0 == 0 && i1 == 0 && i2 == 0) ? fe_df64(0.0f, 0.0f) : u[i0 * FE_NVAL];")
        w("      fe_mac(a_, uu, sMr[q0 * 3 + i0]); fe_mac(b_, uu, sMr[9 + q0 * 3 + i0]); }")
        w(f"    Ia[el * {SA} + o] = fe_norm(a_); Ia[el * {SA} + 27 + o] = fe_norm(b_);")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // axis 1: AA, AB, BA [i2][q0][q1]")
        w("    const int el = p / 27, o = p - el * 27, i2 = o / 9, q0 = (o / 3) % 3, q1 = o % 3;")
        w(f"    const fe_df64* A = Ia + el * {SA} + i2 * 3 + q0;")
        w("    fe_df64 aa = fe_df64(0.0f, 0.0f), ab = fe_df64(0.0f, 0.0f), ba = fe_df64(0.0f, 0.0f);")
        w("    #pragma unroll")
        w("    for (int i1 = 0; i1 < 3; ++i1) {")
        w("      const fe_df64 av = A[i1 * 9], bv = A[27 + i1 * 9];")
        w("      fe_mac(aa, av, sMr[q1 * 3 + i1]); fe_mac(ab, av, sMr[9 + q1 * 3 + i1]); fe_mac(ba, bv, sMr[q1 * 3 + i1]); }")
        w(f"    Ib[el * {SB} + o] = fe_norm(aa); Ib[el * {SB} + 27 + o] = fe_norm(ab); Ib[el * {SB} + 54 + o] = fe_norm(ba);")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // axis 2: value, d0, d1, d2 at knot q")
        w("    const int el = p / 27, q = p - el * 27, q0 = q / 9, q1 = (q / 3) % 3, q2 = q % 3;")
        w(f"    const fe_df64* B = Ib + el * {SB} + q0 * 3 + q1;")
        w("    fe_df64 v = fe_df64(0.0f, 0.0f), d0 = v, d1 = v, d2 = v;")
        w("    #pragma unroll")
        w("    for (int i2 = 0; i2 < 3; ++i2) {")
        w("      const fe_df64 aa = B[i2 * 9], ab = B[27 + i2 * 9], ba = B[54 + i2 * 9];")
        w("      const fe_df64 m0 = sMr[q2 * 3 + i2], m1 = sMr[9 + q2 * 3 + i2];")
        w("      fe_mac(v, aa, m0); fe_mac(d2, aa, m1); fe_mac(d1, ab, m0); fe_mac(d0, ba, m0); }")
        w(f"    fe_df64* C = Ic + el * {SC} + q;")
        w("    C[0] = fe_norm(v); C[27] = fe_norm(d0); C[54] = fe_norm(d1); C[81] = fe_norm(d2);")
        w("  }")
        w("  __syncthreads(); }")
    elif sfi:
        SA, SB, SC = sfs
        # ---------------- phase I: sum-factorised interpolation ----------------
        # u at node l = i0 + 3 i1 + 9 i2; knot q = 9 q0 + 3 q1 + q2; shapes
        # psi_l(q) = M0[q0][i0] M0[q1][i1] M0[q2][i2] (M1: derivatives)
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // axis 0: A, B [i1][i2][q0]")
        w("    const int el = p / 27, o = p - el * 27, i1 = o / 9, i2 = (o / 3) % 3, q0 = o % 3;")
        w("    const double* u = sU + el * FE_NN * FE_NVAL + (3 * i1 + 9 * i2) * FE_NVAL;")
        w("    double a_ = 0.0, b_ = 0.0;")
        w("    #pragma unroll")
        w("    for (int i0 = 0; i0 < 3; ++i0) {")
        w("      const double uu = u[i0 * FE_NVAL];")
        w("      a_ = fma(uu, sM[q0 * 3 + i0], a_); b_ = fma(uu, sM[9 + q0 * 3 + i0], b_); }")
        w(f"    sIa[el * {SA} + o] = a_; sIa[el * {SA} + 27 + o] = b_;")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // axis 1: AA, AB, BA [i2][q0][q1]")
        w("    const int el = p / 27, o = p - el * 27, i2 = o / 9, q0 = (o / 3) % 3, q1 = o % 3;")
        w(f"    const double* A = sIa + el * {SA} + i2 * 3 + q0;")
        w("    double aa = 0.0, ab = 0.0, ba = 0.0;")
        w("    #pragma unroll")
        w("    for (int i1 = 0; i1 < 3; ++i1) {")
        w("      const double av = A[i1 * 9], bv = A[27 + i1 * 9];")
        w("      aa = fma(av, sM[q1 * 3 + i1], aa); ab = fma(av, sM[9 + q1 * 3 + i1], ab); ba = fma(bv, sM[q1 * 3 + i1], ba); }")
        w(f"    sIb[el * {SB} + o] = aa; sIb[el * {SB} + 27 + o] = ab; sIb[el * {SB} + 54 + o] = ba;")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // axis 2: value, d0, d1, d2 at knot q")
        w("    const int el = p / 27, q = p - el * 27, q0 = q / 9, q1 = (q / 3) % 3, q2 = q % 3;")
        w(f"    const double* B = sIb + el * {SB} + q0 * 3 + q1;")
        w("    double v = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0;")
        w("    #pragma unroll")
        w("    for (int i2 = 0; i2 < 3; ++i2) {")
        w("      const double aa = B[i2 * 9], ab = B[27 + i2 * 9], ba = B[54 + i2 * 9];")
        w("      const double m0 = sM[q2 * 3 + i2], m1 = sM[9 + q2 * 3 + i2];")
        w("      v = fma(aa, m0, v); d2 = fma(aa, m1, d2); d1 = fma(ab, m0, d1); d0 = fma(ba, m0, d0); }")
        w(f"    double* C = sIc + el * {SC} + q;")
        w("    C[0] = v; C[27] = d0; C[54] = d1; C[81] = d2;")
        w("  }")
        w("  __syncthreads();")
    # ---------------- phase A ----------------
    w("  for (int p = threadIdx.x; p < nel * FE_NQ; p += FE_NT) {")
    w("    const int el = p / FE_NQ, q = p - el * FE_NQ;")
    w("    const double* X = sX + el * FE_NN * FE_DIM;")
    w("    const double* dps = sDps2 + q * FE_NN * FE_DIM;")
    w("    double g[FE_DIM][FE_DIM]; double J;")
    if affine:
        w("    { const double* sg = sG + el * (FE_DIM * FE_DIM + 1);")
        w("      #pragma unroll")
        w("      for (int b = 0; b < FE_DIM; ++b)")
        w("        #pragma unroll")
        w("        for (int i = 0; i < FE_DIM; ++i) g[b][i] = sg[b * FE_DIM + i];")
        w("      J = sg[FE_DIM * FE_DIM]; }")
    else:
        w("    fe_metric_geometry<FE_DIM, FE_NN>(X, dps, g, J);")
        w("    if (!(J > 0.0)) atomicExch(a.status, 1);")
    w("    const double wq = sW[q] * J;")
    w("    double Xq[3] = {0.0, 0.0, 0.0};")
    if pw.uses_x:
        if affine:
            # the affine map is reproduced exactly by the vertex (C1) shapes
            for l, node in enumerate(et.c1_index):
                for i in range(dim):
                    w(f"    Xq[{i}] += X[{node * dim + i}] * sPsi1[q * FE_NN1 + {l}];")
        else:
            w("    #pragma unroll")
            w("    for (int l = 0; l < FE_NN; ++l) {")
            w("      const double ps = sPsi2[q * FE_NN + l];")
            w("      #pragma unroll")
            w("      for (int i = 0; i < FE_DIM; ++i) Xq[i] += X[l * FE_DIM + i] * ps;")
            w("    }")
    def interp(dst, src, ind, with_dt=False):
        with_dt = with_dt and transient
        w(f"{ind}double {dst}[{nu if with_dt else 'FE_NTC'}];")
        for f, (fname, fsp) in enumerate(fields):
            base = f * nc
            zeros = ", ".join(["0.0"] * dim)
            fdt = with_dt and f in pw.dt_fields
            w(f"{ind}{{ double v = 0.0, gs[FE_DIM] = {{{zeros}}};" + (" double vt = 0.0;" if fdt else ""))
            if fsp == "C2":
                w(f"{ind}  #pragma unroll")
                w(f"{ind}  for (int l = 0; l < FE_NN; ++l) {{")
                w(f"{ind}    const double u = {src}[(el * FE_NN + l) * FE_NVAL + {f}];")
                w(f"{ind}    v += u * sPsi2[q * FE_NN + l];")
                if fdt:
                    w(f"{ind}    vt += sUt[(el * FE_NN + l) * FE_NVAL + {f}] * sPsi2[q * FE_NN + l];")
                w(f"{ind}    #pragma unroll")
                w(f"{ind}    for (int b = 0; b < FE_DIM; ++b) gs[b] += u * dps[l * FE_DIM + b];")
                w(f"{ind}  }}")
            else:
                # C1 nodes by literal element slot (no constant-memory index in the loop)
                w(f"{ind}  const double* ps1 = sPsi1 + q * FE_NN1;")
                w(f"{ind}  const double* dp1 = sDps1 + q * FE_NN1 * FE_DIM;")
                for l, node in enumerate(et.c1_index):
                    w(f"{ind}  {{ const double u = {src}[(el * FE_NN + {node}) * FE_NVAL + {f}];")
                    w(f"{ind}    v += u * ps1[{l}];")
                    if fdt:
                        w(f"{ind}    vt += sUt[(el * FE_NN + {node}) * FE_NVAL + {f}] * ps1[{l}];")
                    for b in range(dim):
                        w(f"{ind}    gs[{b}] += u * dp1[{l * dim + b}];")
                    w(f"{ind}  }}")
            w(f"{ind}  {dst}[{base}] = v;")
            if fdt:
                w(f"{ind}  {dst}[{ntc + f}] = vt;")
            w(f"{ind}  #pragma unroll")
            w(f"{ind}  for (int i = 0; i < FE_DIM; ++i) {{ double s = 0.0;")
            w(f"{ind}    #pragma unroll")
            w(f"{ind}    for (int b = 0; b < FE_DIM; ++b) s += g[b][i] * gs[b];")
            w(f"{ind}    {dst}[{base} + 1 + i] = s; }}")
            w(f"{ind}}}")

    def interp_r():
        # u = u_0 + sum_{l>0} d_l psi_l, grad u = sum_{l>0} d_l grad psi_l
        # (d_l = u_l - u_0 as staged), renormalised every 4 nodes
        w("    fe_df64 gr[FE_DIM][FE_DIM];")
        w("    #pragma unroll")
        w("    for (int b = 0; b < FE_DIM; ++b)")
        w("      #pragma unroll")
        w("      for (int i = 0; i < FE_DIM; ++i) gr[b][i] = fe_df64(g[b][i]);")
        w("    fe_df64 U[FE_NTC];")
        for f, (fname, fsp) in enumerate(fields):
            base = f * nc
            w(f"    {{ fe_df64 v = sUr[(el * FE_NN) * FE_NVAL + {f}];")
            w("      fe_df64 gs[FE_DIM];")
            w("      #pragma unroll")
            w("      for (int b = 0; b < FE_DIM; ++b) gs[b] = fe_df64(0.0f, 0.0f);")
            if fsp == "C2":
                w("      #pragma unroll")
                w("      for (int l = 1; l < FE_NN; ++l) {")
                w(f"        const fe_df64 u = sUr[(el * FE_NN + l) * FE_NVAL + {f}];")
                w("        fe_mac(v, u, sPsi2r[q * FE_NN + l]);")
                w("        #pragma unroll")
                w("        for (int b = 0; b < FE_DIM; ++b) fe_mac(gs[b], u, sDps2r[(q * FE_NN + l) * FE_DIM + b]);")
                w("        if ((l & 3) == 0) {")
                w("          v = fe_norm(v);")
                w("          #pragma unroll")
                w("          for (int b = 0; b < FE_DIM; ++b) gs[b] = fe_norm(gs[b]); }")
                w("      }")
            else:
                w("      const fe_df64* ps1 = sPsi1r + q * FE_NN1;")
                w("      const fe_df64* dp1 = sDps1r + q * FE_NN1 * FE_DIM;")
                for l, node in enumerate(et.c1_index):
                    if l == 0:
                        continue
                    w(f"      {{ const fe_df64 u = sUr[(el * FE_NN + {node}) * FE_NVAL + {f}];")
                    w(f"        fe_mac(v, u, ps1[{l}]);")
                    for b in range(dim):
                        w(f"        fe_mac(gs[{b}], u, dp1[{l * dim + b}]);")
                    if l % 4 == 0:
                        w("        v = fe_norm(v);")
                        for b in range(dim):
                            w(f"        gs[{b}] = fe_norm(gs[{b}]);")
                    w("      }")
            w(f"      U[{base}] = fe_norm(v);")
            w("      #pragma unroll")
            w("      for (int b = 0; b < FE_DIM; ++b) gs[b] = fe_norm(gs[b]);")
            w("      #pragma unroll")
            w("      for (int i = 0; i < FE_DIM; ++i) { fe_df64 s_ = fe_df64(0.0f, 0.0f);")
            w("        #pragma unroll")
            w("        for (int b = 0; b < FE_DIM; ++b) fe_mac(s_, gr[b][i], gs[b]);")
            w(f"        U[{base} + 1 + i] = fe_norm(s_); }}")
            w("    }")

    if rdf and sfi:
        # value = u_0 + the interpolated differences; gradients from phase I
        w("    fe_df64 gr[FE_DIM][FE_DIM];")
        w("    #pragma unroll")
        w("    for (int b = 0; b < FE_DIM; ++b)")
        w("      #pragma unroll")
        w("      for (int i = 0; i < FE_DIM; ++i) gr[b][i] = fe_df64(g[b][i]);")
        w("    fe_df64 U[FE_NTC];")
        w(f"    {{ const fe_df64* C = reinterpret_cast<const fe_df64*>(sIc) + el * {SC} + q;")
        w("      U[0] = C[0] + sUr[(el * FE_NN) * FE_NVAL];")
        w("      const fe_df64 gs[3] = {C[27], C[54], C[81]};")
        w("      #pragma unroll")
        w("      for (int i = 0; i < FE_DIM; ++i) { fe_df64 s_ = fe_df64(0.0f, 0.0f);")
        w("        #pragma unroll")
        w("        for (int b = 0; b < FE_DIM; ++b) fe_mac(s_, gr[b][i], gs[b]);")
        w("        U[1 + i] = fe_norm(s_); }")
        w("    }")
    elif rdf:
        interp_r()
    elif sfi:
        w(f"    double U[{nu if transient else 'FE_NTC'}];")
        w(f"    {{ const double* C = sIc + el * {SC} + q;")
        w("      const double gs[3] = {C[27], C[54], C[81]};")
        w("      U[0] = C[0];")
        w("      #pragma unroll")
        w("      for (int i = 0; i < FE_DIM; ++i) { double s = 0.0;")
        w("        #pragma unroll")
        w("        for (int b = 0; b < FE_DIM; ++b) s += g[b][i] * gs[b];")
        w("        U[1 + i] = s; }")
        w("    }")
        if transient:
            # du/dt at the knot: the value only, one plain pass over the nodes
            w("    { double vt = 0.0;")
            w("      #pragma unroll")
            w("      for (int l = 0; l < FE_NN; ++l) vt += sUt[(el * FE_NN + l) * FE_NVAL] * sPsi2[q * FE_NN + l];")
            w(f"      U[{ntc}] = vt; }}")
    else:
        interp("U", "sU", "    ", with_dt=True)
    w("    const double* Pe = a.params + (a.replica_elems > 0 ? ((e0 + el) / a.replica_elems) * a.params_stride : 0);")
    if rdf:
        w(f"    fe_df64 r[FE_NTC]; {'fe_df64' if df64 else 'jreal'} D[FE_NDNZ];")
        w("    if (dpar) {")
        w("      double Ud[FE_NTC], rt[FE_NTC];")
        w("      #pragma unroll")
        w("      for (int k = 0; k < FE_NTC; ++k) Ud[k] = fe_widen(U[k]);")
        w("      fe_pointwise_dparam(Ud, Xq, Pe, rt, a.aux);")
        w("      #pragma unroll")
        w("      for (int k = 0; k < FE_NTC; ++k) r[k] = fe_df64(rt[k]);")
        if gsep:
            w("    } else {")
            w("      int qI[FE_DIM];")
            w("      { int qq = q;")
            w("        #pragma unroll")
            w("        for (int d = FE_DIM - 1; d >= 0; --d) { qI[d] = qq % 3; qq /= 3; } }")
            w(f"      fe_pointwise(U, Xq, Pe, r, D, flag, sGe + el * {gsd}, qI);")
            w("    }")
        else:
            w("    } else fe_pointwise(U, Xq, Pe, r, D, flag, nullptr, nullptr);")
        w("    fe_df64* rh = sRhr + (el * FE_NQ + q) * FE_NTC;")
        w("    const fe_df64 wqr = fe_df64(wq);")
        w("    #pragma unroll")
        w("    for (int f = 0; f < FE_NF; ++f) {")
        w("      rh[f * (1 + FE_DIM)] = wqr * r[f * (1 + FE_DIM)];")
        w("      #pragma unroll")
        w("      for (int b = 0; b < FE_DIM; ++b) { fe_df64 s_ = fe_df64(0.0f, 0.0f);")
        w("        #pragma unroll")
        w("        for (int i = 0; i < FE_DIM; ++i) fe_mac(s_, gr[b][i], r[f * (1 + FE_DIM) + 1 + i]);")
        w("        rh[f * (1 + FE_DIM) + 1 + b] = wqr * fe_norm(s_); }")
        w("    }")
    else:
        w("    double r[FE_NTC]; jreal D[FE_NDNZ];")
    if rdf:
        pass
    elif gsep:
        w("    int qI[FE_DIM];")
        w("    { int qq = q;")
        w("      #pragma unroll")
        w("      for (int d = FE_DIM - 1; d >= 0; --d) { qI[d] = qq % 3; qq /= 3; } }")
        w(f"    if (dpar) fe_pointwise_dparam(U, Xq, Pe, r, a.aux);")
        w(f"    else fe_pointwise(U, Xq, Pe, r, D, flag, sGe + el * {gsd}, qI);")
    else:
        w("    if (dpar) fe_pointwise_dparam(U, Xq, Pe, r, a.aux);")
        w("    else fe_pointwise(U, Xq, Pe, r, D, flag, nullptr, nullptr);")
    if not rdf:
        w("    double* rh = sRh + (el * FE_NQ + q) * FE_NTC;")
        w("    #pragma unroll")
        w("    for (int f = 0; f < FE_NF; ++f) {")
        w("      rh[f * (1 + FE_DIM)] = wq * r[f * (1 + FE_DIM)];")
        w("      #pragma unroll")
        w("      for (int b = 0; b < FE_DIM; ++b) { double s = 0.0;")
        w("        #pragma unroll")
        w("        for (int i = 0; i < FE_DIM; ++i) s += g[b][i] * r[f * (1 + FE_DIM) + 1 + i];")
        w("        rh[f * (1 + FE_DIM) + 1 + b] = wq * s; }")
        w("    }")
    w("    if (flag) {")
    if jreal == "float":
        w("      if (flag != 4) fe_pointwise_jac(U, Xq, Pe, D, flag);")
    w("      if (flag == 4) {")
    interp("V", "sY", "        ")
    if rdf:
        w("        double Ud[FE_NTC];")
        w("        #pragma unroll")
        w("        for (int k = 0; k < FE_NTC; ++k) Ud[k] = fe_widen(U[k]);")
        if df64:
            w("        double Dh[FE_NDNZ];")
            w("        fe_pointwise_hvp(Ud, V, Xq, Pe, Dh);")
            w("        #pragma unroll")
            w("        for (int k = 0; k < FE_NDNZ; ++k) D[k] = fe_df64(Dh[k]);")
        else:
            w("        fe_pointwise_hvp(Ud, V, Xq, Pe, D);")
    else:
        w("        fe_pointwise_hvp(U, V, Xq, Pe, D);")
    w("      }")
    w("      const jreal wj = (jreal)wq;")
    if jref:
        # Dhat = T^T D T, T = diag(1, g) per field: d/dx_i = sum_b g[b][i] d/ds_b
        # (df64: the pull-back itself in double-float -- D, g and the weight
        # are converted once, the products run on the FP32 pipes)
        w("      jacc* Dq = sD + (el * FE_NQ + q) * FE_NDNZH;")
        tT = "jacc" if df64 else "jreal"
        w(f"      {tT} T[FE_DIM][FE_DIM];")
        w("      #pragma unroll")
        w("      for (int i = 0; i < FE_DIM; ++i)")
        w("        #pragma unroll")
        w(f"        for (int b = 0; b < FE_DIM; ++b) T[i][b] = ({tT})g[b][i];")
        dsym = "D"
        if df64:
            w("      jacc Dd[FE_NDNZ];")
            w("      #pragma unroll")
            w("      for (int k = 0; k < FE_NDNZ; ++k) Dd[k] = (jacc)D[k];")
            w("      const jacc wjd = (jacc)wq;")
            dsym = "Dd"

        def cT(a_, h_):
            if a_ == 0 and h_ == 0:
                return ""
            if a_ == 0 or h_ == 0:
                return None
            return f"T[{a_ - 1}][{h_ - 1}]"
        for kk, (tf_, gf_, ah, bh) in enumerate(hat):
            terms = []
            for a_, b_, k in blocks[(tf_, gf_)]:
                ca, cb = cT(a_, ah), cT(b_, bh)
                if ca is None or cb is None:
                    continue
                terms.append(" * ".join([x_ for x_ in (ca, f"{dsym}[{k}]", cb) if x_]))
            if df64:
                w(f"      Dq[{kk}] = {'wjd * (' + ' + '.join(terms) + ')' if terms else '(jacc)0'};")
            else:
                w(f"      Dq[{kk}] = (jacc)(wj * ({' + '.join(terms) if terms else '(jreal)0'}));")
    else:
        w("      jreal* Dq = sD + (el * FE_NQ + q) * FE_NDNZ;")
        w("      #pragma unroll")
        w("      for (int k = 0; k < FE_NDNZ; ++k) Dq[k] = wj * D[k];")
        w("      fe_phys_grad<FE_DIM, FE_NN, jreal>(g, dps, sDx2 + (el * FE_NQ + q) * FE_NN * FE_DIM);")
        if has_c1:
            w("      fe_phys_grad<FE_DIM, FE_NN1, jreal>(g, sDps1 + q * FE_NN1 * FE_DIM, sDx1 + (el * FE_NQ + q) * FE_NN1 * FE_DIM);")
    w("    }")
    w("  }")
    w("  __syncthreads();")
    if use_tc:
        # ---------------- phase T: Dhat out, for the tensor-core contraction ----------------
        w("  if (flag == 1 || flag == 4) {")
        w("    if (a.dhat == nullptr) {")
        w("      if (threadIdx.x == 0) atomicExch(a.status, 4);   // no contraction buffer attached")
        w("    } else {")
        w("      float* dh = a.dhat + e0 * (FE_NQ * FE_NDNZH);")
        w("      for (int k = threadIdx.x; k < nel * FE_NQ * FE_NDNZH; k += FE_NT) dh[k] = sD[k];")
        w("    }")
        w("  }")
    if sfi and rdf:
        SA, SB, SC = sfs
        # ---------------- phase R (double-float): sum-factorised residual ----------------
        w("  { fe_df64* Ia = reinterpret_cast<fe_df64*>(sIa); fe_df64* Ib = reinterpret_cast<fe_df64*>(sIb);")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // knot axis 2 -> node i2: T0, T1, T2 [q0][q1][i2]")
        w("    const int el = p / 27, o = p - el * 27, q0 = o / 9, q1 = (o / 3) % 3, i2 = o % 3;")
        w("    const fe_df64* rh = sRhr + (el * FE_NQ + q0 * 9 + q1 * 3) * FE_NTC;")
        w("    fe_df64 t0 = fe_df64(0.0f, 0.0f), t1 = t0, t2 = t0;")
        w("    #pragma unroll")
        w("    for (int q2 = 0; q2 < 3; ++q2) {")
        w("      const fe_df64* r = rh + q2 * FE_NTC;")
        w("      const fe_df64 m0 = sMr[q2 * 3 + i2], m1 = sMr[9 + q2 * 3 + i2];")
        w("      fe_mac(t0, r[3], m1); fe_mac(t0, r[0], m0); fe_mac(t1, r[1], m0); fe_mac(t2, r[2], m0); }")
        w(f"    Ib[el * {SB} + o] = fe_norm(t0); Ib[el * {SB} + 27 + o] = fe_norm(t1); Ib[el * {SB} + 54 + o] = fe_norm(t2);")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // knot axis 1 -> node i1: S0, S1 [q0][i1][i2]")
        w("    const int el = p / 27, o = p - el * 27, q0 = o / 9, i1 = (o / 3) % 3, i2 = o % 3;")
        w(f"    const fe_df64* T = Ib + el * {SB} + q0 * 9 + i2;")
        w("    fe_df64 s0 = fe_df64(0.0f, 0.0f), s1 = s0;")
        w("    #pragma unroll")
        w("    for (int q1 = 0; q1 < 3; ++q1) {")
        w("      const fe_df64 m0 = sMr[q1 * 3 + i1], m1 = sMr[9 + q1 * 3 + i1];")
        w("      fe_mac(s0, T[54 + q1 * 3], m1); fe_mac(s0, T[q1 * 3], m0); fe_mac(s1, T[27 + q1 * 3], m0); }")
        w(f"    Ia[el * {SA} + o] = fe_norm(s0); Ia[el * {SA} + 27 + o] = fe_norm(s1);")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // knot axis 0 -> node i0: R at node l")
        w("    const int el = p / 27, l = p - el * 27, i0 = l % 3, i1 = (l / 3) % 3, i2 = l / 9;")
        w(f"    const fe_df64* S = Ia + el * {SA} + i1 * 3 + i2;")
        w("    fe_df64 r = fe_df64(0.0f, 0.0f);")
        w("    #pragma unroll")
        w("    for (int q0 = 0; q0 < 3; ++q0) { fe_mac(r, S[27 + q0 * 9], sMr[9 + q0 * 3 + i0]); fe_mac(r, S[q0 * 9], sMr[q0 * 3 + i0]); }")
        w("    a.rbuf[(e0 + el) * FE_NLOC + l] = fe_widen(fe_norm(r));")
        w("  }")
        w("  __syncthreads(); }")
    elif sfi:
        SA, SB, SC = sfs
        # ---------------- phase R: sum-factorised residual ----------------
        # R_l = sum_q [rh0 psi_l + rh1 d0psi_l + rh2 d1psi_l + rh3 d2psi_l], one axis at a time
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // knot axis 2 -> node i2: T0, T1, T2 [q0][q1][i2]")
        w("    const int el = p / 27, o = p - el * 27, q0 = o / 9, q1 = (o / 3) % 3, i2 = o % 3;")
        w("    const double* rh = sRh + (el * FE_NQ + q0 * 9 + q1 * 3) * FE_NTC;")
        w("    double t0 = 0.0, t1 = 0.0, t2 = 0.0;")
        w("    #pragma unroll")
        w("    for (int q2 = 0; q2 < 3; ++q2) {")
        w("      const double* r = rh + q2 * FE_NTC;")
        w("      const double m0 = sM[q2 * 3 + i2], m1 = sM[9 + q2 * 3 + i2];")
        w("      t0 = fma(r[0], m0, fma(r[3], m1, t0)); t1 = fma(r[1], m0, t1); t2 = fma(r[2], m0, t2); }")
        w(f"    sIb[el * {SB} + o] = t0; sIb[el * {SB} + 27 + o] = t1; sIb[el * {SB} + 54 + o] = t2;")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // knot axis 1 -> node i1: S0, S1 [q0][i1][i2]")
        w("    const int el = p / 27, o = p - el * 27, q0 = o / 9, i1 = (o / 3) % 3, i2 = o % 3;")
        w(f"    const double* T = sIb + el * {SB} + q0 * 9 + i2;")
        w("    double s0 = 0.0, s1 = 0.0;")
        w("    #pragma unroll")
        w("    for (int q1 = 0; q1 < 3; ++q1) {")
        w("      const double m0 = sM[q1 * 3 + i1], m1 = sM[9 + q1 * 3 + i1];")
        w("      s0 = fma(T[q1 * 3], m0, fma(T[54 + q1 * 3], m1, s0)); s1 = fma(T[27 + q1 * 3], m0, s1); }")
        w(f"    sIa[el * {SA} + o] = s0; sIa[el * {SA} + 27 + o] = s1;")
        w("  }")
        w("  __syncthreads();")
        w("  for (int p = threadIdx.x; p < nel * 27; p += FE_NT) {  // knot axis 0 -> node i0: R at node l")
        w("    const int el = p / 27, l = p - el * 27, i0 = l % 3, i1 = (l / 3) % 3, i2 = l / 9;")
        w(f"    const double* S = sIa + el * {SA} + i1 * 3 + i2;")
        w("    double r = 0.0;")
        w("    #pragma unroll")
        w("    for (int q0 = 0; q0 < 3; ++q0)")
        w("      r = fma(S[q0 * 9], sM[q0 * 3 + i0], fma(S[27 + q0 * 9], sM[9 + q0 * 3 + i0], r));")
        w("    a.rbuf[(e0 + el) * FE_NLOC + l] = r;")
        w("  }")
        w("  __syncthreads();")
    if sumfac:
        # ---------------- phase B': sum-factorised Jacobian, one (a, b) block at a time ----------------
        w("  if (flag) {")
        for kk, (_, _, ah, bh) in enumerate(hat):
            cx = 2 * (ah == 1) + (bh == 1)
            cy = 2 * (ah == 2) + (bh == 2)
            cz = 2 * (ah == 3) + (bh == 3)
            w(f"    // block (a={ah}, b={bh})")
            w("    for (int p = threadIdx.x; p < nel * 81; p += FE_NT) {")
            w("      const int el = p / 81, o = p - el * 81, qxy = o / 9, izjz = o - qxy * 9;")
            w("      const int iz = izjz / 3, jz = izjz - iz * 3;")
            w("      const jacc* Dq = sD + (el * FE_NQ + 3 * qxy) * FE_NDNZH;")
            w(f"      const jacc* F = sF + {cz * 27} + iz * 3 + jz;")
            if df64:
                w(f"      jacc t = (jacc)0; fe_mac(t, F[0], Dq[{kk}]); fe_mac(t, F[9], Dq[FE_NDNZH + {kk}]);")
                w(f"      fe_mac(t, F[18], Dq[2 * FE_NDNZH + {kk}]); sS1[p] = fe_norm(t);")
            else:
                w(f"      sS1[p] = F[0] * Dq[{kk}] + F[9] * Dq[FE_NDNZH + {kk}] + F[18] * Dq[2 * FE_NDNZH + {kk}];")
            w("    }")
            w("    __syncthreads();")
            w("    for (int p = threadIdx.x; p < nel * 243; p += FE_NT) {")
            w("      const int el = p / 243, o = p - el * 243, qx = o / 81, r = o - qx * 81, iyjy = r / 9;")
            w("      const int izjz = r - iyjy * 9, iy = iyjy / 3, jy = iyjy - iy * 3;")
            w("      const jacc* S1 = sS1 + el * 81 + qx * 27 + izjz;")
            w(f"      const jacc* F = sF + {cy * 27} + iy * 3 + jy;")
            if df64:
                w("      jacc t = (jacc)0; fe_mac(t, F[0], S1[0]); fe_mac(t, F[9], S1[9]); fe_mac(t, F[18], S1[18]);")
                w("      sS2[p] = fe_norm(t);")
            else:
                w("      sS2[p] = F[0] * S1[0] + F[9] * S1[9] + F[18] * S1[18];")
            w("    }")
            w("    __syncthreads();")
            w("    for (int p = threadIdx.x; p < nel * 729; p += FE_NT) {")
            w("      const int el = p / 729, o = p - el * 729, i = o / 27, j = o - i * 27;")
            w("      const int ix = i % 3, iy = (i / 3) % 3, iz = i / 9, jx = j % 3, jy = (j / 3) % 3, jz = j / 9;")
            w("      const jacc* S2 = sS2 + el * 243 + (iy * 3 + jy) * 9 + iz * 3 + jz;")
            w(f"      const jacc* F = sF + {cx * 27} + ix * 3 + jx;")
            if df64:
                # one accumulator over all (a, b) blocks: each thread owns its entries
                w(f"      jacc v = {'(jacc)0' if kk == 0 else 'sJe[p]'};")
                w("      fe_mac(v, F[0], S2[0]); fe_mac(v, F[9], S2[81]); fe_mac(v, F[18], S2[162]);")
                w("      sJe[p] = fe_norm(v);")
            elif kk == 0:
                w("      sJe[p] = F[0] * S2[0] + F[9] * S2[81] + F[18] * S2[162];")
            else:
                w("      sJe[p] = fe_fma(F[18], S2[162], fe_fma(F[9], S2[81], fe_fma(F[0], S2[0], sJe[p])));")
            w("    }")
            w("    __syncthreads();")
        w("  }")
    # ---------------- phase B: field-major rows ----------------
    if use_tc and sfi:
        # the residual came from phase R, the Jacobian comes from the tensor cores
        w("}")
        source = "\n".join(src) + "\n"
        return KernelSpec(name=name, source=source, et=et, layout=layout, pointwise=pw, epb=epb,
                          threads=threads, smem_bytes=smem, jac_precision=jac_precision,
                          tables=et.packed_tables(), sumfac_blocks=0, gauss_sep=gs_n if gsep else 0,
                          sum_fact_interp=sfi, tc_pairs=[(ah, bh) for (_, _, ah, bh) in hat],
                          min_blocks=int(min_blocks or 0), residual_precision=residual_precision)
    w("  for (int p = threadIdx.x; p < nel * FE_NLOC; p += FE_NT) {")
    w("    int tf = 0, rel = p;")
    for f in range(nf - 1):
        w(f"    if (tf == {f} && rel >= nel * {nsub[f]}) {{ rel -= nel * {nsub[f]}; tf = {f + 1}; }}")
    w("    int tn = 0, toff = 0;")
    for f in range(nf):
        w(f"    if (tf == {f}) {{ tn = {nsub[f]}; toff = {loc_off[f]}; }}")
    w("    const int el = rel / tn, lt = rel - el * tn;")
    w("    const int i = c_loc_of[toff + lt];")
    w("    const int t1 = (tn == FE_NN1) && (FE_NN1 != FE_NN) ? 1 : 0;")
    if not has_c1:
        w("    (void)t1;")
    w("    const double* tpsi = t1 ? sPsi1 : sPsi2;")
    w("    const double* tdps = t1 ? sDps1 : sDps2;")
    if rdf and not sfi:
        w("    const fe_df64* tpsir = t1 ? sPsi1r : sPsi2r;")
        w("    const fe_df64* tdpsr = t1 ? sDps1r : sDps2r;")
        w("    (void)tpsi; (void)tdps;")
        w("    fe_df64 Racc = fe_df64(0.0f, 0.0f);")
    else:
        w("    double Racc = 0.0;")
    w("    jacc Jr[FE_NLOC];")
    w("    #pragma unroll")
    w("    for (int k = 0; k < FE_NLOC; ++k) Jr[k] = (jacc)0;")
    if sfi:
        w("    (void)Racc; (void)tpsi; (void)tdps;")
    # (sum-factorised Jacobian and residual: nothing is left per knot here)
    w(f"    for (int q = 0; q < {'0' if (sfi and sumfac) else 'FE_NQ'}; ++q) {{")
    if rdf and not sfi:
        w("      const fe_df64* rh = sRhr + (el * FE_NQ + q) * FE_NTC + tf * (1 + FE_DIM);")
        w("      fe_mac(Racc, rh[0], tpsir[q * tn + lt]);")
        w("      #pragma unroll")
        w("      for (int b = 0; b < FE_DIM; ++b) fe_mac(Racc, rh[1 + b], tdpsr[(q * tn + lt) * FE_DIM + b]);")
        w("      Racc = fe_norm(Racc);")
    elif not sfi:
        w("      const double* rh = sRh + (el * FE_NQ + q) * FE_NTC + tf * (1 + FE_DIM);")
        w("      const double pv = tpsi[q * tn + lt];")
        w("      double racc = rh[0] * pv;")
        w("      #pragma unroll")
        w("      for (int b = 0; b < FE_DIM; ++b) racc += rh[1 + b] * tdps[(q * tn + lt) * FE_DIM + b];")
        w("      Racc += racc;")
    if sumfac or use_tc:
        pass
    elif jref:
        w("      if (flag) {")
        w("        const jacc* Dq = sD + (el * FE_NQ + q) * FE_NDNZH;")
        w(f"        const {tabt}* tpj = t1 ? (sPsi1j + q * FE_NN1) : (sPsi2j + q * FE_NN);")
        w(f"        const {tabt}* tdj = t1 ? (sDps1j + (q * FE_NN1 + lt) * FE_DIM) : (sDps2j + (q * FE_NN + lt) * FE_DIM);")
        w("        const jacc phi0 = (jacc)tpj[lt];")
        for d in range(dim):
            w(f"        const jacc phi{d + 1} = (jacc)tdj[{d}];")
        used_h = sorted({(gf_, bh) for (_, gf_, _, bh) in hat})
        for gf_, bh in used_h:
            w(f"        jacc h{gf_}_{bh} = (jacc)0;")
        for f in range(nf):
            ents = [(kk, ah, gf_, bh) for kk, (tf_, gf_, ah, bh) in enumerate(hat) if tf_ == f]
            if not ents:
                continue
            w(f"        if (tf == {f}) {{")
            for kk, ah, gf_, bh in ents:
                if df64:
                    w(f"          fe_mac(h{gf_}_{bh}, phi{ah}, Dq[{kk}]);")
                else:
                    w(f"          h{gf_}_{bh} += phi{ah} * Dq[{kk}];")
            w("        }")
        if df64:
            for gf_, bh in used_h:
                w(f"        h{gf_}_{bh} = fe_norm(h{gf_}_{bh});")
        for f, (fname, fsp) in enumerate(fields):
            comps = [bh for (gf_, bh) in used_h if gf_ == f]
            if not comps:
                continue
            w("        {")
            if fsp == "C2":
                w(f"          const {tabt}* psi = sPsi2j + q * FE_NN;")
                w(f"          const {tabt}* dps_ = sDps2j + q * FE_NN * FE_DIM;")
                cnt = nn
            else:
                w(f"          const {tabt}* psi = sPsi1j + q * FE_NN1;")
                w(f"          const {tabt}* dps_ = sDps1j + q * FE_NN1 * FE_DIM;")
                cnt = nn1
            for ls in range(cnt):
                terms = []
                for bh in comps:
                    if bh == 0:
                        terms.append((f"h{f}_0", f"(jacc)psi[{ls}]"))
                    else:
                        terms.append((f"h{f}_{bh}", f"(jacc)dps_[{ls * dim + bh - 1}]"))
                if df64:
                    # renormalised after each group of multiply-adds: the
                    # compensation word's error then grows linearly, not
                    # quadratically, with the number of knots
                    col = layout.loc_of[f][ls]
                    w("          " + " ".join(f"fe_mac(Jr[{col}], {x_}, {y_});" for x_, y_ in terms)
                      + f" Jr[{col}] = fe_norm(Jr[{col}]);")
                else:
                    w(f"          Jr[{layout.loc_of[f][ls]}] {_jacc_update(terms, f'Jr[{layout.loc_of[f][ls]}]', jacc)};")
            w("        }")
    else:
        w("      if (flag) {")
        w("        const jreal* Dq = sD + (el * FE_NQ + q) * FE_NDNZ;")
        w("        const jreal* tdx = t1 ? (sDx1 + ((el * FE_NQ + q) * FE_NN1 + lt) * FE_DIM)")
        w("                             : (sDx2 + ((el * FE_NQ + q) * FE_NN + lt) * FE_DIM);")
        w("        const jreal phi0 = (jreal)pv;")
        for d in range(dim):
            w(f"        const jreal phi{d + 1} = tdx[{d}];")
        for ic in used_ic:
            w(f"        jreal a{ic} = (jreal)0;")
        # per test field: only its own D entries (warp-uniform branch)
        for f in range(nf):
            ents = [(k, tc, ic) for k, (tc, ic, _) in enumerate(pw.d_entries) if tc // nc == f]
            if not ents:
                continue
            w(f"        if (tf == {f}) {{")
            for k, tc, ic in ents:
                w(f"          a{ic} += phi{tc % nc} * Dq[{k}];")
            w("        }")
        for f, (fname, fsp) in enumerate(fields):
            comps = [ic for ic in used_ic if ic // nc == f]
            if not comps:
                continue
            if fsp == "C2":
                w("        {")
                w("          const double* psi = sPsi2 + q * FE_NN;")
                w("          const jreal* dx = sDx2 + (el * FE_NQ + q) * FE_NN * FE_DIM;")
                cnt = nn
            else:
                w("        {")
                w("          const double* psi = sPsi1 + q * FE_NN1;")
                w("          const jreal* dx = sDx1 + (el * FE_NQ + q) * FE_NN1 * FE_DIM;")
                cnt = nn1
            for ls in range(cnt):
                terms = []
                for ic in comps:
                    c = ic % nc
                    if c == 0:
                        terms.append((f"a{ic}", f"(jreal)psi[{ls}]"))
                    else:
                        terms.append((f"a{ic}", f"dx[{ls * dim + c - 1}]"))
                w(f"          Jr[{layout.loc_of[f][ls]}] {_jacc_update(terms, f'Jr[{layout.loc_of[f][ls]}]', jacc)};")
            w("        }")
    if not (sumfac or use_tc):
        w("      }")
    w("    }")
    w("    const long long row = (e0 + el) * FE_NLOC + i;")
    if rdf and not sfi:
        w("    a.rbuf[row] = fe_widen(Racc);")
    elif not sfi:
        w("    a.rbuf[row] = Racc;")
    w("    if (flag && !" + ("true" if use_tc else "false") + ") {")
    w("      jstore* jb = reinterpret_cast<jstore*>(a.jbuf) + row * FE_NLOC;")
    if sumfac:
        w("      const jacc* Jrow = sJe + el * 729 + i * 27;")
        w("      for (int k = 0; k < FE_NLOC; ++k) jb[k] = fe_jstore(Jrow[k]);")
    else:
        w("      #pragma unroll")
        w("      for (int k = 0; k < FE_NLOC; ++k) jb[k] = fe_jstore(Jr[k]);")
    w("    }")
    w("  }")
    w("}")
    source = "\n".join(src) + "\n"
    return KernelSpec(name=name, source=source, et=et, layout=layout, pointwise=pw, epb=epb,
                      threads=threads, smem_bytes=smem, jac_precision=jac_precision,
                      tables=et.packed_tables(), sumfac_blocks=len(hat) if sumfac else 0,
                      gauss_sep=gs_n if gsep else 0, sum_fact_interp=sfi,
                      tc_pairs=[(ah, bh) for (_, _, ah, bh) in hat] if use_tc else None,
                      min_blocks=int(min_blocks or 0), residual_precision=residual_precision)


def _jacc_update(terms, acc: str, jacc: str) -> str:
    """The right-hand side of a Jacobian accumulator update acc += sum x*y.
    FP64 (bound by FP64 issue on GB300): nested fused multiply-adds into the
    accumulator, one FP64 add fewer than adding a separate sum of products
    (NS 256^2 2.06 -> 1.72 ms).  FP32 (latency-bound): the sum of products
    formed apart and added once, which keeps the accumulator's dependency
    chain short (the nested form measured 0.48 -> 0.62 ms)."""
    if jacc == "double":
        out = acc
        for x_, y_ in terms:
            out = f"fe_fma({x_}, {y_}, {out})"
        return "= " + out
    return "+= " + " + ".join(f"{x_} * {y_}" for x_, y_ in terms)


def estimate_flops(ks: KernelSpec, affine: bool) -> Dict[str, float]:
    """Floating-point operations per element of a generated kernel, counted
    from its structure (an FMA counts 2).  Keys: ``fp64`` (geometry,
    interpolation, pointwise residual, residual contraction; plus the
    Jacobian when it is FP64, its D and pull-back when it is df64), ``jac``
    (the Jacobian-only work) and, for df64, ``df64`` (the contraction done in
    double-float).  With the double-float residual, ``df64_residual`` holds
    the residual path's flops (done in double-float, counted as the FP64
    flops they replace) and ``fp64`` the geometry only."""
    et, pw, lay = ks.et, ks.pointwise, ks.layout
    D, NN, N1, NQ = et.dim, et.nnode, et.nnode_c1, et.nq
    nc = 1 + D
    fields = pw.fields
    geo = 2 * NN * D * D + 2 * D ** 3 + (D ** 3 + 10) + 2 * D ** 3 + 10
    per_q = 0.0 if affine else geo
    if pw.uses_x:
        per_q += 2 * (N1 if affine else NN) * D
    for _, s in fields:
        n = NN if s == "C2" else N1
        # sum-factorised: the interpolation stages are counted per element below
        per_q += (0 if ks.sum_fact_interp else 2 * n * nc) + 2 * D * D
    ops_r = 0
    for e in pw.r_exprs:
        gs = list(e.atoms(E.GaussianSum))
        for g in gs:
            k0 = next(i for i, a in enumerate(g.args) if a.is_Integer)
            # separable: D products and a sum per Gaussian and knot (the
            # factors are counted per element below)
            ops_r += int(g.args[k0]) * ((D + 1) if ks.gauss_sep else (3 * D + 45))
        ops_r += sp.count_ops(e.subs({g: 0 for g in gs}))
    per_q += ops_r
    per_q += len(fields) * (1 + 2 * D * D)
    rows = lay.n
    # residual contraction; sum-factorised: 3 stages of 27 x (12, 9, 6) FMAs,
    # plus the 3 interpolation stages of 27 x (6, 9, 12) FMAs
    resid = 2 * 27 * (12 + 9 + 6) * 2 if ks.sum_fact_interp else rows * NQ * 2 * nc
    fp64 = NQ * per_q + (geo if affine else 0) + resid
    if ks.gauss_sep:
        # per element: 3 D factors per Gaussian (the affine map along the axis, exp)
        fp64 += ks.gauss_sep * D * 3 * (2 * N1 + 48)
    ops_d = sum(sp.count_ops(d) for (_, _, d) in pw.d_entries)
    jac_q = ops_d + len(pw.d_entries) + 2 * NN * D * D + (2 * N1 * D * D if any(s == "C1" for _, s in fields) else 0)
    used_ic = sorted({ic for (_, ic, _) in pw.d_entries})
    per_row_q = 0.0
    for f, (_, s) in enumerate(fields):
        comps = [ic for ic in used_ic if ic // nc == f]
        per_row_q += 2 * (NN if s == "C2" else N1) * len(comps)
    a_ops = 2 * len(pw.d_entries) / max(1, len(fields))
    jac_a = NQ * jac_q                              # D and its pull-back, per knot
    jac_b = rows * NQ * (per_row_q + a_ops)         # the contraction into J
    if ks.sumfac_blocks:
        # pulled-back D per knot, then per (a, b) block 3 x (81 + 243 + 729) multiply-adds
        jac_a = NQ * (ops_d + 4 * ks.sumfac_blocks)
        jac_b = ks.sumfac_blocks * 2 * 3 * (81 + 243 + 729)
    if ks.tc_pairs:
        # the contraction on the tensor cores: A = Dhat Phi built in FP32
        # (2 flops per pair, knot and trial function), then the useful
        # multiply-adds of J_e = Phi^T A (rows x rows x knots x active test
        # components); each one runs as three TF32 products
        nact = len({a_ for a_, _ in ks.tc_pairs})
        jac_b = rows * NQ * len(ks.tc_pairs) * 2
        out = {"fp64": float(fp64), "jac": float(jac_a + jac_b),
               "tensor": float(2 * rows * rows * NQ * nact),
               "tensor_issued": float(3 * 2 * 128 // 4 * 32 * (-(-(NQ * nact) // 8) * 8))}
        return out
    out = {"fp64": float(fp64), "jac": float(jac_a + jac_b)}
    if ks.residual_precision == "df64":
        geo_only = float(geo if affine else NQ * geo)
        out["df64_residual"] = float(fp64) - geo_only
        out["fp64"] = geo_only
        if ks.jac_precision == "df64":
            out["df64"] = float(jac_a + jac_b)
        return out
    if ks.jac_precision == "f64":
        out["fp64"] += out["jac"]
    elif ks.jac_precision == "df64":
        # D in FP64; the contraction in double-float on the FP32 pipes
        # (counted as the FP64 flops it replaces)
        out["fp64"] += float(jac_a)
        out["df64"] = float(jac_b)
    return out
