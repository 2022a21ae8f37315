"""CPU emulation of a generated element kernel (test infrastructure).

The generated kernels run their phases as block-strided loops
``for (p = threadIdx.x; p < n; p += FE_NT)`` separated by __syncthreads().
Compiled as plain C++ with FE_NT = 1 and threadIdx = 0, one host thread runs
every iteration of each phase in order, which is exactly the block's
result.  This lets the CPU test suite check the generated code element by
element against the oracle without a GPU.  It is never part of the product.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pyoomph_gb300", "csrc")
OUT = os.path.join(ROOT, "_build", "emu")

PRELUDE = r"""
#include <math.h>
#include <cmath>
#include <cstring>
struct fe_emu_dim3 { unsigned x, y, z; };
static fe_emu_dim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, gridDim = {1, 1, 1};
#define __global__
#define __device__
#define __host__
#define __constant__ static
#define __forceinline__ inline
#define __noinline__
#define __launch_bounds__(...)
#define __restrict__ __restrict
#define __align__(n) alignas(n)
#define __syncthreads() do {} while (0)
#define __shared__
static inline int atomicExch(int *p, int v) { int o = *p; *p = v; return o; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline long long __double_as_longlong(double d) { long long u; std::memcpy(&u, &d, 8); return u; }
static inline double __longlong_as_double(long long u) { double d; std::memcpy(&d, &u, 8); return d; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
alignas(16) unsigned char fe_smem[232448];
"""


def _headers() -> str:
    """The device headers the generated code includes (part of the cache key:
    a changed argument block must rebuild every emulator library)."""
    out = ""
    for f in ("fe_abi.h", "fe_device.cuh", "fe_df64.cuh"):
        with open(os.path.join(CSRC, f)) as fp:
            out += fp.read()
    return out


class _Args(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("conn", ctypes.c_void_p), ("values", ctypes.c_void_p),
                ("params", ctypes.c_void_p), ("tables", ctypes.c_void_p), ("rbuf", ctypes.c_void_p),
                ("jbuf", ctypes.c_void_p), ("n_elem", ctypes.c_longlong), ("nval", ctypes.c_int),
                ("flag", ctypes.c_int), ("status", ctypes.c_void_p), ("replica_elems", ctypes.c_longlong),
                ("params_stride", ctypes.c_int), ("hist", ctypes.c_void_p), ("x0", ctypes.c_void_p),
                ("n_hist", ctypes.c_int), ("hist_stride", ctypes.c_longlong), ("aux", ctypes.c_int), ("n_nodes", ctypes.c_longlong), ("dir", ctypes.c_void_p),
                ("dhat", ctypes.c_void_p)]


def build(ks) -> ctypes.CDLL:
    src = re.sub(r"#define FE_NT \d+", "#define FE_NT 1", ks.source)
    src = src.replace("extern __shared__ __align__(16) unsigned char fe_smem[];", "")
    body = PRELUDE + src + (
        f'\nextern "C" void fe_emu_run(const FeElemArgs *a, int nblocks) {{\n'
        f'  for (int b = 0; b < nblocks; ++b) {{\n'
        f'    memset(fe_smem, 0xff, sizeof(fe_smem)); /* NaN garbage: uninitialised reads show */\n'
        f'    blockIdx.x = b; {ks.name}(*a); }}\n}}\n')
    h = hashlib.sha1((body + _headers()).encode()).hexdigest()[:16]
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, f"emu_{h}.so")
    if not os.path.exists(so):
        cpp = os.path.join(OUT, f"emu_{h}.cpp")
        with open(cpp, "w") as f:
            f.write(body)
        subprocess.run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-I", CSRC, cpp,
                        "-o", so + ".tmp"], check=True)
        os.replace(so + ".tmp", so)
    L = ctypes.CDLL(so)
    L.fe_emu_run.argtypes = [ctypes.POINTER(_Args), ctypes.c_int]
    return L


def run(ks, x, conn, values, params, flag: int = 1, direction=None, aux: int = 0, hist=None):
    """Element residuals [E, nloc] and matrices [E, nloc, nloc] of the
    generated kernel ks on the given mesh data (host arrays); ``hist``
    [levels, n_nodes, nval]: previous time levels of the values."""
    L = build(ks)
    E = conn.shape[0]
    nloc = ks.layout.n
    jt = np.float32 if ks.jac_precision == "f32" else np.float64
    x = np.ascontiguousarray(x, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    values = np.ascontiguousarray(values, dtype=np.float64)
    params = np.ascontiguousarray(params if len(params) else np.zeros(1), dtype=np.float64)
    tables = np.ascontiguousarray(ks.tables, dtype=np.float64)
    rbuf = np.zeros((E, nloc))
    jbuf = np.zeros((E, nloc, nloc), dtype=jt)
    status = np.zeros(4, dtype=np.int32)
    if direction is not None:
        direction = np.ascontiguousarray(direction, dtype=np.float64)
    nh = 0
    if hist is not None:
        hist = np.ascontiguousarray(hist, dtype=np.float64)
        assert hist.shape[1:] == values.shape
        nh = hist.shape[0]
    dhat = None
    if ks.tc_pairs:
        # the kernel writes the pulled-back derivatives; the tensor-core
        # contraction (csrc/fe_tc.cuh) is emulated exactly below
        dhat = np.zeros((E, ks.et.nq, len(ks.tc_pairs)), dtype=np.float32)
    a = _Args(x.ctypes.data, conn.ctypes.data, values.ctypes.data, params.ctypes.data, tables.ctypes.data,
              rbuf.ctypes.data, jbuf.ctypes.data, E, values.shape[1], flag, status.ctypes.data, 0, 0,
              None if hist is None else hist.ctypes.data, None, nh, values.size, aux,
              x.shape[0], values.ctypes.data if direction is None else direction.ctypes.data,
              None if dhat is None else dhat.ctypes.data)
    L.fe_emu_run(ctypes.byref(a), (E + ks.epb - 1) // ks.epb)
    if ks.tc_pairs and flag in (1, 4):
        from pyoomph_gb300.codegen import tc_tables
        pa, pb, phi = tc_tables(ks)
        jbuf[:] = np.einsum("qpi,eqp,qpj->eij", phi[:, pa, :], dhat.astype(np.float64), phi[:, pb, :])
    return rbuf, jbuf, status


class _FusedArgs(ctypes.Structure):
    _fields_ = [("d", _Args * 4), ("block_start", ctypes.c_int * 5), ("n_domains", ctypes.c_int)]


def build_fused(fk, defines=()) -> ctypes.CDLL:
    """Emulator library of a fused multi-domain kernel (pyoomph_gb300.ale)."""
    src = re.sub(r"#define FE_NT \d+", "#define FE_NT 1", fk.source)
    src = src.replace("extern __shared__ __align__(16) unsigned char fe_smem[];", "")
    body = "".join(f"#define {d_} 1\n" for d_ in defines) + PRELUDE + src + (
        f'\nextern "C" void fe_emu_run_fused(const FeFusedArgs *a, int nblocks) {{\n'
        f'  for (int b = 0; b < nblocks; ++b) {{\n'
        f'    memset(fe_smem, 0xff, sizeof(fe_smem));\n'
        f'    blockIdx.x = b; gridDim.x = nblocks; {fk.name}(*a); }}\n}}\n')
    h = hashlib.sha1((body + _headers()).encode()).hexdigest()[:16]
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, f"emu_{h}.so")
    if not os.path.exists(so):
        cpp = os.path.join(OUT, f"emu_{h}.cpp")
        with open(cpp, "w") as f:
            f.write(body)
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-ffp-contract=off", "-I", CSRC, cpp,
                        "-o", so + ".tmp"], check=True)
        os.replace(so + ".tmp", so)
    L = ctypes.CDLL(so)
    L.fe_emu_run_fused.argtypes = [ctypes.POINTER(_FusedArgs), ctypes.c_int]
    return L


def run_fused(fk, conns, values, hist, x0, params, flag: int = 1, aux: int = 0, defines=()):
    """Element residuals and matrices of every domain of a fused kernel.
    values, hist[k]: [n_nodes, nval]; x0: [n_nodes, dim]; conns: per domain
    [E_k, nnode_k]."""
    L = build_fused(fk, defines)
    nval = values.shape[1]
    values = np.ascontiguousarray(values, dtype=np.float64)
    hist_arr = np.ascontiguousarray(np.stack(hist), dtype=np.float64)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    params = np.ascontiguousarray(params, dtype=np.float64)
    status = np.zeros(4, dtype=np.int32)
    fa = _FusedArgs()
    keep, outs = [], []
    nb = 0
    jt = np.float32 if fk.jac_precision == "f32" else np.float64
    for k, (dc, conn) in enumerate(zip(fk.domains, conns)):
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        tables = np.ascontiguousarray(dc.dtype.tables(), dtype=np.float64)
        E = conn.shape[0]
        rbuf = np.zeros((E, dc.nloc))
        jbuf = np.zeros((E, dc.nloc, dc.nloc), dtype=jt)
        keep += [conn, tables]
        outs.append((rbuf, jbuf))
        fa.d[k] = _Args(x0.ctypes.data, conn.ctypes.data, values.ctypes.data, params.ctypes.data,
                        tables.ctypes.data, rbuf.ctypes.data, jbuf.ctypes.data, E, nval, flag,
                        status.ctypes.data, 0, 0, hist_arr.ctypes.data, x0.ctypes.data, len(hist),
                        values.size, aux, values.shape[0], values.ctypes.data, None)
        fa.block_start[k] = nb
        nb += (E + dc.epb - 1) // dc.epb
    fa.block_start[len(fk.domains)] = nb
    fa.n_domains = len(fk.domains)
    L.fe_emu_run_fused(ctypes.byref(fa), nb)
    return outs, status
