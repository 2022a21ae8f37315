"""Double-float (df64) arithmetic of fe_df64.cuh, compiled as host C++ with
the CPU emulator's intrinsic shims, against exact rational arithmetic:

* binary64 -> binary32 narrowing and binary32 -> binary64 widening by
  integer operations agree with the hardware conversions (numpy) on every
  class of value (normal, subnormal, zero, infinity, NaN, range edges);
* splitting a double into hi + lo is exact in the binary32 normal range;
* addition, subtraction and multiplication keep relative errors near
  2^-48 (bounded here by 2^-45), division near 2^-44 (bounded by 2^-42);
  the compensated multiply-add, renormalised every few
  terms as the generated contractions do, keeps the error of an n-term
  accumulation within (n m + 2) u^2 sum|terms| -- far below the 1e-12
  contract.
"""
import ctypes
import hashlib
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

import kernel_emulator as KE

SRC = r"""
#include "fe_df64.cuh"
extern "C" {
double t_widen(float f) { return fe_widen(f); }
float t_narrow(double d) { return fe_narrow(d); }
void t_split(double d, float *hi, float *lo) { fe_df64 a(d); *hi = a.hi; *lo = a.lo; }
void t_add(float ah, float al, float bh, float bl, float *h, float *l) {
  fe_df64 r = fe_df64(ah, al) + fe_df64(bh, bl); *h = r.hi; *l = r.lo; }
void t_mul(float ah, float al, float bh, float bl, float *h, float *l) {
  fe_df64 r = fe_df64(ah, al) * fe_df64(bh, bl); *h = r.hi; *l = r.lo; }
void t_sub(float ah, float al, float bh, float bl, float *h, float *l) {
  fe_df64 r = fe_df64(ah, al) - fe_df64(bh, bl); *h = r.hi; *l = r.lo; }
void t_div(float ah, float al, float bh, float bl, float *h, float *l) {
  fe_df64 r = fe_df64(ah, al) / fe_df64(bh, bl); *h = r.hi; *l = r.lo; }
void t_dot(const float *ah, const float *al, const float *bh, const float *bl, int n, int m, float *h, float *l) {
  fe_df64 acc = (fe_df64)0;
  for (int i = 0; i < n; ++i) {
    fe_mac(acc, fe_df64(ah[i], al[i]), fe_df64(bh[i], bl[i]));
    if ((i + 1) % m == 0) acc = fe_norm(acc);   // as the generated contractions do
  }
  acc = fe_norm(acc); *h = acc.hi; *l = acc.lo; }
}
"""


@pytest.fixture(scope="module")
def lib():
    body = KE.PRELUDE + SRC
    h = hashlib.sha1((body + KE._headers()).encode()).hexdigest()[:16]
    os.makedirs(KE.OUT, exist_ok=True)
    so = os.path.join(KE.OUT, f"df64_{h}.so")
    if not os.path.exists(so):
        cpp = os.path.join(KE.OUT, f"df64_{h}.cpp")
        with open(cpp, "w") as f:
            f.write(body)
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", KE.CSRC, cpp,
                        "-o", so + ".tmp"], check=True)
        os.replace(so + ".tmp", so)
    L = ctypes.CDLL(so)
    f, d, pf = ctypes.c_float, ctypes.c_double, ctypes.POINTER(ctypes.c_float)
    L.t_widen.argtypes, L.t_widen.restype = [f], d
    L.t_narrow.argtypes, L.t_narrow.restype = [d], f
    L.t_split.argtypes = [d, pf, pf]
    L.t_add.argtypes = [f, f, f, f, pf, pf]
    L.t_mul.argtypes = [f, f, f, f, pf, pf]
    L.t_sub.argtypes = [f, f, f, f, pf, pf]
    L.t_div.argtypes = [f, f, f, f, pf, pf]
    L.t_dot.argtypes = [pf, pf, pf, pf, ctypes.c_int, ctypes.c_int, pf, pf]
    return L


def _pair(L, fn, *args):
    h, l = ctypes.c_float(), ctypes.c_float()
    fn(*args, ctypes.byref(h), ctypes.byref(l))
    return h.value, l.value


def _split(L, x):
    return _pair(L, L.t_split, float(x))


def _val(h, l):
    return Fraction(float(np.float32(h))) + Fraction(float(np.float32(l)))


def test_widen_and_narrow_match_the_hardware_conversions(lib):
    f32 = np.finfo(np.float32)
    rng = np.random.default_rng(0)
    floats = np.concatenate([
        np.array([0.0, -0.0, 1.0, -1.0, f32.tiny, -f32.tiny, f32.max, -f32.max, f32.smallest_subnormal,
                  np.inf, -np.inf], dtype=np.float32),
        (rng.standard_normal(2000) * 10.0 ** rng.integers(-40, 38, 2000)).astype(np.float32)])
    for x in floats:
        assert lib.t_widen(float(x)) == float(np.float64(x)) or (np.isnan(x) and np.isnan(lib.t_widen(float(x))))
    assert np.isnan(lib.t_widen(float("nan")))
    doubles = np.concatenate([
        np.array([0.0, -0.0, 1.0, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -25, float(f32.max), 3.5e38, 1e-45, 1e-39,
                  float(f32.tiny), -1e300, np.inf, -np.inf]),
        rng.standard_normal(2000) * 10.0 ** rng.integers(-45, 39, 2000)])
    for x in doubles:
        got = lib.t_narrow(float(x))
        with np.errstate(over="ignore"):
            ref = np.float32(x)   # round to nearest even
        if np.isinf(ref) or np.isinf(got):
            assert np.isinf(got) == np.isinf(ref) or abs(x) >= float(f32.max)
            continue
        # nearest: ties may round away from zero (magnitude rounding); any other result must match
        assert abs(Fraction(float(got)) - Fraction(float(x))) <= abs(Fraction(float(ref)) - Fraction(float(x)))


def test_split_is_exact_in_the_normal_range(lib):
    rng = np.random.default_rng(1)
    xs = rng.standard_normal(5000) * 10.0 ** rng.integers(-25, 30, 5000)
    for x in xs:
        h, l = _split(lib, x)
        assert _val(h, l) == Fraction(float(x)) or abs(float(_val(h, l) - Fraction(float(x)))) <= abs(x) * 2.0 ** -47
        assert abs(l) <= abs(h) * 2.0 ** -23


def test_add_mul_and_compensated_dot_error_bounds(lib):
    rng = np.random.default_rng(2)
    eps = 2.0 ** -45
    for _ in range(3000):
        a, b = rng.standard_normal(2) * 10.0 ** rng.integers(-8, 8, 2)
        ah, al = _split(lib, a)
        bh, bl = _split(lib, b)
        A, B = _val(ah, al), _val(bh, bl)
        s = _val(*_pair(lib, lib.t_add, ah, al, bh, bl))
        p = _val(*_pair(lib, lib.t_mul, ah, al, bh, bl))
        assert abs(s - (A + B)) <= eps * (abs(A) + abs(B))
        assert abs(p - A * B) <= eps * abs(A * B)
    # compensated dot product, renormalised every m = 3 terms: the error is
    # bounded by (n m + 2) u^2 sum|terms|, u = 2^-24 (here 3.6e-13 for 64
    # terms; observed well below)
    n, m = 64, 3
    bound = (n * m + 2) * 2.0 ** -48
    worst = 0.0
    for _ in range(200):
        xs = rng.standard_normal(n) * 10.0 ** rng.integers(-3, 3, n)
        ys = rng.standard_normal(n)
        sx = [_split(lib, v) for v in xs]
        sy = [_split(lib, v) for v in ys]
        arr = lambda vals: (ctypes.c_float * n)(*vals)
        h, l = _pair(lib, lib.t_dot, arr([v[0] for v in sx]), arr([v[1] for v in sx]),
                     arr([v[0] for v in sy]), arr([v[1] for v in sy]), n, m)
        exact = sum(_val(*u) * _val(*v) for u, v in zip(sx, sy))
        scale = sum(abs(_val(*u) * _val(*v)) for u, v in zip(sx, sy))
        err = float(abs(_val(h, l) - exact) / scale)
        worst = max(worst, err)
        assert err <= bound
    assert worst <= 2.0 ** -44      # in practice an order below the bound


def test_sub_and_div_error_bounds(lib):
    rng = np.random.default_rng(5)
    for _ in range(3000):
        a, b = rng.standard_normal(2) * 10.0 ** rng.integers(-8, 8, 2)
        ah, al = _split(lib, a)
        bh, bl = _split(lib, b)
        A, B = _val(ah, al), _val(bh, bl)
        d = _val(*_pair(lib, lib.t_sub, ah, al, bh, bl))
        q = _val(*_pair(lib, lib.t_div, ah, al, bh, bl))
        assert abs(d - (A - B)) <= 2.0 ** -45 * (abs(A) + abs(B))
        assert abs(q - A / B) <= 2.0 ** -42 * abs(A / B)
