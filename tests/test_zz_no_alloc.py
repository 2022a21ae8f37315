"""The allocation-free residual max-norm, fe_residual_max_noalloc.

Some callers cannot allocate device memory: fe_residual_max needs a problem
handle, and creating one allocates.  The no-alloc entry point keeps its
scratch in a static device array of the library instead.  This test calls it
through the C-ABI and checks it against the existing entry point
fe_residual_max on the same device vectors, twice in a row (the second call
reuses the scratch the first one left behind), plus NaN handling and the
size limit.  It sits in a file of its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_no_alloc_max_norm_matches_problem_entry_point_on_two_calls():
    import torch
    from pyoomph_gb300 import _native as N
    from pyoomph_gb300 import workloads as W
    L = N.load()
    P = W.poisson_problem(N=4)
    P.initialise()  # a handle for the existing entry point
    rng = np.random.default_rng(3)
    # multi-block sizes first, then small ones; two calls in a row each
    for n in (5_000_003, 8192 * 7 + 1, 1000, 1):
        R = torch.as_tensor(rng.normal(0.0, 1.0, n) * 10.0 ** rng.integers(-3, 3), device="cuda")
        for _ in range(2):
            ref = ctypes.c_double(-1.0)
            N.check(L.fe_residual_max(P._h, R.data_ptr(), n, ctypes.byref(ref), _stream(torch)))
            out = ctypes.c_double(-1.0)
            N.check(L.fe_residual_max_noalloc(R.data_ptr(), n, ctypes.byref(out), _stream(torch)))
            # a max is exact: the tolerance of the parity tests (1e-12) holds with equality
            assert out.value == ref.value == float(torch.max(torch.abs(R)).item())
    # NaN -> +inf, as DoubleVector::max
    R = torch.zeros(100_000, dtype=torch.float64, device="cuda")
    R[77_777] = float("nan")
    out = ctypes.c_double()
    N.check(L.fe_residual_max_noalloc(R.data_ptr(), R.numel(), ctypes.byref(out), _stream(torch)))
    ref = ctypes.c_double()
    N.check(L.fe_residual_max(P._h, R.data_ptr(), R.numel(), ctypes.byref(ref), _stream(torch)))
    assert out.value == float("inf") and ref.value == float("inf")


def test_no_alloc_rejects_sizes_beyond_its_scratch():
    import torch
    from pyoomph_gb300 import _native as N
    L = N.load()
    R = torch.zeros(16, dtype=torch.float64, device="cuda")
    limit = L.fe_residual_max_noalloc_limit()
    assert limit == (32768 - 1) * 8192
    out = ctypes.c_double(-1.0)
    rc = L.fe_residual_max_noalloc(R.data_ptr(), limit + 1, ctypes.byref(out), _stream(torch))
    assert rc == N.FE_ERR_ARG
    assert b"exceeds the maximum" in L.fe_last_error()
    assert out.value == -1.0
