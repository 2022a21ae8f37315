"""Element Jacobians contracted on the tensor cores (tcgen05, 3xTF32 split,
FP32 accumulation; csrc/fe_tc.cuh) against the same contraction in FP64
numpy: J_e[i][j] = sum_q sum_p phi[q][a_p][i] Dhat_e[q][p] phi[q][b_p][j],
the reference-coordinate form of the generated Jacobian loop
(codegen.cpp:1883-2258).  Contract: 1e-5 relative in the max norm (the FP32
Jacobian's); the split keeps it near 1e-6."""
import ctypes

import numpy as np
import pytest




def _hex_pairs():
    # nonlinear diffusion on Q2 hexes: test gradient x (trial value, trial gradient)
    pa, pb = [], []
    for a in (1, 2, 3):
        for b in (0, 1, 2, 3):
            pa.append(a)
            pb.append(b)
    return pa, pb


def _contract_numpy(phi, dhat, pa, pb):
    A = phi[:, pa, :]                    # [nq][npair][n]
    B = phi[:, pb, :]
    return np.einsum("qpi,eqp,qpj->eij", A, dhat.astype(np.float64), B)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["hex27", "quad9", "ragged"])
def test_tc_contraction_matches_fp64(case):
    import torch
    from pyoomph_gb300 import _native as N
    rng = np.random.default_rng(7)
    if case == "hex27":
        n, nq, nc, E = 27, 27, 4, 1001
        pa, pb = _hex_pairs()
    elif case == "quad9":
        n, nq, nc, E = 9, 9, 3, 64
        pa, pb = [1, 1, 2, 2, 0], [1, 2, 1, 2, 0]
    else:   # every component active, odd sizes, a partial last tile
        n, nq, nc, E = 20, 13, 4, 7
        pa = [0, 1, 2, 3, 0, 2]
        pb = [0, 1, 2, 3, 3, 1]
    phi = rng.normal(0.0, 1.0, (nq, nc, n))
    dhat = rng.normal(0.0, 1.0, (E, nq, len(pa))).astype(np.float32) * np.float32(1e-3)
    ref = _contract_numpy(phi, dhat, np.array(pa), np.array(pb))
    dd = torch.as_tensor(dhat, device="cuda").contiguous()
    jb = torch.full((E, n, n), float("nan"), dtype=torch.float32, device="cuda")
    L = N.load()
    pa_ = np.array(pa, dtype=np.int32)
    pb_ = np.array(pb, dtype=np.int32)
    ph = np.ascontiguousarray(phi)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):                   # twice: the result does not depend on what the buffers held
        N.check(L.fe_tc_contract(dd.data_ptr(), jb.data_ptr(), E, n, nq, nc, ph.ctypes.data, len(pa),
                                 pa_.ctypes.data, pb_.ctypes.data, st))
        got = jb.cpu().numpy().astype(np.float64)
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= 1e-5, err
    # the 3xTF32 split is far inside the FP32 contract (one TF32 product alone would be ~1e-3)
    assert err <= 2e-6, err


@pytest.mark.gpu
def test_tc_contraction_rejects_bad_sizes():
    import torch
    from pyoomph_gb300 import _native as N
    L = N.load()
    dd = torch.zeros(4, device="cuda")
    phi = np.zeros(64)
    pa = np.zeros(1, dtype=np.int32)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.fe_tc_contract(dd.data_ptr(), dd.data_ptr(), 1, 40, 1, 1, phi.ctypes.data, 1, pa.ctypes.data,
                          pa.ctypes.data, st)
    assert rc == N.FE_ERR_ARG


def test_generator_chooses_the_tensor_cores_for_fp32_hex_jacobians_only():
    """Lowering only (no GPU): the Q2 hex FP32 Jacobian is contracted on the
    tensor cores by default; FP64/df64 Jacobians, the 9-node quad and
    multi-field forms keep their kernels; forcing it where it does not apply
    is an error."""
    from pyoomph_gb300 import workloads as W
    P = W.nonlinear_diffusion_problem(N=3, jacobian_precision="fp32")
    ks = P.lower()
    assert ks.tc_pairs == [(a, b) for a in (1, 2, 3) for b in (0, 1, 2, 3)]
    assert "a.dhat" in ks.source and "fe_jstore" not in ks.source     # no Jacobian stored by the kernel
    pa, pb, phi = P.tensor_contraction_tables()
    assert phi.shape == (27, 4, 27) and np.allclose(phi[:, 0, :].sum(axis=1), 1.0)   # partition of unity
    for prec in ("fp64", "df64"):
        assert W.nonlinear_diffusion_problem(N=3, jacobian_precision=prec).lower().tc_pairs is None
    assert W.poisson_problem(N=3, jacobian_precision="fp32").lower().tc_pairs is None
    assert W.navier_stokes_problem(N=3, jacobian_precision="fp32").lower().tc_pairs is None
    Q = W.nonlinear_diffusion_problem(N=3, jacobian_precision="fp32")
    Q.tensor_cores = False
    assert Q.lower().tc_pairs is None
    R = W.navier_stokes_problem(N=3, jacobian_precision="fp32")
    R.tensor_cores = True
    with pytest.raises(ValueError):
        R.lower()
