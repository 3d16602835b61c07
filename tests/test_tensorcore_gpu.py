"""The tcgen05 split-BF16x3 GEMM and the mixed-precision nonlocal term on GB300.

* Raw GEMM against the exact (float64) value of the split-BF16x3 formula: the
  only differences left are FP32 accumulation (tolerance 1e-5 relative), so
  this pins descriptors, swizzle, pipeline and epilogue.
* Mixed nonlocal term (complex64) against the FP64 oracle: 2e-5 relative.
"""
import ctypes as ct

import numpy as np
import pytest
import torch

from oracle import hpsi as oh
from qimpy_gb300 import _lib, ops, workloads as wl

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _split(x: torch.Tensor):
    hi = x.to(torch.bfloat16)
    lo = (x - hi.float()).to(torch.bfloat16)
    return hi, lo


def _pad_cols(x, ld):
    out = torch.zeros((x.shape[0], ld), dtype=x.dtype, device=x.device)
    out[:, : x.shape[1]] = x
    return out.contiguous()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (200, 48, 1000), (384, 64, 4160)])
def test_tc_gemm_bf16x3_exact_split(M, N, K):
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = torch.randn((M, K), generator=g).to(DEV)
    B = torch.randn((N, K), generator=g).to(DEV)
    a_hi, a_lo = _split(A)
    b_hi, b_lo = _split(B)
    lda = ldb = (K + 7) // 8 * 8
    a_hi, a_lo, b_hi, b_lo = (_pad_cols(t, lda) for t in (a_hi, a_lo, b_hi, b_lo))
    D = torch.empty((M, N), dtype=torch.float32, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    ws = torch.empty(((M + 127) // 128 * 128) * 64, dtype=torch.float32, device=DEV)
    rc = _lib.aux().qgb_tc_gemm_bf16x3(a_hi.data_ptr(), a_lo.data_ptr(), b_hi.data_ptr(), b_lo.data_ptr(), M, N, K,
                                        lda, ldb, D.data_ptr(), err.data_ptr(), ws.data_ptr(), ws.numel() * 4,
                                        torch.cuda.current_stream().cuda_stream)
    _lib.check(rc, "tc_gemm")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ah, al, bh, bl = (t[:, :K].double() for t in (a_hi, a_lo, b_hi, b_lo))
    exact = ah @ bh.T + ah @ bl.T + al @ bh.T
    scale = (A.double().abs() @ B.double().abs().T).max()
    assert float((D.double() - exact).abs().max() / scale) < 1e-5
    true = A.double() @ B.double().T
    assert float((D.double() - true).abs().max() / scale) < 1e-4


@pytest.mark.parametrize("name,nb", [("tiny_fcc", 8), ("si2", 18), ("cu32", 200)])
def test_nonlocal_tc_matches_oracle(name, nb):
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    beta = wl.make_projectors(p, b)
    C = wl.make_wavefunctions(p, b, nb)
    betad = torch.from_numpy(beta).to(DEV, torch.complex64)
    Cd = torch.from_numpy(C).to(DEV, torch.complex64)
    Dd = torch.from_numpy(p.D_atom).to(DEV, torch.complex64)
    split = ops.beta_split(betad)
    HC = torch.zeros_like(Cd)
    projT = ops.apply_nonlocal_tc(split, Dd, Cd, HC)
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    proj_ref = oh.project(beta, C)
    nl_ref = oh.apply_nonlocal(beta, p.D_all(), proj_ref)
    got_proj = projT.transpose(1, 2).cpu().numpy()
    assert np.abs(got_proj - proj_ref).max() / np.abs(proj_ref).max() < 2e-5
    got = HC.cpu().numpy()
    assert np.abs(got - nl_ref).max() / np.abs(nl_ref).max() < 2e-5


def test_bounded_wait_times_out_cleanly():
    """A pipeline wait that runs out: the test launch's producer issues no
    copies, so the MMA issuer's first wait gives up after 1 ms and records
    error 3; the kernel frees its tensor memory and returns (no copy or MMA in
    flight), and the context stays usable: a normal GEMM afterwards is exact."""
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    ops_ = torch.zeros((192, 64), dtype=torch.bfloat16, device=DEV)
    ws = torch.empty((128, 64), dtype=torch.float32, device=DEV)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.aux().qgb_tc_wait_timeout_test(ops_.data_ptr(), ws.data_ptr(), err.data_ptr(), 1_000_000, st),
               "tc_wait_timeout_test")
    torch.cuda.synchronize()
    assert int(err.item()) == 3
    err.zero_()
    test_tc_gemm_bf16x3_exact_split(128, 64, 64)
    assert int(err.item()) == 0
