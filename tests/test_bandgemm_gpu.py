"""Hand-written band-space products (qgb_dot, qgb_matmul, qgb_project,
qgb_apply_nonlocal) against numpy FP64 products of the same inputs.

Tolerances (max-norm, relative to the largest |value| of the exact result):
FP64 1e-13; FP32 inputs 1e-5 (dot, FP32 sums per basis range added in FP64)
and 5e-6 (matmul).  Shapes cover tile edges (sizes not multiples of the
64-wide tiles or of 16-wide basis stages), one and several k-points, the
split-K path (long bases) and the single-range path (short ones).
"""
import numpy as np
import pytest
import torch

from qimpy_gb300 import ops

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _rand(shape, seed, dtype):
    g = np.random.default_rng(seed)
    x = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    return x.astype(np.complex128 if dtype == torch.complex128 else np.complex64)


def _err(got, want):
    return float(np.abs(got - want).max() / np.abs(want).max())


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-13), (torch.complex64, 1e-5)])
@pytest.mark.parametrize("nk,nx,ny,n", [(1, 7, 5, 33), (2, 65, 130, 1000), (1, 176, 352, 37073), (3, 18, 36, 1152)])
def test_dot_matches_numpy(dtype, tol, nk, nx, ny, n):
    X = _rand((nk, nx, n), 1, dtype)
    Y = _rand((nk, ny, n), 2, dtype)
    got = ops.dot(torch.from_numpy(X).to(DEV), torch.from_numpy(Y).to(DEV)).cpu().numpy()
    want = np.einsum("kig,kjg->kij", X.astype(np.complex128).conj(), Y.astype(np.complex128))
    assert got.dtype == np.complex128
    assert _err(got, want) < tol


@pytest.mark.parametrize("nk,nx,ny,n", [(1, 7, 5, 33), (2, 65, 130, 1000), (1, 352, 176, 37073), (8, 36, 18, 1152)])
def test_dot_tensor_cores_match_numpy(nk, nx, ny, n):
    """qgb_dot_tc (split-BF16x3 on tcgen05, FP32 accumulation, FP64 split sums):
    within 5e-5 of the FP64 product (max-norm relative)."""
    X = _rand((nk, nx, n), 5, torch.complex64)
    Y = _rand((nk, ny, n), 6, torch.complex64)
    got = ops.dot(torch.from_numpy(X).to(DEV), torch.from_numpy(Y).to(DEV), tc=True).cpu().numpy()
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    want = np.einsum("kig,kjg->kij", X.astype(np.complex128).conj(), Y.astype(np.complex128))
    assert got.dtype == np.complex128
    assert _err(got, want) < 5e-5


@pytest.mark.parametrize("accumulate", [False, True])
@pytest.mark.parametrize("nk,n_in,n_out,n", [(1, 7, 5, 33), (2, 130, 65, 1001), (1, 352, 176, 37073), (8, 36, 18, 1152)])
def test_matmul_tensor_cores_match_numpy(nk, n_in, n_out, n, accumulate):
    """qgb_matmul_tc (transposed split of C, split-BF16x3 GEMM accumulating into
    out): within 5e-5 of the FP64 product (max-norm relative)."""
    C = _rand((nk, n_in, n), 7, torch.complex64)
    M = _rand((nk, n_in, n_out), 8, torch.complex64)
    O = _rand((nk, n_out, n), 9, torch.complex64)
    out = torch.from_numpy(O).to(DEV)
    got = ops.matmul(torch.from_numpy(C).to(DEV), torch.from_numpy(M).to(DEV), out=out, accumulate=accumulate,
                     tc=True).cpu().numpy()
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    want = np.einsum("kij,kig->kjg", M.astype(np.complex128), C.astype(np.complex128))
    if accumulate:
        want = want + O
    assert _err(got.astype(np.complex128), want) < 5e-5


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-13), (torch.complex64, 5e-6)])
@pytest.mark.parametrize("nk,n_in,n_out,n", [(1, 7, 5, 33), (2, 130, 65, 1001), (1, 352, 176, 37073)])
def test_matmul_matches_numpy(dtype, tol, nk, n_in, n_out, n):
    C = _rand((nk, n_in, n), 3, dtype)
    M = _rand((nk, n_in, n_out), 4, dtype)
    Cd, Md = torch.from_numpy(C).to(DEV), torch.from_numpy(M).to(DEV)
    want = np.einsum("kij,kig->kjg", M.astype(np.complex128), C.astype(np.complex128))
    got = ops.matmul(Cd, Md).cpu().numpy()
    assert _err(got, want) < tol
    acc = torch.from_numpy(C[:, :n_out] if n_out <= n_in else _rand((nk, n_out, n), 5, dtype)).to(DEV).contiguous()
    base = acc.cpu().numpy().astype(np.complex128)
    ops.matmul(Cd, Md, out=acc, accumulate=True)
    assert _err(acc.cpu().numpy(), want + base) < tol


def test_matmul_zero_inputs_and_deterministic():
    C = torch.from_numpy(_rand((2, 40, 777), 6, torch.complex128)).to(DEV)
    M = torch.from_numpy(_rand((2, 40, 24), 7, torch.complex128)).to(DEV)
    a = ops.matmul(C, M)
    b = ops.matmul(C, M)
    assert torch.equal(a, b)
    d1 = ops.dot(C, C)
    d2 = ops.dot(C, C)
    assert torch.equal(d1, d2)
    z = ops.matmul(C[:, :0].contiguous(), M[:, :0].contiguous())  # no input bands: zeros
    assert z.shape == (2, 24, 777) and int(torch.count_nonzero(z)) == 0


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-13), (torch.complex64, 5e-6)])
def test_project_and_nonlocal_match_numpy(dtype, tol):
    nk, P, nb, n, pa = 2, 36, 20, 3001, 4
    beta = _rand((nk, P, n), 8, dtype)
    C = _rand((nk, nb, n), 9, dtype)
    D = _rand((P // pa, pa, pa), 10, dtype)
    betad, Cd, Dd = (torch.from_numpy(x).to(DEV) for x in (beta, C, D))
    projT = ops.project(betad, Cd).cpu().numpy()
    want_p = np.einsum("kpg,kbg->kbp", beta.astype(np.complex128).conj(), C.astype(np.complex128))
    assert _err(projT, want_p) < tol
    out = torch.from_numpy(_rand((nk, nb, n), 11, dtype)).to(DEV)
    base = out.cpu().numpy().astype(np.complex128)
    ops.apply_nonlocal(betad, Dd, torch.from_numpy(projT).to(DEV), out)
    D_all = np.zeros((P, P), complex)
    for a in range(P // pa):
        D_all[a * pa:(a + 1) * pa, a * pa:(a + 1) * pa] = D[a]
    want = base + np.einsum("kpg,kbp->kbg", beta.astype(np.complex128), np.einsum("pq,kbq->kbp", D_all, projT))
    assert _err(out.cpu().numpy(), want) < tol


def test_matmul_resolves_lazy_conjugate():
    """A conjugate transpose of a column-major matrix is contiguous yet carries
    torch's lazy conjugate bit; the rotation must use the conjugated values."""
    C = torch.from_numpy(_rand((2, 8, 77), 12, torch.complex128)).to(DEV)
    A = torch.from_numpy(_rand((2, 8, 8), 13, torch.complex128)).to(DEV)
    M = A.transpose(1, 2).contiguous().transpose(1, 2).conj().transpose(1, 2)  # contiguous, conj bit set
    assert M.is_conj() and M.is_contiguous()
    want = torch.matmul(M.resolve_conj().transpose(1, 2), C)
    got = ops.matmul(C, M)
    assert float((got - want).abs().max() / want.abs().max()) < 1e-13
    with pytest.raises(ValueError):
        ops.dot(C.conj(), C)
