"""Batched FP64 subspace eigensolver (qgb_subspace_eigh) against torch.linalg.eigh."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nk,n", [(1, 1), (1, 40), (4, 96), (8, 352), (3, 17)])
def test_subspace_eigh_matches_torch(nk, n):
    from qimpy_gb300.linalg import eigh

    dev = torch.device("cuda:0")
    g = torch.Generator(device="cpu").manual_seed(1000 * nk + n)
    a = torch.randn(nk, n, 2 * n, dtype=torch.complex128, generator=g)
    A = (a @ a.conj().transpose(-2, -1) / n - 1.5 * torch.eye(n)).to(dev)
    W, V = eigh(A)
    W0, _ = torch.linalg.eigh(A)
    scale = float(W0.abs().max())
    assert torch.allclose(W, W0, rtol=0, atol=1e-12 * scale)
    # Eigenvectors: A V = V diag(W) and V^H V = I (vectors are unique only up to phase).
    res = A @ V - V * W[:, None, :]
    assert float(res.abs().max()) < 1e-11 * scale
    eye = torch.eye(n, dtype=V.dtype, device=dev)
    assert float((V.conj().transpose(-2, -1) @ V - eye).abs().max()) < 1e-12 * max(n, 10)
    assert torch.equal(A, A.clone())  # input untouched


def test_subspace_eigh_rejects_non_fp64():
    from qimpy_gb300.linalg import eigh

    with pytest.raises(TypeError):
        eigh(torch.eye(4, dtype=torch.complex64, device="cuda:0"))
