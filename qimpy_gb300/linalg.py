"""Subspace linear algebra in FP64 on the GPU (cuSOLVER through torch.linalg).

Restates qimpy/math/_linalg.py:110-183 (``ortho_matrix``, ``eighg``): the
Cholesky orthonormaliser U = (L^-1)^H of the overlap O, then eigh of U^H H U.
Both precision forms keep these steps in FP64.
"""
from __future__ import annotations

import torch


def dagger(x: torch.Tensor) -> torch.Tensor:
    return x.conj().transpose(-2, -1)


def ortho_matrix(O: torch.Tensor, use_cholesky: bool = True) -> torch.Tensor:
    """Orthonormalisation matrix of a basis with overlap O (qimpy/math/_linalg.py:110-140)."""
    if use_cholesky:
        eye = torch.eye(O.shape[-1], device=O.device, dtype=O.dtype).expand(O.shape)
        return dagger(torch.linalg.solve_triangular(torch.linalg.cholesky(O), eye, upper=False))
    lbda, V = torch.linalg.eigh(O)
    return V @ ((1.0 / torch.sqrt(lbda))[..., None] * dagger(V))


def eighg(H, O: torch.Tensor, use_cholesky: bool = True):
    """Solve H V = O V E (qimpy/math/_linalg.py:143-183); H may be a Waitable."""
    U = ortho_matrix(O, use_cholesky)
    Hr = H.wait() if hasattr(H, "wait") else H
    E, V = torch.linalg.eigh(dagger(U) @ (Hr @ U))
    return E, U @ V
