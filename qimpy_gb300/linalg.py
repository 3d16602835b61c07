"""Subspace linear algebra in FP64 on the GPU.

Restates qimpy/math/_linalg.py:110-183 (``ortho_matrix``, ``eighg``): the
Cholesky orthonormaliser U = (L^-1)^H of the overlap O (cuSOLVER through
torch.linalg), then eigh of U^H H U through the library's batched cuSOLVER
entry point (qgb_subspace_eigh: all k-points in one call).  Both precision
forms keep these steps in FP64.
"""
from __future__ import annotations

import ctypes as ct
import math

import torch

from . import _lib


def eigh(A: torch.Tensor, check: bool = True):
    """Eigenvalues (ascending) and eigenvectors of Hermitian FP64 matrices
    A [..., n, n] on a CUDA device, one batched cuSOLVER call
    (qgb_subspace_eigh) for all leading indices.  Raises if any fails to
    converge (as torch.linalg.eigh does); with check=False it returns
    (E, V, failed) instead, `failed` a device bool per matrix, without the host
    synchronisation the check needs."""
    if A.device.type != "cuda" or A.dtype not in (torch.complex128, torch.float64):
        raise TypeError(f"eigh needs complex128 or float64 CUDA matrices, got {A.dtype} on {A.device}")
    if A.dtype == torch.float64:
        # Real symmetric (the overlaps of real wavefunctions): real eigenvectors,
        # so that rotations keep the bands real.  cuSOLVER through torch.linalg.
        W, V = torch.linalg.eigh(A)
        return (W, V) if check else (W, V, torch.zeros(A.shape[:-2], dtype=torch.bool, device=A.device))
    n = A.shape[-1]
    lead = A.shape[:-2]
    X = A.reshape(-1, n, n).clone(memory_format=torch.contiguous_format)
    nk = X.shape[0]
    W = torch.empty((nk, n), dtype=torch.float64, device=A.device)
    if nk == 0 or n == 0:
        if not check:
            return W.reshape(*lead, n), X.reshape(*lead, n, n), torch.zeros(lead, dtype=torch.bool, device=A.device)
        return W.reshape(*lead, n), X.reshape(*lead, n, n)
    info = torch.empty(nk, dtype=torch.int32, device=A.device)
    lib = _lib.lib()
    ws_bytes = int(lib.qgb_subspace_eigh_workspace_bytes(nk, n))
    if ws_bytes == 0:
        raise _lib.QgbError(f"subspace_eigh workspace query failed: {lib.qgb_last_error().decode()}")
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=A.device)
    st = torch.cuda.current_stream(A.device).cuda_stream
    _lib.check(lib.qgb_subspace_eigh(X.data_ptr(), W.data_ptr(), info.data_ptr(), nk, n, ws.data_ptr(),
                                     ws_bytes, ct.c_void_p(st)), "subspace_eigh")
    # X holds V^H row-major (the column-major solve saw conj(A)).
    V = X.conj().transpose(-2, -1).reshape(*lead, n, n)
    if not check:
        return W.reshape(*lead, n), V, (info != 0).reshape(lead)
    bad = torch.nonzero(info).flatten().tolist()
    if bad:
        raise RuntimeError(f"subspace eigh: (Batch element {bad[0]}) did not converge (info {int(info[bad[0]])})")
    return W.reshape(*lead, n), V


def dagger(x: torch.Tensor) -> torch.Tensor:
    return x.conj().transpose(-2, -1)


def ortho_matrix(O: torch.Tensor, use_cholesky: bool = True) -> torch.Tensor:
    """Orthonormalisation matrix of a basis with overlap O (qimpy/math/_linalg.py:110-140)."""
    if use_cholesky:
        eye = torch.eye(O.shape[-1], device=O.device, dtype=O.dtype).expand(O.shape)
        return dagger(torch.linalg.solve_triangular(torch.linalg.cholesky(O), eye, upper=False))
    lbda, V = eigh(O)
    return V @ ((1.0 / torch.sqrt(lbda))[..., None] * dagger(V))


def _canonical_ortho(O: torch.Tensor, drop_below: float):
    """Canonical orthogonalisation (Loewdin, Int. J. Quantum Chem. 4, 1970):
    U = V_kept diag(lambda_kept^-1/2) from the eigenpairs of O, dropping the
    directions with lambda < drop_below * max_i O_ii.  Dropped columns of U are
    zero, so U keeps its square shape across the batch; `keep` marks the rest."""
    lbda, V = eigh(O)
    floor = drop_below * O.diagonal(dim1=-2, dim2=-1).real.amax(dim=-1, keepdim=True)
    keep = lbda > floor
    scale = torch.where(keep, 1.0 / torch.sqrt(torch.where(keep, lbda, torch.ones_like(lbda))),
                        torch.zeros_like(lbda))
    return V * scale[..., None, :].to(V.dtype), keep


def eighg(H, O: torch.Tensor, use_cholesky: bool = True, drop_below: float = 0.0, check: bool = True,
          defer_canonical: bool = False, force_canonical: bool = False):
    """Solve H V = O V E (qimpy/math/_linalg.py:143-183); H may be a Waitable.

    drop_below > 0 is for overlaps of FP32 vectors.  Their rounding (and the
    drift of supposedly orthonormal vectors) is ~1e-5 of O, so directions the
    subspace barely spans cannot be resolved: Cholesky fails on them, or
    amplifies their noise by lambda^-1/2.  When the Cholesky pivots show such a
    direction (min L_ii^2 < drop_below * max O_ii, or a failed factorisation),
    the basis is orthonormalised canonically instead, dropping directions with
    eigenvalue below that floor.  Dropped directions come last, with
    eigenvalue +inf and eigenvector zero.

    check=False returns (E, V, failed) with `failed` a device bool per k (a
    failed Cholesky factorisation of O, or an eigensolve that did not
    converge), so that the caller can fold the test into its own host
    synchronisation; check=True raises as the reference does.

    defer_canonical=True (with drop_below > 0, check=False) takes the Cholesky
    path without deciding on the host and returns (E, V, failed, canonical):
    `canonical` is a device bool that is set when the pivots call for the
    canonical orthogonalisation; the caller then solves again with
    force_canonical=True.  The common case thus needs no host synchronisation."""
    Hr = H.wait() if hasattr(H, "wait") else H
    keep = None
    chol_failed = None
    if use_cholesky:
        eye = torch.eye(O.shape[-1], device=O.device, dtype=O.dtype).expand(O.shape)
        canonical_flag = None
        if force_canonical:
            U, keep = _canonical_ortho(O, drop_below)
            L, info = None, torch.zeros(O.shape[:-2], dtype=torch.int32, device=O.device)
        else:
            L, info = torch.linalg.cholesky_ex(O)
        if drop_below > 0.0 and not force_canonical:
            pivot = L.diagonal(dim1=-2, dim2=-1).real.square().amin(dim=-1)
            floor = drop_below * O.diagonal(dim1=-2, dim2=-1).real.amax(dim=-1)
            bad = ((info != 0) | (pivot < floor)).any()
            if defer_canonical:
                canonical_flag = bad
            elif bool(bad):
                U, keep = _canonical_ortho(O, drop_below)
        elif check:
            bad = torch.nonzero(info).flatten().tolist()
            if bad:
                raise RuntimeError(f"linalg.cholesky: (Batch element {bad[0]}): the overlap is not positive-definite")
        else:
            chol_failed = info != 0
        if keep is None:
            U = dagger(torch.linalg.solve_triangular(L, eye, upper=False))
    else:
        U = ortho_matrix(O, use_cholesky)
    Hs = dagger(U) @ (Hr @ U)
    if keep is not None:
        # Dropped directions: zero rows/columns of Hs; give them a diagonal above
        # the spectral norm of the rest so that they sort last, then mark them +inf.
        big = 10.0 * (torch.linalg.matrix_norm(Hs).amax() + 1.0)
        Hs = Hs + torch.diag_embed((~keep).to(torch.float64) * big).to(Hs.dtype)
    if check:
        E, V = eigh(Hs)
        failed = None
    else:
        E, V, failed = eigh(Hs, check=False)
        if chol_failed is not None:
            failed = failed | chol_failed
    if keep is not None:
        n_keep = keep.sum(dim=-1, keepdim=True)
        E = torch.where(torch.arange(E.shape[-1], device=E.device) >= n_keep, torch.full_like(E, math.inf), E)
    if check:
        return E, U @ V
    if defer_canonical:
        flag = canonical_flag if canonical_flag is not None else torch.zeros((), dtype=torch.bool, device=E.device)
        return E, U @ V, failed, flag
    return E, U @ V, failed
