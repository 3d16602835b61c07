"""FP64 CPU restatement of the reference's CheFSI eigensolver (test infrastructure only).

Follows qimpy/dft/electrons/_chefsi.py:72-176: a Davidson warm-up to
`init_threshold` (oracle.davidson), then per iteration a scaled Chebyshev
filter of degree filter_order - 1 in H on the bands not yet converged, with
the window [min eig, max eig] per k amplified and [max eig, Ecut + max V]
suppressed, then Rayleigh-Ritz (eighg with the filtered vectors' overlap) and
the largest-eigenvalue-change test on the first n_bands.
Arrays drop the singleton spin/spinor axes: C[k, b, g].
"""
from __future__ import annotations

from typing import Callable

import numpy as np

from . import davidson as od


def chefsi(hamiltonian: Callable[[np.ndarray], np.ndarray], C: np.ndarray, ke: np.ndarray, n: np.ndarray,
           n_bands: int, ke_cutoff: float, V_max: float, n_iterations: int = 100, eig_threshold: float = 1e-8,
           filter_order: int = 10, init_threshold: float = 1e-1, gweight: np.ndarray | None = None,
           symmetrize=None) -> od.DavidsonResult:
    """CheFSI from orthonormal start vectors C[k, n_bands + n_bands_extra, g];
    `gweight` / `symmetrize` for real (Gamma-point) wavefunctions as in
    oracle.davidson.davidson."""
    dot_ = od.dot if gweight is None else (lambda A, B: od.dot_real(A, B, gweight))
    warm = od.davidson(hamiltonian, C, ke, n, n_bands, n_iterations, init_threshold,
                       gweight=gweight, symmetrize=symmetrize)  # _chefsi.py:86-92
    C, HC, eig = warm.C, warm.HC, warm.eig
    hpsi_bands = warm.hpsi_bands
    nk = C.shape[0]
    b_up = ke_cutoff + V_max  # _chefsi.py:103-104
    n_eigs_done = 0
    deig_max = np.inf
    converged = False
    i_iter = warm.iterations
    for i_iter in range(warm.iterations + 1, n_iterations + 1):
        b_lo = eig.max(axis=1)[:, None, None]  # _chefsi.py:109-112
        a_lo = eig.min(axis=1)[:, None, None]
        b_diff = 0.5 * (b_up - b_lo)
        b_mid = 0.5 * (b_lo + b_up)
        sigma = b_diff / (b_mid - a_lo)
        tau = 2.0 / sigma
        C0, HC0 = C[:, :n_eigs_done], HC[:, :n_eigs_done]
        X, HX = C[:, n_eigs_done:], HC[:, n_eigs_done:]
        Y = (HX - b_mid * X) * (sigma / b_diff)  # _chefsi.py:125-147
        for _ in range(filter_order - 2):
            sigma_new = 1.0 / (tau - sigma)
            HY = hamiltonian(Y)
            hpsi_bands += nk * Y.shape[1]
            Yt = (HY - b_mid * Y) * (2.0 * sigma_new / b_diff) - (sigma * sigma_new) * X
            X, Y, sigma = Y, Yt, sigma_new
        HY = hamiltonian(Y)
        hpsi_bands += nk * Y.shape[1]
        C = np.concatenate((C0, Y), axis=1)
        HC = np.concatenate((HC0, HY), axis=1)
        eig_prev = eig
        eig, V = od.eighg(dot_(C, HC), dot_(C, C))  # _chefsi.py:157-161
        C = od.matmul(C, V)
        HC = od.matmul(HC, V)
        deig = np.abs(eig - eig_prev)[:, :n_bands]  # _check_deig, _davidson.py:126-139
        deig_max = float(deig.max())
        pending = np.where((deig > eig_threshold).any(axis=0))[0]
        n_eigs_done = int(pending[0]) if len(pending) else n_bands
        if n_eigs_done >= n_bands:
            converged = True
            break
    return od.DavidsonResult(eig, C, i_iter, converged, deig_max, hpsi_bands, HC)
