"""Chebyshev-filtered subspace iteration (CheFSI) on the GPU H.psi path.

Restates qimpy/dft/electrons/_chefsi.py:72-176, the second caller of the
Hamiltonian in the reference:

* warm-up: Davidson to `init_threshold` when the eigenvalues are not yet that
  accurate, else a subspace diagonalisation of the current vectors;
* each iteration filters the not-yet-converged bands with a scaled Chebyshev
  polynomial of degree `filter_order - 1` in H: the window [a_lo, b_lo] of the
  current eigenvalues (per k) is amplified and [b_lo, b_up] suppressed, with
  b_up = Ecut + max V(r) bounding the spectrum from above;
* then Rayleigh-Ritz in the filtered subspace (overlap and Hamiltonian
  matrices, ``eighg``), and the reference's convergence test on the largest
  eigenvalue change of the first n_bands.

The filter recursion (three-term, with the scaling sigma_{i+1} =
1 / (2 / sigma_1 - sigma_i)) is the reference's.  Mixed precision: the
vectors and H.psi are FP32 and the subspace algebra FP64, as in the mixed
Davidson; an FP32 run stops at FP32's floor (no new minimum of the eigenvalue
change for 10 iterations, or an overlap that FP32 cannot factor) and is
finished by ``refine_fp64``.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from .davidson import Davidson, DavidsonStats
from .electrons import Electrons
from .linalg import eigh, eighg


class CheFSI(Davidson):
    """CheFSI diagonalisation of ``electrons`` (qimpy/dft/electrons/_chefsi.py:14-176)."""

    def __init__(self, electrons: Electrons, n_iterations: int = 100, eig_threshold: float = 1e-8,
                 filter_order: int = 10, init_threshold: float = 1e-1):
        super().__init__(electrons, n_iterations=n_iterations, eig_threshold=eig_threshold)
        if filter_order < 2:
            raise ValueError("filter_order must be at least 2")
        self.filter_order = int(filter_order)
        self.init_threshold = float(init_threshold)

    def __call__(self, n_iterations: Optional[int] = None) -> DavidsonStats:
        el = self.electrons
        n_bands = el.n_bands
        n_iterations = n_iterations or self.n_iterations
        fp32 = el.C.coeff.dtype == torch.complex64
        hpsi = 0
        if el.deig_max > self.init_threshold:  # _chefsi.py:86-92
            warm = Davidson(el, n_iterations=n_iterations, eig_threshold=self.init_threshold)
            stats = warm(n_iterations)
            HC = warm._HC
            hpsi += stats.hpsi_bands
            i_start = stats.iterations
        else:  # _chefsi.py:93-101
            HC = el.hamiltonian(el.C)
            hpsi += el.C.n_bands() * el.basis.nk
            el.eig, V = eigh((el.C ^ HC).wait())
            el.deig_max = np.inf
            el.C = el.C @ V
            HC = HC @ V
            i_start = 0

        KEmax = float(el.basis.ke_cutoff)  # upper bound on KE in the sphere
        V_r = el.V_r if isinstance(el.V_r, torch.Tensor) else torch.from_numpy(np.asarray(el.V_r))
        PEmax = float(V_r.max())
        n_eigs_done = 0
        converged = stalled = False
        min_deig, i_best = np.inf, i_start
        self._i_iter = i_start
        for self._i_iter in range(i_start + 1, n_iterations + 1):
            # Filter window per k (_chefsi.py:109-123).
            b_up = KEmax + PEmax
            b_lo = el.eig.max(dim=1).values
            a_lo = el.eig.min(dim=1).values
            b_diff = (0.5 * (b_up - b_lo))[:, None]
            b_mid = (0.5 * (b_lo + b_up))[:, None]
            sigma = b_diff / (b_mid - a_lo[:, None])
            tau = 2.0 / sigma
            prev = (el.C, el.eig, HC, el.deig_max)
            if n_eigs_done:  # converged leading bands are not filtered
                C0, C = el.C.bands(0, n_eigs_done), el.C.bands(n_eigs_done)
                HC0, HC = HC.bands(0, n_eigs_done), HC.bands(n_eigs_done)
            else:
                C = el.C
            # Scaled three-term Chebyshev recursion (_chefsi.py:125-147).
            Y = (HC - C * b_mid) * (sigma / b_diff)
            for _ in range(self.filter_order - 2):
                sigma_new = 1.0 / (tau - sigma)
                HY = el.hamiltonian(Y)
                hpsi += Y.n_bands() * el.basis.nk
                Yt = (HY - Y * b_mid) * (2.0 * sigma_new / b_diff) - C * (sigma * sigma_new)
                C, Y = Y, Yt
                sigma = sigma_new
            HC = el.hamiltonian(Y)
            hpsi += Y.n_bands() * el.basis.nk
            C = Y
            if n_eigs_done:
                C = C0.cat(C)
                HC = HC0.cat(HC)
            # Rayleigh-Ritz in the filtered subspace (_chefsi.py:157-161).
            eig_prev = el.eig
            eig_new, V = eighg((C ^ HC).wait(), (C ^ C).wait(), drop_below=1e-6 if fp32 else 0.0)
            if fp32 and bool(torch.isinf(eig_new).any()):
                stalled = True  # the filtered basis is degenerate at FP32 precision
                el.C, el.eig, HC, el.deig_max = prev
                break
            el.eig = eig_new
            el.C = C @ V
            HC = HC @ V
            d = torch.abs(el.eig - eig_prev)[:, :n_bands]  # _check_deig, _davidson.py:126-139
            el.deig_max = float(d.max())
            if fp32 and min_deig < 1e-3 and el.deig_max > 100.0 * min_deig:
                el.C, el.eig, HC, el.deig_max = prev
                stalled = True
                break
            if el.deig_max < min_deig:
                min_deig, i_best = el.deig_max, self._i_iter
            pending = torch.where((d > self.eig_threshold).any(dim=0))[0]
            n_eigs_done = int(pending[0]) if len(pending) else n_bands
            converged = n_eigs_done >= n_bands
            if converged:
                break
            if fp32 and self._i_iter - i_best >= 10:
                stalled = True
                break
        self._HC = HC
        return DavidsonStats(self._i_iter, converged, el.deig_max, np.inf, hpsi, stalled)
