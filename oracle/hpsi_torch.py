"""The reference's H.psi restated with torch CPU operations (test and baseline infrastructure only).

The reference computes H.psi with torch on the host (qimpy/dft/electrons/
_hamiltonian.py:7-29): KE * C (_basis_ops.py:29-36); the local potential as a
zero-filled FFT grid per band block, a scatter of the coefficients at
fft_index, ``torch.fft.ifftn(norm="forward")``, the product with V(r),
``torch.fft.fftn(norm="forward")`` and a gather (_basis_ops.py:39-113,
152-204; one band per FFT, the block size the reference picks on a CPU,
_basis.py:289-306); the nonlocal term ``beta @ (D_all @ (beta ^ C))`` as complex matrix
products (_hamiltonian.py:22-24, _wavefunction_dot.py:18-191).  This module
does the same operations in the same library, on every host thread, so that
the CPU baseline runs at the speed of the reference's own implementation on
the host that has no copy of the reference.  ``oracle.hpsi`` (numpy) is the
checker; this port is checked against it.
"""
from __future__ import annotations

import numpy as np
import torch


def set_threads(n: int) -> None:
    torch.set_num_threads(int(n))


class Hamiltonian:
    """H of one problem, inputs converted to torch tensors once."""

    def __init__(self, ke, V_r, fft_index, n, beta, D_all, fft_block: int = 1):
        self.ke = torch.from_numpy(np.ascontiguousarray(ke))
        self.V = torch.from_numpy(np.ascontiguousarray(V_r))
        self.shape = tuple(V_r.shape)
        self.N = int(np.prod(self.shape))
        self.fft_index = torch.from_numpy(np.ascontiguousarray(fft_index, dtype=np.int64))
        self.n = [int(x) for x in n]
        self.beta = None if beta is None or beta.shape[1] == 0 else torch.from_numpy(np.ascontiguousarray(beta))
        self.D = None if self.beta is None else torch.from_numpy(np.asarray(D_all, dtype=np.complex128))
        self.fft_block = int(fft_block)

    def __call__(self, C: np.ndarray) -> np.ndarray:
        Ct = torch.from_numpy(np.ascontiguousarray(C))
        nk, nb, n_tot = Ct.shape
        HC = self.ke[:, None, :] * Ct
        for k in range(nk):
            idx = self.fft_index[k]
            for b0 in range(0, nb, self.fft_block):
                blk = Ct[k, b0:b0 + self.fft_block]
                grid = torch.zeros((blk.shape[0], self.N), dtype=torch.complex128)
                grid[:, idx] = blk
                psi = torch.fft.ifftn(grid.view((-1,) + self.shape), dim=(1, 2, 3), norm="forward")
                psi *= self.V
                VC = torch.fft.fftn(psi, dim=(1, 2, 3), norm="forward").flatten(1)[:, idx]
                VC[:, self.n[k]:] = 0.0
                HC[k, b0:b0 + self.fft_block] += VC
        if self.beta is not None:
            proj = self.beta.conj() @ Ct.transpose(1, 2)  # (nk, P, nb)
            HC += (self.beta.transpose(1, 2) @ (self.D @ proj)).transpose(1, 2)
        return HC.numpy()
