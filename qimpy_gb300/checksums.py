"""Size-independent checks of band arrays: per-band checksums that compare a
full-size H.psi result without storing it.

For coefficients X[k, b, g] (padding beyond n[k] ignored) the checksum of band
(k, b) is (sum_g |X|^2, Re sum_g w_g X, Im sum_g w_g X) with fixed weights
w_g in (0, 1) from the splitmix64 stream (seed 0, stream 999).
"""
from __future__ import annotations

import numpy as np

from .workloads import splitmix_uniform


def checksum_weights(n_tot: int) -> np.ndarray:
    return splitmix_uniform(0, 999, n_tot)


def band_checksums(X: np.ndarray, n: np.ndarray) -> np.ndarray:
    """(nk, nb, 3) float64 checksums of complex X (nk, nb, n_tot)."""
    nk, nb, n_tot = X.shape
    w = checksum_weights(n_tot)
    out = np.zeros((nk, nb, 3))
    for k in range(nk):
        Xk = X[k, :, : int(n[k])]
        out[k, :, 0] = np.square(np.abs(Xk)).sum(axis=1)
        s = Xk @ w[: int(n[k])]
        out[k, :, 1] = s.real
        out[k, :, 2] = s.imag
    return out
