"""FP64 CPU restatement of the reference's projector construction (test infrastructure only).

Restates Ions.get_projectors (qimpy/dft/ions/_ions_projectors.py:14-72) with
its pieces: the quintic blip spline (qimpy/math/quintic_spline.py:13-130:
get_coeff and Interpolator), the real solid harmonics times the reciprocal
phase i^l (qimpy/math/spherical_harmonics.py:41-137, get_harmonics_tilde; l <= 2
here) and the translation phases exp(-2 pi i (iG + k).tau) / sqrt(Omega)
(qimpy/dft/ions/_ions.py:304-311).  A shell is (l, ("gauss", sigma)) or
(l, ("blip", coeff, dq)); a Gaussian shell's radial part is the analytic
(-1)^l (2 pi)^{3/2} sigma^{2l+3} exp(-sigma^2 q^2 / 2).
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import solve_banded

#: Quintic B-spline pieces (weights of 6 consecutive coefficients at fractional
#: position t: t^p @ _BLIP / 66), quintic_spline.py:86-96.
_BLIP = np.array([[1.0, 26.0, 66.0, 26.0, 1.0, 0.0], [-5.0, -50.0, 0.0, 50.0, 5.0, 0.0],
                  [10.0, 20.0, -60.0, 20.0, 10.0, 0.0], [-10.0, 20.0, 0.0, -20.0, 10.0, 0.0],
                  [5.0, -20.0, 30.0, -20.0, 5.0, 0.0], [-1.0, 5.0, -10.0, 10.0, -5.0, 1.0]]) / 66.0


def blip_coeff(samples: np.ndarray) -> np.ndarray:
    """Blip coefficients (N + 4) of uniformly spaced samples (N): mirror
    symmetry at the left end, natural (zero 3rd and 4th derivative) at the
    right (quintic_spline.py:13-54)."""
    N = samples.shape[-1]
    off1, off2 = 13.0 / 33, 1.0 / 66
    band = np.tile(np.array([[off2, off1, 1.0, off1, off2]]).T, (1, N))
    band[2, 1] += off2
    band[1, 1] += off1
    band[0, 2] += off2
    extrap = np.array(((1.0, -3.0, 3.0), (3.0, -8.0, 6.0)))
    band[(3, 2, 1), (-3, -2, -1)] += off2 * extrap[0]
    band[(4, 3, 2), (-3, -2, -1)] += (off1, off2) @ extrap
    c = solve_banded((2, 2), band, samples)
    return np.concatenate((c[2:0:-1], c, extrap @ c[-3:]))


def blip_eval(coeff: np.ndarray, dq: float, x: np.ndarray) -> np.ndarray:
    """Spline value at x from blip coefficients on spacing dq (Interpolator,
    quintic_spline.py:57-130)."""
    u = np.asarray(x, dtype=np.float64) / dq
    i = np.floor(u).astype(np.int64)
    t = u - i
    f = (t[:, None] ** np.arange(6)[None, :]) @ _BLIP  # (n, 6)
    return (coeff[i[:, None] + np.arange(6)[None, :]] * f).sum(axis=1)


def solid_harmonics_tilde(l: int, q: np.ndarray) -> np.ndarray:
    """i^l |q|^l Y_lm(q) for m = -l..l, l = 1 as (y, z, x), l = 2 as
    (xy, yz, 3z^2 - r^2, xz, x^2 - y^2) (spherical_harmonics.py:41-137)."""
    x, y, z = q[:, 0], q[:, 1], q[:, 2]
    if l == 0:
        S = np.full((1, x.size), 0.5 / np.sqrt(np.pi))
    elif l == 1:
        S = np.sqrt(3.0 / (4.0 * np.pi)) * np.stack((y, z, x))
    elif l == 2:
        a, b, c = np.sqrt(15.0 / (4.0 * np.pi)), np.sqrt(5.0 / (16.0 * np.pi)), np.sqrt(15.0 / (16.0 * np.pi))
        S = np.stack((a * x * y, a * y * z, b * (3.0 * z * z - (x * x + y * y + z * z)), a * x * z, c * (x * x - y * y)))
    else:
        raise ValueError(f"l = {l} not restated")
    return S * (1j ** l)


def radial(shell, qmag: np.ndarray) -> np.ndarray:
    l, (kind, *par) = shell
    if kind == "gauss":
        sigma = par[0]
        return (-1.0) ** l * (2.0 * np.pi) ** 1.5 * sigma ** (2 * l + 3) * np.exp(-0.5 * sigma * sigma * qmag ** 2)
    coeff, dq = par
    return blip_eval(coeff, dq, qmag)


def projectors(iG: np.ndarray, k: np.ndarray, Gbasis: np.ndarray, n: np.ndarray, positions: np.ndarray,
               shells, volume: float) -> np.ndarray:
    """beta[k, a pa + j, g] for one species on every atom (get_projectors,
    _ions_projectors.py:14-72); padding entries zero."""
    nk, n_tot = iG.shape[:2]
    pa = sum(2 * l + 1 for l, _ in shells)
    beta = np.zeros((nk, len(positions) * pa, n_tot), dtype=np.complex128)
    for ik in range(nk):
        m = int(n[ik])
        kiG = iG[ik, :m] + k[ik][None, :]
        q = kiG @ Gbasis.T
        qmag = np.sqrt(np.square(q).sum(axis=1))
        tmpl = np.concatenate([solid_harmonics_tilde(l, q) * radial((l, r), qmag)[None, :] for l, r in shells])
        trans = np.exp(-2j * np.pi * (kiG @ positions.T)).T / np.sqrt(volume)  # (atom, g)
        beta[ik, :, :m] = (tmpl[None, :, :] * trans[:, None, :]).reshape(-1, m)
    return beta
