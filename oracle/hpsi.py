"""FP64 CPU restatement of the reference's Hamiltonian apply (test infrastructure only).

Layouts follow the reference with the singleton spin and spinor axes dropped:
coefficients C[k, b, g] complex128 with g over the padded basis n_tot,
projectors beta[k, p, g], projections proj[k, p, b], D_all[p, p'].
"""
from __future__ import annotations

import os

import numpy as np
import scipy.fft as sfft

_WORKERS = int(os.environ.get("ORACLE_THREADS", "1"))


def set_threads(n: int) -> None:
    """Threads used by the FFTs of the oracle (1 = scalar port)."""
    global _WORKERS
    _WORKERS = max(1, int(n))


def constrain(C: np.ndarray, n: np.ndarray) -> np.ndarray:
    """Zero padded coefficients beyond n[k] (qimpy/dft/electrons/_wavefunction.py:264-275)."""
    for k in range(C.shape[0]):
        C[k, ..., int(n[k]) :] = 0.0
    return C


def apply_ke(ke: np.ndarray, C: np.ndarray) -> np.ndarray:
    """KE(k, g) * C (qimpy/dft/electrons/_basis_ops.py:29-36; KE from _basis.py:256-270)."""
    return C * ke[:, None, :]


def apply_potential(V_r: np.ndarray, fft_index: np.ndarray, n: np.ndarray, C: np.ndarray) -> np.ndarray:
    """gather(fft(V * ifft(scatter(C)))) then zero padding.

    Follows qimpy/dft/electrons/_basis_ops.py:39-113 and 152-199: scatter every
    padded coefficient to its grid point (fft_index), inverse FFT with
    norm="forward" (no scaling; qimpy/grid/_fft.py:298), multiply by the real
    V(r), forward FFT with norm="forward" (scale 1/N; qimpy/grid/_fft.py:239),
    gather at fft_index, then ``constrain``."""
    nk, nb, n_tot = C.shape
    shape = V_r.shape
    N = int(np.prod(shape))
    out = np.empty_like(C)
    for k in range(nk):
        grid = np.zeros((nb, N), dtype=np.complex128)
        grid[:, fft_index[k]] = C[k]
        psi_r = sfft.ifftn(grid.reshape((nb,) + shape), axes=(1, 2, 3), norm="forward", workers=_WORKERS)
        # real V times complex psi, as pairs of doubles (one pass, no complex promotion of V)
        psi_r.view(np.float64).reshape(psi_r.shape + (2,))[...] *= V_r[None, ..., None]
        VC = sfft.fftn(psi_r, axes=(1, 2, 3), norm="forward", workers=_WORKERS).reshape(nb, N)
        out[k] = VC[:, fft_index[k]]
    return constrain(out, n)


def project(beta: np.ndarray, C: np.ndarray) -> np.ndarray:
    """<beta|C>: proj[k, p, b] = sum_g conj(beta[k, p, g]) C[k, b, g]
    (qimpy/dft/electrons/_wavefunction.py:106-123 via _wavefunction_dot.py:18-107),
    evaluated as conj(beta[k] @ conj(C[k])^T) so that only the band block is
    conjugated (one BLAS product per k)."""
    out = np.empty((beta.shape[0], beta.shape[1], C.shape[1]), dtype=np.result_type(beta, C))
    for k in range(beta.shape[0]):
        out[k] = np.conj(beta[k] @ np.conj(C[k]).T)
    return out


def apply_nonlocal(beta: np.ndarray, D_all: np.ndarray, proj: np.ndarray) -> np.ndarray:
    """beta @ (D_all @ proj): out[k, b, g] = sum_p beta[k, p, g] (D proj)[k, p, b]
    (qimpy/dft/electrons/_hamiltonian.py:22-24; matmul of _wavefunction_dot.py:137-191)."""
    Dp = np.matmul(D_all[None], proj)
    return np.matmul(np.swapaxes(Dp, 1, 2), beta)


def hamiltonian(ke, V_r, fft_index, n, beta, D_all, C) -> np.ndarray:
    """HC = KE C + V C + beta D <beta|C> (qimpy/dft/electrons/_hamiltonian.py:7-29;
    the meta-GGA tau and DFT+U terms are absent for a fixed LDA-like potential)."""
    HC = apply_ke(ke, C)
    HC += apply_potential(V_r, fft_index, n, C)
    if beta is not None and beta.shape[1]:
        HC += apply_nonlocal(beta, D_all, project(beta, C))
    return HC


def collect_density(fft_index: np.ndarray, shape, C: np.ndarray, prefac: np.ndarray) -> np.ndarray:
    """rho(r) = sum_kb prefac[k, b] |psi_kb(r)|^2 with psi = ifft(scatter(C)) (no
    scaling), prefac = f * w_sk / Omega; real-space grid in natural order.

    Follows qimpy/dft/electrons/_basis_ops.py:207-296 (single spin, no spinor):
    expand_ifft of every band (152-163) and accum_norm_ (qimpy/math/_linalg.py:31-58)."""
    nk, nb, n_tot = C.shape
    N = int(np.prod(shape))
    rho = np.zeros(tuple(shape))
    for k in range(nk):
        grid = np.zeros((nb, N), dtype=np.complex128)
        grid[:, fft_index[k]] = C[k]
        psi_r = sfft.ifftn(grid.reshape((nb,) + tuple(shape)), axes=(1, 2, 3), norm="forward", workers=_WORKERS)
        rho += np.einsum("b,bxyz->xyz", prefac[k], np.abs(psi_r) ** 2)
    return rho


# ---------------------------------------------------------------------------
# Real (Gamma-point) wavefunctions: half-mesh basis, r2c / c2r FFTs
# (qimpy/dft/electrons/_basis_real.py:10-106, _basis_ops.py:119-163 with
# shapeH, qimpy/grid/_fft.py real dispatch, _wavefunction_dot.py:55-88).
# ---------------------------------------------------------------------------


def real_gweight(iG: np.ndarray, n: int, n_tot: int) -> np.ndarray:
    """Overlap weight of each basis entry: 1 on the Gz = 0 plane, 2 elsewhere
    (the implicit -G partner), 0 on padding (_basis_real.py:62-66)."""
    w = np.where(iG[:, 2] == 0, 1.0, 2.0)
    w[n:] = 0.0
    return w[:n_tot]


def real_symmetrize(C: np.ndarray, iG: np.ndarray, shape) -> np.ndarray:
    """Hermitian Gz = 0 plane, c(G) = (c(G) + conj(c(-G))) / 2, in place
    (BasisReal.symmetrize, _basis_real.py:68-106); iG is the k = 0 basis."""
    N0, N1 = shape[0], shape[1]
    z0 = np.flatnonzero(iG[:, 2] == 0)
    key = (iG[z0, 0] % N0) * N1 + (iG[z0, 1] % N1)
    key_conj = ((-iG[z0, 0]) % N0) * N1 + ((-iG[z0, 1]) % N1)
    where = {int(kk): i for i, kk in enumerate(key)}
    partner = np.array([where[int(kk)] for kk in key_conj])
    cz = C[..., z0]
    C[..., z0] = 0.5 * (cz + np.conj(cz[..., partner]))
    return C


def apply_potential_real(V_r: np.ndarray, fft_index: np.ndarray, n: np.ndarray, iG: np.ndarray,
                         C: np.ndarray) -> np.ndarray:
    """gather(rfft(V * irfft(scatter(C)))) on the half grid, then constrain
    (padding zeroed, Gz = 0 plane symmetrised); norms as apply_potential."""
    nk, nb, n_tot = C.shape
    shape = V_r.shape
    half = (shape[0], shape[1], shape[2] // 2 + 1)
    out = np.empty_like(C)
    for k in range(nk):
        grid = np.zeros((nb, int(np.prod(half))), dtype=np.complex128)
        grid[:, fft_index[k]] = C[k]
        psi_r = sfft.irfftn(grid.reshape((nb,) + half), s=shape, axes=(1, 2, 3), norm="forward", workers=_WORKERS)
        VC = sfft.rfftn(psi_r * V_r[None], axes=(1, 2, 3), norm="forward", workers=_WORKERS).reshape(nb, -1)
        out[k] = VC[:, fft_index[k]]
    constrain(out, n)
    return real_symmetrize(out, iG[0], shape)


def project_real(beta: np.ndarray, C: np.ndarray, gweight: np.ndarray) -> np.ndarray:
    """<beta|C> of real wavefunctions: Re sum_G w_G conj(beta) C, as proj[k, p, b]
    (the real-basis branch of _wavefunction_dot.py:55-88)."""
    r = np.matmul(beta.conj() * gweight[None, None, :], np.swapaxes(C, 1, 2))
    return r.real.astype(np.complex128)


def hamiltonian_real(ke, V_r, fft_index, n, iG, beta, D_all, C, gweight) -> np.ndarray:
    """HC = KE C + V C + beta D <beta|C> for real (Gamma-point) wavefunctions."""
    HC = apply_ke(ke, C)
    HC += apply_potential_real(V_r, fft_index, n, iG, C)
    if beta is not None and beta.shape[1]:
        HC += apply_nonlocal(beta, D_all, project_real(beta, C, gweight))
    return HC


def collect_density_real(fft_index: np.ndarray, shape, C: np.ndarray, prefac: np.ndarray) -> np.ndarray:
    """Density of real (Gamma-point) wavefunctions: psi = irfft(scatter(C)) on
    the half grid (no scaling), rho = sum_b prefac |psi|^2 (_basis_ops.py:207-296
    with the real-basis expand of _basis_ops.py:119-163)."""
    nk, nb, n_tot = C.shape
    half = (shape[0], shape[1], shape[2] // 2 + 1)
    rho = np.zeros(tuple(shape))
    for k in range(nk):
        grid = np.zeros((nb, int(np.prod(half))), dtype=np.complex128)
        grid[:, fft_index[k]] = C[k]
        psi_r = sfft.irfftn(grid.reshape((nb,) + half), s=tuple(shape), axes=(1, 2, 3), norm="forward",
                            workers=_WORKERS)
        rho += np.einsum("b,bxyz->xyz", prefac[k], psi_r ** 2)
    return rho
