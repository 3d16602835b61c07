"""FP64 CPU restatement of the reference's block Davidson eigensolver (test infrastructure only).

Follows qimpy/dft/electrons/_davidson.py:141-235 step by step, with the
subspace linear algebra of qimpy/math/_linalg.py:110-183 (``ortho_matrix``,
``eighg``) and the wavefunction helpers of qimpy/dft/electrons/_wavefunction*.py.
Arrays drop the singleton spin/spinor axes: C[k, b, g], subspace matrices [k, m, m].
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import numpy as np
import scipy.linalg as sla


def dot(C1: np.ndarray, C2: np.ndarray) -> np.ndarray:
    """[k, b1, b2] = sum_g conj(C1[k,b1,g]) C2[k,b2,g] (qimpy/dft/electrons/_wavefunction_dot.py:18-107)."""
    return np.matmul(C1.conj(), np.swapaxes(C2, 1, 2))


def matmul(C: np.ndarray, M: np.ndarray) -> np.ndarray:
    """C @ M along bands: out[k, b', g] = sum_b M[k, b, b'] C[k, b, g]
    (qimpy/dft/electrons/_wavefunction_dot.py:137-191)."""
    return np.matmul(np.swapaxes(M, 1, 2), C)


def dagger(x: np.ndarray) -> np.ndarray:
    return np.conj(np.swapaxes(x, -1, -2))


def ortho_matrix(O: np.ndarray) -> np.ndarray:
    """(L^-1)^H with L = cholesky(O) (qimpy/math/_linalg.py:110-136)."""
    out = np.empty_like(O)
    eye = np.eye(O.shape[-1], dtype=O.dtype)
    for k in range(O.shape[0]):
        L = np.linalg.cholesky(O[k])
        out[k] = dagger(sla.solve_triangular(L, eye, lower=True))
    return out


def eigh(H: np.ndarray):
    E = np.empty(H.shape[:-1])
    V = np.empty_like(H)
    for k in range(H.shape[0]):
        E[k], V[k] = np.linalg.eigh(H[k])
    return E, V


def eighg(H: np.ndarray, O: np.ndarray):
    """Generalised Hermitian eigenproblem H V = O V E (qimpy/math/_linalg.py:143-183)."""
    U = ortho_matrix(O)
    E, V = eigh(dagger(U) @ (H @ U))
    return E, U @ V


def orthonormalize(C: np.ndarray) -> np.ndarray:
    """C @ ortho_matrix(C^C) (qimpy/dft/electrons/_wavefunction_dot.py:194-199)."""
    return matmul(C, ortho_matrix(dot(C, C)))


def band_ke(C: np.ndarray, ke: np.ndarray) -> np.ndarray:
    """sum_g |C|^2 KE (qimpy/dft/electrons/_wavefunction.py:238-247)."""
    return np.einsum("kbg,kg->kb", np.square(C.real) + np.square(C.imag), ke)


def band_norm(C: np.ndarray) -> np.ndarray:
    """sqrt(sum_g |C|^2) (qimpy/dft/electrons/_wavefunction.py:226-236)."""
    return np.sqrt((np.square(C.real) + np.square(C.imag)).sum(axis=-1))


def precondition(Cerr: np.ndarray, ke: np.ndarray, KEref: np.ndarray) -> np.ndarray:
    """Cerr / (x + exp(-x)), x = KE / KEref (qimpy/dft/electrons/_davidson.py:92-99)."""
    x = ke[:, None, :] / KEref[..., None]
    x = x + np.exp(-x)
    return Cerr / x


def _xorshift_randn(x: np.ndarray) -> np.ndarray:
    """Complex normal from signed 64-bit xorshift state, advanced in place
    (qimpy/dft/electrons/_wavefunction_init.py:11-24; torch int64 shifts are arithmetic)."""
    u = []
    with np.errstate(over="ignore"):
        for _ in range(2):
            x ^= x << np.int64(13)
            x ^= x >> np.int64(7)
            x ^= x << np.int64(17)
            u.append((0.5**64) * x.astype(np.float64) + 0.5)
    return np.sqrt(-2.0 * np.log(u[0])) * np.exp((2j * np.pi) * u[1])


def randomize_selected(C, i_k, i_band, seed, n, n_max, nk_tot, ke):
    """Re-randomise selected bands (qimpy/dft/electrons/_wavefunction_init.py:127-188),
    one spin and one spinor component."""
    n_bands, n_tot = C.shape[1], C.shape[2]
    i_basis = np.arange(n_tot, dtype=np.int64)
    x = ((1 + seed) + i_basis[None, :] + n_max * (i_band[:, None] + n_bands * i_k[:, None])).astype(np.int64)
    _xorshift_randn(x)
    vals = _xorshift_randn(x)
    for j, (k, b) in enumerate(zip(i_k, i_band)):
        v = vals[j].copy()
        v[int(n[k]) :] = 0.0
        C[k, b] = v / (1.0 + ((4.0 / 3) * ke[k]) ** 6)


def tile_expansion(C_XC: np.ndarray, Cnew_XCexp: np.ndarray) -> np.ndarray:
    """Assemble the expanded subspace matrix (qimpy/dft/electrons/_davidson.py:240-264)."""
    nk, n_new, n_exp = Cnew_XCexp.shape
    n_cur = n_new - n_exp
    out = np.zeros((nk, n_new, n_new), dtype=np.complex128)
    out[:, :n_cur, :n_cur] += C_XC
    out[:, :n_cur, n_cur:] = Cnew_XCexp[:, :n_cur]
    out[:, n_cur:, :n_cur] = dagger(Cnew_XCexp[:, :n_cur])
    out[:, n_cur:, n_cur:] = Cnew_XCexp[:, n_cur:]
    return out


@dataclass
class DavidsonResult:
    eig: np.ndarray  #: (nk, n_bands + n_bands_extra)
    C: np.ndarray
    iterations: int
    converged: bool
    deig_max: float
    hpsi_bands: int  #: band-applications of H performed
    HC: np.ndarray = None  #: H C carried through the rotations (as the reference keeps it)


def dot_real(C1: np.ndarray, C2: np.ndarray, gweight: np.ndarray) -> np.ndarray:
    """Real-wavefunction overlap: Re sum_G w_G conj(C1) C2 (the implicit -G
    partners), imaginary part zeroed (qimpy/dft/electrons/_wavefunction_dot.py:55-88)."""
    return np.matmul(C1.conj() * gweight, np.swapaxes(C2, 1, 2)).real.astype(np.complex128)


def davidson(
    hamiltonian: Callable[[np.ndarray], np.ndarray],
    C: np.ndarray,
    ke: np.ndarray,
    n: np.ndarray,
    n_bands: int,
    n_iterations: int = 100,
    eig_threshold: float = 1e-8,
    gweight: np.ndarray | None = None,
    symmetrize: Callable[[np.ndarray], np.ndarray] | None = None,
) -> DavidsonResult:
    """Block Davidson (qimpy/dft/electrons/_davidson.py:141-235) on orthonormal
    start vectors C[k, n_bands + n_bands_extra, g].

    Real (Gamma-point) wavefunctions: `gweight` (1 on Gz = 0, 2 elsewhere, 0 on
    padding) weights the overlaps, norms and kinetic energies and `symmetrize`
    makes the Gz = 0 plane Hermitian in constrain (_wavefunction.py:226-275)."""
    if gweight is not None:
        dot_, band_norm_ = (lambda A, B: dot_real(A, B, gweight)), \
            (lambda A: np.sqrt(((np.square(A.real) + np.square(A.imag)) * gweight).sum(axis=-1)))
        band_ke_ = lambda A, kin: band_ke(A, kin * gweight)  # noqa: E731
    else:
        dot_, band_norm_, band_ke_ = dot, band_norm, band_ke
    nk, n_bands_max, n_tot = C.shape
    if 2 * n_bands_max >= int(n.min()):
        raise ValueError(
            f"n_bands + n_bands_extra = {n_bands_max} exceeds min(n_basis)/2 = {int(n.min()) // 2} in Davidson"
        )
    norm_cut = np.sqrt(n_tot * 1e-15)  # _davidson.py:56-58
    hpsi_bands = nk * n_bands_max
    HC = hamiltonian(C)
    eig, V = eigh(dot_(C, HC))  # _davidson.py:164-168
    C = matmul(C, V)
    HC = matmul(HC, V)
    n_eigs_done = 0
    deig_max = np.inf
    converged = False
    i_iter = 0
    for i_iter in range(1, n_iterations + 1):
        n_bands_cur = C.shape[1]
        eig_sel = eig[:, n_eigs_done:, None]
        C_sel = C[:, n_eigs_done:]
        HC_sel = HC[:, n_eigs_done:]
        KEref = band_ke_(C_sel, ke)
        Cexp = precondition(HC_sel - C_sel * eig_sel, ke, KEref)
        norm_exp = band_norm_(Cexp)
        low_k, low_b = np.where(norm_exp < norm_cut)  # _davidson.py:101-115
        if len(low_k):
            # Real wavefunctions draw the same numbers: the reference's extra
            # conjugate-seeded Gz = 0 term (_wavefunction_init.py:175-181) is added
            # to an advanced-indexing copy and does not reach the coefficients;
            # the Hermitian symmetrisation of constrain below follows.
            randomize_selected(Cexp, low_k, low_b, i_iter, n, int(n.max()), nk, ke)
            norm_exp[low_k, low_b] = 1.0
        Cexp = Cexp * (1.0 / norm_exp)[..., None]
        for k in range(nk):
            Cexp[k, :, int(n[k]) :] = 0.0
        if symmetrize is not None:
            symmetrize(Cexp)
        n_bands_exp = Cexp.shape[1]
        n_bands_new = n_bands_cur + n_bands_exp
        Cnew = np.concatenate((C, Cexp), axis=1)
        C_OC_new = tile_expansion(np.eye(n_bands_cur)[None], dot_(Cnew, Cexp))
        HCexp = hamiltonian(Cexp)
        hpsi_bands += nk * n_bands_exp
        C_HC_new = tile_expansion(np.stack([np.diag(e) for e in eig]), dot_(Cnew, HCexp))
        eig_new, V_new = eighg(C_HC_new, C_OC_new)
        n_bands_next = min(n_bands_new, n_bands_max)
        V_new = V_new[..., :n_bands_next]
        Vcur, Vexp = V_new[:, :n_bands_cur], V_new[:, n_bands_cur:]
        C = matmul(Cnew, V_new)
        HC = matmul(HC, Vcur) + matmul(HCexp, Vexp)
        deig = np.abs(eig - eig_new[:, :n_bands_cur])
        eig = eig_new[:, :n_bands_next]
        # _check_deig (_davidson.py:126-139):
        deig_max = float(deig[:, :n_bands].max())
        pending = np.where((deig[:, :n_bands] > eig_threshold).any(axis=0))[0]
        n_eigs_done = int(pending[0]) if len(pending) else n_bands
        if n_eigs_done >= n_bands:
            converged = True
            break
    return DavidsonResult(eig, C, i_iter, converged, deig_max, hpsi_bands, HC)
