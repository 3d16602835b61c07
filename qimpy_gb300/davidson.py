"""Block Davidson on the GPU, the reference's algorithm on the CUDA H.psi path.

Follows qimpy/dft/electrons/_davidson.py:141-235 step for step (subspace
expansion by the inverse-kinetic preconditioner, expanded generalised
eigenproblem, retention of n_bands + n_bands_extra, convergence on the maximum
eigenvalue change).  Additions:

* an optional residual-norm stop (max_b ||H psi_b - eps_b psi_b|| over the
  first n_bands, in FP64) beside the reference's eigenvalue-change stop;
* for FP32 (mixed-precision) vectors: span(C) projected out of the
  expansion vectors (same subspace, better conditioned), canonical
  orthogonalisation of the expanded basis where its overlap is still too
  ill-conditioned for FP32 (directions below 1e-4 of the overlap dropped), and
  a stop at FP32's floor that leaves the rest to the FP64 refinement;
* real (Gamma-point) wavefunctions (Basis(real=True)): weighted overlaps,
  norms and kinetic energies, real subspace matrices and eigenvectors, and the
  Gz = 0 plane symmetrised after every expansion (the reference's Davidson in
  real-wavefunction mode, _basis_real.py with _wavefunction_dot.py:55-88);
* ``refine_fp64``: FP64 refinement of a mixed-precision solve (Cholesky
  orthonormalisation, then FP64 Davidson sweeps: FP64 H.psi, Rayleigh-Ritz,
  residual expansion, expanded Rayleigh-Ritz).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import ops
from .electrons import Electrons, Wavefunction
from .linalg import eigh, eighg


@dataclass
class DavidsonStats:
    iterations: int
    converged: bool
    deig_max: float
    residual_max: float
    hpsi_bands: int
    #: FP32 only: stopped at the precision floor (basis too ill-conditioned for
    #: FP32, or eigenvalue changes growing again); el holds the last good state.
    stalled: bool = False


def _xorshift_randn(x: torch.Tensor) -> torch.Tensor:
    """Complex normal deviates from a signed 64-bit xorshift state, advanced in
    place (qimpy/dft/electrons/_wavefunction_init.py:11-24: shifts of torch
    int64 are arithmetic, overflow wraps; Box-Muller from two uniforms)."""
    u = []
    for _ in range(2):
        x ^= x << 13
        x ^= x >> 7
        x ^= x << 17
        u.append((0.5 ** 64) * x.to(torch.float64) + 0.5)
    return torch.sqrt(-2.0 * torch.log(u[0])) * torch.exp((2j * np.pi) * u[1])


def randomize_selected(C: Wavefunction, i_k: torch.Tensor, i_band: torch.Tensor, seed: int) -> None:
    """Seeded random bands (k, band) of C in place, one spin and one spinor
    (qimpy/dft/electrons/_wavefunction_init.py:127-188): the state of every
    coefficient is (1 + seed) + g + n_max (band + n_bands k), one warm-up draw,
    then a complex normal; padding zeroed, damped by 1 / (1 + (4/3 KE)^6)."""
    basis = C.basis
    n_bands, n_tot = C.coeff.shape[1], C.coeff.shape[2]
    dev = C.coeff.device
    i_k, i_band = i_k.to(dev, torch.int64), i_band.to(dev, torch.int64)
    n_max = int(basis.n_max)
    g = torch.arange(n_tot, dtype=torch.int64, device=dev)
    x = (1 + seed) + g[None, :] + n_max * (i_band[:, None] + n_bands * i_k[:, None])
    _xorshift_randn(x)  # warm-up: discard one output after seeding
    vals = _xorshift_randn(x)
    vals = vals * basis.mask[i_k].to(vals.real.dtype) / (1.0 + ((4.0 / 3) * basis.ke[i_k]) ** 6)
    C.coeff[i_k, i_band] = vals.to(C.coeff.dtype)
    C._projT = None


def _sub(M: torch.Tensor, real: bool) -> torch.Tensor:
    """Subspace matrix as the eigensolver takes it: real wavefunctions' overlaps
    are real (their imaginary parts are zero by construction)."""
    return M.real.contiguous() if real else M


def _tile_expansion(C_XC: torch.Tensor, Cnew_XCexp: torch.Tensor) -> torch.Tensor:
    """Expanded subspace matrix (qimpy/dft/electrons/_davidson.py:240-264)."""
    nk, n_new, n_exp = Cnew_XCexp.shape
    n_cur = n_new - n_exp
    out = torch.zeros((nk, n_new, n_new), dtype=Cnew_XCexp.dtype, device=Cnew_XCexp.device)
    out[:, :n_cur, :n_cur] += C_XC
    out[:, :n_cur, n_cur:] = Cnew_XCexp[:, :n_cur]
    out[:, n_cur:, :n_cur] = Cnew_XCexp[:, :n_cur].conj().transpose(-2, -1)
    out[:, n_cur:, n_cur:] = Cnew_XCexp[:, n_cur:]
    return out


class Davidson:
    """Davidson diagonalisation of ``electrons`` (qimpy/dft/electrons/_davidson.py:16-237)."""

    def __init__(self, electrons: Electrons, n_iterations: int = 100, eig_threshold: float = 1e-8,
                 residual_threshold: Optional[float] = None):
        self.electrons = electrons
        self.n_iterations = n_iterations
        self.eig_threshold = eig_threshold
        self.residual_threshold = residual_threshold
        # Expansion vectors shorter than this are treated as null and re-randomised
        # (_davidson.py:56-58, 101-115).  The reference's round-off estimate
        # sqrt(n_tot * 1e-15) is also a floor on reachable residuals, so a
        # residual target below it lowers the cut to 1% of the target.
        self._norm_cut = float(np.sqrt(electrons.basis.n_tot * 1e-15))
        if residual_threshold is not None:
            self._norm_cut = min(self._norm_cut, 0.01 * residual_threshold)
        self._i_iter = 0

    def precondition(self, Cerr: Wavefunction, KEref: torch.Tensor) -> Wavefunction:
        """Cerr / (x + exp(-x)), x = KE / KEref (qimpy/dft/electrons/_davidson.py:92-99),
        one pass of qgb_residual (with zero eigenvalues, the residual of Cerr is Cerr)."""
        out = torch.empty_like(Cerr.coeff)
        zero = torch.zeros((Cerr.coeff.shape[0], Cerr.n_bands()), dtype=torch.float64, device=out.device)
        ops.residual(Cerr.coeff, Cerr.coeff, zero, self.electrons.basis.ke, KEref, out=out,
                     weight=self.electrons.basis.weight)
        return Wavefunction(Cerr.basis, coeff=out)

    def _regularize(self, C: Wavefunction, norm: torch.Tensor, i_iter: int) -> None:
        """Re-randomise null bands (qimpy/dft/electrons/_davidson.py:101-115) with
        the reference's seeded generator (randomize_selected, seed = i_iter)."""
        low = norm < self._norm_cut
        if not bool(low.any()):
            return
        i_k, i_b = torch.where(low)
        randomize_selected(C, i_k, i_b, i_iter)
        norm[i_k, i_b] = 1.0  # just an estimate, as in the reference

    def __call__(self, n_iterations: Optional[int] = None) -> DavidsonStats:
        """Run to convergence with direct H.psi calls."""
        el = self.electrons
        gen = self.steps(n_iterations)
        block = next(gen)
        while True:
            try:
                block = gen.send(el.hamiltonian(block))
            except StopIteration as stop:
                return stop.value

    def steps(self, n_iterations: Optional[int] = None):
        """The Davidson iteration as a generator: it yields every block of
        vectors it needs H applied to and expects the H.psi result sent back;
        its return value is the DavidsonStats.  A driver can therefore batch the
        H.psi of many concurrent eigensolves (the serving loop does)."""
        el = self.electrons
        n_bands = el.n_bands
        n_bands_max = n_bands + el.n_bands_extra
        n_iterations = n_iterations or self.n_iterations
        if 2 * n_bands_max >= el.basis.n_min:
            raise ValueError(
                f"n_bands + n_bands_extra = {n_bands_max} exceeds min(n_basis)/2 = {el.basis.n_min // 2} in Davidson"
            )
        hpsi_bands = el.C.n_bands() * el.basis.nk
        real = el.basis.real is not None
        w = el.basis.weight
        cdt = torch.float64 if real else torch.complex128
        HC = yield el.C
        el.eig, V = eigh(_sub((el.C ^ HC).wait(), real))  # _davidson.py:164-168
        el.deig_max = np.inf
        el.C = el.C @ V
        HC = HC @ V
        n_eigs_done = 0
        converged = False
        res_max = np.inf
        self._i_iter = 0
        fp32 = el.C.coeff.dtype == torch.complex64
        stalled = False
        min_deig, i_best = np.inf, 0
        for self._i_iter in range(1, n_iterations + 1):
            n_bands_cur = el.C.n_bands()
            basis = el.basis
            # Expansion from the unconverged bands [n_eigs_done, n_bands_cur)
            # (_davidson.py:177-183), in three band-wise passes: reference KE,
            # preconditioned residual (with its norm), then null-band
            # randomisation, normalisation and constrain; no host sync.
            KEref = ops.band_norm_ke(el.C.coeff, basis.ke, b0=n_eigs_done, norm=False, weight=w)[1]
            Cexp = Wavefunction(basis, coeff=torch.empty((basis.nk, n_bands_cur - n_eigs_done, basis.n_tot),
                                                         dtype=el.C.coeff.dtype, device=el.C.coeff.device))
            norm_exp = ops.residual(HC.coeff, el.C.coeff, el.eig, basis.ke, KEref, b0=n_eigs_done, out=Cexp.coeff,
                                    norm=not fp32, weight=w)
            if fp32:
                # Project span(C) out of the expansion (twice: classical
                # Gram-Schmidt with re-orthogonalisation).  span(C, Cexp) and
                # hence the Ritz pairs are unchanged, but near convergence the
                # new directions are a small part of Cexp, and keeping the rest
                # would leave the overlap too ill-conditioned for FP32.
                for _ in range(2):
                    ops.matmul(el.C.coeff, -_sub((el.C ^ Cexp).wait(), real), out=Cexp.coeff, accumulate=True,
                               tc=basis.tc_subspace and not real)
                norm_exp = Cexp.band_norm()
            ops.normalize_bands(Cexp.coeff, basis.n_device, norm_exp, self._norm_cut, self._i_iter, basis.n_max,
                                basis.ke)
            if real:
                ops.symmetrize_real(basis.real, Cexp.coeff)
            n_bands_exp = Cexp.n_bands()
            n_bands_new = n_bands_cur + n_bands_exp
            Cnew = el.C.cat(Cexp)
            C_OC = torch.eye(n_bands_cur, device=V.device, dtype=cdt)[None]
            C_OC_new = _tile_expansion(C_OC, _sub((Cnew ^ Cexp).wait(), real))
            HCexp = yield Cexp
            hpsi_bands += n_bands_exp * el.basis.nk
            C_HC = torch.diag_embed(el.eig).to(cdt)
            C_HC_new = _tile_expansion(C_HC, _sub((Cnew ^ HCexp).wait(), real))
            # FP32 vectors: directions the expanded basis barely spans are below
            # its rounding and are dropped (canonical orthogonalisation).
            n_bands_next = min(n_bands_new, n_bands_max)
            # FP32 vectors: the Cholesky path first; if its pivots call for the
            # canonical orthogonalisation (known at the one host transfer of the
            # iteration), the subspace problem is solved again that way.
            for canonical in (False, True):
                eig_new, V_new, failed, canon = eighg(C_HC_new, C_OC_new, drop_below=1e-4 if fp32 else 0.0,
                                                      check=False, defer_canonical=True, force_canonical=canonical)
                # Everything the host needs from this iteration in one transfer:
                # _check_deig (_davidson.py:126-139), the factorisation status and,
                # for FP32, whether fewer usable directions than bands remain.
                d = torch.abs(el.eig - eig_new[..., :n_bands_cur])[:, :n_bands]
                pend = (d > self.eig_threshold).any(dim=0)
                first_pending = torch.where(pend.any(), pend.int().argmax(),
                                            torch.full((), n_bands, dtype=torch.int64, device=pend.device))
                host = torch.stack((d.max(), first_pending.to(torch.float64), failed.any().to(torch.float64),
                                    torch.isinf(eig_new[:, n_bands_next - 1]).any().to(torch.float64),
                                    canon.to(torch.float64))).tolist()
                if not host[4]:
                    break
            if host[2]:
                raise RuntimeError("subspace eigenproblem failed: overlap not positive-definite or eigh did not converge")
            if fp32 and host[3]:
                # Fewer usable directions than retained bands: no usable update
                # at FP32 precision.  Keep the current state.
                stalled = True
                break
            deig_max = host[0]
            if fp32 and min_deig < 1e-3 and deig_max > 100.0 * min_deig:
                # FP32 rounding has started to feed back: keep the current state and stop.
                stalled = True
                break
            V_new = V_new[..., :n_bands_next]
            Vcur, Vexp = V_new[:, :n_bands_cur], V_new[:, n_bands_cur:]
            el.C = Cnew @ V_new
            HC = HC @ Vcur
            HC += HCexp @ Vexp
            el.eig = eig_new[..., :n_bands_next].contiguous()
            el.deig_max = deig_max
            if el.deig_max < min_deig:
                min_deig, i_best = el.deig_max, self._i_iter
            n_eigs_done = int(host[1])
            converged = n_eigs_done >= n_bands
            if converged and self.residual_threshold is not None:
                # HC is carried by rotations and drifts from H C over many
                # iterations; test residuals against a fresh H C.
                HC = yield el.C
                hpsi_bands += el.C.n_bands() * el.basis.nk
                res = ops.residual(HC.coeff, el.C.coeff, el.eig, norm=True, weight=w)
                res_band = res[:, :n_bands].amax(dim=0)  # worst k-point per band
                host_res = torch.stack((res_band.max(), (res_band >= self.residual_threshold).int().argmax()
                                        .to(torch.float64))).tolist()
                res_max = host_res[0]
                if res_max >= self.residual_threshold:
                    converged = False
                    # Eigenvalues settled, residuals not yet: the bands below the
                    # first one above the target stay converged; the rest expand.
                    n_eigs_done = int(host_res[1])
            if converged:
                break
            if fp32 and self._i_iter - i_best >= 10:
                stalled = True  # no progress for 10 iterations: FP32's floor
                break
        self._HC = HC
        return DavidsonStats(self._i_iter, converged, el.deig_max, res_max, hpsi_bands, stalled)


def refine_fp64(el_mixed: Electrons, el_fp64: Electrons, C: Optional[Wavefunction] = None,
                eig_threshold: float = 1e-8, max_sweeps: int = 40, residual_threshold: Optional[float] = None,
                method: str = "fp64_sweeps", reset_every: int = 8):
    """FP64 refinement of mixed-precision eigenvectors.

    Upcasts the vectors to complex128 and orthonormalises them (Cholesky,
    FP64).  FP32 H.psi leaves eigenvalues with noise near eps_f32 * Ecut
    (~1e-6 Ha); the sweeps below remove it.  Two methods:

    * ``"fp64_sweeps"`` (default): FP64 Davidson sweeps (the plain form's H.psi
      for the current vectors and every expansion).
    * ``"mixed_expansion"``: FP64 H C once, then sweeps whose
      expansion vectors (the FP64 preconditioned residuals) go through the
      mixed H.psi only.  The Rayleigh-Ritz matrices are FP64: the coupling block
      C^H H X is formed as (H C)^H X from the carried FP64 H C, so it is exact
      to FP64; only the small expansion-expansion block X^H H X carries FP32
      H.psi error (symmetrised), which perturbs the update at second order in
      the residual.  H C is carried through the FP64 rotations; its error grows
      by ~eps_f32 |H| times the size of each update, so a fresh FP64 H C replaces
      it every `reset_every` sweeps and to confirm convergence (a Rayleigh-Ritz
      with it, then the eigenvalue and residual tests).

    Stops when the eigenvalues change by less than `eig_threshold` (and, with
    `residual_threshold`, every requested band's FP64 residual norm is below
    it), at most `max_sweeps` sweeps.  Returns (eigenvalues (nk, nb) FP64,
    refined FP64 Wavefunction); el_fp64 holds the refined state and
    `el_fp64.last_refine` the sweep statistics."""
    C = C or el_mixed.C
    C64 = Wavefunction(el_fp64.basis, coeff=C.coeff.to(torch.complex128))
    C64.constrain()
    el_fp64.C = C64.orthonormalize()
    if method == "fp64_sweeps":
        el_fp64.last_refine = Davidson(el_fp64, n_iterations=max_sweeps, eig_threshold=eig_threshold,
                                       residual_threshold=residual_threshold)()
    elif method == "mixed_expansion":
        el_fp64.last_refine = _refine_mixed_expansion(el_mixed, el_fp64, eig_threshold, max_sweeps,
                                                      residual_threshold, reset_every)
    else:
        raise ValueError(f"unknown refinement method {method!r}")
    return el_fp64.eig, el_fp64.C


def _refine_mixed_expansion(el32: Electrons, el: Electrons, eig_threshold: float, max_sweeps: int,
                            residual_threshold: Optional[float], reset_every: int) -> DavidsonStats:
    basis = el.basis
    real = basis.real is not None
    w = basis.weight
    cdt = torch.float64 if real else torch.complex128
    n_bands = el.n_bands
    n_bands_max = n_bands + el.n_bands_extra
    norm_cut = float(np.sqrt(basis.n_tot * 1e-15))
    if residual_threshold is not None:
        norm_cut = min(norm_cut, 0.01 * residual_threshold)
    hpsi64 = hpsi32 = 0

    def fresh_rr():
        """FP64 H C and a Rayleigh-Ritz rotation with it (eigenvalues to FP64)."""
        nonlocal hpsi64
        HC = el.hamiltonian(el.C)
        hpsi64 += el.C.n_bands() * basis.nk
        eig, V = eigh(_sub((el.C ^ HC).wait(), real))
        el.C = el.C @ V
        return eig, HC @ V

    el.eig, HC = fresh_rr()
    deig_max, res_max, converged = np.inf, np.inf, False
    n_eigs_done = 0
    sweeps = 0
    since_reset = 0
    fresh = True  # HC is a fresh FP64 H C (no carried FP32 error yet)
    while sweeps < max_sweeps:
        sweeps += 1
        since_reset += 1
        n_cur = el.C.n_bands()
        KEref = ops.band_norm_ke(el.C.coeff, basis.ke, b0=n_eigs_done, norm=False, weight=w)[1]
        Cexp = Wavefunction(basis, coeff=torch.empty((basis.nk, n_cur - n_eigs_done, basis.n_tot),
                                                     dtype=el.C.coeff.dtype, device=el.C.coeff.device))
        norm_exp = ops.residual(HC.coeff, el.C.coeff, el.eig, basis.ke, KEref, b0=n_eigs_done, out=Cexp.coeff,
                                norm=True, weight=w)
        ops.normalize_bands(Cexp.coeff, basis.n_device, norm_exp, norm_cut, sweeps, basis.n_max, basis.ke)
        if real:
            ops.symmetrize_real(basis.real, Cexp.coeff)
        # The expansion's H.psi in the mixed form, upcast.
        HCexp32 = el32.hamiltonian(Wavefunction(el32.basis, coeff=Cexp.coeff.to(el32.basis.dtype)))
        hpsi32 += Cexp.n_bands() * basis.nk
        HCexp = Wavefunction(basis, coeff=HCexp32.coeff.to(torch.complex128))
        n_exp = Cexp.n_bands()
        Cnew = el.C.cat(Cexp)
        O = _tile_expansion(torch.eye(n_cur, device=HC.coeff.device, dtype=cdt)[None], _sub((Cnew ^ Cexp).wait(), real))
        coup = _sub((HC ^ Cexp).wait(), real)  # C^H H X = (H C)^H X, FP64
        ee = _sub((Cexp ^ HCexp).wait(), real)
        ee = 0.5 * (ee + ee.conj().transpose(-2, -1))
        Hn = _tile_expansion(torch.diag_embed(el.eig).to(cdt), torch.cat((coup, ee), dim=1))
        eig_new, V_new, failed = eighg(Hn, O, check=False)
        n_next = min(n_cur + n_exp, n_bands_max)
        d = torch.abs(el.eig - eig_new[..., :n_cur])[:, :n_bands]
        pend = (d > eig_threshold).any(dim=0)
        first_pending = torch.where(pend.any(), pend.int().argmax(),
                                    torch.full((), n_bands, dtype=torch.int64, device=pend.device))
        host = torch.stack((d.max(), first_pending.to(torch.float64), failed.any().to(torch.float64))).tolist()
        if host[2]:
            raise RuntimeError("refinement subspace problem failed: overlap not positive-definite")
        V_new = V_new[..., :n_next]
        Vcur, Vexp = V_new[:, :n_cur], V_new[:, n_cur:]
        el.C = Cnew @ V_new
        HC = HC @ Vcur
        HC += HCexp @ Vexp
        el.eig = eig_new[..., :n_next].contiguous()
        deig_max = host[0]
        n_eigs_done = int(host[1])
        if n_eigs_done >= n_bands and fresh:
            # Converged in a sweep that started from a fresh FP64 H C: its
            # eigenvalue changes carry no accumulated FP32 error.  The residual
            # from the carried H C (one update since the fresh one) is accurate
            # to ~eps_f32 |H| relative to the update.
            converged = True
            if residual_threshold is not None:
                res = ops.residual(HC.coeff, el.C.coeff, el.eig, norm=True, weight=w)
                res_max = float(res[:, :n_bands].max())
                converged = res_max < residual_threshold
            if converged:
                break
        fresh = False
        if n_eigs_done >= n_bands or since_reset >= reset_every:
            # Replace the carried H C by a fresh FP64 one (and Rayleigh-Ritz
            # with it); the next sweep then decides convergence.
            el.eig, HC = fresh_rr()
            since_reset, fresh, n_eigs_done = 0, True, 0
    el.deig_max = deig_max
    return DavidsonStats(sweeps, converged, deig_max, res_max, hpsi32 + hpsi64, False)

