"""GPU-resident mirror of QimPy's electronic operator API for the H.psi path.

Class and method names follow the reference so the eigensolver reads the same:

* ``Basis`` (qimpy/dft/electrons/_basis.py) - G-sphere per k, ``apply_ke`` and
  ``apply_potential`` (qimpy/dft/electrons/_basis_ops.py:29-113) on the CUDA path;
* ``Wavefunction`` (qimpy/dft/electrons/_wavefunction*.py) - coefficients
  (nk, nb, n_tot) on the device with ``dot`` / ``^``, ``matmul`` / ``@``,
  ``band_norm``, ``band_ke``, ``constrain``, ``cat``, arithmetic and
  ``orthonormalize``;
* ``Ions`` - projectors ``beta`` and per-atom ``D`` blocks with ``beta_version``
  (qimpy/dft/ions/_ions.py:41-44);
* ``Electrons.hamiltonian`` (qimpy/dft/electrons/_hamiltonian.py:7-29).

Coefficients drop the reference's singleton spin and spinor axes (one spin
channel, no spinors); ``Wavefunction.coeff5`` gives the reference's 5D view.
``Basis(..., real=True)`` is the reference's real-wavefunction (Gamma-point)
mode (qimpy/dft/electrons/_basis_real.py): coefficients on the half basis
Gz >= 0, overlaps and norms weighted by 1 (Gz = 0) / 2, real overlap
matrices, constrain symmetrising the Gz = 0 plane.
Precision: ``complex128`` is the plain FP64 drop-in; ``complex64`` runs H.psi
in FP32 while the subspace algebra (``dot`` results, ``eighg``) is FP64.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import ops
from . import sphere as sp
from . import workloads as wl


class Waitless:
    """Trivial Waitable (qimpy/mpi/_waitable.py:18-25): the result is ready."""

    def __init__(self, result):
        self.result = result

    def wait(self):
        return self.result


class Basis:
    """Plane-wave basis of one cell at all its k-points, resident on one GPU."""

    def __init__(self, Rbasis, k, wk, ke_cutoff: float, grid_shape, device="cuda",
                 dtype: torch.dtype = torch.complex128, fft_factors=None, layout=None, real: bool = False):
        Rbasis = np.asarray(Rbasis, dtype=np.float64)
        self.Rbasis = Rbasis
        self.Gbasis = 2.0 * np.pi * np.linalg.inv(Rbasis.T)
        self.volume = abs(float(np.linalg.det(Rbasis)))
        self.k = np.asarray(k, dtype=np.float64).reshape(-1, 3)
        self.wk = np.asarray(wk, dtype=np.float64)
        self.ke_cutoff = float(ke_cutoff)
        self.grid_shape = tuple(int(x) for x in grid_shape)
        self.device = torch.device(device)
        self.dtype = dtype
        #: Mixed form: subspace overlaps and rotations of complex64 vectors on the
        #: tensor cores (split-BF16x3, qgb_dot_tc / qgb_matmul_tc) instead of the
        #: FP32 CUDA-core kernels.
        self.tc_subspace = dtype == torch.complex64 and not real
        self.real = None  #: DeviceRealBasis of the real-wavefunction mode
        self.weight = None  #: FP64 overlap weights of the half basis (real mode)
        if real:
            from .real_basis import DeviceRealBasis, gamma_bases

            if self.k.shape[0] != 1 or np.any(self.k != 0.0):
                raise ValueError("real wavefunctions need the Gamma point alone")
            half, full = gamma_bases(self.Gbasis, self.ke_cutoff, self.grid_shape)
            self.real = DeviceRealBasis(half, full, self.device, dtype, fft_factors)
            self.weight = self.real.weight
            layout = half
        self.layout = layout or wl.make_basis(self.Gbasis, self.k, self.ke_cutoff, self.grid_shape)
        self.n = self.layout.n
        self.n_tot = self.layout.n_tot
        self.n_min = int(self.n.min())
        self.n_max = int(self.n.max())
        self.fft_index = self.layout.fft_index
        self.iG = self.layout.iG
        if self.real is None:
            self.tables = sp.build_tables(self.fft_index, self.n, self.grid_shape, fft_factors)
            self.sphere = sp.DeviceSphere(self.tables, self.layout.ke, self.device, dtype)
        else:  # transforms run on the full Gamma sphere
            self.sphere = self.real.sphere
            self.tables = self.sphere.tables
        self.ke = torch.from_numpy(self.layout.ke).to(self.device)  # FP64 always
        pad = torch.arange(self.n_tot)[None, :] < torch.from_numpy(self.n)[:, None]
        self.mask = pad.to(self.device)  # True inside the sphere
        self._V_id = None

    @property
    def nk(self) -> int:
        return int(self.k.shape[0])

    @property
    def n_device(self) -> torch.Tensor:
        """Sphere sizes n per k as an int32 device tensor."""
        nd = getattr(self, "_n_device", None)
        if nd is None:
            nd = self._n_device = torch.from_numpy(np.asarray(self.n, dtype=np.int32)).to(self.device)
        return nd

    def get_ke(self) -> torch.Tensor:
        """0.5 |k+G|^2 per k and basis entry (qimpy/dft/electrons/_basis.py:256-270)."""
        return self.ke

    def set_potential(self, V_r) -> None:
        """Install the real-space local potential V(r) for apply_potential."""
        V = V_r if isinstance(V_r, torch.Tensor) else torch.from_numpy(np.asarray(V_r))
        self.sphere.set_potential(V)
        self._V_id = id(V_r)

    def apply_ke(self, C: "Wavefunction") -> "Wavefunction":
        """KE * C (qimpy/dft/electrons/_basis_ops.py:29-36) on the GPU."""
        self._complex_only("apply_ke")
        return Wavefunction(self, coeff=ops.apply_ke(self.sphere, C.coeff))

    def apply_potential(self, V, C: "Wavefunction") -> "Wavefunction":
        """V * C on the G-sphere (qimpy/dft/electrons/_basis_ops.py:39-113)."""
        self._complex_only("apply_potential")
        if V is not None and id(V) != self._V_id:
            self.set_potential(V)
        return Wavefunction(self, coeff=ops.apply_potential(self.sphere, C.coeff))

    def _complex_only(self, what: str) -> None:
        if self.real is not None:
            raise NotImplementedError(f"{what} of real wavefunctions runs inside Electrons.hamiltonian "
                                      "(qgb_hamiltonian_real)")

    def collect_density(self, C: "Wavefunction", f: torch.Tensor, need_Mvec: bool = False) -> torch.Tensor:
        """Electron density (qimpy/dft/electrons/_basis_ops.py:207-296) of the bands
        of C with occupations f (nk, nb): rho(r) = sum_kb f w_sk / Omega |psi(r)|^2,
        w_sk = 2 w_k (one spin, no spinors), as an FP64 (1, N0, N1, N2) tensor (the
        reference's FieldR data with its one density component)."""
        if need_Mvec:
            raise NotImplementedError("magnetization densities need spinorial wavefunctions")
        self._complex_only("collect_density")
        f = f.reshape(C.coeff.shape[0], C.n_bands()).to(torch.float64)
        w_sk = 2.0 * torch.from_numpy(self.wk).to(f.device)
        prefac = f * (w_sk[:, None] / self.volume)
        return ops.collect_density(self.sphere, C.coeff, prefac)[None]


class Ions:
    """Projectors and D matrix of the nonlocal pseudopotential."""

    def __init__(self, basis: Basis, beta: Optional[torch.Tensor], D_atom: Optional[torch.Tensor]):
        self.basis = basis
        if beta is None or beta.shape[1] == 0:
            self.beta = None
            self.D = None
            self.n_projectors = 0
        else:
            self.beta = beta.to(basis.device, basis.dtype).contiguous()
            self.D = D_atom.to(basis.device, basis.dtype).contiguous()
            self.n_projectors = int(beta.shape[1])
        # Mixed form: bf16 hi/lo projector operands for the tensor-core GEMMs.
        self.beta_split = (ops.beta_split(self.beta)
                           if self.beta is not None and basis.dtype == torch.complex64 else None)
        self.beta_version = 0

    def D_all(self) -> torch.Tensor:
        """Dense block-diagonal D (qimpy/dft/ions/_ions_update.py:229-243)."""
        return torch.block_diag(*self.D)


class Wavefunction:
    """Band coefficients (nk, nb, n_tot) of one spin channel on the GPU."""

    def __init__(self, basis: Basis, *, coeff: Optional[torch.Tensor] = None, n_bands: int = 0):
        self.basis = basis
        if coeff is None:
            coeff = torch.zeros((basis.nk, n_bands, basis.n_tot), dtype=basis.dtype, device=basis.device)
        if coeff.dim() == 5:
            coeff = coeff[0, :, :, 0, :]
        self.coeff = coeff if coeff.is_contiguous() else coeff.contiguous()
        self._projT = None
        self._proj_version = -1

    # --- reference-shaped views -------------------------------------------------
    @property
    def coeff5(self) -> torch.Tensor:
        """(spin=1, k, band, spinor=1, basis) view, the reference's layout."""
        return self.coeff[None, :, :, None, :]

    def n_bands(self) -> int:
        return int(self.coeff.shape[1])

    def bands(self, start: int, stop: Optional[int] = None) -> "Wavefunction":
        """Band slice (contiguous copy unless nk == 1)."""
        return Wavefunction(self.basis, coeff=self.coeff[:, start:stop].contiguous())

    def clone(self) -> "Wavefunction":
        return Wavefunction(self.basis, coeff=self.coeff.clone())

    def zeros_like(self, n_bands: int = 0) -> "Wavefunction":
        return Wavefunction(self.basis, n_bands=n_bands or self.n_bands())

    # --- projections (cached like Wavefunction.proj, _wavefunction.py:106-132) ---
    def projT(self, ions: Ions) -> torch.Tensor:
        """<beta|self> as (nk, nb, P), cached per ions.beta_version."""
        if self._projT is None or self._proj_version != ions.beta_version:
            self._projT = ops.project(ions.beta, self.coeff)
            self._proj_version = ions.beta_version
        return self._projT

    # --- algebra --------------------------------------------------------------
    def dot(self, other: "Wavefunction") -> Waitless:
        """[k, b1, b2] = sum_g conj(self) other (qimpy/dft/electrons/_wavefunction_dot.py:18-107);
        FP64 result for both precisions (qgb_dot).  Real wavefunctions: weighted
        and imaginary part zero (qgb_dot_real)."""
        if self.basis.real is not None:
            return Waitless(ops.dot_real(self.coeff, other.coeff, self.basis.weight))
        tc = self.basis.tc_subspace and self.coeff.dtype == torch.complex64
        return Waitless(ops.dot(self.coeff, other.coeff, tc=tc))

    __xor__ = dot
    dot_O = dot

    def overlap(self) -> "Wavefunction":
        return self  # norm-conserving: identity (_wavefunction_dot.py:127-134)

    def matmul(self, mat: torch.Tensor) -> "Wavefunction":
        """C @ M along bands (qimpy/dft/electrons/_wavefunction_dot.py:137-191; qgb_matmul, or
        qgb_matmul_tc for complex64 vectors of a basis with tc_subspace)."""
        tc = self.basis.tc_subspace and self.coeff.dtype == torch.complex64
        return Wavefunction(self.basis, coeff=ops.matmul(self.coeff, mat, tc=tc))

    __matmul__ = matmul

    def band_norm(self) -> torch.Tensor:
        """sqrt(sum_g |c|^2), FP64 (qimpy/dft/electrons/_wavefunction.py:226-236; qgb_band_norm_ke)."""
        return ops.band_norm_ke(self.coeff, weight=self.basis.weight)[0]

    def band_ke(self) -> torch.Tensor:
        """sum_g |c|^2 KE, FP64 (qimpy/dft/electrons/_wavefunction.py:238-247; qgb_band_norm_ke)."""
        return ops.band_norm_ke(self.coeff, self.basis.ke, norm=False, weight=self.basis.weight)[1]

    def constrain(self) -> None:
        """Zero padded coefficients (qimpy/dft/electrons/_wavefunction.py:264-275);
        real wavefunctions: Gz = 0 plane made Hermitian (BasisReal.symmetrize)."""
        self.coeff.mul_(self.basis.mask[:, None, :])
        if self.basis.real is not None:
            ops.symmetrize_real(self.basis.real, self.coeff)
        self._projT = None

    def cat(self, other: "Wavefunction") -> "Wavefunction":
        return Wavefunction(self.basis, coeff=torch.cat((self.coeff, other.coeff), dim=1))

    def orthonormalize(self) -> "Wavefunction":
        from .linalg import ortho_matrix

        O = self.dot(self).wait()
        return self @ ortho_matrix(O.real if self.basis.real is not None else O)

    def __mul__(self, scale):
        if isinstance(scale, torch.Tensor) and scale.dim() == 2:  # per (k, band)
            scale = scale[..., None]
        if isinstance(scale, torch.Tensor):
            scale = scale.to(self.coeff.real.dtype if not scale.is_complex() else self.coeff.dtype)
        return Wavefunction(self.basis, coeff=self.coeff * scale)

    __rmul__ = __mul__

    def __imul__(self, scale):
        if isinstance(scale, torch.Tensor) and scale.dim() == 2:
            scale = scale[..., None]
        if isinstance(scale, torch.Tensor):
            scale = scale.to(self.coeff.real.dtype if not scale.is_complex() else self.coeff.dtype)
        self.coeff.mul_(scale)
        self._projT = None
        return self

    def __add__(self, other):
        return Wavefunction(self.basis, coeff=self.coeff + other.coeff)

    def __iadd__(self, other):
        self.coeff.add_(other.coeff)
        self._projT = None
        return self

    def __sub__(self, other):
        return Wavefunction(self.basis, coeff=self.coeff - other.coeff)

    def __isub__(self, other):
        self.coeff.sub_(other.coeff)
        self._projT = None
        return self


class Electrons:
    """Owner of the basis, ions, potential and wavefunctions; ``hamiltonian``
    is H = KE + V_loc + beta D beta^dagger (qimpy/dft/electrons/_hamiltonian.py:7-29)."""

    def __init__(self, basis: Basis, ions: Ions, V_r, n_bands: int, n_bands_extra: int):
        self.basis = basis
        self.ions = ions
        self.V_r = V_r
        basis.set_potential(V_r)
        self.n_bands = int(n_bands)
        self.n_bands_extra = int(n_bands_extra)
        self.C: Optional[Wavefunction] = None
        self.eig: Optional[torch.Tensor] = None
        self.deig_max = np.inf
        self.hpsi_band_count = 0  # band-applications performed (all k)

    def hamiltonian(self, C: Wavefunction) -> Wavefunction:
        """HC in one C-ABI call: fused KE + local potential, then the nonlocal
        term (FP64: ZGEMMs; mixed: tcgen05 split-BF16x3 GEMMs)."""
        ions = self.ions
        if self.basis.real is not None and self.basis.dtype == torch.complex64:
            HC, projT = ops.hamiltonian_real_mixed(self.basis.real, C.coeff, ions.beta_split, ions.D)
        elif self.basis.real is not None:
            beta = ions.beta if ions.n_projectors else None
            HC, projT = ops.hamiltonian_real(self.basis.real, C.coeff, beta, ions.D)
        elif self.basis.dtype == torch.complex64:
            HC, projT = ops.hamiltonian_mixed(self.basis.sphere, C.coeff, ions.beta_split, ions.D)
        else:
            beta = ions.beta if ions.n_projectors else None
            HC, projT = ops.hamiltonian(self.basis.sphere, C.coeff, beta, ions.D)
        if projT is not None:
            C._projT, C._proj_version = projT, ions.beta_version
        self.hpsi_band_count += C.n_bands() * self.basis.nk
        return Wavefunction(self.basis, coeff=HC)


def from_problem(prob: wl.Problem, device="cuda", dtype=torch.complex128, n_bands_total: Optional[int] = None,
                 real: bool = False):
    """Build (electrons, C0) for a synthetic problem (real=True: real
    wavefunctions on the half basis, Gamma-only problems)."""
    basis = Basis(prob.Rbasis, prob.k, prob.wk, prob.ke_cutoff, prob.grid_shape, device, dtype, real=real)
    beta = wl.make_projectors_device(prob, basis.layout, basis.device, dtype)  # qgb_make_projectors
    ions = Ions(basis, beta, torch.from_numpy(prob.D_atom).to(torch.complex128))
    el = Electrons(basis, ions, torch.from_numpy(prob.V_r), prob.n_bands, prob.n_bands_extra)
    nbt = n_bands_total or (prob.n_bands + prob.n_bands_extra)
    C0 = torch.from_numpy(wl.make_wavefunctions(prob, basis.layout, nbt))
    return el, C0
