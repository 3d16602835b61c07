"""Real (Gamma-point) wavefunctions on the half-sphere basis, on the device.

The reference stores a real wavefunction by its coefficients on the half mesh
Gz >= 0 (qimpy/dft/electrons/_basis_real.py:10-106, basis on the H mesh at
_basis.py:168); the partner c(-G) = conj(c(G)) is implied, the Gz = 0 plane
holds both G and -G and is kept Hermitian by ``symmetrize``, and overlaps take
the weight 2 off that plane (_basis_real.py:62-66, _wavefunction_dot.py:55-88).

Here the local potential of such bands runs on the full Gamma sphere with two
real bands per complex transform (``qgb_hamiltonian_real``): the tables below
map every full-sphere entry to its half-basis coefficient and back.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from . import sphere as sp
from . import workloads as wl

#: Bit 31 of a pack entry's first index: use the conjugate of that coefficient.
CONJ = np.int64(1) << 31


@dataclass
class RealMapTables:
    """Host copy of ``struct qgb_real_map``'s tables (see include/qimpy_gb300.h)."""

    n_half: int
    n_tot_half: int
    n_full: int
    n_tot_full: int
    pack: np.ndarray  #: (n_full, 2) int32
    unpack: np.ndarray  #: (n_half, 2) int32
    plane: np.ndarray  #: (n_plane, 2) int32
    ke: np.ndarray  #: (n_tot_half,) float64
    weight: np.ndarray  #: (n_tot_half,) float64

    @property
    def n_plane(self) -> int:
        return int(self.plane.shape[0])


def _keys(iG: np.ndarray, shape) -> np.ndarray:
    N0, N1, N2 = shape
    return ((iG[:, 0] % N0) * N1 + (iG[:, 1] % N1)) * N2 + (iG[:, 2] % N2)


def build_real_map(half: wl.BasisLayout, full: wl.BasisLayout) -> RealMapTables:
    """Tables between the half basis (``make_basis(..., real=True)`` at k = 0)
    and the full Gamma sphere (``make_basis`` at k = 0) of the same cell,
    cutoff and grid.  Raises if the sphere reaches a Nyquist plane (its -G
    would not be a distinct grid point) or is not closed under G -> -G."""
    if half.fft_index.shape[0] != 1 or full.fft_index.shape[0] != 1:
        raise ValueError("real wavefunctions have one k-point (Gamma)")
    shape = tuple(full.grid_shape)
    n_half, n_full = int(half.n[0]), int(full.n[0])
    iGh, iGf = half.iG[0, :n_half], full.iG[0, :n_full]
    for a in range(3):
        if shape[a] % 2 == 0 and (np.abs(iGf[:, a]) >= shape[a] // 2).any():
            raise ValueError(f"the sphere reaches the Nyquist plane of axis {a}: grid too small for the cutoff")
    if (iGh[:, 2] < 0).any():
        raise ValueError("half basis has Gz < 0 entries")
    if 2 * n_half - int((iGh[:, 2] == 0).sum()) != n_full:
        raise ValueError("half and full spheres do not match (different cutoff or grid?)")
    pos_h = {int(k): i for i, k in enumerate(_keys(iGh, shape))}
    pos_f = {int(k): i for i, k in enumerate(_keys(iGf, shape))}
    kf, kf_neg = _keys(iGf, shape), _keys(-iGf, shape)
    pack = np.full((n_full, 2), -1, np.int64)
    try:
        for j in range(n_full):
            gz = iGf[j, 2]
            if gz > 0:
                pack[j, 0] = pos_h[int(kf[j])]
            elif gz < 0:
                pack[j, 0] = pos_h[int(kf_neg[j])] | CONJ
            else:
                pack[j] = (pos_h[int(kf[j])], pos_h[int(kf_neg[j])])
        kh, kh_neg = _keys(iGh, shape), _keys(-iGh, shape)
        unpack = np.array([(pos_f[int(a)], pos_f[int(b)]) for a, b in zip(kh, kh_neg)], np.int64).reshape(-1, 2)
        z0 = np.flatnonzero(iGh[:, 2] == 0)
        plane = np.array([(h, pos_h[int(kh_neg[h])]) for h in z0], np.int64).reshape(-1, 2)
    except KeyError as e:
        raise ValueError(f"sphere not closed under G -> -G (missing grid point {e})") from None
    weight = np.where(half.iG[0, :, 2] == 0, 1.0, 2.0)
    weight[n_half:] = 0.0
    return RealMapTables(n_half, int(half.n_tot), n_full, int(full.n_tot),
                         pack.astype(np.uint32).view(np.int32), unpack.astype(np.int32), plane.astype(np.int32),
                         half.ke[0].copy(), weight)


class DeviceRealBasis:
    """A real-wavefunction basis on one device: the full Gamma sphere (a
    ``DeviceSphere`` that runs the transforms and holds V), the half/full
    tables and the ``qgb_real_map`` struct pointing at them."""

    def __init__(self, half: wl.BasisLayout, full: wl.BasisLayout, device, dtype: torch.dtype,
                 fft_factors=None):
        self.map = build_real_map(half, full)
        self.half, self.full_layout = half, full
        self.device = torch.device(device)
        self.sphere = sp.DeviceSphere(sp.build_tables(full.fft_index, full.n, full.grid_shape, fft_factors), full.ke,
                                      self.device, dtype)
        self.cdtype, self.rdtype, self.qdtype = self.sphere.cdtype, self.sphere.rdtype, self.sphere.qdtype
        m = self.map

        def dev(a, dt):
            return torch.from_numpy(np.ascontiguousarray(a)).to(self.device, dt)

        self._pack, self._unpack = dev(m.pack, torch.int32), dev(m.unpack, torch.int32)
        self._plane = dev(m.plane if m.n_plane else np.zeros((1, 2), np.int32), torch.int32)
        self.ke = dev(m.ke, self.rdtype)
        self.weight = dev(m.weight, torch.float64)
        s = _lib.QgbRealMap()
        s.n_half, s.n_tot_half, s.n_full, s.n_tot_full, s.n_plane = m.n_half, m.n_tot_half, m.n_full, \
            m.n_tot_full, m.n_plane
        s.pack, s.unpack, s.plane = self._pack.data_ptr(), self._unpack.data_ptr(), self._plane.data_ptr()
        s.ke, s.weight = self.ke.data_ptr(), self.weight.data_ptr()
        self.struct = s

    @property
    def n_tot(self) -> int:
        return self.map.n_tot_half

    def set_potential(self, V_r: torch.Tensor) -> None:
        """Install the real-space local potential V(r) (N0, N1, N2)."""
        self.sphere.set_potential(V_r)

    def workspace_bytes(self, nb: int, P: int) -> int:
        return int(_lib.lib().qgb_hamiltonian_real_workspace_bytes(ct.byref(self.sphere.struct),
                                                                   ct.byref(self.struct), nb, P, self.qdtype))


def gamma_bases(Gbasis: np.ndarray, ke_cutoff: float, shape) -> tuple:
    """(half basis, full sphere) of a Gamma-only cell, both at k = 0."""
    k0 = np.zeros((1, 3))
    return wl.make_basis(Gbasis, k0, ke_cutoff, shape, real=True), wl.make_basis(Gbasis, k0, ke_cutoff, shape)
