"""Device-resident G-sphere tables (``struct qgb_sphere``) for the CUDA kernels.

Built once per basis from the reference-ordered ``fft_index``
(qimpy/dft/electrons/_basis.py:186-193): in-sphere points come first in
ascending linear grid index, so points sharing the first grid index i0 (a
"slab") are contiguous.  The tables list each slab's basis range and i0, the
(i1, i2) of every point, and the distinct i1 rows each slab touches.
"""
from __future__ import annotations

import ctypes as ct
import dataclasses
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

CODELET_SIZES = (1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16)


def factor_axis(N: int, prefer: tuple | None = None) -> tuple[int, int]:
    """(L1, L2) with L1 * L2 = N, both codelet sizes: one pass when N is itself a
    codelet size, else the most balanced split with L1 >= L2."""
    if prefer is not None:
        if prefer[0] * prefer[1] != N or prefer[0] not in CODELET_SIZES or prefer[1] not in CODELET_SIZES:
            raise ValueError(f"bad factorisation {prefer} for N={N}")
        return tuple(prefer)
    if N in CODELET_SIZES:
        return (N, 1)
    best = None
    for L1 in CODELET_SIZES:
        if N % L1 == 0 and (N // L1) in CODELET_SIZES and L1 >= N // L1:
            cand = (L1, N // L1)
            if best is None or abs(cand[0] - cand[1]) < abs(best[0] - best[1]):
                best = cand
    if best is None:
        raise ValueError(
            f"grid size {N} is not a product of two sizes in {CODELET_SIZES}; "
            "choose a 2,3,5,7-smooth grid up to 256"
        )
    return best


def permutation(N: int, L1: int, L2: int) -> np.ndarray:
    """Real-space index stored at each position p: p // L1 + L2 * (p % L1)."""
    p = np.arange(N)
    return p // L1 + L2 * (p % L1)


def twiddle_table(N: int, L1: int, L2: int) -> np.ndarray:
    """W[n1][k2] = exp(+2 pi i n1 k2 / N) (float64 host trigonometry, exact reduction)."""
    m = (np.arange(L1)[:, None] * np.arange(L2)[None, :]) % N
    ang = 2.0 * np.pi * m / N
    return (np.cos(ang) + 1j * np.sin(ang)).reshape(-1)


@dataclass
class SphereTables:
    """Host (numpy) form of the sphere tables."""

    nk: int
    n_tot: int
    shape: tuple
    fac: tuple  # ((L1, L2) per axis)
    n: np.ndarray
    n_slabs: np.ndarray
    slab_start: np.ndarray  # (nk, max_slabs + 1)
    slab_i0: np.ndarray  # (nk, max_slabs)
    yz: np.ndarray  # (nk, n_tot)
    row_start: np.ndarray  # (nk, max_slabs + 1) absolute offsets into rows
    rows: np.ndarray
    max_slabs: int
    max_rows: int
    #: axes with a validated codelet factorisation; the others carry the
    #: placeholder (N, 1) and are not complex-transformable
    fft_axes: tuple = (0, 1, 2)


def build_tables(fft_index: np.ndarray, n: np.ndarray, shape, fac=None, fft_axes=(0, 1, 2)) -> SphereTables:
    """Sphere tables of a basis on the grid `shape` (N2 fastest).  Axes outside
    `fft_axes` get the placeholder factorisation (N, 1) without validation:
    the half-width z axis of a real-wavefunction grid (N2/2 + 1 complex points)
    is transformed as a real length-N2 axis instead."""
    fft_index = np.asarray(fft_index, dtype=np.int64)
    n = np.asarray(n, dtype=np.int64)
    nk, n_tot = fft_index.shape
    N0, N1, N2 = (int(x) for x in shape)
    if max(N1, N2) >= 1 << 15:
        raise ValueError("grid too large for packed (i1, i2) indices")
    fac = tuple((factor_axis(int(Na), None if fac is None else fac[a]) if a in fft_axes else (int(Na), 1))
                for a, Na in enumerate(shape))
    per_k = []
    for k in range(nk):
        idx = fft_index[k, : n[k]]
        if np.any(np.diff(idx) <= 0):
            raise ValueError("in-sphere fft_index must be strictly ascending (reference ordering)")
        i0, rem = np.divmod(idx, N1 * N2)
        i1, i2 = np.divmod(rem, N2)
        bounds = np.flatnonzero(np.diff(i0)) + 1
        starts = np.concatenate(([0], bounds, [len(idx)]))
        slab_rows = [np.unique(i1[starts[s] : starts[s + 1]]) for s in range(len(starts) - 1)]
        per_k.append((i0[starts[:-1]], starts, (i1 << 16) | i2, slab_rows))
    max_slabs = max(len(p[0]) for p in per_k)
    slab_start = np.zeros((nk, max_slabs + 1), np.int32)
    slab_i0 = np.zeros((nk, max_slabs), np.int32)
    n_slabs = np.zeros(nk, np.int32)
    yz = np.zeros((nk, n_tot), np.int32)
    row_start = np.zeros((nk, max_slabs + 1), np.int32)
    rows = []
    off = 0
    max_rows = 0
    for k, (i0s, starts, packed, slab_rows) in enumerate(per_k):
        ns = len(i0s)
        n_slabs[k] = ns
        slab_i0[k, :ns] = i0s
        slab_start[k, : ns + 1] = starts
        slab_start[k, ns + 1 :] = starts[-1]
        yz[k, : n[k]] = packed
        for s, r in enumerate(slab_rows):
            row_start[k, s] = off
            rows.append(r)
            off += len(r)
            max_rows = max(max_rows, len(r))
        row_start[k, ns:] = off
    rows_arr = np.concatenate(rows).astype(np.int32) if rows else np.zeros(1, np.int32)
    return SphereTables(nk, n_tot, (N0, N1, N2), fac, n.astype(np.int32), n_slabs, slab_start, slab_i0,
                        yz, row_start, rows_arr, max_slabs, max_rows, tuple(sorted(fft_axes)))


class DeviceSphere:
    """Sphere tables, twiddles, KE and the permuted potential on one device,
    plus the ``qgb_sphere`` struct pointing at them."""

    def __init__(self, tables: SphereTables, ke: np.ndarray, device, dtype: torch.dtype):
        if dtype not in (torch.complex128, torch.complex64):
            raise ValueError("dtype must be complex128 or complex64")
        if tuple(tables.fft_axes) != (0, 1, 2):
            # Half-width (real-wavefunction) tables: their z axis is not a
            # complex FFT axis, and the complex kernels would transform it as one.
            raise ValueError(f"sphere tables with fft_axes={tables.fft_axes} are not complex-transformable "
                             "on every axis; the complex-wavefunction kernels need all three")
        self.tables = tables
        self.device = torch.device(device)
        self.cdtype = dtype
        self.rdtype = torch.float64 if dtype == torch.complex128 else torch.float32
        self.qdtype = _lib.QGB_F64 if dtype == torch.complex128 else _lib.QGB_F32
        t = tables

        def i32(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(self.device)

        self._n = i32(t.n)
        self._n_slabs = i32(t.n_slabs)
        self._slab_start = i32(t.slab_start)
        self._slab_i0 = i32(t.slab_i0)
        self._yz = i32(t.yz)
        self._row_start = i32(t.row_start)
        self._rows = i32(t.rows)
        tw = np.concatenate([twiddle_table(t.shape[a], *t.fac[a]) for a in range(3)])
        self._tw = torch.from_numpy(tw).to(dtype).to(self.device)
        self.ke = torch.from_numpy(np.ascontiguousarray(ke)).to(self.rdtype).to(self.device)
        self.perms = [permutation(t.shape[a], *t.fac[a]) for a in range(3)]
        self._V = None
        s = _lib.QgbSphere()
        s.nk, s.n_tot = t.nk, t.n_tot
        for a in range(3):
            s.N[a] = t.shape[a]
            s.L1[a], s.L2[a] = t.fac[a]
        s.max_slabs, s.max_rows = t.max_slabs, t.max_rows
        s.tw_off[0], s.tw_off[1], s.tw_off[2] = 0, t.shape[0], t.shape[0] + t.shape[1]
        s.n, s.n_slabs, s.slab_start = self._n.data_ptr(), self._n_slabs.data_ptr(), self._slab_start.data_ptr()
        s.slab_i0, s.yz, s.row_start = self._slab_i0.data_ptr(), self._yz.data_ptr(), self._row_start.data_ptr()
        s.rows, s.twiddle, s.ke = self._rows.data_ptr(), self._tw.data_ptr(), self.ke.data_ptr()
        s.V = 0
        self.struct = s

    @property
    def shape(self) -> tuple:
        return self.tables.shape

    def set_factors(self, fac) -> None:
        """Change the per-axis FFT factorisation (L1, L2): new twiddles, new
        real-space permutation, potential re-permuted.  Sphere tables unchanged."""
        fac = tuple(factor_axis(self.shape[a], tuple(fac[a])) for a in range(3))
        V_real = None
        if self._V is not None:  # undo the old permutation
            inv = [np.argsort(p) for p in self.perms]
            p0, p1, p2 = (torch.from_numpy(i).to(self._V.device) for i in inv)
            V_real = self._V[p0][:, p1][:, :, p2]
        self.tables = dataclasses.replace(self.tables, fac=fac)  # the caller's tables stay as they were
        tw = np.concatenate([twiddle_table(self.shape[a], *fac[a]) for a in range(3)])
        self._tw = torch.from_numpy(tw).to(self.cdtype).to(self.device)
        self.perms = [permutation(self.shape[a], *fac[a]) for a in range(3)]
        for a in range(3):
            self.struct.L1[a], self.struct.L2[a] = fac[a]
        self.struct.twiddle = self._tw.data_ptr()
        if V_real is not None:
            self.set_potential(V_real)

    def permute_real(self, V_r: torch.Tensor) -> torch.Tensor:
        """V in the kernels' digit-permuted real-space order (a gather on device)."""
        p0, p1, p2 = (torch.from_numpy(p).to(V_r.device) for p in self.perms)
        return V_r[p0][:, p1][:, :, p2].contiguous()

    def set_potential(self, V_r: torch.Tensor) -> None:
        """Install the real-space local potential V(r) (N0, N1, N2)."""
        if tuple(V_r.shape) != tuple(self.shape):
            raise ValueError(f"potential shape {tuple(V_r.shape)} != grid {self.shape}")
        V = V_r.to(device=self.device, dtype=self.rdtype)
        self._V = self.permute_real(V)
        self.struct.V = self._V.data_ptr()

    #: Default bound on the slab planes of one band chunk (1 GB: a whole block of
    #: bands in one chunk).  A budget that kept a chunk's planes inside the 126 MB
    #: L2 measured slower on si64 than one chunk per 32-band block (whose 97 MB
    #: of planes mostly stay in L2).  Callers may lower it per sphere, e.g. to a
    #: 32-band FFT block when one call covers many more bands.
    plane_budget_bytes = 1 << 30

    def workspace_bytes(self, nb: int, budget: int | None = None) -> int:
        """Workspace for `nb` bands, capped at the plane budget (the kernels then
        process the bands in chunks that fit)."""
        per_band = int(_lib.lib().qgb_potential_workspace_bytes(ct.byref(self.struct), 1, self.qdtype))
        budget = self.plane_budget_bytes if budget is None else budget
        chunk = max(1, min(nb, budget // max(per_band, 1)))
        return per_band * chunk

    def hamiltonian_workspace_bytes(self, nb: int, P: int) -> int:
        """qgb_hamiltonian workspace: the nonlocal part plus capped slab planes."""
        lib = _lib.lib()
        full = int(lib.qgb_hamiltonian_workspace_bytes(ct.byref(self.struct), nb, P, self.qdtype))
        planes = int(lib.qgb_potential_workspace_bytes(ct.byref(self.struct), nb, self.qdtype))
        return full - planes + self.workspace_bytes(nb)

    def hamiltonian_mixed_workspace_bytes(self, nb: int, P: int) -> int:
        """qgb_hamiltonian_mixed workspace: tensor-core nonlocal part plus capped planes."""
        lib = _lib.lib()
        full = int(lib.qgb_hamiltonian_mixed_workspace_bytes(ct.byref(self.struct), nb, P))
        planes = int(lib.qgb_potential_workspace_bytes(ct.byref(self.struct), nb, _lib.QGB_F32))
        return full - planes + self.workspace_bytes(nb)


def sphere_stats(t: SphereTables) -> dict:
    """Counts used for the algorithmic-work accounting of the local kernel."""
    N0, N1, N2 = t.shape
    rows = sum(int(t.row_start[k, t.n_slabs[k]] - t.row_start[k, 0]) for k in range(t.nk))
    slabs = int(t.n_slabs.sum())
    return dict(slabs=slabs, rows=rows, n=int(t.n.sum()), N=N0 * N1 * N2,
                log2N=math.log2(N0 * N1 * N2))
