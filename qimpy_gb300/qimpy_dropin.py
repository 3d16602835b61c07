"""Drop-in binding of the GB300 path into QimPy's own classes.

QimPy assigns its hot functions as class attributes, so a binding replaces
those attributes and leaves the eigensolvers untouched.  ``install()``
replaces, with calls through the C ABI of ``libqimpy_gb300.so``:

* ``Basis.apply_ke`` / ``Basis.apply_potential`` / ``Basis.collect_density``
  (qimpy/dft/electrons/_basis.py:55-58; _basis_ops.py:29-113, 207-296) -> ``qgb_apply_ke`` /
  ``qgb_apply_potential`` / ``qgb_collect_density``;
* ``Electrons.hamiltonian`` (qimpy/dft/electrons/_electrons.py:45; _hamiltonian.py:7-29)
  -> one ``qgb_hamiltonian`` call (KE, local potential and the nonlocal term
  ``beta @ (D_all @ (beta ^ C))``);
* ``Wavefunction.dot`` / ``__xor__`` / ``dot_O`` and ``Wavefunction.matmul`` /
  ``__matmul__`` (qimpy/dft/electrons/_wavefunction.py:277-298; _wavefunction_dot.py:18-191)
  -> ``qgb_dot`` / ``qgb_matmul``;
* ``eighg`` as the Davidson and CheFSI modules bind it (_davidson.py:12, _chefsi.py:10;
  qimpy/math/_linalg.py:143-183) -> Cholesky of O and the batched cuSOLVER eigensolve
  (``qgb_subspace_eigh``).

The eigensolvers themselves (``Davidson``, ``CheFSI``), the remaining
Wavefunction arithmetic and the preconditioner stay QimPy's own code.

Scope: one spin channel, no spinors, the full basis of one process (no basis
division), norm-conserving pseudopotentials (overlap = identity), no
kinetic-energy-density or DFT+U terms.  Wavefunctions may be complex, or real
at the Gamma point (``basis.real_wavefunctions``, the half-mesh basis of
qimpy/dft/electrons/_basis_real.py): there ``Electrons.hamiltonian`` runs
through ``qgb_hamiltonian_real`` (two real bands per complex transform on the
full Gamma sphere) and the overlaps through ``qgb_dot_real`` (the G-weighted
real products of _wavefunction_dot.py:55-88); ``apply_ke``, ``apply_potential``
and ``collect_density`` are replaced for complex wavefunctions only.  Anything
else raises ``NotImplementedError``: the binding has no path other than the C
ABI, and every call needs CUDA tensors (QimPy's ``rc.device`` a CUDA device).
``uninstall()`` restores the original attributes.
"""
from __future__ import annotations

import numpy as np
import torch

from . import linalg, ops
from . import workloads as wl
from .real_basis import DeviceRealBasis
from .sphere import DeviceSphere, build_tables

#: (owner, attribute name) -> the attribute install() replaced
_ORIGINAL: dict = {}


def _require(ok: bool, what: str) -> None:
    if not ok:
        raise NotImplementedError(f"qimpy_gb300 drop-in: {what}")


def _single_process(basis) -> None:
    division = getattr(basis, "division", None)
    _require(division is None or division.n_procs == 1, "basis divided across processes")


def _coeff3(C) -> torch.Tensor:
    """C.coeff (1, nk, nb, 1, n_tot) as a contiguous (nk, nb, n_tot) tensor."""
    c = C.coeff
    _require(c.dim() == 5 and c.shape[0] == 1 and c.shape[3] == 1,
             f"wavefunction shape {tuple(c.shape)} (one spin channel, no spinors)")
    _require(c.shape[-1] == C.basis.n_tot, "wavefunction on part of the basis")
    _single_process(C.basis)
    return c[0, :, :, 0, :].resolve_conj().resolve_neg().contiguous()


def _wavefunction(like, coeff3: torch.Tensor):
    return type(like)(like.basis, coeff=coeff3[None, :, :, None, :], band_division=like.band_division)


def _sphere(basis, dtype: torch.dtype, device: torch.device) -> DeviceSphere:
    """Sphere tables of `basis` on `device` (built once per basis, dtype and device)."""
    cache = basis.__dict__.setdefault("_qgb_spheres", {})
    key = (dtype, str(device))
    ds = cache.get(key)
    if ds is None:
        tables = build_tables(basis.fft_index.cpu().numpy(), basis.n.cpu().numpy(), tuple(basis.grid.shape))
        ke = basis.get_ke().detach().cpu().numpy()
        ds = cache[key] = DeviceSphere(tables, ke, device, dtype)
        ds._qgb_V_key = None
    return ds


def _real_basis(basis, dtype: torch.dtype, device: torch.device) -> DeviceRealBasis:
    """The real-wavefunction tables of a Gamma-point `basis` on `device`: its
    half-mesh basis (the reference's own fft_index, iG and kinetic energies)
    against the full Gamma sphere of the same lattice, cutoff and grid, built
    once per basis, dtype and device."""
    cache = basis.__dict__.setdefault("_qgb_real", {})
    key = (dtype, str(device))
    rb = cache.get(key)
    if rb is None:
        k = basis.k.detach().cpu().numpy()
        _require(k.shape[0] == 1 and not k.any(), "real wavefunctions away from the Gamma point")
        shape = tuple(int(x) for x in basis.grid.shape)
        half = wl.BasisLayout(grid_shape=shape, n=basis.n.cpu().numpy().astype(np.int64), n_tot=int(basis.n_tot),
                              fft_index=basis.fft_index.cpu().numpy().astype(np.int64),
                              iG=basis.iG.cpu().numpy().astype(np.int64), ke=basis.get_ke().detach().cpu().numpy())
        full = wl.make_basis(basis.lattice.Gbasis.detach().cpu().numpy(), np.zeros((1, 3)), float(basis.ke_cutoff),
                             shape)
        rb = cache[key] = DeviceRealBasis(half, full, device, dtype)
        rb._qgb_V_key = None
    return rb


def _set_potential(ds: DeviceSphere, basis, V) -> None:
    """Install V(r) = ~V on the basis grid (as _basis_ops.py:44), when V changed:
    another field object, another data tensor, or an in-place update (torch's
    version counter).  The cache holds the field and its tensor, so that
    neither object identity nor storage can be recycled by a new potential."""
    data = V.data
    cached = ds._qgb_V_key
    if cached is not None and cached[0] is V and cached[1] is data and cached[2] == data._version:
        return
    Vr = (~(V.to(basis.grid))).data
    _require(Vr.shape[0] == 1, f"{Vr.shape[0]} potential channels (one spin channel only)")
    ds.set_potential(Vr[0])
    ds._qgb_V_key = (V, data, data._version)


def _d_blocks(D_all: torch.Tensor) -> torch.Tensor:
    """D_all (P x P, block diagonal over atoms) as (n_atoms, pa, pa) blocks:
    the finest uniform partition whose off-block entries are all zero (one
    dense block when there is none)."""
    D = D_all
    while D.dim() > 2:
        _require(D.shape[0] == 1, f"D_all of shape {tuple(D_all.shape)}")
        D = D[0]
    P = D.shape[-1]
    if P == 0:
        return D.reshape(0, 0, 0)
    nz = (D != 0).cpu().numpy()
    for n_atoms in range(P, 0, -1):
        if P % n_atoms:
            continue
        pa = P // n_atoms
        blk = np.arange(P) // pa
        if not nz[blk[:, None] != blk[None, :]].any():
            idx = torch.arange(n_atoms, device=D.device)
            Db = D.reshape(n_atoms, pa, n_atoms, pa)[idx, :, idx, :]
            return Db.contiguous()
    return D[None].contiguous()


def _nonlocal(basis, dtype: torch.dtype, device: torch.device):
    """(beta (nk, P, n_tot), D blocks) of the basis' ions, cached per beta_version."""
    ions = basis.ions
    beta_wf = getattr(ions, "beta", None)
    if beta_wf is None or ions.n_projectors == 0:
        return None, None
    cache = basis.__dict__.setdefault("_qgb_beta", {})
    key = (dtype, str(device))
    hit = cache.get(key)
    if hit is not None and hit[0] == ions.beta_version and hit[1] is beta_wf:
        return hit[2], hit[3]
    b = beta_wf.coeff
    _require(b.dim() == 5 and b.shape[0] == 1 and b.shape[3] == 1, f"projector shape {tuple(b.shape)}")
    beta = b[0, :, :, 0, :].to(device=device, dtype=dtype).contiguous()
    D = _d_blocks(ions.D_all.to(device=device, dtype=dtype))
    cache[key] = (ions.beta_version, beta_wf, beta, D)
    return beta, D


# ---------------------------------------------------------------------------
# The replacements
# ---------------------------------------------------------------------------

def apply_ke(self, C):
    """Basis.apply_ke (_basis_ops.py:29-36) through qgb_apply_ke."""
    _require(not self.real_wavefunctions, "apply_ke of real wavefunctions")
    C3 = _coeff3(C)
    ds = _sphere(self, C3.dtype, C3.device)
    return _wavefunction(C, ops.apply_ke(ds, C3))


def apply_potential(self, V, C):
    """Basis.apply_potential (_basis_ops.py:39-113) through qgb_apply_potential."""
    _require(not self.real_wavefunctions, "apply_potential of real wavefunctions")
    C3 = _coeff3(C)
    ds = _sphere(self, C3.dtype, C3.device)
    _set_potential(ds, self, V)
    return _wavefunction(C, ops.apply_potential(ds, C3))


def collect_density(self, C, f: torch.Tensor, need_Mvec: bool):
    """Basis.collect_density (_basis_ops.py:207-296) through qgb_collect_density:
    rho(r) = sum_kb f w_sk / Omega |psi_kb(r)|^2 of one spin channel, FP64."""
    from qimpy.grid import FieldR

    _require(not need_Mvec, "magnetization vector (spinors)")
    _require(not self.real_wavefunctions, "collect_density of real wavefunctions")
    C3 = _coeff3(C)
    assert tuple(f.shape) == tuple(C.coeff.shape[:3])
    ds = _sphere(self, C3.dtype, C3.device)
    prefac = (f * (self.w_sk / self.lattice.volume))[0]  # (nk, nb), as _basis_ops.py:229
    rho = ops.collect_density(ds, C3, prefac)
    return FieldR(self.grid, data=rho[None])


def hamiltonian(self, C):
    """Electrons.hamiltonian (_hamiltonian.py:7-29) as one C-ABI call:
    qgb_hamiltonian, or qgb_hamiltonian_real for real Gamma-point wavefunctions."""
    _require(not self.xc.need_tau, "kinetic-energy-density functionals")
    _require(not self.xc.plus_U, "DFT+U")
    basis = C.basis
    C3 = _coeff3(C)
    beta, D = _nonlocal(basis, C3.dtype, C3.device)
    if basis.real_wavefunctions:
        rb = _real_basis(basis, C3.dtype, C3.device)
        _set_potential(rb, basis, self.n_tilde.grad)
        HC, _ = ops.hamiltonian_real(rb, C3, beta, D)
        return _wavefunction(C, HC)
    ds = _sphere(basis, C3.dtype, C3.device)
    _set_potential(ds, basis, self.n_tilde.grad)
    HC, _ = ops.hamiltonian(ds, C3, beta, D)
    return _wavefunction(C, HC)


class _Ready:
    """A result that is ready now: QimPy's Waitable protocol (qimpy/mpi/_waitable.py,
    ``wait()`` returns the result), as its ``Waitless`` is for one process."""

    __slots__ = ("result",)

    def __init__(self, result):
        self.result = result

    def wait(self):
        return self.result


def dot(self, other):
    """Wavefunction.dot / ^ / dot_O (_wavefunction_dot.py:18-123): the overlap
    matrices (1, nk, nb_self, nb_other) through qgb_dot."""
    if not isinstance(other, type(self)):
        return NotImplemented
    assert self.basis is other.basis
    X, Y = _coeff3(self), _coeff3(other)
    _require(X.dtype == Y.dtype, f"operands of dtypes {X.dtype} and {Y.dtype}")
    if self.basis.real_wavefunctions:
        out = ops.dot_real(X, Y, _real_basis(self.basis, X.dtype, X.device).weight)
    else:
        out = ops.dot(X, Y)
    return _Ready(out[None] if X.dtype == torch.complex128 else out[None].to(torch.complex64))


def matmul(self, mat):
    """Wavefunction.matmul / @ (_wavefunction_dot.py:137-191) through qgb_matmul.
    The cached projections are not carried over; they are recomputed on use."""
    if not isinstance(mat, torch.Tensor):
        return NotImplemented
    C3 = _coeff3(self)
    M = mat
    while M.dim() > 3:
        _require(M.shape[0] == 1, f"band matrix of shape {tuple(mat.shape)}")
        M = M[0]
    if M.dim() == 3 and M.shape[0] == 1 and C3.shape[0] > 1:
        M = M.expand(C3.shape[0], *M.shape[1:])
    return _wavefunction(self, ops.matmul(C3, M))


def eighg(H, O: torch.Tensor, use_cholesky: bool = True):
    """qimpy.math.eighg (_linalg.py:143-183): Cholesky orthonormaliser of O and
    the batched FP64 eigensolve of U^H H U."""
    return linalg.eighg(H, O, use_cholesky=use_cholesky)


# ---------------------------------------------------------------------------

def _replace(owner, name: str, fn) -> None:
    _ORIGINAL.setdefault((owner, name), owner.__dict__[name])
    setattr(owner, name, fn)


def install() -> None:
    """Replace QimPy's hot functions by the C-ABI calls (idempotent)."""
    from qimpy.dft import electrons
    from qimpy.dft.electrons import _chefsi, _davidson

    Basis, Electrons, Wavefunction = electrons.Basis, electrons.Electrons, electrons.Wavefunction
    _replace(Basis, "apply_ke", apply_ke)
    _replace(Basis, "apply_potential", apply_potential)
    _replace(Basis, "collect_density", collect_density)
    _replace(Electrons, "hamiltonian", hamiltonian)
    for name in ("dot", "__xor__", "dot_O"):
        _replace(Wavefunction, name, dot)
    for name in ("matmul", "__matmul__"):
        _replace(Wavefunction, name, matmul)
    _replace(_davidson, "eighg", eighg)
    _replace(_chefsi, "eighg", eighg)


def uninstall() -> None:
    """Put back every attribute install() replaced."""
    for (owner, name), fn in list(_ORIGINAL.items()):
        setattr(owner, name, fn)
    _ORIGINAL.clear()
