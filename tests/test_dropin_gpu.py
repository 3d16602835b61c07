"""The drop-in binding's device path (qimpy_gb300.qimpy_dropin) on the GPU.

The reference's classes are not importable here, so minimal stand-ins carry
the attributes the binding reads from QimPy's Basis, Ions, Wavefunction,
Electrons and FieldH objects (the same attributes that
``tests/test_dropin_cpu.py`` exercises on the real classes).  Each replaced
function runs through the C ABI and is compared with the oracle: FP64 within
1e-12 relative.
"""
import sys
import types

import numpy as np
import pytest
import torch

from oracle import davidson as od
from oracle import hpsi as oh
from qimpy_gb300 import qimpy_dropin as dropin
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


class _Grid:
    def __init__(self, shape):
        self.shape = tuple(shape)


class _FieldR:
    def __init__(self, data):
        self.data = data


class _FieldH:
    """Stands in for FieldH: ``~V.to(grid)`` gives the real-space field."""

    def __init__(self, V_r):
        self.data = torch.from_numpy(V_r)[None].clone()

    def to(self, grid):
        return self

    def __invert__(self):
        return _FieldR(self.data)


class _Basis:
    def __init__(self, p, b, ions):
        self.fft_index = torch.from_numpy(b.fft_index)
        self.n = torch.from_numpy(b.n)
        self.grid = _Grid(p.grid_shape)
        self.n_tot = int(b.fft_index.shape[1])
        self.real_wavefunctions = False
        self.division = None
        self.ions = ions
        self._ke = torch.from_numpy(b.ke)

    def get_ke(self):
        return self._ke


class _Wavefunction:
    def __init__(self, basis, *, coeff, band_division=None):
        self.basis, self.coeff, self.band_division = basis, coeff, band_division


class _Ions:
    pass


class _Xc:
    need_tau = False
    plus_U = None


class _Electrons:
    def __init__(self, V):
        self.xc = _Xc()
        self.n_tilde = type("NTilde", (), {})()
        self.n_tilde.grad = V


def _setup(name, nb):
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    beta = wl.make_projectors(p, b)
    ions = _Ions()
    basis = _Basis(p, b, ions)
    ions.beta = _Wavefunction(basis, coeff=torch.from_numpy(beta)[None, :, :, None, :].to(DEV))
    ions.D_all = torch.from_numpy(p.D_all()).to(DEV, torch.complex128)
    ions.beta_version = 0
    ions.n_projectors = beta.shape[1]
    C0 = wl.make_wavefunctions(p, b, nb)
    C = _Wavefunction(basis, coeff=torch.from_numpy(C0)[None, :, :, None, :].to(DEV))
    return p, b, beta, basis, C, C0


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name,nb", [("tiny_fcc", 6), ("si2", 8)])
def test_dropin_hamiltonian_and_parts(name, nb):
    p, b, beta, basis, C, C0 = _setup(name, nb)
    V = _FieldH(p.V_r)
    el = _Electrons(V)
    want = oh.hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all(), C0)
    HC = dropin.hamiltonian(el, C)
    assert isinstance(HC, _Wavefunction) and tuple(HC.coeff.shape) == (1, p.nk, nb, 1, C0.shape[2])
    assert _rel(HC.coeff[0, :, :, 0, :].cpu().numpy(), want) <= 1e-12
    ke = dropin.apply_ke(basis, C).coeff[0, :, :, 0, :].cpu().numpy()
    assert _rel(ke, oh.apply_ke(b.ke, C0)) <= 1e-14
    vc = dropin.apply_potential(basis, V, C).coeff[0, :, :, 0, :].cpu().numpy()
    assert _rel(vc, oh.apply_potential(p.V_r, b.fft_index, b.n, C0)) <= 1e-12
    # The potential is converted again after an in-place change (torch's version counter).
    V.data.mul_(2.0)
    vc2 = dropin.apply_potential(basis, V, C).coeff[0, :, :, 0, :].cpu().numpy()
    assert _rel(vc2, oh.apply_potential(2.0 * p.V_r, b.fft_index, b.n, C0)) <= 1e-12


def test_dropin_dot_matmul_eighg():
    p, b, beta, basis, C, C0 = _setup("si2", 8)
    C0b = wl.make_wavefunctions(p, b, 5) * (0.5 - 0.25j)
    C2 = _Wavefunction(basis, coeff=torch.from_numpy(C0b)[None, :, :, None, :].to(DEV))
    O = dropin.dot(C, C2).wait()
    assert tuple(O.shape) == (1, p.nk, 8, 5) and O.dtype == torch.complex128
    assert _rel(O[0].cpu().numpy(), od.dot(C0, C0b)) <= 1e-12
    g = torch.Generator().manual_seed(7)
    M = torch.randn((1, p.nk, 8, 3), dtype=torch.complex128, generator=g)
    out = dropin.matmul(C, M.to(DEV)).coeff[0, :, :, 0, :].cpu().numpy()
    assert _rel(out, od.matmul(C0, M[0].numpy())) <= 1e-12
    # A band slice of a wider block (not contiguous) and a conjugated matrix.
    Cs = _Wavefunction(basis, coeff=C.coeff[:, :, 2:7])
    Mc = M[..., :5, :].to(DEV).conj()
    out2 = dropin.matmul(Cs, Mc).coeff[0, :, :, 0, :].cpu().numpy()
    assert _rel(out2, od.matmul(C0[:, 2:7], np.conj(M[0, :, :5].numpy()))) <= 1e-12
    # eighg of the expanded-subspace shape: H = C^H C + shift, O = C^H C.
    Ok = dropin.dot(C, C).wait()
    Hk = Ok + 0.3 * torch.eye(8, dtype=torch.complex128, device=DEV)
    E, Vv = dropin.eighg(dropin._Ready(Hk), Ok)
    Ew, _ = od.eighg(Hk[0].cpu().numpy(), Ok[0].cpu().numpy())
    assert tuple(E.shape) == (1, p.nk, 8) and float(np.abs(E[0].cpu().numpy() - Ew).max()) <= 1e-10
    res = Hk @ Vv - Ok @ Vv * E[..., None, :]
    assert float(res.abs().max()) <= 1e-10


def test_dropin_collect_density(monkeypatch):
    """Basis.collect_density through qgb_collect_density; FieldR comes from a
    stand-in qimpy.grid module."""
    grid_mod = types.ModuleType("qimpy.grid")

    class FieldR:
        def __init__(self, grid, data):
            self.grid, self.data = grid, data

    grid_mod.FieldR = FieldR
    qimpy_mod = types.ModuleType("qimpy")
    qimpy_mod.grid = grid_mod
    monkeypatch.setitem(sys.modules, "qimpy", qimpy_mod)
    monkeypatch.setitem(sys.modules, "qimpy.grid", grid_mod)
    p, b, beta, basis, C, C0 = _setup("si2", 8)
    wk = np.linspace(0.5, 1.5, p.nk) / p.nk
    basis.w_sk = torch.from_numpy(wk).reshape(1, p.nk, 1).to(DEV)
    basis.lattice = type("Lattice", (), {"volume": float(p.volume)})()
    f = torch.from_numpy(wl.make_fillings(p, 8))[None].to(DEV)
    rho = dropin.collect_density(basis, C, f, False)
    assert isinstance(rho, FieldR) and tuple(rho.data.shape) == (1,) + tuple(p.grid_shape)
    prefac = f[0].cpu().numpy() * wk[:, None] / p.volume
    want = oh.collect_density(b.fft_index, tuple(p.grid_shape), C0, prefac)
    assert _rel(rho.data[0].cpu().numpy(), want) <= 1e-12
    with pytest.raises(NotImplementedError, match="magnetization"):
        dropin.collect_density(basis, C, f, True)


def test_dropin_real_wavefunctions():
    """Real (Gamma-point) wavefunctions on the half-mesh basis: hamiltonian
    through qgb_hamiltonian_real and the weighted real overlaps through
    qgb_dot_real, against the oracle's real-mode H.psi and overlap (1e-12)."""
    p = wl.get("tiny_gamma")
    half = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    beta = wl.make_projectors(p, half)
    ions = _Ions()
    basis = _Basis(p, half, ions)
    basis.real_wavefunctions = True
    basis.iG = torch.from_numpy(half.iG)
    basis.k = torch.zeros((1, 3), dtype=torch.float64)
    basis.ke_cutoff = p.ke_cutoff
    basis.lattice = type("Lattice", (), {"Gbasis": torch.from_numpy(np.asarray(p.Gbasis))})()
    ions.beta = _Wavefunction(basis, coeff=torch.from_numpy(beta)[None, :, :, None, :].to(DEV))
    ions.D_all = torch.from_numpy(p.D_all()).to(DEV, torch.complex128)
    ions.beta_version = 0
    ions.n_projectors = beta.shape[1]
    C0 = wl.make_wavefunctions(p, half, 5)
    oh.constrain(C0, half.n)
    oh.real_symmetrize(C0, half.iG[0], p.grid_shape)
    C = _Wavefunction(basis, coeff=torch.from_numpy(C0)[None, :, :, None, :].to(DEV))
    el = _Electrons(_FieldH(p.V_r))
    gw = oh.real_gweight(half.iG[0], int(half.n[0]), half.n_tot)
    want = oh.hamiltonian_real(half.ke, p.V_r, half.fft_index, half.n, half.iG, beta, p.D_all(), C0, gw)
    HC = dropin.hamiltonian(el, C)
    assert _rel(HC.coeff[0, :, :, 0, :].cpu().numpy(), want) <= 1e-12
    O = dropin.dot(C, HC).wait()
    Ow = od.dot_real(C0, want, gw)
    assert O.dtype == torch.complex128 and not O.imag.any()
    assert _rel(O[0].cpu().numpy(), Ow) <= 1e-12
    with pytest.raises(NotImplementedError, match="real wavefunctions"):
        dropin.apply_ke(basis, C)
