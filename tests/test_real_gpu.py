"""GPU parity of real (Gamma-point) wavefunctions on the half basis.

``qgb_hamiltonian_real`` (two real bands per complex full-sphere transform,
weighted real projections) against the reference's own real-wavefunction
H.psi (tests/golden/real_tiny_gamma.npz) and against the oracle's r2c/c2r
restatement on Gamma-only copies of the si2 and si64 cells; ``qgb_dot_real``,
``qgb_symmetrize_real`` and the weighted band norms against numpy.
Tolerances: FP64 1e-12 relative (max-norm), FP32 2e-5.
"""
import os

import numpy as np
import pytest
import torch

from oracle import davidson as od
from oracle import hpsi as oh
from qimpy_gb300 import ops
from qimpy_gb300 import real_basis as rbm
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEV = "cuda:0"
TOL = {torch.complex128: 1e-12, torch.complex64: 2e-5}


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _setup(name, dtype):
    p = wl.get(name)
    p.k = np.zeros((1, 3))  # Gamma only (si64 already is)
    half, full = rbm.gamma_bases(p.Gbasis, p.ke_cutoff, p.grid_shape)
    rb = rbm.DeviceRealBasis(half, full, DEV, dtype)
    rb.set_potential(torch.from_numpy(p.V_r))
    beta = wl.make_projectors(p, half)
    return p, half, rb, beta


def _oracle(p, half, beta, C):
    gw = oh.real_gweight(half.iG[0], int(half.n[0]), half.n_tot)
    return oh.hamiltonian_real(half.ke, p.V_r, half.fft_index, half.n, half.iG, beta, p.D_all(), C, gw), \
        oh.project_real(beta, C, gw)


def test_real_hamiltonian_matches_reference_golden():
    """FP64 H.psi and <beta|psi> of the reference's real-wavefunction run."""
    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p, half, rb, beta = _setup("tiny_gamma", torch.complex128)
    assert np.array_equal(half.fft_index, g["fft_index"])
    C = torch.from_numpy(g["C0"]).to(DEV)
    HC, projT = ops.hamiltonian_real(rb, C, torch.from_numpy(beta).to(DEV),
                                     torch.from_numpy(p.D_atom).to(DEV, torch.complex128))
    assert _rel(HC.cpu().numpy(), g["hpsi"]) <= 1e-12
    assert _rel(projT.cpu().numpy().transpose(0, 2, 1), g["proj"]) <= 1e-12


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
@pytest.mark.parametrize("name,nb,hermitian", [("tiny_gamma", 5, False), ("tiny_gamma", 6, True),
                                              ("si2", 7, True), ("si64", 4, True)])
def test_real_hamiltonian_matches_oracle(name, nb, hermitian, dtype):
    """Odd and even band counts; a Gz = 0 plane that is not Hermitian gives the
    reference's result too (its c2r transform uses the Hermitian part)."""
    p, half, rb, beta = _setup(name, dtype)
    C = wl.make_wavefunctions(p, half, nb)
    oh.constrain(C, half.n)
    if hermitian:
        oh.real_symmetrize(C, half.iG[0], p.grid_shape)
    want, want_proj = _oracle(p, half, beta, C)
    HC, projT = ops.hamiltonian_real(rb, torch.from_numpy(C).to(DEV, dtype), torch.from_numpy(beta).to(DEV, dtype),
                                     torch.from_numpy(p.D_atom).to(DEV, dtype))
    assert _rel(HC.cpu().numpy().astype(np.complex128), want) <= TOL[dtype]
    assert _rel(projT.cpu().numpy().astype(np.complex128).transpose(0, 2, 1), want_proj) <= TOL[dtype]


@pytest.mark.parametrize("name,nb,hermitian", [("tiny_gamma", 5, False), ("si2", 7, True), ("si64", 32, True)])
def test_real_hamiltonian_mixed_matches_oracle(name, nb, hermitian):
    """Mixed form: FP32 local potential, weighted real projection and
    back-projection on the tcgen05 split-BF16x3 GEMMs; within 2e-5 of the
    oracle's FP64 H.psi, projections included."""
    p, half, rb, beta = _setup(name, torch.complex64)
    C = wl.make_wavefunctions(p, half, nb)
    oh.constrain(C, half.n)
    if hermitian:
        oh.real_symmetrize(C, half.iG[0], p.grid_shape)
    want, want_proj = _oracle(p, half, beta, C)
    split = ops.beta_split(torch.from_numpy(beta).to(DEV, torch.complex64))
    # The nonlocal term is stored into HC beside the local potential, whose
    # unpack then adds to it: every entry is written (NaN before the call).
    out = torch.full(C.shape, float("nan"), dtype=torch.complex64, device=DEV)
    HC, projT = ops.hamiltonian_real_mixed(rb, torch.from_numpy(C).to(DEV, torch.complex64), split,
                                           torch.from_numpy(p.D_atom).to(DEV, torch.complex64), out=out)
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    HCn = HC.cpu().numpy().astype(np.complex128)
    assert np.isfinite(HCn).all() and not HCn[0, :, int(half.n[0]):].any()
    assert _rel(HCn, want) <= TOL[torch.complex64]
    pr = projT.cpu().numpy().astype(np.complex128).transpose(0, 2, 1)
    assert _rel(pr, want_proj) <= TOL[torch.complex64] and not pr.imag.any()


def test_real_hamiltonian_without_projectors_and_errors():
    p, half, rb, beta = _setup("tiny_gamma", torch.complex128)
    C = wl.make_wavefunctions(p, half, 3)
    oh.real_symmetrize(C, half.iG[0], p.grid_shape)
    HC, _ = ops.hamiltonian_real(rb, torch.from_numpy(C).to(DEV), None, None)
    want = oh.apply_ke(half.ke, C) + oh.apply_potential_real(p.V_r, half.fft_index, half.n, half.iG, C)
    assert _rel(HC.cpu().numpy(), want) <= 1e-12
    Cd = torch.from_numpy(C).to(DEV)
    with pytest.raises(Exception, match="alias"):
        ops.hamiltonian_real(rb, Cd, None, None, out=Cd)
    with pytest.raises(Exception, match="workspace"):
        ops.hamiltonian_real(rb, Cd, None, None, ws=torch.empty(16, dtype=torch.uint8, device=DEV))


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_dot_real_symmetrize_and_weighted_norms(dtype):
    p, half, rb, beta = _setup("si2", dtype)
    gw = oh.real_gweight(half.iG[0], int(half.n[0]), half.n_tot)
    X = wl.make_wavefunctions(p, half, 6)
    Y = wl.make_wavefunctions(p, half, 9) * 0.5
    Xd, Yd = torch.from_numpy(X).to(DEV, dtype), torch.from_numpy(Y).to(DEV, dtype)
    tol = TOL[dtype]
    got = ops.dot_real(Xd, Yd, rb.weight).cpu().numpy()
    want = od.dot_real(Xd.cpu().numpy().astype(np.complex128), Yd.cpu().numpy().astype(np.complex128), gw)
    assert _rel(got, want) <= tol and not got.imag.any()
    nrm, bke = ops.band_norm_ke(Xd, torch.from_numpy(half.ke).to(DEV), weight=rb.weight)
    Xh = Xd.cpu().numpy().astype(np.complex128)
    assert _rel(nrm.cpu().numpy(), np.sqrt((np.abs(Xh) ** 2 * gw).sum(-1))) <= tol
    assert _rel(bke.cpu().numpy(), (np.abs(Xh) ** 2 * gw * half.ke[0]).sum(-1)) <= tol
    ops.symmetrize_real(rb, Xd)
    want_sym = oh.real_symmetrize(Xh.copy(), half.iG[0], p.grid_shape)
    assert _rel(Xd.cpu().numpy().astype(np.complex128), want_sym) <= (0 if dtype == torch.complex128 else 1e-7)


def _real_solve(name, dtype, threshold, C0=None):
    from qimpy_gb300 import davidson as dv
    from qimpy_gb300 import electrons as E

    p = wl.get(name)
    el, C_start = E.from_problem(p, DEV, dtype, real=True)
    C = E.Wavefunction(el.basis, coeff=(C_start if C0 is None else torch.from_numpy(C0)).to(DEV, dtype))
    C.constrain()
    el.C = C.orthonormalize()
    stats = dv.Davidson(el, n_iterations=300, eig_threshold=threshold)()
    return p, el, stats


def test_real_davidson_fp64_matches_reference():
    """The reference's Davidson in real-wavefunction mode: eigenvalues within
    1e-10 Ha and the same iteration count (within 2) from the same start."""
    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p, el, stats = _real_solve("tiny_gamma", torch.complex128, float(g["eig_threshold"]), g["C0"])
    assert stats.converged
    assert np.abs(el.eig.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
    assert abs(stats.iterations - int(g["davidson_iterations"])) <= 2
    assert not el.C.coeff.isnan().any()


def test_real_davidson_mixed_refined_within_1e6():
    from qimpy_gb300 import davidson as dv
    from qimpy_gb300 import electrons as E

    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p, el, stats = _real_solve("tiny_gamma", torch.complex64, 1e-6, g["C0"])
    assert stats.converged or stats.stalled
    el64, _ = E.from_problem(p, DEV, torch.complex128, real=True)
    eig, _ = dv.refine_fp64(el, el64)
    err = np.abs(eig.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    assert err <= 1e-6, err


def test_real_davidson_si64_matches_reference_eigenvalues():
    """The 64-atom Si cell (Gamma only, 160 + 16 bands) solved with real
    wavefunctions on the half basis has the reference's (complex-mode)
    eigenvalues: the Gamma-point Hamiltonian is real, so both bases give the
    same spectrum.  Within 1e-8 Ha at eig_threshold 1e-9."""
    g = np.load(os.path.join(GOLDEN, "si64.npz"))
    p, el, stats = _real_solve("si64", torch.complex128, 1e-9)
    assert stats.converged
    assert np.abs(el.eig.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-8
