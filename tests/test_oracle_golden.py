"""The CPU oracle against golden fixtures produced by running the reference itself.

Pins the oracle: H.psi (KE + local potential + nonlocal) within 1e-12 relative
and Davidson eigenvalues within 1e-10 Ha of the reference on the same inputs;
the basis layout (n, fft_index) exactly.
"""
import os

import numpy as np
import pytest

from oracle import davidson as od
from oracle import hpsi as oh
from qimpy_gb300 import workloads as wl
from qimpy_gb300.checksums import band_checksums

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def _problem(name, nb):
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    return p, b, wl.make_projectors(p, b), wl.make_wavefunctions(p, b, nb)


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2", "si64", "cu32"])
def test_basis_layout_matches_reference(name):
    g = _load(name)
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    assert np.array_equal(b.n, g["n"])
    assert np.array_equal(b.fft_index, g["fft_index"])
    assert np.allclose(b.ke[:, :8], g["ke_ref"], rtol=1e-13, atol=0)
    assert np.allclose(p.Gbasis, g["Gbasis_ref"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho"])
def test_oracle_hpsi_full_arrays(name):
    g = _load(name)
    nb = int(g["hpsi_bands"])
    p, b, beta, C = _problem(name, nb)
    assert np.array_equal(C, g["C0"]) and np.array_equal(p.V_r, g["V_r"]) and np.array_equal(beta, g["beta"])
    HC = oh.hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all(), C)
    assert np.abs(HC - g["hpsi"]).max() <= 1e-12 * np.abs(g["hpsi"]).max()
    proj = oh.project(beta, C)
    assert np.abs(proj - g["proj"]).max() <= 1e-12 * np.abs(g["proj"]).max()


@pytest.mark.parametrize("name", ["si2", "si64", "cu32"])
def test_oracle_hpsi_checksums(name):
    g = _load(name)
    nb = int(g["hpsi_bands"])
    p, b, beta, C = _problem(name, nb)
    HC = oh.hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all(), C)
    cs = band_checksums(HC, b.n)
    assert np.abs(cs - g["hpsi_checksums"]).max() <= 1e-12 * np.abs(g["hpsi_checksums"]).max()
    for (k, bb), ref in zip(g["hpsi_sample_kb"], g["hpsi_sample"]):
        assert np.abs(HC[k, bb] - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2"])
def test_oracle_davidson_eigenvalues(name):
    g = _load(name)
    pw = wl.get(name)
    p, b, beta, C = _problem(name, pw.n_bands + pw.n_bands_extra)
    H = lambda X: oh.hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all(), X)  # noqa: E731
    r = od.davidson(H, od.orthonormalize(C), b.ke, b.n, p.n_bands, 300, float(g["eig_threshold"]))
    assert r.converged
    assert np.abs(r.eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
    assert r.iterations == int(g["davidson_iterations"])


def test_oracle_davidson_rejects_oversized_subspace():
    p, b, beta, C = _problem("tiny_fcc", 60)
    with pytest.raises(ValueError):
        od.davidson(lambda X: X, C, b.ke, b.n, 50)


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2"])
def test_oracle_chefsi_matches_reference_chefsi(name):
    from oracle import chefsi as oc

    g = np.load(os.path.join(GOLDEN, f"chefsi_{name}.npz"))
    pw = wl.get(name)
    p, b, beta, C = _problem(name, pw.n_bands + pw.n_bands_extra)
    H = lambda X: oh.hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all(), X)  # noqa: E731
    r = oc.chefsi(H, od.orthonormalize(C), b.ke, b.n, p.n_bands, p.ke_cutoff, float(p.V_r.max()),
                  int(g["n_iterations"]), float(g["eig_threshold"]), int(g["filter_order"]),
                  float(g["init_threshold"]))
    assert r.converged
    assert np.abs(r.eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
    assert r.iterations == int(g["iterations"])


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2"])
def test_oracle_density_matches_reference(name):
    g = np.load(os.path.join(GOLDEN, f"density_{name}.npz"))
    pw = wl.get(name)
    p, b, beta, C = _problem(name, pw.n_bands + pw.n_bands_extra)
    assert np.allclose(g["w_sk"], 2.0 * p.wk) and abs(float(g["volume"]) - p.volume) < 1e-12 * p.volume
    f = wl.make_fillings(p, C.shape[1])
    assert np.array_equal(f, g["f"])
    rho = oh.collect_density(b.fft_index, p.grid_shape, C, f * (2.0 * p.wk[:, None] / p.volume))
    scale = np.abs(rho).max()
    if "rho" in g:
        assert np.abs(rho - g["rho"]).max() <= 1e-12 * scale
    else:
        i = g["sample_idx"]
        assert np.abs(rho[i[:, 0], i[:, 1], i[:, 2]] - g["sample"]).max() <= 1e-12 * scale
    assert np.abs(rho.sum(axis=(1, 2)) - g["plane_sums"]).max() <= 1e-12 * np.abs(g["plane_sums"]).max()


def test_oracle_real_wavefunctions_match_reference():
    """Gamma-point real wavefunctions (half-mesh basis, r2c/c2r FFTs, weighted
    projections): the oracle's basis, symmetrisation, <beta|psi> and H.psi
    against the reference run with real-wavefunctions: true."""
    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p = wl.get("tiny_gamma")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    assert np.array_equal(b.n, g["n"]) and np.array_equal(b.fft_index, g["fft_index"])
    gw = oh.real_gweight(b.iG[0], int(b.n[0]), b.n_tot)
    assert np.array_equal(gw, g["Gweight"][: b.n_tot])
    beta = wl.make_projectors(p, b)
    assert np.abs(beta - g["beta"]).max() <= 1e-14 * np.abs(beta).max()
    C = wl.make_wavefunctions(p, b, p.n_bands + p.n_bands_extra)
    oh.constrain(C, b.n)
    oh.real_symmetrize(C, b.iG[0], p.grid_shape)
    assert np.abs(C - g["C0"]).max() <= 1e-15 * np.abs(C).max()
    proj = oh.project_real(beta, C, gw)
    assert np.abs(proj - g["proj"]).max() <= 1e-12 * np.abs(g["proj"]).max()
    HC = oh.hamiltonian_real(b.ke, p.V_r, b.fft_index, b.n, b.iG, beta, p.D_all(), C, gw)
    assert np.abs(HC - g["hpsi"]).max() <= 1e-12 * np.abs(g["hpsi"]).max()


def test_oracle_real_wavefunction_davidson_matches_reference():
    """Davidson with real (Gamma-point) wavefunctions: weighted overlaps, norms
    and kinetic energies, Hermitian Gz = 0 plane; eigenvalues and iteration
    count against the reference's real-wavefunction Davidson, and eigenvalues
    against the oracle's complex-basis Davidson of the same cell."""
    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p = wl.get("tiny_gamma")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    gw = oh.real_gweight(b.iG[0], int(b.n[0]), b.n_tot)
    beta = wl.make_projectors(p, b)
    H = lambda X: oh.hamiltonian_real(b.ke, p.V_r, b.fft_index, b.n, b.iG, beta, p.D_all(), X, gw)  # noqa: E731
    sym = lambda X: oh.real_symmetrize(X, b.iG[0], p.grid_shape)  # noqa: E731
    C = g["C0"].copy()
    C = od.matmul(C, od.ortho_matrix(od.dot_real(C, C, gw)))
    r = od.davidson(H, C, b.ke, b.n, p.n_bands, 200, float(g["eig_threshold"]), gweight=gw, symmetrize=sym)
    assert r.converged
    assert np.abs(r.eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
    assert r.iterations == int(g["davidson_iterations"])
    # The same Hamiltonian in the complex (full-mesh) basis has the same spectrum.
    bc = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    bec = wl.make_projectors(p, bc)
    Hc = lambda X: oh.hamiltonian(bc.ke, p.V_r, bc.fft_index, bc.n, bec, p.D_all(), X)  # noqa: E731
    Cc = od.orthonormalize(wl.make_wavefunctions(p, bc, p.n_bands + p.n_bands_extra))
    rc = od.davidson(Hc, Cc, bc.ke, bc.n, p.n_bands, 200, 1e-12)
    assert np.abs(rc.eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-9


def test_oracle_real_wavefunction_density_matches_reference():
    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p = wl.get("tiny_gamma")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    assert np.allclose(g["w_sk"], 2.0 * p.wk)
    rho = oh.collect_density_real(b.fft_index, p.grid_shape, g["C0"], g["f"] * (2.0 * p.wk[:, None] / p.volume))
    assert np.abs(rho - g["rho"]).max() <= 1e-12 * np.abs(g["rho"]).max()


def test_oracle_real_wavefunction_chefsi_matches_reference():
    from oracle import chefsi as oc

    g = np.load(os.path.join(GOLDEN, "real_tiny_gamma.npz"))
    p = wl.get("tiny_gamma")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    gw = oh.real_gweight(b.iG[0], int(b.n[0]), b.n_tot)
    beta = wl.make_projectors(p, b)
    H = lambda X: oh.hamiltonian_real(b.ke, p.V_r, b.fft_index, b.n, b.iG, beta, p.D_all(), X, gw)  # noqa: E731
    sym = lambda X: oh.real_symmetrize(X, b.iG[0], p.grid_shape)  # noqa: E731
    C = g["C0"].copy()
    C = od.matmul(C, od.ortho_matrix(od.dot_real(C, C, gw)))
    r = oc.chefsi(H, C, b.ke, b.n, p.n_bands, p.ke_cutoff, float(p.V_r.max()), 100, 1e-11, 10, 1e-1,
                  gweight=gw, symmetrize=sym)
    assert r.converged
    assert np.abs(r.eig[:, : p.n_bands] - g["chefsi_eig"][:, : p.n_bands]).max() < 1e-10
    assert r.iterations == int(g["chefsi_iterations"])


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_gamma"])
def test_oracle_projectors_match_reference(name):
    """The oracle's projector construction against the reference's own
    Ions.get_projectors (tests/golden/projectors_*.npz): the blip coefficients
    of the Gaussian shells' radial samples (get_coeff), beta from those tables
    (Interpolator, harmonics with the i^l phase, translation phases), and the
    analytic-radial form against the workloads' projectors, which the spline
    approximates to ~1e-9."""
    from oracle import projectors as op

    g = np.load(os.path.join(GOLDEN, f"projectors_{name}.npz"))
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=bool(p.extra.get("real_wavefunctions")))
    assert np.array_equal(b.fft_index, g["fft_index"])
    dq = float(g["dq"])
    q = np.arange(g["coeff"].shape[1] - 4) * dq
    for s, sh in enumerate(p.shells):
        samples = (-1.0) ** sh.l * (2 * np.pi) ** 1.5 * sh.sigma ** (2 * sh.l + 3) * np.exp(-0.5 * sh.sigma ** 2 * q ** 2)
        c = op.blip_coeff(samples)
        assert np.abs(c - g["coeff"][s]).max() <= 1e-14 * np.abs(g["coeff"][s]).max()
    blip = [(sh.l, ("blip", g["coeff"][s], dq)) for s, sh in enumerate(p.shells)]
    gauss = [(sh.l, ("gauss", sh.sigma)) for sh in p.shells]
    beta_b = op.projectors(b.iG, p.k, p.Gbasis, b.n, p.positions, blip, p.volume)
    beta_g = op.projectors(b.iG, p.k, p.Gbasis, b.n, p.positions, gauss, p.volume)
    ref = g["beta"]
    assert np.abs(beta_b - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(beta_g - wl.make_projectors(p, b)).max() <= 1e-14 * np.abs(ref).max()
    assert np.abs(beta_g - ref).max() <= 1e-8 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho"])
def test_torch_port_matches_reference(name):
    """The torch restatement used as the CPU baseline gives the reference's H.psi."""
    from oracle import hpsi_torch as oht

    g = _load(name)
    p, b, beta, C = _problem(name, int(g["hpsi_bands"]))
    HC = oht.Hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all())(C)
    assert np.abs(HC - g["hpsi"]).max() <= 1e-12 * np.abs(g["hpsi"]).max()
