"""GPU parity of the H.psi path against the oracle and the reference's golden vectors.

Tolerances: FP64 H.psi within 1e-12 relative (max-norm over the block) of the
oracle and of the reference; FP32 within 2e-5 relative.
"""
import os

import numpy as np
import pytest
import torch

from oracle import hpsi as oh
from qimpy_gb300 import ops
from qimpy_gb300 import sphere as sp
from qimpy_gb300 import workloads as wl
from qimpy_gb300.checksums import band_checksums

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEV = "cuda:0"
TOL = {torch.complex128: 1e-12, torch.complex64: 2e-5}


def _setup(name, dtype, nbands=None, shape=None):
    p = wl.get(name) if shape is None else wl.get(name, shape=shape)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    beta = wl.make_projectors(p, b)
    nb = nbands or (p.n_bands + p.n_bands_extra)
    C = wl.make_wavefunctions(p, b, nb)
    t = sp.build_tables(b.fft_index, b.n, p.grid_shape)
    ds = sp.DeviceSphere(t, b.ke, DEV, dtype)
    ds.set_potential(torch.from_numpy(p.V_r))
    return p, b, beta, C, ds


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
@pytest.mark.parametrize("name,shape", [("tiny_fcc", None), ("tiny_ortho", None), ("tiny_fcc", (18, 24, 20)),
                                        ("si2", None)])
def test_apply_potential_matches_oracle(name, shape, dtype):
    p, b, beta, C, ds = _setup(name, dtype, nbands=5, shape=shape)
    Cd = torch.from_numpy(C).to(DEV, dtype)
    out = ops.apply_potential(ds, Cd).cpu().numpy()
    want = oh.apply_potential(p.V_r, b.fft_index, b.n, C)
    assert _rel(out, want) < TOL[dtype]
    out2 = ops.apply_potential(ds, Cd, add_ke=True).cpu().numpy()
    assert _rel(out2, want + oh.apply_ke(b.ke, C)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho"])
def test_hamiltonian_matches_reference_golden(name, dtype):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p, b, beta, C, ds = _setup(name, dtype)
    assert np.array_equal(b.fft_index, g["fft_index"])
    Cd = torch.from_numpy(C).to(DEV, dtype)
    betad = torch.from_numpy(beta).to(DEV, dtype)
    Dd = torch.from_numpy(p.D_atom).to(DEV, dtype)
    HC, projT = ops.hamiltonian(ds, Cd, betad, Dd)
    assert _rel(HC.cpu().numpy(), g["hpsi"]) < TOL[dtype]
    assert _rel(projT.transpose(1, 2).cpu().numpy(), g["proj"]) < TOL[dtype]


@pytest.mark.parametrize("name", ["si2", "si64", "cu32"])
def test_hamiltonian_checksums_fp64(name):
    """Full-size H.psi against the reference's per-band checksums (1e-12 relative)."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    nb = int(g["hpsi_bands"])
    p, b, beta, C, ds = _setup(name, torch.complex128, nbands=nb)
    assert np.array_equal(b.fft_index, g["fft_index"])
    Cd = torch.from_numpy(C).to(DEV)
    HC, _ = ops.hamiltonian(ds, Cd, torch.from_numpy(beta).to(DEV), torch.from_numpy(p.D_atom).to(DEV, torch.complex128))
    HC = HC.cpu().numpy()
    cs = band_checksums(HC, b.n)
    assert np.abs(cs - g["hpsi_checksums"]).max() <= 1e-12 * np.abs(g["hpsi_checksums"]).max()
    for (k, bb), ref in zip(g["hpsi_sample_kb"], g["hpsi_sample"]):
        assert _rel(HC[k, bb], ref) < 1e-12


def test_inplace_and_accumulate_and_padding():
    p, b, beta, C, ds = _setup("tiny_fcc", torch.complex128, nbands=3)
    Cd = torch.from_numpy(C).to(DEV)
    ref = ops.apply_potential(ds, Cd, add_ke=True)
    X = Cd.clone()
    ops.apply_potential(ds, X, out=X, add_ke=True)
    assert torch.equal(X, ref)
    acc = torch.ones_like(Cd)
    ops.apply_potential(ds, Cd, out=acc, add_ke=True, accumulate=True)
    want = ref.clone()
    for k in range(p.nk):
        want[k, :, : b.n[k]] += 1.0
        want[k, :, b.n[k]:] = 1.0
    assert torch.allclose(acc, want, rtol=0, atol=1e-13)
    for k in range(p.nk):
        assert torch.count_nonzero(ref[k, :, b.n[k]:]) == 0


def test_small_workspace_chunks_bands():
    p, b, beta, C, ds = _setup("tiny_ortho", torch.complex128, nbands=5)
    Cd = torch.from_numpy(C).to(DEV)
    full = ops.apply_potential(ds, Cd)
    ws = ops.workspace(ds.workspace_bytes(2), DEV)  # two bands per launch
    chunked = ops.apply_potential(ds, Cd, ws=ws)
    assert torch.equal(full, chunked)
    with pytest.raises(RuntimeError):
        ops.apply_potential(ds, Cd, ws=ops.workspace(16, DEV))


def test_deterministic():
    p, b, beta, C, ds = _setup("si2", torch.complex128, nbands=4)
    Cd = torch.from_numpy(C).to(DEV)
    a = ops.apply_potential(ds, Cd, add_ke=True)
    c = ops.apply_potential(ds, Cd, add_ke=True)
    assert torch.equal(a, c)
