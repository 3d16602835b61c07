"""Electron density (qgb_collect_density) against the reference's
Basis.collect_density (golden fixtures) and the oracle.

Tolerances (max-norm relative to the largest density value): FP64 1e-12,
FP32 2e-6."""
import os

import numpy as np
import pytest
import torch

from oracle import hpsi as oh
from qimpy_gb300 import electrons as E
from qimpy_gb300 import ops
from qimpy_gb300 import sphere as sp
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEV = "cuda:0"
TOL = {torch.complex128: 1e-12, torch.complex64: 2e-6}


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2"])
def test_density_matches_reference(name, dtype):
    g = np.load(os.path.join(GOLDEN, f"density_{name}.npz"))
    p = wl.get(name)
    el, C0 = E.from_problem(p, DEV, dtype)
    C = E.Wavefunction(el.basis, coeff=C0.to(DEV, dtype))
    rho = el.basis.collect_density(C, torch.from_numpy(g["f"]))[0].cpu().numpy()
    scale = np.abs(rho).max()
    if "rho" in g:
        assert np.abs(rho - g["rho"]).max() <= TOL[dtype] * scale
    else:
        i = g["sample_idx"]
        assert np.abs(rho[i[:, 0], i[:, 1], i[:, 2]] - g["sample"]).max() <= TOL[dtype] * scale
    assert np.abs(rho.sum(axis=(1, 2)) - g["plane_sums"]).max() <= TOL[dtype] * np.abs(g["plane_sums"]).max()


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_density_large_grid_chunked_and_accumulate(dtype):
    """si64-sized grid (96^3) against the oracle on a few bands, with a
    workspace of one band (chunked) and accumulation over two calls."""
    p = wl.get("si64")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    C = wl.make_wavefunctions(p, b, 5)
    t = sp.build_tables(b.fft_index, b.n, p.grid_shape)
    ds = sp.DeviceSphere(t, b.ke, DEV, dtype)
    pref = np.linspace(0.2, 1.0, 5)[None, :] * (2.0 / p.volume)
    want = oh.collect_density(b.fft_index, p.grid_shape, C, pref)
    Cd = torch.from_numpy(C).to(DEV, dtype)
    ws = ops.workspace(ds.workspace_bytes(1), DEV)
    rho = ops.collect_density(ds, Cd[:, :2].contiguous(), torch.from_numpy(pref[:, :2]), ws=ws)
    ops.collect_density(ds, Cd[:, 2:].contiguous(), torch.from_numpy(pref[:, 2:]), rho=rho, accumulate=True, ws=ws)
    got = rho.cpu().numpy()
    assert np.abs(got - want).max() <= TOL[dtype] * np.abs(want).max()


def test_density_rejects_bad_prefactor_shape():
    p = wl.get("tiny_fcc")
    el, C0 = E.from_problem(p, DEV, torch.complex128)
    with pytest.raises(ValueError):
        ops.collect_density(el.basis.sphere, C0.to(DEV), torch.ones(3, 3))
