"""Projectors generated on the device (qgb_make_projectors) against the oracle.

The oracle's restatement of Ions.get_projectors is pinned to the reference's
own get_projectors (tests/golden/projectors_*.npz).  FP64 within 1e-12
relative (max-norm), FP32 within 1e-6; padding entries exactly zero.
"""
import os

import numpy as np
import pytest
import torch

from oracle import projectors as op
from qimpy_gb300 import ops
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEV = "cuda:0"


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_gamma"])
def test_blip_projectors_match_reference(name):
    """Blip-spline radial tables, as the reference's get_projectors uses them:
    the device result against the reference's own beta."""
    g = np.load(os.path.join(GOLDEN, f"projectors_{name}.npz"))
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=bool(p.extra.get("real_wavefunctions")))
    shells = [(sh.l, ("blip", g["coeff"][s], float(g["dq"]))) for s, sh in enumerate(p.shells)]
    beta = ops.make_projectors(b.iG, p.k, p.Gbasis, b.n, p.positions, shells, p.volume, torch.complex128, DEV)
    assert _rel(beta.cpu().numpy(), g["beta"]) <= 1e-12


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-12), (torch.complex64, 1e-6)])
@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2", "cu32"])
def test_gaussian_projectors_match_oracle(name, dtype, tol):
    """Analytic Gaussian shells (every workload's projectors): s, p, d shells,
    several k-points with ragged bases (padding zero), 18 projectors per atom
    on the 32-atom Cu-like cell."""
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    shells = [(sh.l, ("gauss", sh.sigma)) for sh in p.shells]
    got = wl.make_projectors_device(p, b, DEV, dtype).cpu().numpy().astype(np.complex128)
    want = op.projectors(b.iG, p.k, p.Gbasis, b.n, p.positions, shells, p.volume)
    assert _rel(got, want) <= tol
    for k in range(p.nk):
        assert not got[k, :, int(b.n[k]):].any()


def test_projector_errors():
    p = wl.get("tiny_fcc")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    with pytest.raises(Exception, match="l = 3"):
        ops.make_projectors(b.iG, p.k, p.Gbasis, b.n, p.positions, [(3, ("gauss", 1.0))], p.volume,
                            torch.complex128, DEV)
    with pytest.raises(Exception, match="sigma"):
        ops.make_projectors(b.iG, p.k, p.Gbasis, b.n, p.positions, [(0, ("gauss", -1.0))], p.volume,
                            torch.complex128, DEV)
