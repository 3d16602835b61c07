"""Band-wise Davidson passes (qgb_band_norm_ke, qgb_residual,
qgb_normalize_bands) against torch FP64 restatements of the reference's
formulas on the same inputs.

Tolerances (relative, max-norm): FP64 1e-13; FP32 inputs 1e-6.  The null-band
randomisation must reproduce the host restatement of the reference's seeded
generator (davidson.randomize_selected, itself checked against the oracle on
CPU) within 1e-13 (FP64) / 1e-6 (FP32).
"""
import pytest
import torch

from qimpy_gb300 import davidson as dv
from qimpy_gb300 import electrons as E
from qimpy_gb300 import ops
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
TOL = {torch.complex128: 1e-13, torch.complex64: 1e-6}


def _setup(dtype, nb=10):
    p = wl.get("si2")
    el, C0 = E.from_problem(p, DEV, dtype, n_bands_total=nb)
    C = C0.to(DEV, dtype).contiguous()
    g = torch.Generator(device="cpu").manual_seed(5)
    HC = (torch.randn(C.shape, generator=g, dtype=torch.complex128).to(DEV, dtype) * el.basis.mask[:, None, :]).contiguous()
    eig = torch.randn((p.nk, nb), generator=g, dtype=torch.float64).to(DEV)
    return p, el, C, HC, eig


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_band_norm_ke(dtype):
    p, el, C, HC, eig = _setup(dtype)
    c2 = C.to(torch.complex128).abs().square()
    nrm, bke = ops.band_norm_ke(C, el.basis.ke, b0=3)
    assert _rel(nrm, c2[:, 3:].sum(-1).sqrt()) < TOL[dtype]
    assert _rel(bke, (c2[:, 3:] * el.basis.ke[:, None, :]).sum(-1)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_residual_and_precondition(dtype):
    p, el, C, HC, eig = _setup(dtype)
    b0 = 4
    C64, H64 = C.to(torch.complex128), HC.to(torch.complex128)
    R = H64[:, b0:] - C64[:, b0:] * eig[:, b0:, None]
    nrm = ops.residual(HC, C, eig, norm=True)
    assert _rel(nrm[:, b0:], R.abs().square().sum(-1).sqrt()) < TOL[dtype]
    KEref = (C64[:, b0:].abs().square() * el.basis.ke[:, None, :]).sum(-1)
    out = torch.empty((p.nk, C.shape[1] - b0, C.shape[2]), dtype=dtype, device=DEV)
    n2 = ops.residual(HC, C, eig, el.basis.ke, KEref, b0=b0, out=out, norm=True)
    x = el.basis.ke[:, None, :] / KEref[..., None]
    want = R / (x + torch.exp(-x))
    tol = TOL[dtype] if dtype == torch.complex128 else 5e-6
    assert _rel(out.to(torch.complex128), want) < tol
    assert _rel(n2, want.abs().square().sum(-1).sqrt()) < tol


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_normalize_bands_randomises_null_bands(dtype):
    p, el, C, HC, eig = _setup(dtype, nb=6)
    X = C.clone()
    norm = ops.band_norm_ke(X)[0]
    low = torch.zeros_like(norm, dtype=torch.bool)
    low[0, 1] = low[3, 4] = low[7, 0] = True
    cut = 1e-3
    norm_in = torch.where(low, torch.full_like(norm, 1e-6), norm)
    n_out = norm_in.clone()
    ops.normalize_bands(X, el.basis.n_device, n_out, cut, 17, el.basis.n_max, el.basis.ke)
    # Host restatement of the reference's randomize_selected for the same bands.
    Wref = E.Wavefunction(el.basis, coeff=C.clone())
    i_k, i_b = torch.where(low)
    dv.randomize_selected(Wref, i_k, i_b, 17)
    want = Wref.coeff.to(torch.complex128) / torch.where(low, torch.ones_like(norm), norm)[..., None]
    want = want * el.basis.mask[:, None, :]
    assert _rel(X.to(torch.complex128), want) < TOL[dtype]
    assert torch.equal(n_out[low], torch.ones(3, dtype=torch.float64, device=DEV))
    assert torch.equal(n_out[~low], norm[~low])
    for k in range(p.nk):
        assert int(torch.count_nonzero(X[k, :, int(el.basis.n[k]):])) == 0
