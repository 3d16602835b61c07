"""Davidson on the GPU against the reference's converged eigenvalues (golden fixtures).

Plain FP64 form: eigenvalues within 1e-10 Ha of the reference.  Mixed form
(FP32 H.psi, FP64 subspace): within 1e-6 Ha after one FP64 Rayleigh-Ritz sweep.
"""
import os

import numpy as np
import pytest
import torch

from qimpy_gb300 import davidson as dv
from qimpy_gb300 import electrons as E
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _solve(name, dtype, threshold=None, residual=None):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p = wl.get(name)
    el, C0 = E.from_problem(p, "cuda:0", dtype)
    el.C = E.Wavefunction(el.basis, coeff=C0.to("cuda:0", dtype)).orthonormalize()
    d = dv.Davidson(el, n_iterations=300, eig_threshold=threshold or float(g["eig_threshold"]),
                    residual_threshold=residual)
    stats = d()
    return g, p, el, stats


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2"])
def test_davidson_fp64_matches_reference(name):
    g, p, el, stats = _solve(name, torch.complex128)
    assert stats.converged
    eig = el.eig.cpu().numpy()
    assert np.abs(eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
    # The same algorithm on the same inputs takes the same number of iterations.
    assert abs(stats.iterations - int(g["davidson_iterations"])) <= 2


def test_davidson_mixed_refined_within_1e6():
    g, p, el, stats = _solve("si2", torch.complex64, threshold=1e-6)
    assert stats.converged
    el64, _ = E.from_problem(p, "cuda:0", torch.complex128)
    eig_ref, _ = dv.refine_fp64(el, el64)
    err_before = np.abs(el.eig.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    err_after = np.abs(eig_ref.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    assert err_after <= 1e-6, (err_before, err_after)


def test_davidson_residual_criterion():
    g, p, el, stats = _solve("tiny_fcc", torch.complex128, threshold=1e-8, residual=1e-8)
    assert stats.converged and stats.residual_max < 1e-8
    eig = el.eig.cpu().numpy()
    assert np.abs(eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
