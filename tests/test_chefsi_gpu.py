"""CheFSI on the GPU against the reference's own CheFSI (golden fixtures made
by running qimpy/dft/electrons/_chefsi.py on the same inputs).

Plain FP64 form: eigenvalues within 1e-10 Ha of the reference's CheFSI with the
same iteration count (Davidson warm-up included).  Mixed form (FP32 H.psi and
filter, FP64 subspace): within 1e-6 Ha after the FP64 refinement.
"""
import os

import numpy as np
import pytest
import torch

from qimpy_gb300 import chefsi as cf
from qimpy_gb300 import davidson as dv
from qimpy_gb300 import electrons as E
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _solve(name, dtype, threshold=None):
    g = np.load(os.path.join(GOLDEN, f"chefsi_{name}.npz"))
    p = wl.get(name)
    el, C0 = E.from_problem(p, "cuda:0", dtype)
    el.C = E.Wavefunction(el.basis, coeff=C0.to("cuda:0", dtype)).orthonormalize()
    solver = cf.CheFSI(el, n_iterations=int(g["n_iterations"]),
                       eig_threshold=threshold or float(g["eig_threshold"]),
                       filter_order=int(g["filter_order"]), init_threshold=float(g["init_threshold"]))
    return g, p, el, solver()


@pytest.mark.parametrize("name", ["tiny_fcc", "tiny_ortho", "si2"])
def test_chefsi_fp64_matches_reference_chefsi(name):
    g, p, el, stats = _solve(name, torch.complex128)
    assert stats.converged
    eig = el.eig.cpu().numpy()
    assert np.abs(eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max() < 1e-10
    assert stats.iterations == int(g["iterations"])


def test_chefsi_mixed_refined_within_1e6():
    g, p, el, stats = _solve("si2", torch.complex64, threshold=1e-6)
    assert stats.converged or stats.stalled
    el64, _ = E.from_problem(p, "cuda:0", torch.complex128)
    eig_ref, _ = dv.refine_fp64(el, el64)
    err = np.abs(eig_ref.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    assert err <= 1e-6, err


def test_chefsi_rejects_bad_filter_order():
    p = wl.get("tiny_fcc")
    el, _ = E.from_problem(p, "cuda:0", torch.complex128)
    with pytest.raises(ValueError):
        cf.CheFSI(el, filter_order=1)
