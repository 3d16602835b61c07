"""Parity on the configurations the throughput figures are quoted on.

* Mixed H.psi (complex64: FP32 KE + local potential, tensor-core split-BF16x3
  nonlocal) on the 64-atom Si cell (96^3, n = 37073, P = 256) and the 32-atom
  Cu-like cell (72^3, 4 k, P = 576) against the reference's own FP64 H.psi:
  per-band checksums and whole sample bands within 2e-5 relative (max-norm).
* Davidson on both cells, plain FP64 against the reference's converged
  eigenvalues (within 1e-10 Ha, the same iteration count within 2), and mixed
  with FP64 refinement (within 1e-6 Ha after refinement; the error before it
  is reported by the assertion message).
* Batched H.psi of instances of the uneven-batch distribution against the
  oracle's FP64 H.psi (2e-5 relative).
* Served eigensolves at the residual target 1e-6.
"""
import os

import numpy as np
import pytest
import torch

from oracle import hpsi as oh
from qimpy_gb300 import batch as bt
from qimpy_gb300 import davidson as dv
from qimpy_gb300 import electrons as E
from qimpy_gb300 import ops
from qimpy_gb300 import serve as sv
from qimpy_gb300 import sphere as sp
from qimpy_gb300 import workloads as wl
from qimpy_gb300.checksums import band_checksums

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEV = "cuda:0"
TOL_MIXED = 2e-5  # relative, max-norm, mixed H.psi against FP64


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name,nb,chunk", [("tiny_fcc", 6, None), ("cu32", 5, 2)])
def test_mixed_hamiltonian_writes_every_entry(name, nb, chunk):
    """qgb_hamiltonian_mixed stores the nonlocal term into HC on a side stream
    while the local potential's transforms run, and the gather adds KE C + V C:
    every entry of HC is written (NaN-filled before the call), the padding is
    exactly zero, and HC matches the oracle, also when the bands pass through
    the local potential in chunks (planes for `chunk` bands)."""
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    beta = wl.make_projectors(p, b)
    C = wl.make_wavefunctions(p, b, nb)
    ds = sp.DeviceSphere(sp.build_tables(b.fft_index, b.n, p.grid_shape), b.ke, DEV, torch.complex64)
    ds.set_potential(torch.from_numpy(p.V_r))
    split = ops.beta_split(torch.from_numpy(beta).to(DEV, torch.complex64))
    P = beta.shape[1]
    ws = None
    if chunk is not None:
        nl = ds.hamiltonian_mixed_workspace_bytes(nb, P) - ds.workspace_bytes(nb)
        ws = ops.workspace(nl + ds.workspace_bytes(chunk), DEV)
    out = torch.full(C.shape, float("nan"), dtype=torch.complex64, device=DEV)
    HC, _ = ops.hamiltonian_mixed(ds, torch.from_numpy(C).to(DEV, torch.complex64), split,
                                  torch.from_numpy(p.D_atom).to(DEV, torch.complex64), out=out, ws=ws)
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    HC = HC.cpu().numpy().astype(np.complex128)
    assert np.isfinite(HC).all()
    for k in range(p.nk):
        assert not HC[k, :, int(b.n[k]):].any()
    want = oh.hamiltonian(b.ke, p.V_r, b.fft_index, b.n, beta, p.D_all(), C)
    assert _rel(HC, want) < TOL_MIXED


@pytest.mark.parametrize("name", ["si64", "cu32"])
def test_mixed_hamiltonian_matches_reference_checksums(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    nb = int(g["hpsi_bands"])
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    assert np.array_equal(b.fft_index, g["fft_index"])
    beta = wl.make_projectors(p, b)
    C = wl.make_wavefunctions(p, b, nb)
    ds = sp.DeviceSphere(sp.build_tables(b.fft_index, b.n, p.grid_shape), b.ke, DEV, torch.complex64)
    ds.set_potential(torch.from_numpy(p.V_r))
    split = ops.beta_split(torch.from_numpy(beta).to(DEV, torch.complex64))
    HC, projT = ops.hamiltonian_mixed(ds, torch.from_numpy(C).to(DEV, torch.complex64), split,
                                      torch.from_numpy(p.D_atom).to(DEV, torch.complex64))
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    HC = HC.cpu().numpy().astype(np.complex128)
    cs = band_checksums(HC, b.n)
    assert np.abs(cs - g["hpsi_checksums"]).max() <= TOL_MIXED * np.abs(g["hpsi_checksums"]).max()
    for (k, bb), ref in zip(g["hpsi_sample_kb"], g["hpsi_sample"]):
        assert _rel(HC[k, bb], ref) < TOL_MIXED
    for (k, bb), ref in zip(g["hpsi_sample_kb"], g["proj_sample"]):
        assert _rel(projT[k, bb].cpu().numpy(), ref) < TOL_MIXED


def _davidson(name, dtype, threshold=None):
    """Davidson from the reference's start vectors; threshold None = the reference run's."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p = wl.get(name)
    el, C0 = E.from_problem(p, DEV, dtype)
    el.C = E.Wavefunction(el.basis, coeff=C0.to(DEV, dtype)).orthonormalize()
    thr = float(g["eig_threshold"]) if threshold is None else threshold
    stats = dv.Davidson(el, n_iterations=300, eig_threshold=thr)()
    return g, p, el, stats


@pytest.mark.parametrize("name", ["si64", "cu32"])
def test_davidson_fp64_matches_reference_full_size(name):
    g, p, el, stats = _davidson(name, torch.complex128)
    assert stats.converged
    eig = el.eig.cpu().numpy()
    err = np.abs(eig[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    assert err < 1e-10, err
    assert abs(stats.iterations - int(g["davidson_iterations"])) <= 2, (stats.iterations, int(g["davidson_iterations"]))


@pytest.mark.parametrize("name", ["si64", "cu32"])
def test_davidson_mixed_refined_full_size(name):
    g, p, el, stats = _davidson(name, torch.complex64, 1e-6)
    assert stats.converged or stats.stalled
    el64, _ = E.from_problem(p, DEV, torch.complex128)
    eig_ref, _ = dv.refine_fp64(el, el64, eig_threshold=1e-8)
    err_before = np.abs(el.eig.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    err_after = np.abs(eig_ref.cpu().numpy()[:, : p.n_bands] - g["eig"][:, : p.n_bands]).max()
    assert err_after <= 1e-6, (err_before, err_after)


def test_batched_instances_match_oracle():
    """Four instances of the 256-instance uneven distribution (the smallest
    grids, two grid shapes at least) run as one batched H.psi; each result
    against the oracle's FP64 H.psi of the same inputs."""
    specs = bt.make_batch_specs(count=256)
    small = sorted(specs, key=lambda s: (s.grid, s.n_bands * len(s.k)))
    pick = small[:2] + [s for s in small if s.grid > small[0].grid][:2]
    insts = [bt.Instance(s, DEV) for s in pick]
    assert len({i.tables.shape for i in insts}) > 1
    bh = bt.BatchedHamiltonian(insts, torch.device(DEV))
    bh.apply()
    torch.cuda.synchronize()
    assert int(ops.device_error_word(DEV).item()) == 0
    for inst, out in zip(insts, bh.outputs):
        lay = inst.layout
        D_all = np.kron(np.eye(inst.spec.n_atoms), inst.D[0].cpu().numpy().astype(np.complex128))
        want = oh.hamiltonian(lay.ke, inst.V_r.cpu().numpy(), lay.fft_index, lay.n,
                              inst.beta.cpu().numpy().astype(np.complex128), D_all,
                              inst.C.cpu().numpy().astype(np.complex128))
        assert _rel(out.cpu().numpy(), want) < TOL_MIXED


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_serving_meets_residual_target(precision):
    """Requests served with the residual target 1e-6 finish with every
    band's FP64 residual norm below it."""
    specs = bt.make_batch_specs(count=4, seed=9, bands_range=(4, 8), k_range=(1, 2), ke_range=(5.0, 9.0),
                                atoms_range=(2, 3), sides=(10.0, 12.0))
    reqs = [sv.EigenRequest(i, s, 6, arrival=0.005 * i) for i, s in enumerate(specs)]
    with sv.EigenServer(DEV, precision=precision, eig_threshold=1e-6, residual_threshold=1e-6) as srv:
        rep = srv.run(reqs, realtime=True)
    assert rep["done"] == len(reqs), [(r.rid, r.status, r.error) for r in reqs]
    assert max(r.residual for r in reqs) < 1e-6
