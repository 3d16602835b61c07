"""Batched H.psi over uneven instances: equal to the per-instance calls.

The batched local-potential kernels run the same per-unit code as the
single-sphere kernels, so results must agree bit for bit; graph replay must
reproduce the eager result.  Also pins the device basis builder against the
host one on the reference's ordering rule.
"""
import numpy as np
import pytest
import torch

from qimpy_gb300 import batch as bt
from qimpy_gb300 import ops
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_device_basis_matches_host():
    p = wl.si2()
    a = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    b = wl.make_basis_device(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, DEV)
    assert np.array_equal(a.n, b.n) and np.array_equal(a.fft_index, b.fft_index)
    assert np.allclose(a.ke, b.ke, rtol=1e-14, atol=0)


def _small_specs():
    specs = bt.make_batch_specs(count=6, seed=5, bands_range=(3, 9), k_range=(1, 3), ke_range=(6.0, 12.0),
                                atoms_range=(2, 4))
    return specs


# plane chunks: 64 MB, one instance per chunk, one chunk per group; solo: none
# batched alone, or the larger half of the instances through the single call
@pytest.mark.parametrize("chunk,solo", [(64 << 20, False), (1, False), (0, False), (0, True)])
def test_batched_equals_individual_and_graph_replay(chunk, solo):
    specs = _small_specs()
    insts = [bt.Instance(s, DEV) for s in specs]
    assert len({i.tables.shape for i in insts}) > 1  # uneven grids
    units = sorted(i.tables.nk * i.nb * i.tables.max_slabs for i in insts)
    bh = bt.BatchedHamiltonian(insts, torch.device(DEV), plane_chunk_bytes=chunk,
                               solo_units=units[len(units) // 2] if solo else 0)
    assert (len(bh.solo) > 0) == solo and (not solo or len(bh.solo) < len(insts))
    if chunk == 1:
        assert sum(len(g._chunks) for g in bh.groups) == len(insts)
    bh.apply()
    torch.cuda.synchronize()
    eager = [o.clone() for o in bh.outputs]
    for inst, out in zip(insts, eager):
        ref, _ = ops.hamiltonian_mixed(inst.sphere, inst.C, inst.split, inst.D)
        assert torch.equal(out, ref)
    for o in bh.outputs:
        o.zero_()
    bh.capture()
    for o in bh.outputs:
        o.zero_()
    bh.replay()
    torch.cuda.synchronize()
    for a, b in zip(bh.outputs, eager):
        assert torch.equal(a, b)
    assert int(ops.device_error_word(DEV).item()) == 0


def test_autotuned_factors_give_same_result():
    from qimpy_gb300 import autotune

    spec = _small_specs()[0]
    inst = bt.Instance(spec, DEV)
    ref, _ = ops.hamiltonian_mixed(inst.sphere, inst.C, inst.split, inst.D)
    fac = autotune.tune_shape(inst.tables.shape, torch.complex64, DEV, nb=2, reps=1, use_cache=False)
    inst.sphere.set_factors(fac)
    got, _ = ops.hamiltonian_mixed(inst.sphere, inst.C, inst.split, inst.D)
    assert float((got - ref).abs().max() / ref.abs().max()) < 2e-6
