"""qgb_apply_potential_static: the local-potential apply for callers that cannot
allocate device memory (their device memory is owned by an outer framework, or
they run where cudaMalloc is not allowed).  It must give the same result as
qgb_apply_potential, whose workspace the caller allocates, on two calls in a
row that reuse its fixed scratch, and reject a sphere too big for that scratch.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as ct

import pytest
import torch

from qimpy_gb300 import _lib, ops, sphere as sp, workloads as wl

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
TOL = {torch.complex128: 1e-12, torch.complex64: 2e-5}


def _sphere(name, dtype):
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    ds = sp.DeviceSphere(sp.build_tables(b.fft_index, b.n, p.grid_shape), b.ke, DEV, dtype)
    ds.set_potential(torch.from_numpy(p.V_r))
    return p, b, ds


@pytest.mark.parametrize("name,dtype", [("si2", torch.complex128), ("si2", torch.complex64),
                                        ("si64", torch.complex128)])
def test_static_scratch_matches_workspace_entry_point(name, dtype):
    p, b, ds = _sphere(name, dtype)
    lib = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    nb = 12  # more bands than fit in the fixed scratch at once for si64 FP64
    flags = _lib.QGB_ADD_KE
    for call in range(2):  # the second call reuses the scratch left by the first
        C = torch.from_numpy(wl.make_wavefunctions(p, b, nb, band_offset=call * nb)).to(DEV, dtype)
        want = ops.apply_potential(ds, C, add_ke=True)
        got = torch.empty_like(C)
        rc = lib.qgb_apply_potential_static(ct.byref(ds.struct), ds.qdtype, C.data_ptr(), got.data_ptr(), nb,
                                            flags, stream)
        _lib.check(rc, "apply_potential_static")
        torch.cuda.synchronize()
        err = float((got - want).abs().max() / want.abs().max())
        assert err <= TOL[dtype], (call, err)


def test_static_scratch_rejects_oversized_sphere():
    lib = _lib.lib()
    p, b, ds = _sphere("tiny_fcc", torch.complex128)
    big = _lib.QgbSphere.from_buffer_copy(ds.struct)
    big.nk, big.max_slabs = 64, 96
    big.N[1], big.N[2] = 96, 96
    need = 64 * 96 * 96 * 96 * 16
    assert need > lib.qgb_static_scratch_bytes()
    C = torch.zeros((1, 1, ds.tables.n_tot), dtype=torch.complex128, device=DEV)
    rc = lib.qgb_apply_potential_static(ct.byref(big), _lib.QGB_F64, C.data_ptr(), C.data_ptr(), 1, 0,
                                        torch.cuda.current_stream().cuda_stream)
    assert rc == 2  # QGB_ERR_WORKSPACE
    assert b"fixed" in lib.qgb_last_error()
