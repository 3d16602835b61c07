"""The C-ABI library builds, loads and exports every entry point include/qimpy_gb300.h declares.

No compute calls (no GPU here): only host-side functions are exercised.
"""
import ctypes as ct
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from qimpy_gb300 import _lib, build

    build.build()
    return _lib.lib()


def declared_symbols(header: str = "qimpy_gb300.h"):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qgb_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    from qimpy_gb300 import _lib

    names = declared_symbols()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(_lib.EXPORTED) | {"qgb_debug_violation"}


def test_aux_library_exports_its_header(lib):
    """Measurement and test aids live in libqimpy_gb300_aux.so, not in the product ABI."""
    from qimpy_gb300 import _lib

    aux = _lib.aux()
    names = declared_symbols("qimpy_gb300_aux.h")
    assert set(names) == set(_lib.AUX_EXPORTED)
    for name in names:
        assert hasattr(aux, name), name
        assert name not in declared_symbols()
    # Errors of the aux library are reported through the main library's message.
    assert aux.qgb_tc_wait_timeout_test(None, None, None, 0, None) == 1
    assert b"timeout" in lib.qgb_last_error()


def test_abi_version_and_error_text(lib):
    assert lib.qgb_abi_version() == 2
    from qimpy_gb300 import _lib

    # An invalid call fails on the host before touching a device.
    rc = lib.qgb_apply_potential(None, 0, None, None, 1, 0, None, 0, None)
    assert rc == 1
    assert b"NULL" in lib.qgb_last_error()
    with pytest.raises(_lib.QgbError):
        _lib.check(rc, "apply_potential")


def test_host_helpers(lib):
    from qimpy_gb300 import _lib, sphere as sp, workloads as wl

    p = wl.tiny_ortho()
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    t = sp.build_tables(b.fft_index, b.n, p.grid_shape)
    s = _lib.QgbSphere()
    s.nk, s.n_tot = t.nk, t.n_tot
    for a in range(3):
        s.N[a] = t.shape[a]
        s.L1[a], s.L2[a] = t.fac[a]
    s.max_slabs = t.max_slabs
    perm = np.zeros(sum(t.shape), dtype=np.int32)
    assert lib.qgb_permute_real_space(ct.byref(s), perm.ctypes.data) == 0
    off = 0
    for a in range(3):
        assert np.array_equal(perm[off: off + t.shape[a]], sp.permutation(t.shape[a], *t.fac[a]))
        off += t.shape[a]
    nbytes = lib.qgb_potential_workspace_bytes(ct.byref(s), 3, 0)
    assert nbytes == 3 * t.nk * t.max_slabs * t.shape[1] * t.shape[2] * 16
    assert lib.qgb_potential_workspace_bytes(ct.byref(s), 3, 1) * 2 == nbytes


def test_band_product_host_checks(lib):
    """Workspace sizing of the split-K products and argument checks that fail
    on the host, before any launch."""
    # Small products need no partial sums; long bases are split over CTAs.
    assert lib.qgb_dot_workspace_bytes(0, 1, 8, 8, 64) == 0
    big = lib.qgb_dot_workspace_bytes(0, 1, 176, 352, 37073)
    assert big > 0 and big % (176 * 352 * 16) == 0
    assert lib.qgb_dot_workspace_bytes(1, 1, 176, 352, 37073) * 2 == big
    assert lib.qgb_project_workspace_bytes(0, 1, 256, 32, 37073) % (256 * 32 * 16) == 0
    assert lib.qgb_dot_workspace_bytes(9, 1, 8, 8, 64) == 0
    assert lib.qgb_dot(9, None, 1, None, 1, 1, 64, None, None, 0, None) == 1
    assert lib.qgb_dot(0, None, 1, None, 1, 1, 0, None, None, 0, None) == 1
    assert lib.qgb_matmul(0, None, 2, 1, 64, None, 2, None, 4, None) == 1  # unknown flag
    assert b"flags" in lib.qgb_last_error()
    # nothing to do: no launch, success
    assert lib.qgb_matmul(0, None, 2, 1, 64, None, 0, None, 0, None) == 0
