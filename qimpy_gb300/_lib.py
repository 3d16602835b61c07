"""ctypes binding of ``libqimpy_gb300.so`` (the C ABI of include/qimpy_gb300.h).

The library is loaded from the package directory only; there is no fallback:
if it is missing, every GPU operation raises.
"""
from __future__ import annotations

import ctypes as ct
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
DEBUG = os.environ.get("QGB_DEBUG_CHECKS", "0") == "1"
LIB_PATH = os.path.join(PKG, "libqimpy_gb300_debug.so" if DEBUG else "libqimpy_gb300.so")

QGB_F64, QGB_F32 = 0, 1
QGB_ADD_KE, QGB_ACCUMULATE = 1, 2
ABI_VERSION = 2

_ERRORS = {1: "invalid argument", 2: "workspace too small", 3: "CUDA error", 4: "cuBLAS error",
           5: "unsupported", 6: "cuSOLVER error"}


class QgbSphere(ct.Structure):
    """Mirror of ``struct qgb_sphere``."""

    _fields_ = [
        ("nk", ct.c_int32), ("n_tot", ct.c_int32),
        ("N", ct.c_int32 * 3), ("L1", ct.c_int32 * 3), ("L2", ct.c_int32 * 3),
        ("max_slabs", ct.c_int32), ("max_rows", ct.c_int32), ("tw_off", ct.c_int32 * 3),
        ("n", ct.c_void_p), ("n_slabs", ct.c_void_p), ("slab_start", ct.c_void_p),
        ("slab_i0", ct.c_void_p), ("yz", ct.c_void_p), ("row_start", ct.c_void_p),
        ("rows", ct.c_void_p), ("twiddle", ct.c_void_p), ("ke", ct.c_void_p), ("V", ct.c_void_p),
    ]


class QgbRealMap(ct.Structure):
    """Mirror of ``struct qgb_real_map``."""

    _fields_ = [("n_half", ct.c_int32), ("n_tot_half", ct.c_int32), ("n_full", ct.c_int32),
                ("n_tot_full", ct.c_int32), ("n_plane", ct.c_int32), ("pack", ct.c_void_p), ("unpack", ct.c_void_p),
                ("plane", ct.c_void_p), ("ke", ct.c_void_p), ("weight", ct.c_void_p)]


class QgbProjectorShell(ct.Structure):
    """Mirror of ``struct qgb_projector_shell``."""

    _fields_ = [("l", ct.c_int32), ("kind", ct.c_int32), ("sigma", ct.c_double), ("coeff", ct.c_void_p),
                ("n_coeff", ct.c_int32), ("dq", ct.c_double)]


QGB_RADIAL_GAUSSIAN, QGB_RADIAL_BLIP = 0, 1


class QgbBatchItem(ct.Structure):
    """Mirror of ``struct qgb_batch_item``."""

    _fields_ = [("sphere", ct.c_void_p), ("C", ct.c_void_p), ("out", ct.c_void_p), ("planes", ct.c_void_p),
                ("nb", ct.c_int32), ("flags", ct.c_uint32)]


class QgbError(RuntimeError):
    """Nonzero status returned by the library."""


_lock = threading.Lock()
_lib = None

_SIGS = {
    "qgb_abi_version": (ct.c_int, []),
    "qgb_last_error": (ct.c_char_p, []),
    "qgb_potential_workspace_bytes": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.c_int, ct.c_int]),
    "qgb_hamiltonian_workspace_bytes": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.c_int, ct.c_int, ct.c_int]),
    "qgb_permute_real_space": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_void_p]),
    "qgb_apply_ke": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_void_p]),
    "qgb_apply_potential": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int,
                                       ct.c_uint, ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_project_workspace_bytes": (ct.c_size_t, [ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int]),
    "qgb_project": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int,
                               ct.c_int, ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_dot_workspace_bytes": (ct.c_size_t, [ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int]),
    "qgb_dot": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p,
                           ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_band_norm_ke": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
                                    ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "qgb_residual": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
                                ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                ct.c_void_p]),
    "qgb_normalize_bands": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p,
                                       ct.c_double, ct.c_longlong, ct.c_longlong, ct.c_void_p, ct.c_void_p]),
    "qgb_matmul_tc_workspace_bytes": (ct.c_size_t, [ct.c_int, ct.c_int, ct.c_int, ct.c_int]),
    "qgb_matmul_tc": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p,
                                 ct.c_uint, ct.c_void_p, ct.c_size_t, ct.c_void_p, ct.c_void_p]),
    "qgb_dot_tc_workspace_bytes": (ct.c_size_t, [ct.c_int, ct.c_int, ct.c_int, ct.c_int]),
    "qgb_dot_tc": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p,
                              ct.c_void_p, ct.c_size_t, ct.c_void_p, ct.c_void_p]),
    "qgb_dot_real": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p,
                                ct.c_void_p, ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_hamiltonian_real_workspace_bytes": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.POINTER(QgbRealMap), ct.c_int,
                                                           ct.c_int, ct.c_int]),
    "qgb_hamiltonian_real": (ct.c_int, [ct.POINTER(QgbSphere), ct.POINTER(QgbRealMap), ct.c_int, ct.c_void_p,
                                        ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int,
                                        ct.c_void_p, ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_hamiltonian_real_mixed_workspace_bytes": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.POINTER(QgbRealMap),
                                                                 ct.c_int, ct.c_int]),
    "qgb_hamiltonian_real_mixed": (ct.c_int, [ct.POINTER(QgbSphere), ct.POINTER(QgbRealMap), ct.c_void_p, ct.c_void_p,
                                              ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p,
                                              ct.c_void_p, ct.c_size_t, ct.c_void_p, ct.c_void_p]),
    "qgb_symmetrize_real": (ct.c_int, [ct.c_int, ct.POINTER(QgbRealMap), ct.c_void_p, ct.c_int, ct.c_void_p]),
    "qgb_make_projectors": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                       ct.POINTER(ct.c_double), ct.c_int, ct.c_void_p, ct.c_int,
                                       ct.POINTER(QgbProjectorShell), ct.c_double, ct.c_void_p, ct.c_void_p]),
    "qgb_matmul": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int,
                              ct.c_void_p, ct.c_uint, ct.c_void_p]),
    "qgb_apply_nonlocal": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p,
                                      ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p]),
    "qgb_hamiltonian": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int,
                                   ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p,
                                   ct.c_size_t, ct.c_void_p]),
    "qgb_apply_potential_static": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int,
                                              ct.c_uint, ct.c_void_p]),
    "qgb_static_scratch_bytes": (ct.c_size_t, []),
    "qgb_collect_density": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p,
                                       ct.c_void_p, ct.c_uint, ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_sphere_smem_bytes": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.c_int]),
    "qgb_sphere_smem_bytes_yz": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.c_int]),
    "qgb_apply_potential_batched": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                               ct.c_void_p, ct.c_longlong, ct.c_longlong, ct.c_int, ct.c_size_t,
                                               ct.c_size_t, ct.c_void_p]),
    "qgb_beta_split_bytes": (ct.c_size_t, [ct.c_int, ct.c_int, ct.c_int]),
    "qgb_beta_split": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_size_t, ct.c_void_p]),
    "qgb_nonlocal_tc_workspace_bytes": (ct.c_size_t, [ct.c_int, ct.c_int, ct.c_int, ct.c_int]),
    "qgb_apply_nonlocal_tc": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p,
                                         ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_size_t,
                                         ct.c_void_p, ct.c_void_p]),
    "qgb_apply_nonlocal_tc_phase": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p,
                                               ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p,
                                               ct.c_size_t, ct.c_void_p, ct.c_int, ct.c_void_p]),
    "qgb_hamiltonian_mixed_workspace_bytes": (ct.c_size_t, [ct.POINTER(QgbSphere), ct.c_int, ct.c_int]),
    "qgb_hamiltonian_mixed": (ct.c_int, [ct.POINTER(QgbSphere), ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_void_p,
                                         ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_size_t,
                                         ct.c_void_p, ct.c_void_p]),
    "qgb_subspace_eigh_workspace_bytes": (ct.c_size_t, [ct.c_int64, ct.c_int64]),
    "qgb_subspace_eigh": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int64, ct.c_void_p,
                                     ct.c_size_t, ct.c_void_p]),
}

#: Every symbol the header declares (checked by the CPU tests).
EXPORTED = tuple(_SIGS)

#: Measurement and test aids of libqimpy_gb300_aux.so (include/qimpy_gb300_aux.h).
AUX_PATH = os.path.join(PKG, "libqimpy_gb300_aux.so")
_AUX_SIGS = {
    "qgb_fma_burn": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p]),
    "qgb_tc_gemm_bf16x3": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int,
                                      ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                      ct.c_size_t, ct.c_void_p]),
    "qgb_tc_wait_timeout_test": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_ulonglong, ct.c_void_p]),
}
AUX_EXPORTED = tuple(_AUX_SIGS)
_aux = None


def aux() -> ct.CDLL:
    """The auxiliary library of measurement and test aids (loads the main one first)."""
    global _aux
    lib()
    if _aux is None:
        with _lock:
            if _aux is None:
                if not os.path.exists(AUX_PATH):
                    raise RuntimeError(f"{AUX_PATH} is missing: build it with `python -m qimpy_gb300.build`")
                handle = ct.CDLL(AUX_PATH)
                for name, (res, args) in _AUX_SIGS.items():
                    fn = getattr(handle, name)
                    fn.restype = res
                    fn.argtypes = args
                _aux = handle
    return _aux


def lib() -> ct.CDLL:
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise RuntimeError(
                        f"{LIB_PATH} is missing: build it with `python -m qimpy_gb300.build` "
                        "(the CUDA extension is required; there is no CPU fallback)"
                    )
                handle = ct.CDLL(LIB_PATH)
                for name, (res, args) in _SIGS.items():
                    fn = getattr(handle, name)
                    fn.restype = res
                    fn.argtypes = args
                if DEBUG:
                    handle.qgb_debug_violation.restype = ct.c_int
                    handle.qgb_debug_violation.argtypes = [ct.POINTER(ct.c_ulonglong)]
                if handle.qgb_abi_version() != ABI_VERSION:
                    raise RuntimeError("libqimpy_gb300.so ABI version mismatch; rebuild it")
                _lib = handle
    return _lib


def debug_violation() -> tuple:
    """(site, index, limit, block) of the first range violation since the last
    call (debug library only); site 0 means none."""
    out = (ct.c_ulonglong * 4)()
    check(lib().qgb_debug_violation(out), "debug_violation")
    return tuple(int(x) for x in out)


def check(status: int, what: str) -> None:
    """Raise QgbError with the library's message for a nonzero status."""
    if status != 0:
        msg = lib().qgb_last_error().decode(errors="replace")
        raise QgbError(f"{what}: {_ERRORS.get(status, status)}: {msg}")
