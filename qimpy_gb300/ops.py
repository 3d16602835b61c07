"""Tensor-level calls into the CUDA library (device tensors in, device tensors out).

Wavefunction tensors are (nk, nb, n_tot) complex, contiguous, on the sphere's
device; every call is asynchronous on the current torch stream and raises
``QgbError`` on a nonzero status.  There is no CPU path.
"""
from __future__ import annotations

import ctypes as ct

import torch

from . import _lib
from .sphere import DeviceSphere


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _qdtype(t: torch.Tensor) -> int:
    if t.dtype == torch.complex128:
        return _lib.QGB_F64
    if t.dtype == torch.complex64:
        return _lib.QGB_F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def _check_wf(sphere: DeviceSphere, C: torch.Tensor, name: str = "C") -> int:
    if not C.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor (no CPU path)")
    if C.dtype != sphere.cdtype:
        raise TypeError(f"{name} dtype {C.dtype} != sphere dtype {sphere.cdtype}")
    if C.dim() != 3 or C.shape[0] != sphere.tables.nk or C.shape[2] != sphere.tables.n_tot:
        raise ValueError(f"{name} shape {tuple(C.shape)} != (nk={sphere.tables.nk}, nb, n_tot={sphere.tables.n_tot})")
    if not C.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return C.shape[1]


def workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


def apply_ke(sphere: DeviceSphere, C: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    nb = _check_wf(sphere, C)
    out = torch.empty_like(C) if out is None else out
    _check_wf(sphere, out, "out")
    _lib.check(_lib.lib().qgb_apply_ke(ct.byref(sphere.struct), sphere.qdtype, C.data_ptr(), out.data_ptr(),
                                       nb, _stream()), "apply_ke")
    return out


def apply_potential(sphere: DeviceSphere, C: torch.Tensor, out: torch.Tensor | None = None,
                    add_ke: bool = False, accumulate: bool = False,
                    ws: torch.Tensor | None = None) -> torch.Tensor:
    """V*C (+ KE*C) on the G-sphere; `out` may alias `C`."""
    if not sphere.struct.V:
        raise RuntimeError("no potential installed (DeviceSphere.set_potential)")
    nb = _check_wf(sphere, C)
    out = torch.empty_like(C) if out is None else out
    _check_wf(sphere, out, "out")
    if ws is None:
        ws = workspace(sphere.workspace_bytes(nb), C.device)
    flags = (_lib.QGB_ADD_KE if add_ke else 0) | (_lib.QGB_ACCUMULATE if accumulate else 0)
    _lib.check(_lib.lib().qgb_apply_potential(ct.byref(sphere.struct), sphere.qdtype, C.data_ptr(),
                                              out.data_ptr(), nb, flags, ws.data_ptr(), ws.numel(),
                                              _stream()), "apply_potential")
    return out


def collect_density(sphere: DeviceSphere, C: torch.Tensor, prefac: torch.Tensor, rho: torch.Tensor | None = None,
                    accumulate: bool = False, ws: torch.Tensor | None = None) -> torch.Tensor:
    """rho(r) (FP64, natural grid order, shape N0 x N1 x N2) = sum_kb prefac[k, b]
    |psi_kb(r)|^2 of the bands in C; prefac (nk, nb) = f * w_sk / Omega."""
    nb = _check_wf(sphere, C)
    pf = prefac.to(device=C.device, dtype=torch.float64).contiguous()
    if tuple(pf.shape) != (C.shape[0], nb):
        raise ValueError(f"prefac shape {tuple(pf.shape)} != (nk, nb) = {(C.shape[0], nb)}")
    if rho is None:
        rho = torch.empty(sphere.shape, dtype=torch.float64, device=C.device)
    elif rho.dtype != torch.float64 or tuple(rho.shape) != tuple(sphere.shape) or not rho.is_contiguous():
        raise ValueError("rho must be a contiguous float64 tensor of the grid shape")
    if ws is None:
        ws = workspace(sphere.workspace_bytes(nb), C.device)
    flags = _lib.QGB_ACCUMULATE if accumulate else 0
    _lib.check(_lib.lib().qgb_collect_density(ct.byref(sphere.struct), sphere.qdtype, C.data_ptr(), nb,
                                              pf.data_ptr(), rho.data_ptr(), flags, ws.data_ptr(), ws.numel(),
                                              _stream()), "collect_density")
    return rho


def project(beta: torch.Tensor, C: torch.Tensor, projT: torch.Tensor | None = None) -> torch.Tensor:
    """projT[k, b, p] = <beta_p|C_b> (band-major projections)."""
    nk, P, n_tot = beta.shape
    nb = C.shape[1]
    if C.dtype != beta.dtype or C.shape[0] != nk or C.shape[2] != n_tot:
        raise ValueError("beta / C mismatch")
    projT = torch.empty((nk, nb, P), dtype=C.dtype, device=C.device) if projT is None else projT
    _lib.check(_lib.lib().qgb_project(_qdtype(C), beta.data_ptr(), C.data_ptr(), projT.data_ptr(), nk, P, nb,
                                      n_tot, _stream()), "project")
    return projT


def apply_nonlocal(beta: torch.Tensor, D_blocks: torch.Tensor, projT: torch.Tensor, out: torch.Tensor,
                   work: torch.Tensor | None = None) -> torch.Tensor:
    """out += beta D <beta|C> with D given as (n_atoms, pa, pa) blocks."""
    nk, P, n_tot = beta.shape
    n_atoms, pa, _ = D_blocks.shape
    nb = projT.shape[1]
    if n_atoms * pa != P:
        raise ValueError("D blocks do not cover the projectors")
    work = torch.empty_like(projT) if work is None else work
    _lib.check(_lib.lib().qgb_apply_nonlocal(_qdtype(out), beta.data_ptr(), D_blocks.data_ptr(), n_atoms, pa,
                                             projT.data_ptr(), out.data_ptr(), nk, nb, n_tot, work.data_ptr(),
                                             _stream()), "apply_nonlocal")
    return out


def hamiltonian(sphere: DeviceSphere, C: torch.Tensor, beta: torch.Tensor | None, D_blocks: torch.Tensor | None,
                out: torch.Tensor | None = None, projT: torch.Tensor | None = None, ws: torch.Tensor | None = None):
    """(HC, projT): HC = KE C + V C + beta D <beta|C> in one C-ABI call."""
    nb = _check_wf(sphere, C)
    out = torch.empty_like(C) if out is None else out
    if beta is None or beta.shape[1] == 0:
        n_atoms, pa, P = 0, 0, 0
        bptr = dptr = pptr = 0
    else:
        n_atoms, pa, _ = D_blocks.shape
        P = beta.shape[1]
        projT = torch.empty((C.shape[0], nb, P), dtype=C.dtype, device=C.device) if projT is None else projT
        bptr, dptr, pptr = beta.data_ptr(), D_blocks.data_ptr(), projT.data_ptr()
    if ws is None:
        ws = workspace(sphere.hamiltonian_workspace_bytes(nb, P), C.device)
    _lib.check(_lib.lib().qgb_hamiltonian(ct.byref(sphere.struct), sphere.qdtype, C.data_ptr(), out.data_ptr(),
                                          nb, bptr, dptr, n_atoms, pa, pptr, ws.data_ptr(), ws.numel(),
                                          _stream()), "hamiltonian")
    return out, projT


# ---------------------------------------------------------------------------
# Mixed precision: tensor-core (tcgen05, split-BF16x3) nonlocal term
# ---------------------------------------------------------------------------

_ERR_WORDS: dict = {}


def device_error_word(device) -> torch.Tensor:
    """Per-device int32 that tensor-core kernels set nonzero if a bounded
    pipeline wait times out (sticky until cleared by the caller)."""
    dev = torch.device(device)
    key = dev.index if dev.index is not None else torch.cuda.current_device()
    if key not in _ERR_WORDS:
        _ERR_WORDS[key] = torch.zeros(1, dtype=torch.int32, device=dev)
    return _ERR_WORDS[key]


def beta_split(beta: torch.Tensor) -> torch.Tensor:
    """Once per basis: complex64 projectors (nk, P, n_tot) -> bf16 hi/lo operands."""
    if beta.dtype != torch.complex64 or not beta.is_cuda or not beta.is_contiguous():
        raise TypeError("beta must be a contiguous complex64 CUDA tensor")
    nk, P, n_tot = beta.shape
    nbytes = int(_lib.lib().qgb_beta_split_bytes(nk, P, n_tot))
    out = torch.empty(nbytes, dtype=torch.uint8, device=beta.device)
    _lib.check(_lib.lib().qgb_beta_split(beta.data_ptr(), nk, P, n_tot, out.data_ptr(), nbytes, _stream()),
               "beta_split")
    return out


def apply_nonlocal_tc(split: torch.Tensor, D_blocks: torch.Tensor, C: torch.Tensor, HC: torch.Tensor,
                      projT: torch.Tensor | None = None, ws: torch.Tensor | None = None, phases: int = 3):
    """HC += beta D <beta|C> on the tensor cores (complex64); returns projT (nk, nb, P).

    phases = 1 runs only the part that reads C (projT and the back-projection
    operand, kept in `ws`), phases = 2 the accumulation into HC from that `ws`."""
    nk, nb, n_tot = C.shape
    n_atoms, pa, _ = D_blocks.shape
    P = n_atoms * pa
    if C.dtype != torch.complex64 or HC.dtype != torch.complex64 or D_blocks.dtype != torch.complex64:
        raise TypeError("tensor-core nonlocal needs complex64 C, HC and D")
    projT = torch.empty((nk, nb, P), dtype=torch.complex64, device=C.device) if projT is None else projT
    if phases != 3 and ws is None:
        raise ValueError("a split nonlocal apply needs a caller-owned workspace")
    if ws is None:
        ws = workspace(int(_lib.lib().qgb_nonlocal_tc_workspace_bytes(nk, P, nb, n_tot)), C.device)
    err = device_error_word(C.device)
    _lib.check(_lib.lib().qgb_apply_nonlocal_tc_phase(split.data_ptr(), D_blocks.data_ptr(), n_atoms, pa,
                                                      C.data_ptr(), HC.data_ptr(), projT.data_ptr(), nk, nb, n_tot,
                                                      ws.data_ptr(), ws.numel(), err.data_ptr(), phases, _stream()),
               "apply_nonlocal_tc")
    return projT


def hamiltonian_mixed(sphere: DeviceSphere, C: torch.Tensor, split: torch.Tensor | None,
                      D_blocks: torch.Tensor | None, out: torch.Tensor | None = None,
                      projT: torch.Tensor | None = None, ws: torch.Tensor | None = None):
    """Mixed-precision H.psi in one C-ABI call: FP32 KE + local potential,
    tensor-core (split-BF16x3) nonlocal.  Returns (HC, projT)."""
    nb = _check_wf(sphere, C)
    if sphere.cdtype != torch.complex64:
        raise TypeError("hamiltonian_mixed needs a complex64 sphere")
    out = torch.empty_like(C) if out is None else out
    if split is None or D_blocks is None:
        n_atoms = pa = P = 0
        sptr = dptr = pptr = 0
    else:
        n_atoms, pa, _ = D_blocks.shape
        P = n_atoms * pa
        projT = torch.empty((C.shape[0], nb, P), dtype=C.dtype, device=C.device) if projT is None else projT
        sptr, dptr, pptr = split.data_ptr(), D_blocks.data_ptr(), projT.data_ptr()
    if ws is None:
        ws = workspace(sphere.hamiltonian_mixed_workspace_bytes(nb, P), C.device)
    err = device_error_word(C.device)
    _lib.check(_lib.lib().qgb_hamiltonian_mixed(ct.byref(sphere.struct), C.data_ptr(), out.data_ptr(), nb, sptr,
                                                dptr, n_atoms, pa, pptr, ws.data_ptr(), ws.numel(), err.data_ptr(),
                                                _stream()), "hamiltonian_mixed")
    return out, projT
