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
    if C.is_conj() or C.is_neg():
        raise ValueError(f"{name} carries a lazy conjugate/negative bit; pass t.resolve_conj()")
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
    beta, C = _plain(beta), _plain(C)
    projT = torch.empty((nk, nb, P), dtype=C.dtype, device=C.device) if projT is None else projT
    lib = _lib.lib()
    ws = workspace(lib.qgb_project_workspace_bytes(_qdtype(C), nk, P, nb, n_tot), C.device)
    _lib.check(lib.qgb_project(_qdtype(C), beta.data_ptr(), C.data_ptr(), projT.data_ptr(), nk, P, nb, n_tot,
                               ws.data_ptr(), ws.numel(), _stream()), "project")
    return projT


def _plain(t: torch.Tensor) -> torch.Tensor:
    """`t` with torch's lazy conjugate / negative bits applied and a dense
    row-major layout: a contiguous tensor can still carry a conjugate bit (the
    conjugate transpose of a column-major matrix is one), and its data pointer
    then holds the unconjugated values."""
    return t.resolve_conj().resolve_neg().contiguous()


def _check_block(X: torch.Tensor, name: str) -> None:
    if X.is_conj() or X.is_neg():
        raise ValueError(f"{name} carries a lazy conjugate/negative bit; pass t.resolve_conj()")
    if not X.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor (no CPU path)")
    if X.dim() != 3 or not X.is_contiguous():
        raise ValueError(f"{name} must be a contiguous (nk, nb, n_tot) tensor")
    _qdtype(X)


def dot(X: torch.Tensor, Y: torch.Tensor, out: torch.Tensor | None = None, tc: bool = False) -> torch.Tensor:
    """out[k, i, j] = sum_g conj(X[k, i, g]) Y[k, j, g] as complex128 (both
    precisions; FP32 inputs are summed in FP32 per basis range, the ranges in FP64).
    tc=True (complex64 only): on the tensor cores as split-BF16x3 GEMMs (qgb_dot_tc)."""
    _check_block(X, "X")
    _check_block(Y, "Y")
    if X.dtype != Y.dtype or X.shape[0] != Y.shape[0] or X.shape[2] != Y.shape[2] or X.device != Y.device:
        raise ValueError(f"dot operands differ: {tuple(X.shape)} {X.dtype} vs {tuple(Y.shape)} {Y.dtype}")
    nk, nx, n_tot = X.shape
    ny = Y.shape[1]
    if out is None:
        out = torch.empty((nk, nx, ny), dtype=torch.complex128, device=X.device)
    elif out.dtype != torch.complex128 or tuple(out.shape) != (nk, nx, ny) or not out.is_contiguous():
        raise ValueError("out must be a contiguous complex128 (nk, nx, ny) tensor")
    if nk == 0 or nx == 0 or ny == 0:
        return out
    lib = _lib.lib()
    qd = _qdtype(X)
    if tc:
        if qd != _lib.QGB_F32:
            raise TypeError("the tensor-core overlap takes complex64 vectors")
        ws = workspace(lib.qgb_dot_tc_workspace_bytes(nk, nx, ny, n_tot), X.device)
        _lib.check(lib.qgb_dot_tc(X.data_ptr(), nx, Y.data_ptr(), ny, nk, n_tot, out.data_ptr(), ws.data_ptr(),
                                  ws.numel(), device_error_word(X.device).data_ptr(), _stream()), "dot_tc")
        return out
    ws = workspace(lib.qgb_dot_workspace_bytes(qd, nk, nx, ny, n_tot), X.device)
    _lib.check(lib.qgb_dot(qd, X.data_ptr(), nx, Y.data_ptr(), ny, nk, n_tot, out.data_ptr(), ws.data_ptr(),
                           ws.numel(), _stream()), "dot")
    return out


def matmul(C: torch.Tensor, M: torch.Tensor, out: torch.Tensor | None = None, accumulate: bool = False,
           tc: bool = False) -> torch.Tensor:
    """out[k, j, g] (+)= sum_i M[k, i, j] C[k, i, g]; M is cast to C's dtype.
    tc=True (complex64 only): one split-BF16x3 tensor-core GEMM (qgb_matmul_tc)."""
    _check_block(C, "C")
    nk, n_in, n_tot = C.shape
    if M.dim() == 2:
        M = M.expand(nk, *M.shape)
    if M.dim() != 3 or M.shape[0] != nk or M.shape[1] != n_in:
        raise ValueError(f"matrix shape {tuple(M.shape)} does not match C {tuple(C.shape)}")
    n_out = M.shape[2]
    Mc = _plain(M.to(device=C.device, dtype=C.dtype))
    if out is None:
        if accumulate:
            raise ValueError("accumulate needs an output tensor")
        out = torch.empty((nk, n_out, n_tot), dtype=C.dtype, device=C.device)
    elif out.dtype != C.dtype or tuple(out.shape) != (nk, n_out, n_tot) or not out.is_contiguous():
        raise ValueError("out must be a contiguous (nk, n_out, n_tot) tensor of C's dtype")
    if nk == 0 or n_out == 0:
        return out
    if n_in == 0:
        if not accumulate:
            out.zero_()
        return out
    flags = _lib.QGB_ACCUMULATE if accumulate else 0
    if tc:
        if C.dtype != torch.complex64:
            raise TypeError("the tensor-core rotation takes complex64 vectors")
        lib = _lib.lib()
        ws = workspace(lib.qgb_matmul_tc_workspace_bytes(nk, n_in, n_out, n_tot), C.device)
        _lib.check(lib.qgb_matmul_tc(C.data_ptr(), n_in, nk, n_tot, Mc.data_ptr(), n_out, out.data_ptr(), flags,
                                     ws.data_ptr(), ws.numel(), device_error_word(C.device).data_ptr(), _stream()),
                   "matmul_tc")
        return out
    _lib.check(_lib.lib().qgb_matmul(_qdtype(C), C.data_ptr(), n_in, nk, n_tot, Mc.data_ptr(), n_out, out.data_ptr(),
                                     flags, _stream()), "matmul")
    return out


def apply_nonlocal(beta: torch.Tensor, D_blocks: torch.Tensor, projT: torch.Tensor, out: torch.Tensor,
                   work: torch.Tensor | None = None) -> torch.Tensor:
    """out += beta D <beta|C> with D given as (n_atoms, pa, pa) blocks."""
    nk, P, n_tot = beta.shape
    n_atoms, pa, _ = D_blocks.shape
    nb = projT.shape[1]
    if n_atoms * pa != P:
        raise ValueError("D blocks do not cover the projectors")
    beta, D_blocks, projT = _plain(beta), _plain(D_blocks), _plain(projT)
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


# ---------------------------------------------------------------------------
# Band-wise Davidson passes
# ---------------------------------------------------------------------------


def band_norm_ke(C: torch.Tensor, ke: torch.Tensor | None = None, b0: int = 0, nb: int | None = None,
                 norm: bool = True, weight: torch.Tensor | None = None):
    """(||C_b||, sum_g |C_bg|^2 KE_g) of bands [b0, b0 + nb) as FP64 (nk, nb)
    tensors in one pass; either is None when not asked for (norm=False / ke None);
    `weight` (FP64 (n_tot,)) weights every |C_bg|^2 (real wavefunctions)."""
    _check_block(C, "C")
    nk, nb_all, n_tot = C.shape
    nb = nb_all - b0 if nb is None else nb
    out_n = torch.empty((nk, nb), dtype=torch.float64, device=C.device) if norm else None
    out_k = torch.empty((nk, nb), dtype=torch.float64, device=C.device) if ke is not None else None
    if ke is not None and (ke.dtype != torch.float64 or tuple(ke.shape) != (nk, n_tot) or not ke.is_contiguous()):
        raise ValueError("ke must be a contiguous float64 (nk, n_tot) tensor")
    _lib.check(_lib.lib().qgb_band_norm_ke(_qdtype(C), C.data_ptr(), nb_all, b0, nb, nk, n_tot,
                                           ke.data_ptr() if ke is not None else None,
                                           _weight_ptr(weight, n_tot),
                                           out_n.data_ptr() if out_n is not None else None,
                                           out_k.data_ptr() if out_k is not None else None, _stream()),
               "band_norm_ke")
    return out_n, out_k


def _weight_ptr(weight: torch.Tensor | None, n_tot: int):
    if weight is None:
        return None
    if weight.dtype != torch.float64 or weight.numel() != n_tot or not weight.is_contiguous() or not weight.is_cuda:
        raise ValueError("weight must be a contiguous float64 CUDA tensor of n_tot entries")
    return weight.data_ptr()


def residual(HC: torch.Tensor, C: torch.Tensor, eig: torch.Tensor, ke: torch.Tensor | None = None,
             KEref: torch.Tensor | None = None, b0: int = 0, out: torch.Tensor | None = None, norm: bool = False,
             weight: torch.Tensor | None = None):
    """R = HC_b - eig_b C_b for bands b0.. of C / HC (eig FP64 (nk, >= nb_all)),
    preconditioned by 1 / (x + exp(-x)), x = KE / KEref_b, when KEref is given;
    stored into `out` (nk, nb, n_tot) if given, its FP64 norms returned if `norm`."""
    _check_block(C, "C")
    _check_block(HC, "HC")
    if HC.shape != C.shape or HC.dtype != C.dtype:
        raise ValueError("HC and C differ in shape or dtype")
    nk, nb_all, n_tot = C.shape
    nb = nb_all - b0
    if eig.dtype != torch.float64 or eig.dim() != 2 or eig.shape[0] != nk or eig.stride(1) != 1:
        raise ValueError("eig must be float64 (nk, n) with unit column stride")
    if KEref is not None:
        if ke is None:
            raise ValueError("preconditioning needs ke")
        KEref = _plain(KEref.to(torch.float64))
    if out is not None:
        if out.dtype != C.dtype or tuple(out.shape) != (nk, nb, n_tot) or not out.is_contiguous():
            raise ValueError("out must be a contiguous (nk, nb, n_tot) tensor of C's dtype")
    nrm = torch.empty((nk, nb), dtype=torch.float64, device=C.device) if norm else None
    _lib.check(_lib.lib().qgb_residual(_qdtype(C), HC.data_ptr(), C.data_ptr(), nb_all, b0, nb, nk, n_tot,
                                       eig.data_ptr(), eig.stride(0), ke.data_ptr() if ke is not None else None,
                                       KEref.data_ptr() if KEref is not None else None,
                                       _weight_ptr(weight, n_tot),
                                       out.data_ptr() if out is not None else None,
                                       nrm.data_ptr() if nrm is not None else None, _stream()), "residual")
    return nrm


def normalize_bands(X: torch.Tensor, n_dev: torch.Tensor, norm: torch.Tensor, norm_cut: float, seed: int,
                    n_max: int, ke: torch.Tensor) -> None:
    """In place: bands of X with norm < norm_cut re-randomised (the reference's
    seeded generator; their norm set to 1), the others divided by their norm;
    padding zeroed.  n_dev: int32 (nk,) sphere sizes on the device."""
    _check_block(X, "X")
    nk, nb, n_tot = X.shape
    if norm.dtype != torch.float64 or tuple(norm.shape) != (nk, nb) or not norm.is_contiguous():
        raise ValueError("norm must be a contiguous float64 (nk, nb) tensor")
    if n_dev.dtype != torch.int32 or n_dev.numel() != nk:
        raise ValueError("n_dev must be int32 (nk,)")
    _lib.check(_lib.lib().qgb_normalize_bands(_qdtype(X), X.data_ptr(), nb, nk, n_tot, n_dev.data_ptr(),
                                              norm.data_ptr(), float(norm_cut), int(seed), int(n_max),
                                              ke.data_ptr(), _stream()), "normalize_bands")


# ---------------------------------------------------------------------------
# Real (Gamma-point) wavefunctions on the half basis
# ---------------------------------------------------------------------------


def _check_real(rb, C: torch.Tensor, name: str = "C") -> int:
    _check_block(C, name)
    if C.dtype != rb.cdtype or C.shape[0] != 1 or C.shape[2] != rb.n_tot:
        raise ValueError(f"{name} {tuple(C.shape)} {C.dtype} is not (1, nb, {rb.n_tot}) {rb.cdtype}")
    return C.shape[1]


def hamiltonian_real(rb, C: torch.Tensor, beta: torch.Tensor | None, D_blocks: torch.Tensor | None,
                     out: torch.Tensor | None = None, projT: torch.Tensor | None = None,
                     ws: torch.Tensor | None = None):
    """(HC, projT) of real wavefunctions C (1, nb, n_tot_half) on the
    ``DeviceRealBasis`` rb: HC = KE C + V C + beta D <beta|C> with the
    weighted real projections (one C-ABI call)."""
    nb = _check_real(rb, C)
    out = torch.empty_like(C) if out is None else out
    _check_real(rb, out, "out")
    if beta is None or beta.shape[1] == 0:
        n_atoms, pa, P = 0, 0, 0
        bptr = dptr = pptr = 0
    else:
        _check_real(rb, beta, "beta")
        n_atoms, pa, _ = D_blocks.shape
        P = beta.shape[1]
        if D_blocks.dtype != C.dtype or not D_blocks.is_contiguous() or n_atoms * pa != P:
            raise ValueError("D_blocks must be contiguous (n_atoms, pa, pa) of C's dtype with n_atoms * pa = P")
        projT = torch.empty((1, nb, P), dtype=C.dtype, device=C.device) if projT is None else projT
        bptr, dptr, pptr = beta.data_ptr(), D_blocks.data_ptr(), projT.data_ptr()
    if ws is None:
        ws = workspace(rb.workspace_bytes(nb, P), C.device)
    _lib.check(_lib.lib().qgb_hamiltonian_real(ct.byref(rb.sphere.struct), ct.byref(rb.struct), rb.qdtype,
                                               C.data_ptr(), out.data_ptr(), nb, bptr, dptr, n_atoms, pa, pptr,
                                               ws.data_ptr(), ws.numel(), _stream()), "hamiltonian_real")
    return out, projT


def hamiltonian_real_mixed(rb, C: torch.Tensor, split: torch.Tensor | None, D_blocks: torch.Tensor | None,
                           out: torch.Tensor | None = None, projT: torch.Tensor | None = None,
                           ws: torch.Tensor | None = None):
    """(HC, projT) of real wavefunctions in the mixed form (complex64): FP32
    local potential, weighted real projection and back-projection as tcgen05
    split-BF16x3 GEMMs on ``beta_split`` operands of the half-basis beta."""
    nb = _check_real(rb, C)
    if C.dtype != torch.complex64:
        raise TypeError("the mixed real form is complex64")
    out = torch.empty_like(C) if out is None else out
    _check_real(rb, out, "out")
    if split is None:
        n_atoms, pa, P = 0, 0, 0
        sptr = dptr = pptr = 0
    else:
        n_atoms, pa, _ = D_blocks.shape
        P = n_atoms * pa
        if D_blocks.dtype != torch.complex64 or not D_blocks.is_contiguous():
            raise ValueError("D_blocks must be contiguous complex64 (n_atoms, pa, pa)")
        projT = torch.empty((1, nb, P), dtype=C.dtype, device=C.device) if projT is None else projT
        sptr, dptr, pptr = split.data_ptr(), D_blocks.data_ptr(), projT.data_ptr()
    lib = _lib.lib()
    if ws is None:
        ws = workspace(lib.qgb_hamiltonian_real_mixed_workspace_bytes(ct.byref(rb.sphere.struct), ct.byref(rb.struct),
                                                                      nb, P), C.device)
    err = device_error_word(C.device)
    _lib.check(lib.qgb_hamiltonian_real_mixed(ct.byref(rb.sphere.struct), ct.byref(rb.struct), C.data_ptr(),
                                              out.data_ptr(), nb, sptr, dptr, n_atoms, pa, pptr, ws.data_ptr(),
                                              ws.numel(), err.data_ptr(), _stream()), "hamiltonian_real_mixed")
    return out, projT


def dot_real(X: torch.Tensor, Y: torch.Tensor, weight: torch.Tensor, out: torch.Tensor | None = None):
    """out[0, i, j] = Re sum_g w_g conj(X[0, i, g]) Y[0, j, g] as complex128
    (imaginary part 0): the overlap of real wavefunctions on the half basis."""
    _check_block(X, "X")
    _check_block(Y, "Y")
    if X.dtype != Y.dtype or X.shape[0] != 1 or Y.shape[0] != 1 or X.shape[2] != Y.shape[2]:
        raise ValueError(f"dot_real operands differ: {tuple(X.shape)} {X.dtype} vs {tuple(Y.shape)} {Y.dtype}")
    _, nx, n_tot = X.shape
    ny = Y.shape[1]
    if out is None:
        out = torch.empty((1, nx, ny), dtype=torch.complex128, device=X.device)
    elif out.dtype != torch.complex128 or tuple(out.shape) != (1, nx, ny) or not out.is_contiguous():
        raise ValueError("out must be a contiguous complex128 (1, nx, ny) tensor")
    lib = _lib.lib()
    ws = workspace(lib.qgb_dot_workspace_bytes(_qdtype(X), 1, nx, ny, n_tot), X.device)
    _lib.check(lib.qgb_dot_real(_qdtype(X), X.data_ptr(), nx, Y.data_ptr(), ny, n_tot, _weight_ptr(weight, n_tot),
                                out.data_ptr(), ws.data_ptr(), ws.numel(), _stream()), "dot_real")
    return out


def symmetrize_real(rb, X: torch.Tensor) -> torch.Tensor:
    """In place: the Gz = 0 plane of X made Hermitian, c(G) = (c(G) + conj(c(-G))) / 2."""
    nb = _check_real(rb, X, "X")
    _lib.check(_lib.lib().qgb_symmetrize_real(rb.qdtype, ct.byref(rb.struct), X.data_ptr(), nb, _stream()),
               "symmetrize_real")
    return X


# ---------------------------------------------------------------------------
# Projectors generated on the device
# ---------------------------------------------------------------------------


def make_projectors(iG, k, Gbasis, n, positions, shells, volume: float, dtype: torch.dtype, device) -> torch.Tensor:
    """beta (nk, n_atoms pa, n_tot) of `dtype` on `device` (qgb_make_projectors,
    replacing Ions.get_projectors): iG (nk, n_tot, 3) integer, k (nk, 3) and
    positions (n_atoms, 3) fractional, n (nk,) sphere sizes; shells a list of
    (l, ("gauss", sigma)) or (l, ("blip", coeff, dq)) with coeff the radial
    function's blip coefficients (1D, FP64) on |q| spacing dq."""
    dev = torch.device(device)
    iG_d = torch.as_tensor(iG).to(dev, torch.int32).contiguous()
    nk, n_tot = int(iG_d.shape[0]), int(iG_d.shape[1])
    if iG_d.dim() != 3 or iG_d.shape[2] != 3:
        raise ValueError("iG must be (nk, n_tot, 3)")
    k_d = torch.as_tensor(k, dtype=torch.float64).to(dev).reshape(nk, 3).contiguous()
    n_d = torch.as_tensor(n).to(dev, torch.int32).reshape(nk).contiguous()
    pos_d = torch.as_tensor(positions, dtype=torch.float64).to(dev).reshape(-1, 3).contiguous()
    arr = (_lib.QgbProjectorShell * max(len(shells), 1))()
    keep = []
    for s, (l, (kind, *par)) in enumerate(shells):
        arr[s].l = int(l)
        if kind == "gauss":
            arr[s].kind, arr[s].sigma = _lib.QGB_RADIAL_GAUSSIAN, float(par[0])
        elif kind == "blip":
            c = torch.as_tensor(par[0], dtype=torch.float64).to(dev).contiguous()
            keep.append(c)
            arr[s].kind, arr[s].coeff, arr[s].n_coeff, arr[s].dq = _lib.QGB_RADIAL_BLIP, c.data_ptr(), c.numel(), \
                float(par[1])
        else:
            raise ValueError(f"unknown radial kind {kind!r}")
    pa = sum(2 * int(l) + 1 for l, _ in shells)
    beta = torch.empty((nk, pos_d.shape[0] * pa, n_tot), dtype=dtype, device=dev)
    Gb = (ct.c_double * 9)(*[float(x) for x in torch.as_tensor(Gbasis, dtype=torch.float64).reshape(-1)])
    with torch.cuda.device(dev):
        _lib.check(_lib.lib().qgb_make_projectors(_qdtype(beta), nk, n_tot, n_d.data_ptr(), iG_d.data_ptr(),
                                                  k_d.data_ptr(), Gb, pos_d.shape[0], pos_d.data_ptr(), len(shells),
                                                  arr, float(volume), beta.data_ptr(), _stream()),
                   "make_projectors")
    return beta
