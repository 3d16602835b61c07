"""Autotuner for the FFT radix schedule of the local-potential kernels.

For a grid shape and precision, every axis has a few valid factorisations
N = L1 * L2 into codelet sizes; the choice changes register pressure, pass
count and twiddle work of the three kernels.  `tune_shape` times the
candidates axis by axis on a representative G-sphere (cubic cell sized so the
grid follows the reference's rule for Ecut 20 Ha) and keeps the fastest;
results are cached per (shape, dtype) in a JSON file so later runs reuse them.
"""
from __future__ import annotations

import json
import math
import os
import threading

import numpy as np
import torch

from . import ops
from . import sphere as sp
from . import workloads as wl

CACHE = os.environ.get("QGB_AUTOTUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "qimpy_gb300", "autotune.json"))
_lock = threading.Lock()
_memo: dict = {}


def candidates(N: int) -> list:
    """All (L1, L2) with L1 * L2 = N, both codelet sizes."""
    out = []
    for L1 in sp.CODELET_SIZES:
        if N % L1 == 0 and (N // L1) in sp.CODELET_SIZES:
            out.append((L1, N // L1))
    return out


def _key(shape, dtype) -> str:
    return f"{shape[0]}x{shape[1]}x{shape[2]}:{'c64' if dtype == torch.complex64 else 'c128'}"


def _load() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table: dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, CACHE)
    except OSError:
        pass  # read-only home: keep the in-memory result


def _time_apply(ds, C, ws, reps: int) -> float:
    st = torch.cuda.current_stream()
    ops.apply_potential(ds, C, add_ke=True, ws=ws)  # warm-up (and module load)
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ops.apply_potential(ds, C, add_ke=True, ws=ws)
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.median(times))


def tune_shape(shape, dtype=torch.complex64, device="cuda", nb: int = 8, reps: int = 3, use_cache: bool = True):
    """Best per-axis factorisation for `shape`: ((L1, L2) x 3)."""
    shape = tuple(int(x) for x in shape)
    key = _key(shape, dtype)
    with _lock:
        if key in _memo:
            return _memo[key]
        if use_cache:
            table = _load()
            if key in table:
                _memo[key] = tuple(tuple(f) for f in table[key]["fac"])
                return _memo[key]
    # Representative sphere: cubic cell whose reference grid for Ecut 20 Ha is ~shape.
    L = shape[0] * math.pi / (2.0 * math.sqrt(40.0))
    R = np.diag([L * shape[0] / shape[0], L * shape[1] / shape[0], L * shape[2] / shape[0]])
    Gb = 2.0 * np.pi * np.linalg.inv(R.T)
    lay = wl.make_basis(Gb, np.zeros((1, 3)), 20.0, shape)
    tables = sp.build_tables(lay.fft_index, lay.n, shape)
    ds = sp.DeviceSphere(tables, lay.ke, device, dtype)
    g = torch.Generator(device="cpu").manual_seed(7)
    ds.set_potential(torch.randn(shape, generator=g, dtype=torch.float64))
    C = (torch.randn((1, nb, lay.n_tot), generator=g, dtype=torch.float64) + 0j).to(device, dtype)
    for k_ in range(1):
        C[k_, :, int(lay.n[k_]):] = 0
    ws = ops.workspace(ds.workspace_bytes(nb), device)
    best = [tuple(f) for f in tables.fac]
    timings = {}
    for a in range(3):
        best_t = None
        for cand in candidates(shape[a]):
            fac = list(best)
            fac[a] = cand
            ds.set_factors(fac)
            t = _time_apply(ds, C, ws, reps)
            timings[f"{a}:{cand[0]}x{cand[1]}"] = t
            if best_t is None or t < best_t:
                best_t, best[a] = t, cand
    result = tuple(best)
    with _lock:
        _memo[key] = result
        table = _load()
        table[key] = {"fac": [list(f) for f in result], "ms": timings, "nb": nb}
        _store(table)
    return result
