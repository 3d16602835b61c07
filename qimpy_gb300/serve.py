"""Continuous-batching eigensolve server on one GPU.

Requests (a cell spec and a band count) arrive over time.  The server admits a
queued request as soon as a slot and its HBM budget are free, keeps the
request's wavefunctions, potential and projectors resident until it is done,
and runs every active request's Davidson (the reference's algorithm,
qimpy/dft/electrons/_davidson.py:141-235, stepped as a generator) in lock
step: each server tick gathers the block every active request needs H applied
to and runs them all as one batched H.psi (local potential in three launches
per grid shape, nonlocal per request), then advances each request.  Requests
that arrive while others are on the GPU join at the next tick, so their work
overlaps on the device.  A mixed-precision request finishes with FP64
refinement sweeps.  A request that fails (bad size, non-finite result,
iteration limit) is reported with its error and leaves the others untouched.
"""
from __future__ import annotations

import ctypes as ct
import math
import time
import traceback
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _lib, ops
from .batch import Instance, InstanceSpec
from .davidson import Davidson, refine_fp64
from .electrons import Wavefunction


@dataclass
class EigenRequest:
    """One eigensolve: lowest `n_bands` eigenpairs of the cell in `spec`."""

    rid: int
    spec: InstanceSpec
    n_bands: int
    arrival: float = 0.0  #: seconds after the stream starts
    status: str = "queued"  #: queued, active, done, failed, rejected
    eig: Optional[np.ndarray] = None  #: (nk, n_bands) FP64
    error: str = ""
    t_admit: float = math.nan
    t_done: float = math.nan
    iterations: int = 0
    hpsi_bands: int = 0
    converged: bool = False
    residual: float = math.nan
    t_solved: float = math.nan  #: the batched Davidson finished (refinement and checks follow)
    refine_sweeps: int = 0  #: FP64 refinement sweeps of a mixed solve

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


@dataclass
class _Active:
    req: EigenRequest
    inst: Instance
    el: object
    gen: object
    block: Wavefunction
    planes: torch.Tensor
    nbytes: int
    sphere_dev: torch.Tensor
    stream: torch.cuda.Stream
    ready: torch.cuda.Event  #: recorded on `stream` after the request's last step
    stats: object = None  #: DavidsonStats once the mixed/FP64 solve has finished


class EigenServer:
    """Continuous batching of Davidson eigensolves (see the module docstring)."""

    def __init__(self, device="cuda", precision: str = "mixed", hbm_budget_bytes: int = 160 << 30,
                 max_active: int = 64, eig_threshold: float = 1e-6, residual_threshold: Optional[float] = None,
                 max_iterations: int = 200, refine: bool = True, refine_threshold: Optional[float] = None,
                 workers: int = 16, real_gamma: bool = True):
        """eig_threshold: Davidson's stop on the largest eigenvalue change (Ha);
        refine_threshold: the same for the FP64 refinement of a mixed solve
        (default eig_threshold / 10); a refinement that ends
        above it but within eig_threshold still completes the request;
        residual_threshold: optional extra stop on the FP64 residual norm
        (FP64 solve, or the refinement).  Every finished request reports its
        final residual.  real_gamma: Gamma-only requests use real wavefunctions
        on the half basis (qimpy/dft/electrons/_basis_real.py); their H.psi runs
        per request rather than in the batched launches."""
        if precision not in ("mixed", "fp64"):
            raise ValueError("precision must be 'mixed' or 'fp64'")
        self.device = torch.device(device)
        self.precision = precision
        self.dtype = torch.complex64 if precision == "mixed" else torch.complex128
        self.qdtype = _lib.QGB_F32 if precision == "mixed" else _lib.QGB_F64
        self.budget = int(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.eig_threshold = eig_threshold
        self.residual_threshold = residual_threshold
        self.max_iterations = max_iterations
        self.refine = refine and precision == "mixed"
        self.refine_threshold = refine_threshold if refine_threshold is not None else eig_threshold / 10
        self.real_gamma = real_gamma
        self.queue: list = []
        self.active: list = []
        self.finished: list = []
        self.in_use = 0
        self.ticks = 0
        self.tick_band_apps: list = []
        # Request steps (Davidson host logic, cuSOLVER subspace algebra, FP64
        # refinement) run concurrently in worker threads, each request on its own
        # CUDA stream; the batched H.psi runs on the server's stream.
        self.workers = workers
        self._pool = ThreadPoolExecutor(max_workers=workers)
        # Finished solves (FP64 refinement, final residual) complete beside the
        # next ticks on a pool of their own.
        self._finisher = ThreadPoolExecutor(max_workers=max(1, workers // 2))
        self._completing: list = []
        self._warm_up()
        self.tick_wall: list = []  #: host seconds per tick
        self._hpsi_events: list = []  #: (start, end) CUDA events around each batched H.psi

    def close(self) -> None:
        """Stop the worker pools (after finishing what they run)."""
        self._pool.shutdown(wait=True)
        self._finisher.shutdown(wait=True)

    def __enter__(self) -> "EigenServer":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def _warm_up(self) -> None:
        """Load the extension and torch's lazily loaded linear-algebra backends
        once on this thread: their first use from several worker threads at
        once races inside torch."""
        _lib.lib()
        x = torch.eye(2, dtype=torch.complex128, device=self.device)[None] * 2.0
        L, _ = torch.linalg.cholesky_ex(x)
        torch.linalg.solve_triangular(L, x, upper=False)
        torch.linalg.cholesky(x)
        torch.cuda.synchronize(self.device)

    # ------------------------------------------------------------------ admission
    def estimate_bytes(self, spec: InstanceSpec, n_bands: int) -> int:
        """HBM held by an active request: wavefunction-sized Davidson arrays, the
        slab planes of one block, projectors (and their bf16 operands), V, tables."""
        N = spec.grid
        nk = len(spec.k)
        n_est = (2.0 * spec.ke_cutoff) ** 1.5 * spec.side ** 3 / (6 * math.pi ** 2) * 1.1
        nbt = n_bands + self.bands_extra(n_bands, int(n_est))
        elem = 8 if self.dtype == torch.complex64 else 16
        wf = 12 * nk * nbt * n_est * elem
        planes = nk * nbt * (N // 2 + 2) * N * N * elem
        P = 4 * spec.n_atoms
        proj = nk * P * n_est * (elem + (8 if self.dtype == torch.complex64 else 0))
        return int(wf + planes + proj + 4 * N ** 3 * 8)

    def submit(self, req: EigenRequest) -> None:
        self.queue.append(req)
        self.queue.sort(key=lambda r: r.arrival)

    def _admit(self, horizon: float, now: float) -> None:
        """Admit queued requests that arrived by `horizon` while slots and memory
        allow; their set-up (cell data, start vectors, first Davidson step) runs
        in the worker pool."""
        admitted = []
        while self.queue and self.queue[0].arrival <= horizon and len(self.active) + len(admitted) < self.max_active:
            req = self.queue[0]
            need = self.estimate_bytes(req.spec, req.n_bands)
            if need > self.budget:
                self.queue.pop(0)
                self._reject(req, f"needs {need / 2**30:.1f} GiB > budget {self.budget / 2**30:.1f} GiB", now)
                continue
            if self.in_use + need > self.budget and (self.active or admitted or self._completing):
                break  # wait for memory to free up
            self.queue.pop(0)
            self.in_use += need
            admitted.append((req, need))
        main = torch.cuda.current_stream()
        for req, need, result in zip([a[0] for a in admitted], [a[1] for a in admitted],
                                     self._pool.map(lambda rn: self._setup(rn[0], main), admitted)):
            if isinstance(result, Exception):
                self.in_use -= need
                self._reject(req, str(result), now)
                continue
            inst, el, gen, block, planes, sd, stream, ready = result
            req.status, req.t_admit = "active", now
            self.active.append(_Active(req, inst, el, gen, block, planes, need, sd, stream, ready))

    def _setup(self, req: EigenRequest, main: torch.cuda.Stream):
        stream = torch.cuda.Stream(device=self.device)
        stream.wait_stream(main)
        try:
            with torch.cuda.stream(stream):
                inst = Instance(req.spec, self.device, dtype=self.dtype, real=self._real(req.spec))
                n_min = int(inst.layout.n.min())
                extra = self.bands_extra(req.n_bands, n_min)
                nbt = req.n_bands + extra
                if req.n_bands < 1 or 2 * nbt >= n_min:  # Davidson's own limit (_davidson.py:159-163)
                    raise ValueError(f"n_bands + n_bands_extra = {nbt} exceeds min(n_basis)/2 = {n_min // 2}")
                el = inst.electrons(req.n_bands, extra)
                precision_is_mixed = self.dtype == torch.complex64
                dav = Davidson(el, n_iterations=self.max_iterations, eig_threshold=self.eig_threshold,
                               residual_threshold=None if precision_is_mixed else self.residual_threshold)
                gen = dav.steps()
                block = next(gen)
                planes = torch.empty(inst.sphere.workspace_bytes(el.C.n_bands(), budget=1 << 62)
                                     if inst.real_basis is None else 1, dtype=torch.uint8, device=self.device)
                sd = torch.frombuffer(bytearray(bytes(inst.sphere.struct)), dtype=torch.uint8).to(self.device)
                ready = torch.cuda.Event()
                ready.record(stream)
            return inst, el, gen, block, planes, sd, stream, ready
        except (ValueError, RuntimeError, torch.cuda.OutOfMemoryError) as e:
            return e

    def _real(self, spec: InstanceSpec) -> bool:
        return self.real_gamma and spec.k.shape[0] == 1 and not np.any(spec.k != 0.0)

    def bands_extra(self, n_bands: int, n_min: int) -> int:
        """Bands kept beyond the requested ones.  Without a residual target this
        is the reference's default max(1, ceil(0.1 n_bands))
        (qimpy/dft/electrons/_fillings.py:236-243).  With one, at least 4 and
        ceil(0.25 n_bands): the residual of the highest requested band falls
        at a rate set by the gap to the first band above the kept block, and a
        single extra band leaves that gap small on many cells (residual 1e-4
        after 200 iterations on a 2-k cell, against 5e-7 after 30 with 4
        extra).  Capped by Davidson's limit 2 (n_bands + extra) < n_min."""
        base = max(1, math.ceil(0.1 * n_bands))
        if self.residual_threshold is None:
            return base
        want = max(base, 4, math.ceil(0.25 * n_bands))
        return max(base, min(want, (n_min - 1) // 2 - n_bands))

    def _reject(self, req: EigenRequest, why: str, now: float) -> None:
        req.status, req.error, req.t_done = "rejected", why, now
        self.finished.append(req)

    # ------------------------------------------------------------------ batched H.psi
    def _batched_hamiltonian(self, acts: list) -> list:
        """H applied to every active request's pending block: the local potential
        of all requests sharing a grid shape in three batched launches, then each
        request's nonlocal term."""
        lib = _lib.lib()
        real = [i for i, a in enumerate(acts) if a.inst.real_basis is not None]
        if real:  # real-wavefunction requests: their own H.psi calls
            outs_real = {i: acts[i].el.hamiltonian(acts[i].block) for i in real}
            rest = [a for a in acts if a.inst.real_basis is None]
            outs_rest = iter(self._batched_hamiltonian(rest)) if rest else iter(())
            return [outs_real[i] if i in outs_real else next(outs_rest) for i in range(len(acts))]
        for a in acts:  # the kernels read every block with the server's element type
            c = a.block.coeff
            if c.dtype != self.dtype or not c.is_contiguous() or c.shape[0] != a.inst.nk or c.shape[2] != a.inst.n_tot:
                raise TypeError(f"request {a.req.rid}: block {tuple(c.shape)} {c.dtype} does not match its sphere")
            if c.shape[1] * a.inst.sphere.workspace_bytes(1, budget=1 << 62) > a.planes.numel():
                raise ValueError(f"request {a.req.rid}: block of {c.shape[1]} bands exceeds its plane workspace")
        outs = [torch.empty_like(a.block.coeff) for a in acts]
        groups: dict = {}
        for i, a in enumerate(acts):
            groups.setdefault(a.inst.tables.shape, []).append(i)
        st = torch.cuda.current_stream().cuda_stream
        for idx in groups.values():
            items = (_lib.QgbBatchItem * len(idx))()
            slab_units, row_units, smem, smem_yz = [0], [0], 0, 0
            for j, i in enumerate(idx):
                a = acts[i]
                t = a.inst.tables
                nb = a.block.n_bands()
                items[j].sphere = a.sphere_dev.data_ptr()
                items[j].C = a.block.coeff.data_ptr()
                items[j].out = outs[i].data_ptr()
                items[j].planes = a.planes.data_ptr()
                items[j].nb = nb
                items[j].flags = _lib.QGB_ADD_KE
                slab_units.append(slab_units[-1] + t.nk * nb * t.max_slabs)
                row_units.append(row_units[-1] + t.nk * nb * t.shape[1])
                smem = max(smem, int(lib.qgb_sphere_smem_bytes(ct.byref(a.inst.sphere.struct), self.qdtype)))
                smem_yz = max(smem_yz, int(lib.qgb_sphere_smem_bytes_yz(ct.byref(a.inst.sphere.struct), self.qdtype)))
            ids = np.arange(len(idx), dtype=np.int32)
            dev_items = torch.frombuffer(bytearray(bytes(items)), dtype=torch.uint8).to(self.device)
            starts_s = torch.tensor(slab_units, dtype=torch.int64, device=self.device)
            starts_r = torch.tensor(row_units, dtype=torch.int64, device=self.device)
            item_s = torch.from_numpy(np.repeat(ids, np.diff(slab_units))).to(self.device)
            item_r = torch.from_numpy(np.repeat(ids, np.diff(row_units))).to(self.device)
            _lib.check(lib.qgb_apply_potential_batched(dev_items.data_ptr(), len(idx), item_s.data_ptr(),
                                                       starts_s.data_ptr(), item_r.data_ptr(), starts_r.data_ptr(),
                                                       slab_units[-1], row_units[-1], self.qdtype, smem_yz, smem, st),
                       "apply_potential_batched")
            for i in idx:
                a, C = acts[i], acts[i].block.coeff
                ions = a.el.ions
                if self.dtype == torch.complex64:
                    ops.apply_nonlocal_tc(ions.beta_split, ions.D, C, outs[i])
                else:
                    projT = ops.project(ions.beta, C)
                    ops.apply_nonlocal(ions.beta, ions.D, projT, outs[i])
        return [Wavefunction(a.el.basis, coeff=o) for a, o in zip(acts, outs)]

    # ------------------------------------------------------------------ main loop
    def tick(self, now_fn) -> None:
        if not self.active:
            return
        t0 = time.perf_counter()
        acts = list(self.active)
        main = torch.cuda.current_stream()
        for a in acts:  # blocks were produced on the requests' streams
            main.wait_event(a.ready)
            a.block.coeff.record_stream(main)
        start_hpsi = torch.cuda.Event(enable_timing=True)
        start_hpsi.record(main)
        results = self._batched_hamiltonian(acts)
        done_hpsi = torch.cuda.Event(enable_timing=True)
        done_hpsi.record(main)
        self._hpsi_events.append((start_hpsi, done_hpsi))
        self.ticks += 1
        self.tick_band_apps.append(sum(a.block.n_bands() * a.inst.nk for a in acts))
        outcome = list(self._pool.map(lambda ar: self._advance(ar[0], ar[1], done_hpsi, now_fn), zip(acts, results)))
        for a, (kind, payload) in zip(acts, outcome):
            if kind == "finished":  # refinement and checks run beside the next ticks
                self.active.remove(a)
                self._completing.append((a, self._finisher.submit(self._complete, a, payload, now_fn)))
            elif kind == "failed":
                self._fail(a, payload, now_fn())
        self.tick_wall.append(time.perf_counter() - t0)

    def _reap(self, wait: bool = False) -> None:
        """Release the memory of requests whose completion has finished."""
        keep = []
        for a, fut in self._completing:
            if wait or fut.done():
                fut.result()
                a.stream.synchronize()
                self.in_use -= a.nbytes
                self.finished.append(a.req)
            else:
                keep.append((a, fut))
        self._completing = keep

    def _advance(self, a: _Active, HC: Wavefunction, done_hpsi, now_fn):
        """One step of a request on its own stream (worker thread)."""
        try:
            with torch.cuda.stream(a.stream):
                a.stream.wait_event(done_hpsi)
                HC.coeff.record_stream(a.stream)
                try:
                    a.block = a.gen.send(HC)
                except StopIteration as stop:
                    return ("finished", stop.value)
                a.ready.record(a.stream)
            return ("continue", None)
        except (ValueError, RuntimeError, TypeError) as e:  # e.g. a non positive-definite overlap
            return ("failed", _describe(e))

    def _complete(self, a: _Active, stats, now_fn) -> None:
        """Finish a request (finisher thread, on the request's stream): FP64
        refinement of a mixed solve, the final residual
        max_b ||H psi_b - eps_b psi_b|| (one more H.psi), result checks, latency."""
        req = a.req
        req.t_solved = now_fn()
        try:
            with torch.cuda.stream(a.stream):
                self._finish_solve(a, stats)
        except (ValueError, RuntimeError) as e:
            req.status, req.error = "failed", _describe(e)
        req.t_done = now_fn()

    def _finish_solve(self, a: _Active, stats) -> None:
        req, el = a.req, a.el
        converged, iterations, why = bool(stats.converged), stats.iterations, ""
        if not converged:
            why = f"not converged in {stats.iterations} iterations (deig_max {stats.deig_max:.2e})"
        if self.refine:
            # A mixed solve that stopped at FP32's floor (stalled) is finished
            # by the FP64 sweeps.
            inst64 = Instance(req.spec, self.device, dtype=torch.complex128, real=a.inst.real_basis is not None)
            el64 = inst64.electrons(req.n_bands, el.n_bands_extra)
            refine_fp64(el, el64, eig_threshold=self.refine_threshold, residual_threshold=self.residual_threshold,
                        max_sweeps=max(40, self.max_iterations - stats.iterations))
            ref = el64.last_refine
            req.refine_sweeps = ref.iterations
            req.hpsi_bands += ref.hpsi_bands
            iterations += ref.iterations
            converged = (converged or stats.stalled) and (ref.converged or ref.deig_max <= self.eig_threshold)
            if not converged:
                why = why or f"FP64 refinement not converged in {ref.iterations} sweeps (deig_max {ref.deig_max:.2e})"
            el = el64
        HC = el.hamiltonian(el.C)
        res = ops.residual(HC.coeff, el.C.coeff, el.eig.contiguous(), norm=True, weight=el.basis.weight)
        req.residual = float(res[:, : req.n_bands].max())
        if converged and self.residual_threshold is not None and not req.residual < self.residual_threshold:
            converged = False
            why = f"residual {req.residual:.2e} above the target {self.residual_threshold:.0e}"
        eig = el.eig[:, : req.n_bands].detach().cpu().numpy()
        if not np.all(np.isfinite(eig)):
            raise RuntimeError("non-finite eigenvalues")
        req.eig, req.iterations, req.converged = eig, iterations, converged
        req.hpsi_bands += stats.hpsi_bands + el.C.n_bands() * el.basis.nk
        req.status = "done" if converged else "failed"
        req.error = "" if converged else why

    def _fail(self, a: _Active, why: str, now: float) -> None:
        a.req.status, a.req.error, a.req.t_done = "failed", why, now
        self._release(a)

    def _release(self, a: _Active) -> None:
        a.stream.synchronize()
        self.active.remove(a)
        self.in_use -= a.nbytes
        self.finished.append(a.req)

    def run(self, requests: list, realtime: bool = True, max_wall_s: float = 3600.0) -> dict:
        """Serve `requests` (arrival times in seconds from now) to completion.

        realtime=True follows the wall clock (a request is admitted only once its
        arrival time has passed); realtime=False admits requests in arrival order
        as soon as slots and memory allow."""
        for r in requests:
            self.submit(r)
        t0 = time.perf_counter()

        def now() -> float:
            return time.perf_counter() - t0

        while self.queue or self.active or self._completing:
            self._reap()
            t = now()
            self._admit(t if realtime else math.inf, t)
            if not self.active:
                if not self.queue and not self._completing:
                    break
                wait = (self.queue[0].arrival - now()) if self.queue else 0.0
                time.sleep(min(max(wait, 0.001), 0.01))  # next arrival, or memory held by finishing requests
                continue
            self.tick(now)
            if now() > max_wall_s:
                for a in list(self.active):
                    self._fail(a, "server time limit", now())
                for r in self.queue:
                    self._reject(r, "server time limit", now())
                self.queue.clear()
        self._reap(wait=True)
        return self.report(now())

    def report(self, wall: float) -> dict:
        done = [r for r in self.finished if r.status == "done"]
        lat = np.array([r.latency for r in done]) if done else np.array([math.nan])
        first = min((r.arrival for r in self.finished), default=0.0)
        last = max((r.t_done for r in done), default=first)
        return dict(requests=len(self.finished), done=len(done),
                    failed=sum(r.status == "failed" for r in self.finished),
                    rejected=sum(r.status == "rejected" for r in self.finished),
                    eigensolves_per_s=len(done) / max(last - first, 1e-9), wall_s=wall,
                    p50_latency_s=float(np.percentile(lat, 50)), p99_latency_s=float(np.percentile(lat, 99)),
                    ticks=self.ticks, mean_band_apps_per_tick=float(np.mean(self.tick_band_apps)) if self.ticks else 0.0,
                    hpsi_band_apps=int(sum(r.hpsi_bands for r in done)),
                    tick_wall_s=float(sum(self.tick_wall)),
                    errors=[f"{r.rid}: {r.error[:160]}" for r in self.finished if r.status != "done"][:8],
                    hpsi_gpu_s=self.hpsi_gpu_seconds())

    def hpsi_gpu_seconds(self) -> float:
        """Device time of the batched H.psi launches (CUDA events on the server's
        stream; the start event may also wait for the requests' blocks)."""
        torch.cuda.synchronize(self.device)
        return float(sum(a.elapsed_time(b) for a, b in self._hpsi_events)) * 1e-3


def _describe(e: Exception) -> str:
    """Error text with the innermost source location it came from."""
    tb = traceback.extract_tb(e.__traceback__)
    where = f" [{tb[-1].filename.rsplit('/', 1)[-1]}:{tb[-1].lineno} {tb[-1].name}]" if tb else ""
    return f"{type(e).__name__}: {e}{where}"


def poisson_stream(specs: list, rate_hz: float, seed: int, bands_choices=(8, 16, 32, 64, 96, 128, 160)) -> list:
    """Requests with exponential inter-arrival times (mean 1/rate) over `specs`;
    each asks for a band count drawn from bands_choices (capped so that
    2 (n_bands + extra) stays below the basis size)."""
    from .workloads import splitmix_uniform

    u = splitmix_uniform(seed, 77, 2 * len(specs))
    t, reqs = 0.0, []
    for i, spec in enumerate(specs):
        t += -math.log(u[2 * i]) / rate_hz
        nb = bands_choices[int(u[2 * i + 1] * len(bands_choices)) % len(bands_choices)]
        n_est = (2.0 * spec.ke_cutoff) ** 1.5 * spec.side ** 3 / (6 * math.pi ** 2)
        nb = int(min(nb, max(4, 0.3 * n_est)))
        reqs.append(EigenRequest(i, spec, nb, arrival=t))
    return reqs
