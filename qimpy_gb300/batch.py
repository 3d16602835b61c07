"""Batched H.psi over many independent problems with uneven grids and bases.

A batch holds independent problems ("instances": a cell with its own k-points,
bands, cutoff and FFT grid), all resident on one GPU.  One batched H.psi runs
the local potential of every instance's band block in three launches (one per
transform phase, work units mapped to CTAs through prefix sums over the
instances) and the tensor-core nonlocal term per instance; the whole
application is captured once in a CUDA graph and replayed.

Instance inputs (V(r), projectors, start vectors) are generated on the device
from seeded specs, because the biggest cells have 100^3 grids.
"""
from __future__ import annotations

import ctypes as ct
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import _lib, ops
from . import sphere as sp
from . import workloads as wl

CUBIC_SIDES = (10.0, 14.0, 18.0, 22.0)


def reference_grid(L: float, ke_cutoff: float) -> int:
    """Smallest codelet-factorable size >= the reference's minimum for a
    wavefunction cutoff: L * 2 sqrt(2 Ecut) / pi rounded up to a multiple of 4
    (qimpy/grid/_grid.py:114-127, density cutoff 4 Ecut)."""
    n_min = int(4 * math.ceil(L * 2.0 * math.sqrt(2.0 * ke_cutoff) / math.pi / 4.0))
    n = n_min
    while True:
        try:
            sp.factor_axis(n)
            return n
        except ValueError:
            n += 4


@dataclass
class InstanceSpec:
    """One independent eigenproblem of a batch."""

    index: int
    side: float
    positions: np.ndarray  # (n_atoms, 3) fractional
    ke_cutoff: float
    n_bands: int
    k: np.ndarray  # (nk, 3)
    seed: int
    grid: int = 0

    @property
    def n_atoms(self) -> int:
        return int(self.positions.shape[0])


def make_batch_specs(count: int = 256, seed: int = 31, sides=CUBIC_SIDES, ke_range=(15.0, 25.0),
                     atoms_range=(2, 16), bands_range=(8, 64), k_range=(1, 8)) -> list:
    """Seeded instance specs: cubic side from `sides`, Gaussian-well atoms at
    random positions, Ecut uniform in ke_range, bands and k-point counts
    uniform in their ranges, k-points random in the Brillouin zone (so basis
    sizes differ per k)."""
    specs = []
    u = wl.splitmix_uniform(seed, 500, count * 8)
    for i in range(count):
        r = u[8 * i : 8 * i + 8]
        side = sides[int(r[0] * len(sides)) % len(sides)]
        n_atoms = atoms_range[0] + int(r[1] * (atoms_range[1] - atoms_range[0] + 1))
        ke = ke_range[0] + (ke_range[1] - ke_range[0]) * r[2]
        nb = bands_range[0] + int(r[3] * (bands_range[1] - bands_range[0] + 1))
        nk = k_range[0] + int(r[4] * (k_range[1] - k_range[0] + 1))
        pos = wl.splitmix_uniform(seed, 1000 + i, 3 * n_atoms).reshape(n_atoms, 3)
        kpts = wl.splitmix_uniform(seed, 5000 + i, 3 * nk).reshape(nk, 3) - 0.5
        if nk == 1:
            kpts[:] = 0.0
        spec = InstanceSpec(i, side, pos, ke, nb, kpts, seed * 100003 + i)
        spec.grid = reference_grid(side, ke)
        specs.append(spec)
    return specs


class Instance:
    """Device-resident data of one instance (complex64 by default)."""

    def __init__(self, spec: InstanceSpec, device, fft_factors=None, tune: bool = False,
                 dtype: torch.dtype = torch.complex64, real: bool = False):
        """real=True (Gamma-only specs): real wavefunctions on the half basis
        (qimpy/dft/electrons/_basis_real.py), the transforms on the full Gamma
        sphere with two real bands per complex transform."""
        self.spec = spec
        dev = torch.device(device)
        L, shape = spec.side, (spec.grid,) * 3
        if fft_factors is None and tune:
            from .autotune import tune_shape

            fft_factors = tune_shape(shape, torch.complex64, dev)
        R = np.eye(3) * L
        Gb = 2.0 * np.pi * np.linalg.inv(R.T)
        self.dtype = dtype
        self.real_basis = None
        if real:
            from .real_basis import DeviceRealBasis, gamma_bases

            if spec.k.shape[0] != 1 or np.any(spec.k != 0.0):
                raise ValueError("real wavefunctions need a Gamma-only instance")
            half, full = gamma_bases(Gb, spec.ke_cutoff, shape)
            self.real_basis = DeviceRealBasis(half, full, dev, dtype, fft_factors)
            self.layout = half
            self.sphere = self.real_basis.sphere
            self.tables = self.sphere.tables
        else:
            self.layout = wl.make_basis_device(Gb, spec.k, spec.ke_cutoff, shape, dev)
            self.tables = sp.build_tables(self.layout.fft_index, self.layout.n, shape, fft_factors)
            self.sphere = sp.DeviceSphere(self.tables, self.layout.ke, dev, dtype)
        self.Rbasis, self.fft_factors = R, self.tables.fac
        self.nk, self.nb, self.n_tot = spec.k.shape[0], spec.n_bands, self.layout.n_tot
        self.volume = L ** 3
        g = torch.Generator(device=dev).manual_seed(spec.seed)
        self.V_r = self._potential(dev, g, L, shape)
        self.sphere.set_potential(self.V_r)
        self.beta, self.D = self._projectors(dev, Gb)
        self.split = ops.beta_split(self.beta) if dtype == torch.complex64 else None
        self.C = self._start_vectors(dev, g)

    def _potential(self, dev, g, L, shape):
        """Gaussian wells (depth 2 Ha, width 1.2 bohr, nearest image) plus
        Fourier modes with amplitude ~ exp(-|G|^2/8), rms 0.3 Ha."""
        N = shape[0]
        x = torch.arange(N, device=dev, dtype=torch.float64) / N
        X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
        V = torch.zeros(shape, dtype=torch.float64, device=dev)
        for tau in self.spec.positions:
            d = [c - float(t) for c, t in zip((X, Y, Z), tau)]
            d = [(t - torch.round(t)) * L for t in d]
            V -= 2.0 * torch.exp(-(d[0] ** 2 + d[1] ** 2 + d[2] ** 2) / (2 * 1.2 ** 2))
        iG = torch.fft.fftfreq(N, d=1.0 / N, device=dev, dtype=torch.float64) * (2 * math.pi / L)
        G2 = iG[:, None, None] ** 2 + iG[None, :, None] ** 2 + iG[None, None, :] ** 2
        c = torch.complex(torch.randn(shape, generator=g, device=dev, dtype=torch.float64),
                          torch.randn(shape, generator=g, device=dev, dtype=torch.float64)) * torch.exp(-G2 / 8)
        modes = torch.fft.ifftn(c, norm="forward").real
        V += modes * (0.3 / modes.square().mean().sqrt())
        return V

    def _projectors(self, dev, Gb):
        """s + p Gaussian projectors (sigma 1) on every atom, generated on the
        device (qgb_make_projectors); D = diag(1.5, -0.8 x3)."""
        lay = self.layout
        shells = [(0, ("gauss", 1.0)), (1, ("gauss", 1.0))]
        beta = ops.make_projectors(lay.iG, self.spec.k, Gb, lay.n, self.spec.positions, shells, self.volume,
                                   self.dtype, dev)
        D = torch.diag(torch.tensor([1.5, -0.8, -0.8, -0.8], dtype=self.dtype, device=dev))
        return beta, D.expand(self.spec.n_atoms, 4, 4).contiguous()

    def _start_vectors(self, dev, g):
        ke = torch.from_numpy(self.layout.ke).to(dev)
        mask = torch.arange(self.n_tot, device=dev)[None, :] < torch.from_numpy(self.layout.n).to(dev)[:, None]
        C = torch.complex(torch.randn((self.nk, self.nb, self.n_tot), generator=g, device=dev),
                          torch.randn((self.nk, self.nb, self.n_tot), generator=g, device=dev))
        return (C / (1 + ke[:, None, :]) * mask[:, None, :]).to(self.dtype).contiguous()

    def electrons(self, n_bands: int, n_bands_extra: Optional[int] = None):
        """Electrons (mirror API) of this instance for an eigensolve of the lowest
        `n_bands` bands, sharing this instance's device data; start vectors
        orthonormalised.  n_bands_extra defaults to max(1, ceil(0.1 n_bands)),
        the reference's default (qimpy/dft/electrons/_fillings.py:236-243)."""
        from . import electrons as E

        spec = self.spec
        basis = E.Basis.__new__(E.Basis)
        basis.Rbasis, basis.Gbasis = self.Rbasis, 2.0 * np.pi * np.linalg.inv(self.Rbasis.T)
        basis.volume, basis.k, basis.wk = self.volume, spec.k, np.full(len(spec.k), 1.0 / len(spec.k))
        basis.ke_cutoff, basis.grid_shape, basis.device, basis.dtype = spec.ke_cutoff, self.tables.shape, \
            self.sphere.device, self.dtype
        basis.layout, basis.n, basis.n_tot = self.layout, self.layout.n, self.layout.n_tot
        basis.n_min, basis.n_max = int(self.layout.n.min()), int(self.layout.n.max())
        basis.fft_index, basis.iG, basis.tables, basis.sphere = self.layout.fft_index, self.layout.iG, \
            self.tables, self.sphere
        basis.ke = torch.from_numpy(self.layout.ke).to(self.sphere.device)
        basis.real = self.real_basis
        basis.weight = self.real_basis.weight if self.real_basis is not None else None
        # Subspace products on the CUDA cores: the tensor-core ones take ~0.2 GB
        # of bf16 operand workspace per call on the largest cells, and with many
        # requests' worker threads each caching its own, served runs exhausted
        # device memory (library handle creation then failed).
        basis.tc_subspace = False
        pad = torch.arange(basis.n_tot)[None, :] < torch.from_numpy(basis.n)[:, None]
        basis.mask = pad.to(self.sphere.device)
        basis._V_id = id(self.V_r)
        ions = E.Ions.__new__(E.Ions)
        ions.basis, ions.beta, ions.D = basis, self.beta, self.D
        ions.n_projectors, ions.beta_split, ions.beta_version = int(self.beta.shape[1]), self.split, 0
        extra = max(1, int(math.ceil(0.1 * n_bands))) if n_bands_extra is None else int(n_bands_extra)
        el = E.Electrons.__new__(E.Electrons)
        el.basis, el.ions, el.V_r = basis, ions, self.V_r
        el.n_bands, el.n_bands_extra = n_bands, extra
        el.eig, el.deig_max, el.hpsi_band_count = None, np.inf, 0
        C = self.C[:, : n_bands + extra]
        if C.shape[1] < n_bands + extra:  # more bands requested than generated: extend deterministically
            g = torch.Generator(device=self.sphere.device).manual_seed(spec.seed + 7)
            more = torch.complex(torch.randn((self.nk, n_bands + extra - C.shape[1], self.n_tot), generator=g,
                                             device=self.sphere.device),
                                 torch.randn((self.nk, n_bands + extra - C.shape[1], self.n_tot), generator=g,
                                             device=self.sphere.device)).to(self.dtype)
            more = (more / (1 + basis.ke[:, None, :]) * basis.mask[:, None, :]).to(self.dtype)
            C = torch.cat((C, more), dim=1)
        C = E.Wavefunction(basis, coeff=C.contiguous())
        if self.real_basis is not None:
            C.constrain()  # Hermitian Gz = 0 plane
        el.C = C.orthonormalize()
        return el

    @property
    def band_apps(self) -> int:
        return self.nk * self.nb


class _Group:
    """Instances sharing one grid shape: one batched launch per transform phase
    and chunk of instances, with that shape's shared-memory size."""

    def __init__(self, instances: list, inputs: list, outputs: list, device, plane_chunk_bytes: int = 64 << 20):
        lib = _lib.lib()
        self.instances, self.inputs, self.outputs = instances, inputs, outputs
        for inst, c, o in zip(instances, inputs, outputs):
            if c.dtype != torch.complex64 or o.dtype != torch.complex64 or c.shape != (inst.nk, inst.nb, inst.n_tot) \
                    or o.shape != c.shape or not (c.is_contiguous() and o.is_contiguous()):
                raise TypeError("batched instances need contiguous complex64 (nk, nb, n_tot) inputs and outputs")
        n = len(instances)
        ssz = ct.sizeof(_lib.QgbSphere)
        host = bytearray(ssz * n)
        for i, inst in enumerate(instances):
            host[i * ssz : (i + 1) * ssz] = bytes(inst.sphere.struct)
        self._spheres = torch.frombuffer(host, dtype=torch.uint8).to(device)
        # Chunks of consecutive instances whose slab planes together fit the
        # chunk budget: a chunk's planes are written by the y/z launch and read
        # back by the x and gather launches while they are still in L2.  Chunks
        # run in order on one stream and share one plane buffer.
        per = [(inst.sphere.workspace_bytes(inst.nb, budget=1 << 62) + 255) // 256 * 256 for inst in instances]
        chunks, cur, cur_bytes = [], [], 0
        for i, b in enumerate(per):
            if cur and cur_bytes + b > plane_chunk_bytes:
                chunks.append(cur)
                cur, cur_bytes = [], 0
            cur.append(i)
            cur_bytes += b
        chunks.append(cur)
        self._planes = torch.empty(max(sum(per[i] for i in c) for c in chunks), dtype=torch.uint8, device=device)
        smem = max(int(lib.qgb_sphere_smem_bytes(ct.byref(i.sphere.struct), _lib.QGB_F32)) for i in instances)
        smem_yz = max(int(lib.qgb_sphere_smem_bytes_yz(ct.byref(i.sphere.struct), _lib.QGB_F32)) for i in instances)
        self.smem, self.smem_yz = smem, smem_yz
        self._chunks = []
        for chunk in chunks:
            items = (_lib.QgbBatchItem * len(chunk))()
            slab_units, row_units, off = [0], [0], 0
            for j, i in enumerate(chunk):
                inst, t = instances[i], instances[i].tables
                items[j].sphere = self._spheres.data_ptr() + i * ssz
                items[j].C = inputs[i].data_ptr()
                items[j].out = outputs[i].data_ptr()
                items[j].planes = self._planes.data_ptr() + off
                items[j].nb = inst.nb
                items[j].flags = _lib.QGB_ADD_KE
                off += per[i]
                slab_units.append(slab_units[-1] + t.nk * inst.nb * t.max_slabs)
                row_units.append(row_units[-1] + t.nk * inst.nb * t.shape[1])
            ids = np.arange(len(chunk), dtype=np.int32)
            self._chunks.append(dict(
                n=len(chunk),
                items=torch.frombuffer(bytearray(bytes(items)), dtype=torch.uint8).to(device),
                slab_starts=torch.tensor(slab_units, dtype=torch.int64, device=device),
                row_starts=torch.tensor(row_units, dtype=torch.int64, device=device),
                slab_item=torch.from_numpy(np.repeat(ids, np.diff(slab_units))).to(device),
                row_item=torch.from_numpy(np.repeat(ids, np.diff(row_units))).to(device),
                n_slab=slab_units[-1], n_row=row_units[-1]))
        self._nl_ws = [ops.workspace(int(lib.qgb_nonlocal_tc_workspace_bytes(i.nk, i.beta.shape[1], i.nb, i.n_tot)),
                                     device) for i in instances]
        self._projT = [torch.empty((i.nk, i.nb, i.beta.shape[1]), dtype=torch.complex64, device=device)
                       for i in instances]
        self._side = torch.cuda.Stream(device=device)

    def apply(self):
        """Projector part of every instance's nonlocal term (it reads only C) on
        a side stream beside the three batched local-potential launches, then
        the accumulation of the nonlocal terms into HC after both."""
        main = torch.cuda.current_stream()
        self._side.wait_stream(main)
        with torch.cuda.stream(self._side):
            for i, inst in enumerate(self.instances):
                ops.apply_nonlocal_tc(inst.split, inst.D, self.inputs[i], self.outputs[i], self._projT[i],
                                      self._nl_ws[i], phases=1)
        st = main.cuda_stream
        for c in self._chunks:
            _lib.check(_lib.lib().qgb_apply_potential_batched(c["items"].data_ptr(), c["n"], c["slab_item"].data_ptr(),
                                                               c["slab_starts"].data_ptr(), c["row_item"].data_ptr(),
                                                               c["row_starts"].data_ptr(), c["n_slab"], c["n_row"],
                                                               _lib.QGB_F32, self.smem_yz, self.smem, st),
                       "apply_potential_batched")
        main.wait_stream(self._side)
        for i, inst in enumerate(self.instances):
            ops.apply_nonlocal_tc(inst.split, inst.D, self.inputs[i], self.outputs[i], self._projT[i],
                                  self._nl_ws[i], phases=2)


@dataclass
class BatchedHamiltonian:
    """H.psi for all instances of a batch in one graph-capturable sequence.

    Instances are grouped by FFT grid shape; each group runs its local
    potential in three batched launches (shared memory sized for that shape)
    followed by the tensor-core nonlocal term of its instances.  Groups run on
    separate streams, so a captured graph has one parallel branch per group.
    Instances large enough to fill the GPU alone (``solo_units``) run through
    the single-instance call on a branch of their own."""

    instances: list
    device: torch.device
    inputs: list = field(default_factory=list)
    outputs: list = field(default_factory=list)
    #: Slab-plane bytes per batched launch chunk (kept within L2 between the
    #: three transform phases); 0 = one chunk per group, the default: on the
    #: 256-instance batch 64 MB chunks measured 11% slower than one chunk.
    plane_chunk_bytes: int = 0
    #: Instances with at least this many (k, band, slab) work units fill the GPU
    #: by themselves (two waves of 152 SMs x 4 CTAs); they run through the
    #: single-instance call (kernel parameters in constant memory, the
    #: asynchronous x-pass without per-unit context staging) inside the same
    #: graph, and only the smaller ones share batched launches.  0 batches all.
    solo_units: int = 2 * 152 * 4

    def __post_init__(self):
        dev = self.device
        self.inputs = [inst.C for inst in self.instances]
        self.outputs = [torch.empty_like(inst.C) for inst in self.instances]
        by_shape: dict = {}
        self.solo = []
        for i, inst in enumerate(self.instances):
            t = inst.tables
            if self.solo_units and t.nk * inst.nb * t.max_slabs >= self.solo_units:
                self.solo.append(i)
            else:
                by_shape.setdefault(inst.tables.shape, []).append(i)
        self._solo_ws = {i: ops.workspace(self.instances[i].sphere.hamiltonian_mixed_workspace_bytes(
            self.instances[i].nb, self.instances[i].beta.shape[1]), dev) for i in self.solo}
        self._solo_projT = {i: torch.empty((self.instances[i].nk, self.instances[i].nb,
                                            self.instances[i].beta.shape[1]), dtype=torch.complex64, device=dev)
                            for i in self.solo}
        # Largest groups first: their branches start earliest.
        order = sorted(by_shape.values(), key=lambda idx: -sum(self.instances[i].band_apps for i in idx))
        chunk = self.plane_chunk_bytes or (1 << 62)
        self.groups = [_Group([self.instances[i] for i in idx], [self.inputs[i] for i in idx],
                              [self.outputs[i] for i in idx], dev, chunk) for idx in order]
        self._streams = [torch.cuda.Stream(device=dev) for _ in self.groups]
        # Solo instances spread over a few streams, so that the smaller of them
        # overlap in the graph as the batched groups do.
        self._solo_streams = [torch.cuda.Stream(device=dev) for _ in range(min(4, len(self.solo)))]
        self.graph = None

    @property
    def band_apps(self) -> int:
        return sum(inst.band_apps for inst in self.instances)

    def launches(self) -> int:
        """Kernels of ours per application: 3 batched local per chunk of a group,
        3 local per solo instance, + 5 nonlocal per instance."""
        return 3 * sum(len(g._chunks) for g in self.groups) + 3 * len(self.solo) + 5 * len(self.instances)

    def apply(self):
        """Out_i = H_i C_i for every instance (inputs/outputs fixed at construction)."""
        main = torch.cuda.current_stream()
        for s in self._solo_streams:
            s.wait_stream(main)
        for j, i in enumerate(self.solo):
            inst = self.instances[i]
            with torch.cuda.stream(self._solo_streams[j % len(self._solo_streams)]):
                ops.hamiltonian_mixed(inst.sphere, self.inputs[i], inst.split, inst.D, out=self.outputs[i],
                                      projT=self._solo_projT[i], ws=self._solo_ws[i])
        for g, s in zip(self.groups, self._streams):
            s.wait_stream(main)
            with torch.cuda.stream(s):
                g.apply()
        for s in self._streams + self._solo_streams:
            main.wait_stream(s)

    def capture(self):
        """Capture apply() in a CUDA graph (after one eager warm-up call)."""
        self.apply()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(device=self.device)
        cap.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap):
                self.apply()
        torch.cuda.current_stream().wait_stream(cap)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
