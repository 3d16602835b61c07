"""Seeded synthetic plane-wave eigenproblems (cells, k-points, V(r), projectors, D, C0).

Every random number comes from a counter-based splitmix64 stream evaluated with
numpy integer arithmetic, so the same seed gives bit-identical uniforms on any
platform and numpy version; Gaussian deviates use Box-Muller (last-ulp libm
differences only).  The same arrays feed the CUDA path, the CPU oracle and the
reference package when golden fixtures are generated.

Named workloads (sizes are the ones the benchmark and tests use):

* ``si2``  - Si diamond primitive cell, FCC a=10.26 bohr, 2 atoms, Ecut 20 Ha,
  36^3 grid, 2x2x2 Monkhorst-Pack k (offset 1/2, no inversion), 16 bands (+2).
* ``si64`` - 64-atom Si cube, side 20.52 bohr, Ecut 20 Ha, 96^3 grid, Gamma only,
  160 bands (blocks of 32).
* ``cu32`` - 32-atom fcc Cu-like cube, side 13.64 bohr, Ecut 30 Ha, 72^3 grid,
  4 k-points, 200 bands, 18 projectors per atom with dense 18x18 D blocks.
* ``tiny_*`` - small cells used as exhaustive parity cases.

Physics conventions follow the reference: lattice vectors are the columns of
``Rbasis`` and ``Gbasis = 2 pi inv(Rbasis^T)`` (qimpy/lattice/_lattice.py:217);
k-points are fractional reciprocal coordinates with the Monkhorst-Pack mesh
wrapped to [-1/2, 1/2) (qimpy/lattice/_kpoints.py:130-138).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix_uniform_grid(seed: int, streams, counters) -> np.ndarray:
    """Uniforms in (0, 1) for broadcastable arrays of stream ids and counters.

    Element (stream, i) is a pure function of (seed, stream, i): no state, no
    platform dependence (integer arithmetic modulo 2^64, then the top 53 bits)."""
    streams = np.asarray(streams, dtype=np.uint64)
    counters = np.asarray(counters, dtype=np.uint64)
    with np.errstate(over="ignore"):
        base = (np.uint64(seed) * np.uint64(0x100000001B3)) ^ (streams * np.uint64(0xC2B2AE3D27D4EB4F))
        x = base + (counters + np.uint64(1)) * _GOLD
        z = (x ^ (x >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return u + 0.5 / 9007199254740992.0  # strictly inside (0, 1)


def make_fillings(prob: "Problem", nb: int, seed_stream: int = 11) -> np.ndarray:
    """Seeded occupations f[k, b] in [0, 1] (one splitmix stream per workload):
    a smeared step from 1 to 0 across the band window, perturbed by up to 5%."""
    u = splitmix_uniform(prob.seed, seed_stream, prob.nk * nb).reshape(prob.nk, nb)
    b = np.arange(nb)[None, :]
    step = 1.0 / (1.0 + np.exp((b - 0.6 * nb) / max(1.0, 0.1 * nb)))
    return np.clip(step * (0.95 + 0.1 * u), 0.0, 1.0)


def splitmix_uniform(seed: int, stream: int, count: int) -> np.ndarray:
    """`count` uniforms in (0, 1) from one counter-based splitmix64 stream."""
    return splitmix_uniform_grid(seed, stream, np.arange(count, dtype=np.uint64))


def splitmix_normal(seed: int, stream: int, count: int) -> np.ndarray:
    """`count` standard-normal deviates (Box-Muller on two uniform streams)."""
    u1 = splitmix_uniform(seed, 2 * stream, count)
    u2 = splitmix_uniform(seed, 2 * stream + 1, count)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos((2.0 * np.pi) * u2)


def splitmix_complex_normal(seed: int, stream: int, count: int) -> np.ndarray:
    """Complex deviates with independent standard-normal real and imaginary parts."""
    return splitmix_normal(seed, 2 * stream, count) + 1j * splitmix_normal(
        seed, 2 * stream + 1, count
    )


# ---------------------------------------------------------------------------
# Projector specification
# ---------------------------------------------------------------------------

#: Real solid-harmonic prefactors, order m = -l..l; l=1 is (y, z, x) and l=2 is
#: (xy, yz, 3z^2-r^2, xz, x^2-y^2), the ordering of the reference's real
#: harmonics (qimpy/math/spherical_harmonics.py:80-83).
_Y00 = 0.5 / np.sqrt(np.pi)
_Y1 = np.sqrt(3.0 / (4.0 * np.pi))
_Y2a = np.sqrt(15.0 / (4.0 * np.pi))
_Y2b = np.sqrt(5.0 / (16.0 * np.pi))
_Y2c = np.sqrt(15.0 / (16.0 * np.pi))


def solid_harmonics(l: int, q: np.ndarray) -> np.ndarray:
    """Real solid harmonics |q|^l Y_lm(q-hat) for all m of `l`, shape (2l+1, ...)."""
    x, y, z = q[..., 0], q[..., 1], q[..., 2]
    if l == 0:
        return np.full((1,) + x.shape, _Y00)
    if l == 1:
        return _Y1 * np.stack((y, z, x))
    if l == 2:
        r2 = x * x + y * y + z * z
        return np.stack(
            (
                _Y2a * x * y,
                _Y2a * y * z,
                _Y2b * (3.0 * z * z - r2),
                _Y2a * x * z,
                _Y2c * (x * x - y * y),
            )
        )
    raise ValueError(f"l={l} not supported")


@dataclass
class ProjectorShell:
    """One radial shell r^l exp(-r^2 / (2 sigma^2)) times all 2l+1 real Y_lm."""

    l: int
    sigma: float


# ---------------------------------------------------------------------------
# Problem description
# ---------------------------------------------------------------------------


@dataclass
class Problem:
    """A synthetic fixed-potential Kohn-Sham problem (one cell, all its k)."""

    name: str
    Rbasis: np.ndarray  #: (3, 3), lattice vectors in columns [bohr]
    positions: np.ndarray  #: (n_atoms, 3) fractional
    k: np.ndarray  #: (nk, 3) fractional reciprocal coordinates
    wk: np.ndarray  #: (nk,) weights summing to 1
    ke_cutoff: float
    grid_shape: tuple
    n_bands: int
    n_bands_extra: int
    shells: list  #: list[ProjectorShell] per atom (same for every atom)
    D_atom: np.ndarray  #: (n_atoms, p_atom, p_atom) real symmetric
    V_r: np.ndarray  #: (N0, N1, N2) float64 local potential
    seed: int
    block_size: int = 0  #: band-block size for H.psi benchmarks (0 = all bands)
    kmesh: tuple = ((1, 1, 1), (0.0, 0.0, 0.0))  #: (size, offset) that generated `k`
    extra: dict = field(default_factory=dict)

    @property
    def Gbasis(self) -> np.ndarray:
        return 2.0 * np.pi * np.linalg.inv(self.Rbasis.T)

    @property
    def volume(self) -> float:
        return abs(float(np.linalg.det(self.Rbasis)))

    @property
    def n_atoms(self) -> int:
        return self.positions.shape[0]

    @property
    def p_atom(self) -> int:
        return sum(2 * s.l + 1 for s in self.shells)

    @property
    def n_projectors(self) -> int:
        return self.n_atoms * self.p_atom

    @property
    def nk(self) -> int:
        return self.k.shape[0]

    def D_all(self) -> np.ndarray:
        """Dense block-diagonal (P, P) D matrix, atom-major projector order
        (the layout qimpy/dft/ions/_ions_update.py:229-243 builds)."""
        P, pa = self.n_projectors, self.p_atom
        D = np.zeros((P, P))
        for a in range(self.n_atoms):
            D[a * pa : (a + 1) * pa, a * pa : (a + 1) * pa] = self.D_atom[a]
        return D


# ---------------------------------------------------------------------------
# Basis (G-sphere) construction
# ---------------------------------------------------------------------------


@dataclass
class BasisLayout:
    """G-sphere for every k, in the reference's ordering.

    ``fft_index[k]`` lists the in-sphere grid points first, in ascending
    linear FFT index, then out-of-sphere points up to the common padded length
    ``n_tot = max(n)``, exactly as qimpy/dft/electrons/_basis.py:167-204 builds
    it.  ``iG`` are the integer reciprocal coordinates of those points
    (wrapped as in qimpy/grid/_fft.py:67-71), ``ke`` the kinetic energies."""

    grid_shape: tuple
    n: np.ndarray  #: (nk,) in-sphere counts
    n_tot: int
    fft_index: np.ndarray  #: (nk, n_tot) int64
    iG: np.ndarray  #: (nk, n_tot, 3) int64
    ke: np.ndarray  #: (nk, n_tot) float64 = 0.5 |(iG + k) Gbasis^T|^2


def grid_iG(shape) -> np.ndarray:
    """Integer reciprocal mesh (N0*N1*N2, 3); index i maps to i if i <= N//2
    else i - N (qimpy/grid/_fft.py:67-71)."""
    iG1 = [np.where(np.arange(s) <= s // 2, np.arange(s), np.arange(s) - s) for s in shape]
    mesh = np.stack(np.meshgrid(*iG1, indexing="ij"), axis=-1)
    return mesh.reshape(-1, 3).astype(np.int64)


def grid_iH(shape) -> np.ndarray:
    """Integer half (Hermitian-symmetric) reciprocal mesh (N0*N1*(N2//2+1), 3) of
    real-wavefunction bases: the full mesh's first N2//2 + 1 z-frequencies
    (qimpy/grid/_grid.py get_mesh("H") with _fft.py:72-76)."""
    iG1 = [np.where(np.arange(s) <= s // 2, np.arange(s), np.arange(s) - s) for s in shape]
    iG1[2] = iG1[2][: shape[2] // 2 + 1]
    mesh = np.stack(np.meshgrid(*iG1, indexing="ij"), axis=-1)
    return mesh.reshape(-1, 3).astype(np.int64)


def make_basis(Gbasis: np.ndarray, k: np.ndarray, ke_cutoff: float, shape, real: bool = False) -> BasisLayout:
    """Plane-wave basis per k (restates qimpy/dft/electrons/_basis.py:167-204);
    real=True: the half-mesh basis of real (Gamma-point) wavefunctions, with
    fft_index into the N0 x N1 x (N2//2+1) half grid (_basis.py:168)."""
    iG_grid = grid_iH(shape) if real else grid_iG(shape)
    n_fft = iG_grid.shape[0]
    G = (iG_grid[None, :, :] + k[:, None, :]) @ Gbasis.T
    ke_grid = 0.5 * np.square(G).sum(axis=-1)
    within = ke_grid < ke_cutoff
    n = within.sum(axis=1)
    n_tot = int(n.max())
    key = np.where(within, 0, n_fft) + np.arange(n_fft)[None, :]
    fft_index = np.argsort(key, axis=1, kind="stable")[:, :n_tot]
    iG = iG_grid[fft_index]
    Gk = (iG + k[:, None, :]) @ Gbasis.T
    ke = 0.5 * np.square(Gk).sum(axis=-1)
    return BasisLayout(tuple(shape), n.astype(np.int64), n_tot, fft_index.astype(np.int64), iG, ke)


def make_basis_device(Gbasis: np.ndarray, k: np.ndarray, ke_cutoff: float, shape, device="cuda") -> BasisLayout:
    """`make_basis` evaluated with torch on a device (for large grids).

    Same ordering rule without the sort: in-sphere points in ascending linear
    index, then the first out-of-sphere points as padding up to n_tot."""
    import torch

    dev = torch.device(device)
    iG_grid = torch.from_numpy(grid_iG(shape)).to(dev)
    Gb = torch.from_numpy(np.ascontiguousarray(Gbasis.T)).to(dev)
    kt = torch.from_numpy(np.asarray(k, dtype=np.float64)).to(dev)
    within = []
    for ik in range(kt.shape[0]):
        G = (iG_grid.to(torch.float64) + kt[ik]) @ Gb
        within.append(0.5 * G.square().sum(dim=1) < ke_cutoff)
    n = torch.stack([w.sum() for w in within]).cpu().numpy().astype(np.int64)
    n_tot = int(n.max())
    fft_index = torch.empty((len(within), n_tot), dtype=torch.int64, device=dev)
    for ik, w in enumerate(within):
        inside = torch.nonzero(w).flatten()
        outside = torch.nonzero(~w).flatten()[: n_tot - inside.numel()]
        fft_index[ik] = torch.cat((inside, outside))
    iG = iG_grid[fft_index]
    Gk = (iG.to(torch.float64) + kt[:, None, :]) @ Gb
    ke = 0.5 * Gk.square().sum(dim=-1)
    return BasisLayout(tuple(shape), n, n_tot, fft_index.cpu().numpy(), iG.cpu().numpy(), ke.cpu().numpy())


# ---------------------------------------------------------------------------
# Field and projector generators
# ---------------------------------------------------------------------------


def make_potential(
    Rbasis: np.ndarray,
    positions: np.ndarray,
    shape,
    depth: float,
    width: float,
    modes_rms: float,
    seed: int,
) -> np.ndarray:
    """V(r) = sum over atoms and the 27 nearest periodic images of
    -depth * exp(-|r - tau|^2 / (2 width^2)), plus seeded Fourier modes with
    amplitude proportional to exp(-|G|^2 / 8), rescaled to rms `modes_rms`."""
    shape = tuple(shape)
    frac = np.stack(
        np.meshgrid(*[np.arange(s) / s for s in shape], indexing="ij"), axis=-1
    ).reshape(-1, 3)
    V = np.zeros(frac.shape[0])
    images = np.array([[a, b, c] for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    for tau in positions:
        d = frac - tau[None, :]
        d -= np.floor(d + 0.5)  # nearest image first
        for img in images:
            r = (d + img[None, :]) @ Rbasis.T
            V -= depth * np.exp(-np.square(r).sum(axis=1) / (2.0 * width * width))
    V = V.reshape(shape)
    if modes_rms > 0.0:
        Gbasis = 2.0 * np.pi * np.linalg.inv(Rbasis.T)
        G = grid_iG(shape) @ Gbasis.T
        amp = np.exp(-np.square(G).sum(axis=1) / 8.0)
        c = splitmix_complex_normal(seed, 101, amp.size) * amp
        modes = np.fft.ifftn(c.reshape(shape), norm="forward").real
        modes *= modes_rms / np.sqrt(np.mean(np.square(modes)))
        V = V + modes
    return np.ascontiguousarray(V)


def make_projectors(prob: Problem, basis: BasisLayout) -> np.ndarray:
    """beta[k, p, g] = (-i)^l (2 pi)^{3/2} sigma^{2l+3} S_lm(q) exp(-sigma^2 q^2 / 2)
    exp(-i q.tau) / sqrt(Omega), q = (iG + k) Gbasis^T: the analytic Fourier
    transform of r^l Y_lm exp(-r^2/(2 sigma^2)) centred on each atom.  Padding
    entries are zero (as qimpy/dft/ions/_ions_projectors.py:14-72 leaves them)."""
    Gb = prob.Gbasis
    nk, n_tot = basis.fft_index.shape
    beta = np.zeros((nk, prob.n_projectors, n_tot), dtype=np.complex128)
    inv_sqrt_vol = 1.0 / np.sqrt(prob.volume)
    for ik in range(nk):
        nkk = int(basis.n[ik])
        kiG = basis.iG[ik, :nkk] + prob.k[ik][None, :]
        q = kiG @ Gb.T
        q2 = np.square(q).sum(axis=1)
        radial = []
        for sh in prob.shells:
            pref = ((-1j) ** sh.l) * (2.0 * np.pi) ** 1.5 * sh.sigma ** (2 * sh.l + 3)
            g = pref * np.exp(-0.5 * sh.sigma**2 * q2)
            radial.append(solid_harmonics(sh.l, q) * g[None, :])
        ang = np.concatenate(radial, axis=0)  # (p_atom, n)
        for a, tau in enumerate(prob.positions):
            phase = np.exp(-2j * np.pi * (kiG @ tau)) * inv_sqrt_vol
            beta[ik, a * prob.p_atom : (a + 1) * prob.p_atom, :nkk] = ang * phase[None, :]
    return beta


def make_projectors_device(prob: Problem, basis: BasisLayout, device, dtype):
    """``make_projectors`` generated on the device by qgb_make_projectors (the
    same analytic Gaussian shells, computed in FP64, stored as `dtype`)."""
    from . import ops

    shells = [(sh.l, ("gauss", sh.sigma)) for sh in prob.shells]
    return ops.make_projectors(basis.iG, prob.k, prob.Gbasis, basis.n, prob.positions, shells, prob.volume,
                               dtype, device)


def make_wavefunctions(prob: Problem, basis: BasisLayout, n_bands: int, seed_stream: int = 7,
                       band_offset: int = 0) -> np.ndarray:
    """C0[k, b, g] = complex Gaussian / (1 + |k+G|^2 / 2); padding zero.

    Every (k, band) draws from its own stream, so band b has the same
    coefficients however many bands are generated (bands start at band_offset)."""
    nk, n_tot = basis.fft_index.shape
    kk = np.arange(nk, dtype=np.uint64)[:, None, None]
    bb = (np.arange(n_bands, dtype=np.uint64) + np.uint64(band_offset))[None, :, None]
    gg = np.arange(n_tot, dtype=np.uint64)[None, None, :]
    sid = (np.uint64(seed_stream) << np.uint64(40)) + (kk << np.uint64(20)) + bb
    u = [splitmix_uniform_grid(prob.seed, sid * np.uint64(4) + np.uint64(j), gg) for j in range(4)]
    nrm = lambda a, b: np.sqrt(-2.0 * np.log(a)) * np.cos((2.0 * np.pi) * b)  # noqa: E731
    C = nrm(u[0], u[1]) + 1j * nrm(u[2], u[3])
    damp = 1.0 / (1.0 + basis.ke)  # |k+G|^2 / 2 = ke
    C = C * damp[:, None, :]
    for ik in range(nk):
        C[ik, :, int(basis.n[ik]) :] = 0.0
    return C


def random_symmetric(seed: int, stream: int, n: int, lo: float, hi: float) -> np.ndarray:
    """Dense real symmetric n x n matrix with eigenvalues drawn in [lo, hi]."""
    A = splitmix_normal(seed, stream, n * n).reshape(n, n)
    Q, R = np.linalg.qr(A)
    Q = Q * np.sign(np.diag(R))[None, :]
    ev = lo + (hi - lo) * splitmix_uniform(seed, stream + 1, n)
    D = (Q * ev[None, :]) @ Q.T
    return 0.5 * (D + D.T)


# ---------------------------------------------------------------------------
# Lattices
# ---------------------------------------------------------------------------


def monkhorst_pack(size, offset) -> np.ndarray:
    """Full k-mesh (no symmetry reduction), wrapped to [-1/2, 1/2)
    (qimpy/lattice/_kpoints.py:130-138)."""
    g1 = [(offset[i] + np.arange(size[i])) / size[i] for i in range(3)]
    mesh = np.stack(np.meshgrid(*g1, indexing="ij")).reshape(3, -1).T
    mesh -= np.floor(0.5 + mesh)
    return mesh


_DIAMOND_BASIS = np.array(
    [[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0],
     [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25]]
)
_FCC_BASIS = _DIAMOND_BASIS[:4]


def supercell_positions(basis_frac: np.ndarray, reps: int) -> np.ndarray:
    """Tile conventional-cell fractional positions `reps` times along each axis."""
    out = []
    for i in range(reps):
        for j in range(reps):
            for l in range(reps):
                out.append((basis_frac + np.array([i, j, l])) / reps)
    return np.concatenate(out, axis=0)


def _finish(prob: Problem, depth: float, width: float, modes_rms: float) -> Problem:
    prob.V_r = make_potential(prob.Rbasis, prob.positions, prob.grid_shape, depth, width, modes_rms, prob.seed)
    return prob


def si2(seed: int = 1) -> Problem:
    """Si diamond primitive cell (2 atoms), Ecut 20 Ha, 36^3, 8 k, 16 bands."""
    a = 10.26
    R = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]]).T
    pos = np.array([[0.0, 0.0, 0.0], [0.25, 0.25, 0.25]])
    km = ((2, 2, 2), (0.5, 0.5, 0.5))
    k = monkhorst_pack(*km)
    D = np.tile(np.diag([1.5, -0.8, -0.8, -0.8])[None], (2, 1, 1))
    prob = Problem("si2", R, pos, k, np.full(len(k), 1.0 / len(k)), 20.0, (36, 36, 36),
                   16, 2, [ProjectorShell(0, 1.0), ProjectorShell(1, 1.0)], D, None, seed,
                   kmesh=km)
    return _finish(prob, 2.0, 1.2, 0.3)


def si64(seed: int = 2) -> Problem:
    """64-atom Si cube (2x2x2 conventional), side 20.52, Ecut 20 Ha, 96^3, Gamma, 160 bands."""
    L = 20.52
    R = np.eye(3) * L
    pos = supercell_positions(_DIAMOND_BASIS, 2)
    D = np.tile(np.diag([1.5, -0.8, -0.8, -0.8])[None], (64, 1, 1))
    prob = Problem("si64", R, pos, np.zeros((1, 3)), np.ones(1), 20.0, (96, 96, 96),
                   160, 16, [ProjectorShell(0, 1.0), ProjectorShell(1, 1.0)], D, None, seed,
                   block_size=32)
    return _finish(prob, 2.0, 1.2, 0.3)


def cu32(seed: int = 3) -> Problem:
    """32-atom fcc Cu-like cube (2x2x2 conventional, a=6.82), Ecut 30 Ha, 72^3,
    4 k-points (2x2x1 mesh, offset 1/2), 200 bands, 18 projectors per atom."""
    L = 13.64
    R = np.eye(3) * L
    pos = supercell_positions(_FCC_BASIS, 2)
    shells = [ProjectorShell(l, s) for s in (0.9, 1.4) for l in (0, 1, 2)]
    D = np.stack([random_symmetric(seed, 200 + 2 * a, 18, -3.0, 3.0) for a in range(32)])
    km = ((2, 2, 1), (0.5, 0.5, 0.0))
    k = monkhorst_pack(*km)
    prob = Problem("cu32", R, pos, k, np.full(4, 0.25), 30.0, (72, 72, 72),
                   200, 20, shells, D, None, seed, block_size=200, kmesh=km)
    return _finish(prob, 4.0, 1.2, 0.3)


def tiny_fcc(seed: int = 11, shape=(18, 18, 18)) -> Problem:
    """Small FCC cell (a=6.0), Ecut 10 Ha, 2 off-Gamma k, s+p+d projectors."""
    a = 6.0
    R = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]]).T
    pos = np.array([[0.0, 0.0, 0.0], [0.25, 0.25, 0.25]])
    shells = [ProjectorShell(0, 0.9), ProjectorShell(1, 0.9), ProjectorShell(2, 1.1)]
    D = np.stack([random_symmetric(seed, 300 + 2 * a_, 9, -2.0, 2.0) for a_ in range(2)])
    km = ((1, 1, 2), (0.0, 0.0, 0.5))
    k = monkhorst_pack(*km)
    prob = Problem("tiny_fcc", R, pos, k, np.full(2, 0.5), 10.0, tuple(shape),
                   6, 2, shells, D, None, seed, kmesh=km)
    return _finish(prob, 2.0, 1.0, 0.2)


def tiny_ortho(seed: int = 12, shape=(15, 20, 25)) -> Problem:
    """Orthorhombic cell with an odd, non-cubic grid (15 x 20 x 25), Gamma + one k."""
    R = np.diag([5.0, 6.5, 8.0])
    pos = np.array([[0.1, 0.2, 0.3], [0.6, 0.55, 0.8], [0.35, 0.9, 0.1]])
    shells = [ProjectorShell(0, 1.0), ProjectorShell(1, 0.8)]
    D = np.stack([random_symmetric(seed, 400 + 2 * a_, 4, -1.5, 1.5) for a_ in range(3)])
    km = ((1, 2, 1), (0.0, 0.0, 0.0))
    k = monkhorst_pack(*km)
    prob = Problem("tiny_ortho", R, pos, k, np.full(2, 0.5), 5.0, tuple(shape),
                   5, 1, shells, D, None, seed, kmesh=km)
    return _finish(prob, 1.5, 1.0, 0.2)


def tiny_gamma(seed: int = 13, shape=(16, 20, 24)) -> Problem:
    """Gamma-only orthorhombic cell for real wavefunctions (half-mesh basis,
    qimpy/dft/electrons/_basis_real.py): even grid 16 x 20 x 24, Ecut 6 Ha,
    s + p projectors on three atoms."""
    R = np.diag([5.5, 6.5, 7.5])
    pos = np.array([[0.1, 0.2, 0.3], [0.6, 0.55, 0.8], [0.35, 0.9, 0.1]])
    shells = [ProjectorShell(0, 1.0), ProjectorShell(1, 0.8)]
    D = np.stack([random_symmetric(seed, 500 + 2 * a_, 4, -1.5, 1.5) for a_ in range(3)])
    km = ((1, 1, 1), (0.0, 0.0, 0.0))
    k = monkhorst_pack(*km)
    prob = Problem("tiny_gamma", R, pos, k, np.full(1, 1.0), 6.0, tuple(shape),
                   5, 1, shells, D, None, seed, kmesh=km, extra={"real_wavefunctions": True})
    return _finish(prob, 1.5, 1.0, 0.2)


WORKLOADS = {"si2": si2, "si64": si64, "cu32": cu32, "tiny_fcc": tiny_fcc, "tiny_ortho": tiny_ortho,
             "tiny_gamma": tiny_gamma}


def get(name: str, **kw) -> Problem:
    """Build the named synthetic problem."""
    return WORKLOADS[name](**kw)
