"""CPU checks of the sphere tables and the local-potential kernel plan.

``emulate_apply_potential`` replays the three CUDA kernels of
qimpy_gb300/csrc/local_potential.cu with numpy on the same tables: slab planes,
z-FFTs only on listed rows, four-step FFT passes leaving real space in the
digit-permuted order, V in that order, slab-only x outputs.  It must agree with
the oracle, which pins the table builder and the index arithmetic before the
kernels run on a GPU.
"""
import numpy as np
import pytest

from oracle import hpsi as oh
from qimpy_gb300 import sphere as sp
from qimpy_gb300 import workloads as wl


def _inv_perm(x, L1, L2, axis):
    """Inverse DFT (unnormalised) natural -> permuted along `axis` (four-step)."""
    x = np.moveaxis(x, axis, -1)
    sh = x.shape[:-1]
    N = L1 * L2
    A = x.reshape(sh + (L2, L1))  # [n2, n1], position n1 + L1 n2
    A = np.fft.ifft(A, axis=-2) * L2  # over n2 -> k2
    W = np.exp(2j * np.pi * (np.arange(L2)[:, None] * np.arange(L1)[None, :] % N) / N)  # [k2, n1]
    A = A * W
    A = np.fft.ifft(A, axis=-1) * L1  # over n1 -> k1; position L1 k2 + k1
    return np.moveaxis(A.reshape(sh + (N,)), -1, axis)


def _fwd_perm(x, L1, L2, axis):
    """Forward DFT (unnormalised) permuted -> natural along `axis`."""
    x = np.moveaxis(x, axis, -1)
    sh = x.shape[:-1]
    N = L1 * L2
    A = x.reshape(sh + (L2, L1))  # [a, b], real index a + L2 b
    A = np.fft.fft(A, axis=-1)  # over b -> c
    W = np.exp(-2j * np.pi * (np.arange(L2)[:, None] * np.arange(L1)[None, :] % N) / N)  # [a, c]
    A = A * W
    A = np.fft.fft(A, axis=-2)  # over a -> d; position c + L1 d
    return np.moveaxis(A.reshape(sh + (N,)), -1, axis)


def emulate_apply_potential(t: sp.SphereTables, V_r, C, ke=None):
    N0, N1, N2 = t.shape
    (a1, a2), (b1, b2), (c1, c2) = t.fac
    perms = [sp.permutation(t.shape[a], *t.fac[a]) for a in range(3)]
    Vp = V_r[perms[0]][:, perms[1]][:, :, perms[2]]
    nk, nb, n_tot = C.shape
    out = np.zeros_like(C)
    for k in range(nk):
        ns = int(t.n_slabs[k])
        for b in range(nb):
            planes = np.zeros((ns, N1, N2), complex)
            for s in range(ns):  # k_ifft_yz
                P = np.zeros((N1, N2), complex)
                g0, g1 = t.slab_start[k, s], t.slab_start[k, s + 1]
                v = t.yz[k, g0:g1]
                P[v >> 16, v & 0xFFFF] = C[k, b, g0:g1]
                rows = t.rows[t.row_start[k, s] : t.row_start[k, s + 1]]
                P[rows] = _inv_perm(P[rows], c1, c2, 1)
                P = _inv_perm(P, b1, b2, 0)
                planes[s] = P
            for r1 in range(N1):  # k_xpass
                X = np.zeros((N0, N2), complex)
                X[t.slab_i0[k, :ns]] = planes[:, r1, :]
                X = _inv_perm(X, a1, a2, 0)
                X *= Vp[:, r1, :]
                X = _fwd_perm(X, a1, a2, 0)
                planes[:, r1, :] = X[t.slab_i0[k, :ns]]
            for s in range(ns):  # k_fft_yz_gather
                P = _fwd_perm(planes[s], b1, b2, 0)
                rows = t.rows[t.row_start[k, s] : t.row_start[k, s + 1]]
                P[rows] = _fwd_perm(P[rows], c1, c2, 1)
                g0, g1 = t.slab_start[k, s], t.slab_start[k, s + 1]
                v = t.yz[k, g0:g1]
                val = P[v >> 16, v & 0xFFFF] / (N0 * N1 * N2)
                if ke is not None:
                    val = val + ke[k, g0:g1] * C[k, b, g0:g1]
                out[k, b, g0:g1] = val
    return out


@pytest.mark.parametrize("name,shape", [("tiny_fcc", None), ("tiny_ortho", None),
                                        ("tiny_fcc", (18, 24, 20)), ("tiny_ortho", (16, 20, 21))])
def test_emulated_plan_matches_oracle(name, shape):
    p = wl.get(name) if shape is None else wl.get(name, shape=shape)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    C = wl.make_wavefunctions(p, b, 3)
    t = sp.build_tables(b.fft_index, b.n, p.grid_shape)
    got = emulate_apply_potential(t, p.V_r, C, b.ke)
    want = oh.apply_potential(p.V_r, b.fft_index, b.n, C) + oh.apply_ke(b.ke, C)
    want = oh.constrain(want, b.n)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_tables_cover_sphere_exactly():
    p = wl.si2()
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    t = sp.build_tables(b.fft_index, b.n, p.grid_shape)
    N0, N1, N2 = p.grid_shape
    for k in range(p.nk):
        ns = int(t.n_slabs[k])
        assert t.slab_start[k, ns] == b.n[k]
        idx = b.fft_index[k, : b.n[k]]
        for s in range(ns):
            g0, g1 = t.slab_start[k, s], t.slab_start[k, s + 1]
            assert np.all(idx[g0:g1] // (N1 * N2) == t.slab_i0[k, s])
            rows = set(t.rows[t.row_start[k, s] : t.row_start[k, s + 1]].tolist())
            assert rows == set(((idx[g0:g1] // N2) % N1).tolist())
        v = t.yz[k, : b.n[k]]
        assert np.array_equal((v >> 16) * N2 + (v & 0xFFFF), idx % (N1 * N2))
    assert t.max_slabs <= N0 and t.max_rows <= N1


@pytest.mark.parametrize("N", [1, 7, 16, 18, 24, 36, 48, 64, 72, 96, 100, 144, 210, 256])
def test_factorisation_and_permutation(N):
    L1, L2 = sp.factor_axis(N)
    assert L1 * L2 == N
    perm = sp.permutation(N, L1, L2)
    assert sorted(perm.tolist()) == list(range(N))
    x = np.random.default_rng(N).standard_normal(N) + 0j
    y = _inv_perm(x, L1, L2, 0)
    assert np.allclose(y[np.argsort(perm)], np.fft.ifft(x) * N)
    z = _fwd_perm(y, L1, L2, 0)
    assert np.allclose(z, x * N)


def test_factorisation_rejects_large_primes():
    with pytest.raises(ValueError):
        sp.factor_axis(17 * 3)


def test_batched_units_per_cta_cover_every_unit_once():
    """CPU replay of the batched launch geometry (launch_batched and the
    QGB_BATCH_UNITS_BEGIN loop): with upc = clamp(n / (152 * 32), 1, 8) units per
    CTA and ceil(n / upc) CTAs, every work unit u < n runs exactly once and no
    CTA touches u >= n."""
    import numpy as np

    for n in [1, 7, 152 * 32 - 1, 152 * 32, 152 * 32 * 3 + 5, 1_300_001]:
        upc = max(1, min(8, n // (152 * 32)))
        ctas = (n + upc - 1) // upc
        seen = np.zeros(n, dtype=np.int64)
        for b in range(ctas):
            u0 = b * upc
            u1 = min(u0 + upc, n)
            assert u0 < n
            seen[u0:u1] += 1
        assert np.all(seen == 1)


def test_density_kernel_index_replay():
    """CPU replay of k_density_x's indexing: the z-split keeps N0 * nz within
    the per-thread register accumulators (64 FP32 / 32 FP64 per thread, 256
    threads), and the incremental (px, c) walk of each thread visits exactly
    e = t + 256 j -> (e // nz, e % nz), covering the tile once."""
    import numpy as np

    threads = 256
    for dtype_regs in (64, 32):
        for N0, N2 in [(18, 18), (15, 25), (36, 36), (96, 96), (100, 100), (144, 120), (160, 160)]:
            zs = 1
            while N0 * ((N2 + zs - 1) // zs) > dtype_regs * threads:
                zs += 1
            nz_max = (N2 + zs - 1) // zs
            covered = np.zeros((N0, N2), dtype=np.int64)
            for zp in range(zs):
                z0 = zp * nz_max
                nz = min(nz_max, N2 - z0)
                if nz <= 0:
                    continue
                total = N0 * nz
                assert total <= dtype_regs * threads
                step_px, step_c = threads // nz, threads - (threads // nz) * nz
                for t in range(threads):
                    px, c = t // nz, t - (t // nz) * nz
                    for j in range(dtype_regs):
                        e = t + j * threads
                        if e < total:
                            assert (px, c) == (e // nz, e % nz)
                            covered[px, z0 + c] += 1
                        px += step_px
                        c += step_c
                        if c >= nz:
                            c -= nz
                            px += 1
            assert np.all(covered == 1), (N0, N2, dtype_regs)


def test_real_wavefunction_slab_plan_matches_oracle():
    """Plan of the real-wavefunction (Gamma-point) local potential, replayed with
    numpy on the half-grid sphere tables: y c2c on the slab planes
    N1 x (N2/2+1); per y-row the x c2c, the z c2r per x-row, V on the real tile,
    the z r2c and the x c2c; then y c2c back and the gather.  The c2r along z
    comes last because a single z-line is not Hermitian by itself.  Must agree
    with the oracle's irfftn/rfftn form (before its constrain)."""
    p = wl.get("tiny_gamma")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    N0, N1, N2 = p.grid_shape
    N2h = N2 // 2 + 1
    t = sp.build_tables(b.fft_index, b.n, (N0, N1, N2h), fft_axes=(0, 1))
    (a1, a2), (b1, b2) = t.fac[0], t.fac[1]
    C = wl.make_wavefunctions(p, b, 3)
    oh.real_symmetrize(C, b.iG[0], p.grid_shape)
    perm_x = sp.permutation(N0, a1, a2)
    perm_y = sp.permutation(N1, b1, b2)
    Vp = p.V_r[perm_x][:, perm_y]  # x, y permuted; z natural
    k = 0
    ns = int(t.n_slabs[k])
    out = np.zeros_like(C)
    for band in range(C.shape[1]):
        planes = np.zeros((ns, N1, N2h), complex)
        for s in range(ns):
            P = np.zeros((N1, N2h), complex)
            g0, g1 = t.slab_start[k, s], t.slab_start[k, s + 1]
            v = t.yz[k, g0:g1]
            P[v >> 16, v & 0xFFFF] = C[k, band, g0:g1]
            planes[s] = _inv_perm(P, b1, b2, 0)  # y c2c
        for r1 in range(N1):
            X = np.zeros((N0, N2h), complex)
            X[t.slab_i0[k, :ns]] = planes[:, r1, :]
            X = _inv_perm(X, a1, a2, 0)  # x c2c
            R = np.fft.irfft(X, n=N2, axis=1) * N2  # z c2r, unnormalised
            R = R * Vp[:, r1, :]
            X = np.fft.rfft(R, axis=1)  # z r2c
            X = _fwd_perm(X, a1, a2, 0)  # x c2c back
            planes[:, r1, :] = X[t.slab_i0[k, :ns]]
        for s in range(ns):
            P = _fwd_perm(planes[s], b1, b2, 0)
            g0, g1 = t.slab_start[k, s], t.slab_start[k, s + 1]
            v = t.yz[k, g0:g1]
            out[k, band, g0:g1] = P[v >> 16, v & 0xFFFF] / (N0 * N1 * N2)
    oh.constrain(out, b.n)
    oh.real_symmetrize(out, b.iG[0], p.grid_shape)
    want = oh.apply_potential_real(p.V_r, b.fft_index, b.n, b.iG, C)
    assert np.abs(out - want).max() <= 1e-12 * np.abs(want).max()


def test_device_sphere_refuses_half_width_tables():
    """Half-width (real-wavefunction) tables leave the z axis unfactorised; the
    complex kernels would transform it as a complex axis, so DeviceSphere
    refuses them before touching a device."""
    import pytest
    import torch

    p = wl.get("tiny_gamma")
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape, real=True)
    N0, N1, N2 = p.grid_shape
    t = sp.build_tables(b.fft_index, b.n, (N0, N1, N2 // 2 + 1), fft_axes=(0, 1))
    assert t.fft_axes == (0, 1)
    with pytest.raises(ValueError, match="fft_axes"):
        sp.DeviceSphere(t, b.ke, "cpu", torch.complex128)
