"""CPU checks of the real-wavefunction (Gamma-point) tables and plan.

``qgb_hamiltonian_real`` runs the local potential of real bands on the full
Gamma sphere, two bands per complex transform (qimpy_gb300/csrc/real_basis.cu).
These tests replay that plan with numpy on the same tables (pack two half-basis
bands into one full-sphere row, the complex oracle's V.psi on the full sphere,
unpack) and compare it with the oracle's r2c/c2r restatement of the reference,
before the kernels run on a GPU.
"""
import numpy as np
import pytest

from oracle import hpsi as oh
from qimpy_gb300 import real_basis as rbm
from qimpy_gb300 import workloads as wl


def _gamma(name):
    p = wl.get(name)
    if name != "tiny_gamma":  # a Gamma-only copy of the cell
        p.k = np.zeros((1, 3))
    half, full = rbm.gamma_bases(p.Gbasis, p.ke_cutoff, p.grid_shape)
    return p, half, full


def _split_pack(m):
    """(half index, conjugate flag, plane partner or -1) of every pack entry."""
    e0 = m.pack[:, 0].view(np.uint32).astype(np.int64)
    return e0 & 0x7FFFFFFF, (e0 >> 31) != 0, m.pack[:, 1].astype(np.int64)


def _pack_rows(m, C):
    """Full-sphere rows z = c_a + i c_b of band pairs (k_pack_real)."""
    nb = C.shape[1]
    h0, conj, h1 = _split_pack(m)
    plane = h1 >= 0
    Z = np.zeros((1, (nb + 1) // 2, m.n_tot_full), complex)
    for q in range((nb + 1) // 2):
        rows = []
        for b in (2 * q, 2 * q + 1):
            if b >= nb:
                rows.append(np.zeros(m.n_full, complex))
                continue
            c = C[0, b]
            v = np.where(conj, np.conj(c[h0]), c[h0])
            v[plane] = 0.5 * (c[h0[plane]] + np.conj(c[h1[plane]]))
            rows.append(v)
        Z[0, q, : m.n_full] = rows[0] + 1j * rows[1]
    return Z


def _unpack_rows(m, W, C):
    """Half-basis V.psi of every band from the transformed pairs, plus KE C
    (k_unpack_real)."""
    nb = C.shape[1]
    out = np.zeros_like(C)
    up = m.unpack
    for b in range(nb):
        w = W[0, b // 2]
        wp, wm = w[up[:, 0]], np.conj(w[up[:, 1]])
        v = 0.5 * (wp + wm) if b % 2 == 0 else -0.5j * (wp - wm)
        out[0, b, : m.n_half] = v + m.ke[: m.n_half] * C[0, b, : m.n_half]
    return out


def test_real_map_tables_are_consistent():
    """pack and unpack are inverse maps between the half basis and the full
    sphere; the plane pairs are an involution; weights 1 / 2 / 0."""
    p, half, full = _gamma("tiny_gamma")
    m = rbm.build_real_map(half, full)
    iGh, iGf = half.iG[0], full.iG[0]
    h0, conj, h1 = _split_pack(m)
    assert np.array_equal(iGf[: m.n_full], np.where(conj, -1, 1)[:, None] * iGh[h0])
    plane = h1 >= 0
    assert np.array_equal(iGh[h1[plane]], -iGf[: m.n_full][plane]) and (iGf[: m.n_full][plane, 2] == 0).all()
    assert np.array_equal(iGf[m.unpack[:, 0]], iGh[: m.n_half])
    assert np.array_equal(iGf[m.unpack[:, 1]], -iGh[: m.n_half])
    assert np.array_equal(iGh[m.plane[:, 1]], -iGh[m.plane[:, 0]])
    assert (iGh[m.plane[:, 0], 2] == 0).all() and m.n_plane == int((iGh[: m.n_half, 2] == 0).sum())
    assert m.n_full == 2 * m.n_half - m.n_plane
    assert set(np.unique(m.weight[: m.n_half])) <= {1.0, 2.0} and not m.weight[m.n_half:].any()


@pytest.mark.parametrize("name,nb,hermitian", [("tiny_gamma", 6, True), ("tiny_gamma", 5, False),
                                              ("si2", 3, False)])
def test_packed_plan_matches_oracle(name, nb, hermitian):
    """Two real bands per complex full-sphere transform reproduce the
    reference's irfftn / rfftn H.psi (KE + local), also for an odd band count
    and for a Gz = 0 plane that is not Hermitian (the c2r transform uses its
    Hermitian part)."""
    p, half, full = _gamma(name)
    m = rbm.build_real_map(half, full)
    C = wl.make_wavefunctions(p, half, nb)
    oh.constrain(C, half.n)
    if hermitian:
        oh.real_symmetrize(C, half.iG[0], p.grid_shape)
    Z = _pack_rows(m, C)
    W = oh.apply_potential(p.V_r, full.fft_index, full.n, Z)
    got = _unpack_rows(m, W, C)
    want = oh.apply_ke(half.ke, C) + oh.apply_potential_real(p.V_r, half.fft_index, half.n, half.iG, C)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_real_map_rejects_nyquist_sphere():
    """A cutoff whose sphere reaches the grid's Nyquist plane has no distinct
    -G partner there; the map builder refuses it."""
    p = wl.get("tiny_gamma")
    half, full = rbm.gamma_bases(p.Gbasis, 12 * p.ke_cutoff, p.grid_shape)
    with pytest.raises(ValueError, match="Nyquist"):
        rbm.build_real_map(half, full)
