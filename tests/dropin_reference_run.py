"""Run the reference's own Davidson with qimpy_gb300.qimpy_dropin installed.

Test infrastructure (``tests/test_dropin_cpu.py`` runs this file in a child
process, where the reference source is present).  The unmodified reference is
imported as ``tests/golden/make_golden.py`` does and given the same seeded
problem as the goldens: V(r), the projectors and D injected, the start vectors
orthonormalised (a ``real_<name>`` case runs the reference's real-wavefunction
mode on the half-mesh basis, a ``chefsi_<name>`` case its CheFSI eigensolver).  ``install()`` then replaces Basis.apply_ke/
apply_potential/collect_density, Electrons.hamiltonian, Wavefunction.dot/^/dot_O/matmul/@ and the eigensolvers'
eighg, and ``electrons.diagonalize()`` (the reference's Davidson,
qimpy/dft/electrons/_davidson.py:141-235) runs to convergence through them.

This host has no GPU, so the binding's device layer (``ops``, the sphere and
``linalg.eighg``, which need CUDA) is swapped in this process for the oracle's
FP64 restatements of the same operations.  What runs is therefore every line of
the binding itself against the reference's own classes: the views of the
reference's tensors, the potential conversion, the projector and D-block
extraction, the Waitable wrapping and the attribute replacement.  That the C ABI
computes what the oracle computes is shown on the GPU by the parity tests.

Prints one JSON line: per case the eigenvalue error against the golden
eigenvalues, the iteration counts, and how often each replaced function ran.
"""
from __future__ import annotations

import json
import os
import sys
import types
from collections import Counter

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as mg  # noqa: E402
from oracle import davidson as od  # noqa: E402
from oracle import hpsi as oh  # noqa: E402
from qimpy_gb300 import qimpy_dropin as dropin  # noqa: E402
from qimpy_gb300 import workloads as wl  # noqa: E402

CALLS: Counter = Counter()


class OracleSphere:
    """Stands in for DeviceSphere: the tables and V(r) in natural order."""

    def __init__(self, tables, ke, device, dtype):
        self.fft_index, self.n, self.shape = tables.fft_index, tables.n, tables.shape
        self.ke = np.asarray(ke)
        self.V = None

    def set_potential(self, V_r):
        self.V = V_r.detach().cpu().numpy().astype(np.float64)


class OracleRealBasis:
    """Stands in for DeviceRealBasis: the half-mesh basis, its overlap weights
    and V(r) in natural order."""

    def __init__(self, half, full, device, dtype):
        self.half = half
        n = int(half.n[0])
        self.weight_np = oh.real_gweight(half.iG[0], n, int(half.n_tot))
        import torch

        self.weight = torch.from_numpy(self.weight_np)
        self.V = None

    def set_potential(self, V_r):
        self.V = V_r.detach().cpu().numpy().astype(np.float64)


def oracle_tables(fft_index, n, shape):
    return types.SimpleNamespace(fft_index=np.asarray(fft_index), n=np.asarray(n), shape=tuple(shape))


def _dense_D(D_blocks):
    n_atoms, pa, _ = D_blocks.shape
    D = np.zeros((n_atoms * pa, n_atoms * pa), dtype=np.complex128)
    for a in range(n_atoms):
        D[a * pa:(a + 1) * pa, a * pa:(a + 1) * pa] = D_blocks[a]
    return D


def make_oracle_ops(torch):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))  # noqa: E731

    class OracleOps:
        @staticmethod
        def apply_ke(ds, C):
            CALLS["apply_ke"] += 1
            return t(oh.apply_ke(ds.ke, C.numpy()))

        @staticmethod
        def apply_potential(ds, C):
            CALLS["apply_potential"] += 1
            return t(oh.apply_potential(ds.V, ds.fft_index, ds.n, C.numpy()))

        @staticmethod
        def hamiltonian(ds, C, beta, D_blocks):
            CALLS["hamiltonian"] += 1
            CALLS[f"D_blocks {tuple(D_blocks.shape)}"] += 1
            HC = oh.hamiltonian(ds.ke, ds.V, ds.fft_index, ds.n, beta.numpy(), _dense_D(D_blocks.numpy()), C.numpy())
            return t(HC), None

        @staticmethod
        def collect_density(ds, C, prefac):
            CALLS["collect_density"] += 1
            return t(oh.collect_density(ds.fft_index, ds.shape, C.numpy(), prefac.numpy()))

        @staticmethod
        def hamiltonian_real(rb, C, beta, D_blocks):
            CALLS["hamiltonian_real"] += 1
            h = rb.half
            HC = oh.hamiltonian_real(h.ke, rb.V, h.fft_index, h.n, h.iG, beta.numpy(), _dense_D(D_blocks.numpy()),
                                     C.numpy(), rb.weight_np)
            return t(HC), None

        @staticmethod
        def dot_real(X, Y, weight):
            CALLS["dot_real"] += 1
            return t(od.dot_real(X.numpy(), Y.numpy(), weight.numpy()))

        @staticmethod
        def dot(X, Y):
            CALLS["dot"] += 1
            return t(od.dot(X.numpy(), Y.numpy()))

        @staticmethod
        def matmul(C, M):
            CALLS["matmul"] += 1
            M = M.resolve_conj().resolve_neg().numpy()
            if M.ndim == 2:
                M = np.broadcast_to(M, (C.shape[0],) + M.shape)
            return t(od.matmul(C.numpy(), M.astype(np.complex128)))

    class OracleLinalg:
        @staticmethod
        def eighg(H, O, use_cholesky=True):
            CALLS["eighg"] += 1
            Hr = H.wait() if hasattr(H, "wait") else H
            lead = Hr.shape[:-2]
            n = Hr.shape[-1]
            E, V = od.eighg(Hr.reshape(-1, n, n).numpy(), O.reshape(-1, n, n).numpy())
            return t(E).reshape(*lead, n), t(V).reshape(*lead, n, n)

    return OracleOps, OracleLinalg


def run(qimpy, name: str) -> dict:
    import torch
    from qimpy.dft.electrons import Wavefunction

    cfg = mg.CASES[name]
    golden = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape)
    system = mg.build_system(qimpy, prob, cfg["davidson"])
    el = mg.inject(qimpy, system, prob, wl.make_projectors(prob, mine))
    C0 = wl.make_wavefunctions(prob, mine, prob.n_bands + prob.n_bands_extra)
    out = {}
    if "hpsi" in golden:
        # The reference's own _hamiltonian over the replaced Basis.apply_ke,
        # Basis.apply_potential and the ^ / @ of the projections (beta ^ C,
        # beta @ (D_all @ proj)), and the replaced Electrons.hamiltonian.
        from qimpy.dft.electrons._hamiltonian import _hamiltonian

        C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
        want = golden["hpsi"]
        scale = np.abs(want).max()
        CALLS.clear()
        parts = _hamiltonian(el, C).coeff[0, :, :, 0, :].numpy()
        out["hpsi_parts_rel_err"] = float(np.abs(parts - want).max() / scale)
        out["hpsi_parts_calls"] = dict(CALLS)
        whole = el.hamiltonian(C).coeff[0, :, :, 0, :].numpy()
        out["hpsi_rel_err"] = float(np.abs(whole - want).max() / scale)
    dens_path = os.path.join(HERE, "golden", f"density_{name}.npz")
    if os.path.exists(dens_path) and "rho" in np.load(dens_path):
        # The replaced Basis.collect_density with the goldens' seeded fillings.
        dg = np.load(dens_path)
        C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
        CALLS.clear()
        rho = el.basis.collect_density(C, torch.from_numpy(dg["f"])[None].clone(), False)
        out["density_rel_err"] = float(np.abs(rho.data[0].numpy() - dg["rho"]).max() / np.abs(dg["rho"]).max())
        out["density_calls"] = dict(CALLS)
    CALLS.clear()
    el.C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
    el.C = el.C.orthonormalize()
    el.diagonalize()
    eig = el.eig[0].numpy()
    out.update(eig_err=float(np.abs(eig - golden["eig"]).max()), iterations=int(el.diagonalize._i_iter),
               golden_iterations=int(golden["davidson_iterations"]), calls=dict(CALLS))
    return out


def run_real(qimpy, name: str) -> dict:
    """Real (Gamma-point) wavefunctions: the reference's own H.psi and Davidson
    on the half-mesh basis, as the real-mode goldens were made."""
    import torch
    from qimpy.dft.electrons import Davidson, Wavefunction

    golden = np.load(os.path.join(HERE, "golden", f"real_{name}.npz"))
    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape, real=True)
    system = mg.build_system(qimpy, prob, None, real=True)
    el = mg.inject(qimpy, system, prob, wl.make_projectors(prob, mine))
    basis = el.basis
    assert basis.real_wavefunctions
    C0s = golden["C0"]
    out = {}
    CALLS.clear()
    C = Wavefunction(basis, coeff=torch.from_numpy(C0s[None, :, :, None, :]).clone())
    HC = el.hamiltonian(C).coeff[0, :, :, 0, :].numpy()
    out["hpsi_rel_err"] = float(np.abs(HC - golden["hpsi"]).max() / np.abs(golden["hpsi"]).max())
    CALLS.clear()
    el.C = Wavefunction(basis, coeff=torch.from_numpy(C0s[None, :, :, None, :]).clone()).orthonormalize()
    el.deig_max = np.inf
    solver = Davidson(electrons=el, n_iterations=200, eig_threshold=float(golden["eig_threshold"]))
    solver()
    out.update(eig_err=float(np.abs(el.eig[0].numpy() - golden["eig"]).max()), iterations=int(solver._i_iter),
               golden_iterations=int(golden["davidson_iterations"]), calls=dict(CALLS))
    return out


def run_chefsi(qimpy, name: str) -> dict:
    """The reference's own CheFSI (qimpy/dft/electrons/_chefsi.py:72-176, its
    Davidson warm-up included) from the goldens' start vectors."""
    import torch
    from qimpy.dft.electrons import CheFSI, Wavefunction

    golden = np.load(os.path.join(HERE, "golden", f"chefsi_{name}.npz"))
    cfg = mg.CHEFSI_CASES[name]
    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape)
    system = mg.build_system(qimpy, prob, None)
    el = mg.inject(qimpy, system, prob, wl.make_projectors(prob, mine))
    C0 = wl.make_wavefunctions(prob, mine, prob.n_bands + prob.n_bands_extra)
    CALLS.clear()
    el.C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone()).orthonormalize()
    el.deig_max = np.inf
    solver = CheFSI(electrons=el, **cfg)
    solver()
    return dict(eig_err=float(np.abs(el.eig[0].numpy() - golden["eig"]).max()), iterations=int(solver._i_iter),
                golden_iterations=int(golden["iterations"]), calls=dict(CALLS))


def main() -> None:
    ref_src = sys.argv[1]
    names = sys.argv[2:] or ["tiny_fcc"]
    qimpy = mg.import_reference(ref_src)
    import torch

    ops_, linalg_ = make_oracle_ops(torch)
    dropin.ops, dropin.linalg = ops_, linalg_
    dropin.DeviceSphere, dropin.build_tables = OracleSphere, oracle_tables
    dropin.DeviceRealBasis = OracleRealBasis
    dropin.install()
    out = {}
    for name in names:
        if name.startswith("real_"):
            out[name] = run_real(qimpy, name[len("real_"):])
        elif name.startswith("chefsi_"):
            out[name] = run_chefsi(qimpy, name[len("chefsi_"):])
        else:
            out[name] = run(qimpy, name)
    dropin.uninstall()
    from qimpy.dft import electrons

    out["restored"] = electrons.Wavefunction.dot.__module__ != dropin.__name__
    print(json.dumps(out))


if __name__ == "__main__":
    main()
