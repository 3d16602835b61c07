"""Generate golden fixtures by running the reference package (nohm-devices/qimpy).

Run in a container where the reference source is available:

    python tests/golden/make_golden.py [--ref /root/reference/src] [--only NAME ...]

The reference is imported unmodified.  Its missing optional dependencies
(mpi4py, h5py, yaml, svg.path) are replaced by the single-rank stand-ins in
``tests/golden/_shims``, and its pybind11 ``BufferView`` by a pass-through.
Inputs come from ``qimpy_gb300.workloads`` (seeded, platform independent): the
same lattice, k-mesh, cutoff and grid build the reference ``System``; the
synthetic V(r), projectors beta and D matrix are injected into it the way the
reference's fixed-Hamiltonian path holds them (``electrons.n_tilde.grad``,
``ions.beta``, ``ions.D_all``, ``ions.beta_version``).

Outputs, one ``.npz`` per workload in ``tests/golden/``:

* ``n``, ``fft_index``: the reference's basis layout (qimpy/dft/electrons/_basis.py:167-204);
* ``ke_pot_nl`` checks: H.psi of the seeded start vectors through
  ``Electrons.hamiltonian`` (qimpy/dft/electrons/_hamiltonian.py:7-29), stored in
  full for small cases and as per-band checksums plus a few full bands otherwise;
* ``proj``: <beta|psi> (qimpy/dft/electrons/_wavefunction.py:106-123) for the same bands;
* ``eig``: converged Davidson eigenvalues (qimpy/dft/electrons/_davidson.py:141-235)
  from the Cholesky-orthonormalised start vectors, with the iteration count.

Nothing here runs at test time; tests read the ``.npz`` files only.
"""
from __future__ import annotations

import argparse
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from qimpy_gb300 import workloads as wl  # noqa: E402
from qimpy_gb300.checksums import band_checksums  # noqa: E402

#: workload -> (bands whose full H.psi is stored, Davidson settings or None)
CASES = {
    "tiny_fcc": dict(full=True, davidson=dict(n_iterations=200, eig_threshold=1e-12)),
    "tiny_ortho": dict(full=True, davidson=dict(n_iterations=200, eig_threshold=1e-12)),
    "si2": dict(full=False, sample=((0, 0), (0, 5), (3, 17), (7, 9)), n_hpsi_bands=18,
                davidson=dict(n_iterations=300, eig_threshold=1e-11)),
    "si64": dict(full=False, sample=((0, 0), (0, 7)), n_hpsi_bands=8,
                 davidson=dict(n_iterations=300, eig_threshold=1e-9)),
    "cu32": dict(full=False, sample=((0, 0), (3, 3)), n_hpsi_bands=4,
                 davidson=dict(n_iterations=300, eig_threshold=1e-9)),
}


def import_reference(ref_src: str):
    sys.path[:0] = [os.path.join(HERE, "_shims"), ref_src]
    bv = types.ModuleType("qimpy.mpi._bufferview")
    bv.BufferView = lambda t: t
    sys.modules["qimpy.mpi._bufferview"] = bv
    import qimpy  # noqa: F401
    import torch

    qimpy.rc.init(cores_override=os.cpu_count())
    torch.set_num_threads(os.cpu_count())
    return qimpy


def build_system(qimpy, prob: wl.Problem, davidson: dict | None, real: bool = False):
    from qimpy.dft import System

    size, offset = prob.kmesh
    el_cfg = {
        "k-mesh": {"size": list(size), "offset": list(offset), "use-inversion": False},
        "basis": {"ke-cutoff": prob.ke_cutoff, "grid": {"shape": list(prob.grid_shape)},
                  **({"real-wavefunctions": True} if real else {})},
        "fillings": {"n-bands": prob.n_bands, "n-bands-extra": prob.n_bands_extra},
        "lcao": False,
    }
    if davidson:
        el_cfg["davidson"] = {k.replace("_", "-"): v for k, v in davidson.items()}
    R = prob.Rbasis
    return System(
        lattice=dict(vector1=list(R[:, 0]), vector2=list(R[:, 1]), vector3=list(R[:, 2])),
        symmetries={"override": "identity"},
        grid={"shape": list(prob.grid_shape)},
        electrons=el_cfg,
        process_grid_shape=(1, 1, 1),
    )


def inject(qimpy, system, prob, beta_np):
    """Install V(r), beta and D into the reference objects."""
    import torch
    from qimpy.grid import FieldR
    from qimpy.dft.electrons import Wavefunction

    el = system.electrons
    basis = el.basis
    shape = tuple(prob.grid_shape)
    el.n_tilde = ~FieldR(basis.grid, data=torch.zeros((1,) + shape, dtype=torch.float64))
    el.n_tilde.grad = ~FieldR(basis.grid, data=torch.from_numpy(prob.V_r)[None].clone())
    ions = system.ions
    beta = torch.from_numpy(beta_np)[None, :, :, None, :].clone()
    ions.beta = Wavefunction(basis, coeff=beta)
    ions.D_all = torch.from_numpy(prob.D_all()).to(torch.complex128)
    ions.beta_version += 1
    # Zero wavefunctions size their cached projections by ions.n_projectors,
    # a property derived from pseudopotential files; report the injected count.
    ions.__class__ = type("InjectedIons", (type(ions),), {"n_projectors": prob.n_projectors})
    return el


def run_case(qimpy, name: str, cfg: dict, out_dir: str) -> None:
    import torch
    from qimpy.dft.electrons import Wavefunction

    t0 = time.time()
    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape)
    system = build_system(qimpy, prob, cfg.get("davidson"))
    el = system.electrons
    basis = el.basis
    ref_n = basis.n.numpy().astype(np.int64)
    ref_index = basis.fft_index.numpy().astype(np.int64)
    assert np.array_equal(ref_n, mine.n), (ref_n, mine.n)
    assert np.array_equal(ref_index, mine.fft_index)
    beta = wl.make_projectors(prob, mine)
    el = inject(qimpy, system, prob, beta)
    n_bands_tot = prob.n_bands + prob.n_bands_extra
    C0 = wl.make_wavefunctions(prob, mine, n_bands_tot)
    out: dict = dict(
        n=ref_n,
        fft_index=ref_index.astype(np.int32),
        ke_ref=basis.get_ke().numpy()[:, :8].copy(),
        Gbasis_ref=system.lattice.Gbasis.numpy(),
        k_ref=basis.k.numpy(),
    )

    # --- H.psi of the (not orthonormalised) start vectors:
    nb = n_bands_tot if cfg["full"] else cfg["n_hpsi_bands"]
    C = Wavefunction(basis, coeff=torch.from_numpy(C0[None, :, :nb, None, :]).clone())
    t1 = time.time()
    HC = el.hamiltonian(C).coeff[0, :, :, 0, :].numpy()
    t_hpsi = time.time() - t1
    proj = C.proj[0].numpy()  # (nk, P, nb)
    out["hpsi_bands"] = np.int64(nb)
    out["hpsi_seconds"] = np.float64(t_hpsi)
    if cfg["full"]:
        out["hpsi"] = HC
        out["proj"] = proj
        out["C0"] = C0
        out["V_r"] = prob.V_r
        out["beta"] = beta
    else:
        sample = cfg["sample"]
        out["hpsi_sample_kb"] = np.array(sample, dtype=np.int64)
        out["hpsi_sample"] = np.stack([HC[k, b] for k, b in sample])
        out["proj_sample"] = np.stack([proj[k, :, b] for k, b in sample])
    out["hpsi_checksums"] = band_checksums(HC, ref_n)

    # --- Davidson:
    dav = cfg.get("davidson")
    if dav:
        el.C = Wavefunction(basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
        el.C = el.C.orthonormalize()
        t1 = time.time()
        el.diagonalize()
        out["davidson_seconds"] = np.float64(time.time() - t1)
        out["eig"] = el.eig[0].numpy().copy()
        out["davidson_iterations"] = np.int64(el.diagonalize._i_iter)
        out["eig_threshold"] = np.float64(dav["eig_threshold"])
    path = os.path.join(out_dir, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: wrote {path} ({os.path.getsize(path) / 1e3:.0f} KB) in {time.time() - t0:.1f} s"
          f"; H.psi {t_hpsi * 1e3:.1f} ms for {nb} bands"
          + (f"; Davidson {out['davidson_iterations']} it, {out['davidson_seconds']:.1f} s" if dav else ""))


#: workload -> CheFSI settings (second caller of the Hamiltonian)
CHEFSI_CASES = {
    "tiny_fcc": dict(n_iterations=100, eig_threshold=1e-11, filter_order=10, init_threshold=1e-1),
    "tiny_ortho": dict(n_iterations=100, eig_threshold=1e-11, filter_order=10, init_threshold=1e-1),
    "si2": dict(n_iterations=100, eig_threshold=1e-10, filter_order=8, init_threshold=1e-1),
}


def run_chefsi_case(qimpy, name: str, cfg: dict, out_dir: str) -> None:
    """Reference CheFSI (qimpy/dft/electrons/_chefsi.py:72-176) from the same
    orthonormalised start vectors as the Davidson case: its Davidson warm-up
    to init_threshold, then Chebyshev-filtered subspace iterations."""
    import torch
    from qimpy.dft.electrons import CheFSI, Wavefunction

    t0 = time.time()
    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape)
    system = build_system(qimpy, prob, None)
    el = inject(qimpy, system, prob, wl.make_projectors(prob, mine))
    C0 = wl.make_wavefunctions(prob, mine, prob.n_bands + prob.n_bands_extra)
    el.C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone()).orthonormalize()
    el.deig_max = np.inf
    solver = CheFSI(electrons=el, **cfg)
    solver()
    out = dict(eig=el.eig[0].numpy().copy(), iterations=np.int64(solver._i_iter),
               **{k: np.float64(v) for k, v in cfg.items()})
    path = os.path.join(out_dir, f"chefsi_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"chefsi {name}: wrote {path}; {solver._i_iter} iterations in {time.time() - t0:.1f} s")


#: workloads whose reference density is stored in full (others: checksums and samples)
DENSITY_CASES = {"tiny_fcc": True, "tiny_ortho": True, "si2": False}


def run_density_case(qimpy, name: str, full: bool, out_dir: str) -> None:
    """Reference Basis.collect_density (qimpy/dft/electrons/_basis_ops.py:207-296)
    of the seeded start vectors with seeded fillings: rho(r) = sum_kb f w_sk / Omega
    |psi_kb(r)|^2 on the real-space grid (natural order)."""
    import torch
    from qimpy.dft.electrons import Wavefunction

    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape)
    system = build_system(qimpy, prob, None)
    el = inject(qimpy, system, prob, wl.make_projectors(prob, mine))
    nb = prob.n_bands + prob.n_bands_extra
    C0 = wl.make_wavefunctions(prob, mine, nb)
    f = wl.make_fillings(prob, nb)
    C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
    rho = el.basis.collect_density(C, torch.from_numpy(f)[None].clone(), False).data[0].numpy()
    out = dict(f=f, w_sk=el.basis.w_sk.numpy().reshape(-1).copy(), volume=np.float64(system.lattice.volume),
               total=np.float64(rho.sum()), abs_total=np.float64(np.abs(rho).sum()),
               plane_sums=rho.sum(axis=(1, 2)))
    if full:
        out["rho"] = rho
    else:
        idx = np.array([[0, 0, 0], [1, 2, 3], [5, 7, 11], [17, 4, 30]]) % np.array(rho.shape)
        out["sample_idx"] = idx
        out["sample"] = rho[idx[:, 0], idx[:, 1], idx[:, 2]]
    path = os.path.join(out_dir, f"density_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"density {name}: wrote {path}; total {rho.sum():.6f}")


#: Gamma-point workloads with real wavefunctions (half-mesh basis)
REAL_CASES = ("tiny_gamma",)


def run_real_case(qimpy, name: str, out_dir: str) -> None:
    """Reference H.psi with real wavefunctions (qimpy/dft/electrons/_basis_real.py,
    half-mesh basis, r2c / c2r FFTs, Gweight-weighted projections): the basis
    layout, the start vectors after the reference's constrain (padding zeroed,
    Gz = 0 plane made Hermitian), their H.psi and <beta|psi>."""
    import torch
    from qimpy.dft.electrons import Wavefunction

    prob = wl.get(name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape, real=True)
    system = build_system(qimpy, prob, None, real=True)
    basis = system.electrons.basis
    assert basis.real_wavefunctions
    assert np.array_equal(basis.n.numpy(), mine.n)
    assert np.array_equal(basis.fft_index.numpy(), mine.fft_index)
    beta = wl.make_projectors(prob, mine)
    el = inject(qimpy, system, prob, beta)
    nb = prob.n_bands + prob.n_bands_extra
    C0 = wl.make_wavefunctions(prob, mine, nb)
    C = Wavefunction(basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
    C.constrain()
    C0s = C.coeff[0, :, :, 0, :].numpy().copy()
    HC = el.hamiltonian(C).coeff[0, :, :, 0, :].numpy()
    out = dict(n=mine.n, fft_index=mine.fft_index.astype(np.int32), C0=C0s, V_r=prob.V_r, beta=beta, hpsi=HC,
               proj=C.proj[0].numpy(), Gweight=basis.real.Gweight.numpy())
    # Density of the symmetrised start vectors with seeded fillings (c2r expand).
    f = wl.make_fillings(prob, nb)
    Cd = Wavefunction(basis, coeff=torch.from_numpy(C0s[None, :, :, None, :]).clone())
    out.update(f=f, rho=basis.collect_density(Cd, torch.from_numpy(f)[None].clone(), False).data[0].numpy(),
               w_sk=basis.w_sk.numpy().reshape(-1).copy(), volume=np.float64(system.lattice.volume))
    # Davidson with real wavefunctions from the orthonormalised, symmetrised start vectors.
    from qimpy.dft.electrons import Davidson

    el.C = Wavefunction(basis, coeff=torch.from_numpy(C0s[None, :, :, None, :]).clone()).orthonormalize()
    el.deig_max = np.inf
    solver = Davidson(electrons=el, n_iterations=200, eig_threshold=1e-12)
    solver()
    out.update(eig=el.eig[0].numpy().copy(), davidson_iterations=np.int64(solver._i_iter),
               eig_threshold=np.float64(1e-12))
    # CheFSI with real wavefunctions from the same start.
    from qimpy.dft.electrons import CheFSI

    el.C = Wavefunction(basis, coeff=torch.from_numpy(C0s[None, :, :, None, :]).clone()).orthonormalize()
    el.deig_max = np.inf
    cf = CheFSI(electrons=el, n_iterations=100, eig_threshold=1e-11, filter_order=10, init_threshold=1e-1)
    cf()
    out.update(chefsi_eig=el.eig[0].numpy().copy(), chefsi_iterations=np.int64(cf._i_iter))
    path = os.path.join(out_dir, f"real_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"real {name}: wrote {path}")


#: workloads whose projectors are also made by the reference's own
#: Ions.get_projectors (blip-spline radial tables of the Gaussian shells)
PROJECTOR_CASES = ("tiny_fcc", "tiny_gamma")
PROJECTOR_DG = 0.02  # the reference's radial spline spacing (qimpy/math/_radial_function.py:22)


def run_projector_case(qimpy, name: str, out_dir: str) -> None:
    """beta from the unmodified Ions.get_projectors
    (qimpy/dft/ions/_ions_projectors.py:14-72), called with a stand-in for the
    ions object that supplies what it reads: one species on the workload's
    atoms whose radial functions are the workload's Gaussian shells, sampled
    on the reference's spline spacing and converted with its get_coeff."""
    import torch
    from qimpy.dft.ions import _ions_projectors as ip
    from qimpy.dft.ions._ions import Ions
    from qimpy.math import quintic_spline

    prob = wl.get(name)
    real = bool(prob.extra.get("real_wavefunctions", False))
    system = build_system(qimpy, prob, None, real=real)
    basis = system.electrons.basis
    iGk = basis.iG + basis.k[:, None]
    qmax = float(((iGk @ torch.from_numpy(prob.Gbasis).T) ** 2).sum(-1).sqrt().max())
    nG = int(np.ceil(qmax / PROJECTOR_DG)) + 5
    q = np.arange(nG) * PROJECTOR_DG
    samples = np.stack([(-1.0) ** sh.l * (2 * np.pi) ** 1.5 * sh.sigma ** (2 * sh.l + 3)
                        * np.exp(-0.5 * sh.sigma ** 2 * q ** 2) for sh in prob.shells])
    coeff = quintic_spline.get_coeff(torch.from_numpy(samples))  # (nG + 4, n_shells)
    i_rf, i_lm = [], []
    for s, sh in enumerate(prob.shells):
        for m in range(2 * sh.l + 1):
            i_rf.append(s)
            i_lm.append(sh.l * sh.l + m)
    pqn = types.SimpleNamespace(n_tot=len(i_rf), i_rf=torch.tensor(i_rf), i_lm=torch.tensor(i_lm))
    ps = types.SimpleNamespace(l_max=max(sh.l for sh in prob.shells), pqn_beta=pqn,
                               beta=types.SimpleNamespace(f_tilde_coeff=coeff))
    ions = types.SimpleNamespace(
        lattice=types.SimpleNamespace(Gbasis=torch.from_numpy(prob.Gbasis), volume=prob.volume),
        positions=torch.from_numpy(prob.positions), n_projectors=prob.n_projectors, pseudopotentials=[ps],
        n_ions_type=[prob.n_atoms], slices=[slice(0, prob.n_atoms)])
    ions.translation_phase = lambda iG, atom_slice=slice(None): Ions.translation_phase(ions, iG, atom_slice)
    beta = ip.get_projectors(ions, basis, full_basis=True).coeff[0, :, :, 0, :].numpy()
    path = os.path.join(out_dir, f"projectors_{name}.npz")
    np.savez_compressed(path, beta=beta, coeff=coeff.numpy().T.copy(), dq=PROJECTOR_DG,
                        fft_index=basis.fft_index.numpy())
    print(f"projectors {name}: wrote {path}")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference/src")
    ap.add_argument("--only", nargs="*", default=None)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--chefsi", action="store_true", help="only the CheFSI goldens")
    ap.add_argument("--density", action="store_true", help="only the density goldens")
    ap.add_argument("--real", action="store_true", help="only the real-wavefunction goldens")
    ap.add_argument("--projectors", action="store_true", help="only the projector goldens")
    args = ap.parse_args()
    qimpy = import_reference(args.ref)
    only_part = args.chefsi or args.density or args.real or args.projectors
    for name, cfg in CASES.items():
        if only_part or (args.only and name not in args.only):
            continue
        run_case(qimpy, name, cfg, args.out)
    for name, cfg in CHEFSI_CASES.items():
        if (only_part and not args.chefsi) or (args.only and name not in args.only):
            continue
        run_chefsi_case(qimpy, name, cfg, args.out)
    for name, full in DENSITY_CASES.items():
        if (only_part and not args.density) or (args.only and name not in args.only):
            continue
        run_density_case(qimpy, name, full, args.out)
    for name in REAL_CASES:
        if (only_part and not args.real) or (args.only and name not in args.only):
            continue
        run_real_case(qimpy, name, args.out)
    for name in PROJECTOR_CASES:
        if (only_part and not args.projectors) or (args.only and name not in args.only):
            continue
        run_projector_case(qimpy, name, args.out)


if __name__ == "__main__":
    main()
