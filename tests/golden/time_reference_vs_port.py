"""Time the reference's own CPU H.psi against the oracle port on the same host.

The reference is Python and is not installed where bench.py runs, so the CPU
baseline there runs a port (oracle/hpsi_torch.py; before it, oracle.hpsi with
numpy/scipy).  This
script measures, on one host, how fast the unmodified reference's
Electrons.hamiltonian (torch CPU, every host thread) is relative to the port on
the same inputs (every host thread), so that the baseline's ratio can be
restated for the reference itself; the torch port (oracle/hpsi_torch.py) is timed
beside both.  It needs the reference source (the
golden-vector recipe's import, single-rank stand-ins for mpi4py and friends).

    python tests/golden/time_reference_vs_port.py [--ref-src PATH] [--name si64] [--bands 2 8]

Prints one JSON line per band count: median seconds of 5 calls after one
warm-up for both, and reference / port throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import build_system, import_reference, inject  # noqa: E402

from oracle import hpsi as oh  # noqa: E402
from oracle import hpsi_torch as oht  # noqa: E402
from qimpy_gb300 import workloads as wl  # noqa: E402


def median_time(fn, reps: int = 5) -> float:
    fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default="/root/reference/src")
    ap.add_argument("--name", default="si64")
    ap.add_argument("--bands", type=int, nargs="+", default=[2, 8])
    args = ap.parse_args()
    qimpy = import_reference(args.ref_src)
    import torch
    from qimpy.dft.electrons import Wavefunction

    prob = wl.get(args.name)
    mine = wl.make_basis(prob.Gbasis, prob.k, prob.ke_cutoff, prob.grid_shape)
    system = build_system(qimpy, prob, None)
    beta = wl.make_projectors(prob, mine)
    el = inject(qimpy, system, prob, beta)
    threads = os.cpu_count()
    oh.set_threads(threads)
    oht.set_threads(threads)
    D = prob.D_all()
    for nb in args.bands:
        C0 = wl.make_wavefunctions(prob, mine, nb)

        def ref_call():
            C = Wavefunction(el.basis, coeff=torch.from_numpy(C0[None, :, :, None, :]).clone())
            return el.hamiltonian(C)

        def port_call():
            return oh.hamiltonian(mine.ke, prob.V_r, mine.fft_index, mine.n, beta, D, C0)

        H_torch = oht.Hamiltonian(mine.ke, prob.V_r, mine.fft_index, mine.n, beta, D)

        def torch_port_call():
            return H_torch(C0)

        t_ref = median_time(ref_call)
        t_port = median_time(port_call)
        t_tport = median_time(torch_port_call)
        apps = nb * prob.nk
        print(json.dumps({"workload": args.name, "bands": nb, "threads": threads,
                          "reference_s": t_ref, "port_s": t_port,
                          "torch_port_s": t_tport, "reference_over_torch_port": t_tport / t_ref,
                          "reference_band_apps_per_s": apps / t_ref, "port_band_apps_per_s": apps / t_port,
                          "reference_over_port": t_port / t_ref}), flush=True)


if __name__ == "__main__":
    main()
