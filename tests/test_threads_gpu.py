"""The C ABI called from several host threads, each on its own CUDA stream (as
the serving loop does): every thread's H.psi equals the single-thread result
bit for bit, FP64 (cuBLAS nonlocal) and mixed (tensor-core nonlocal on a side
stream), and for grids of different shared-memory sizes at once."""
from concurrent.futures import ThreadPoolExecutor

import pytest
import torch

from qimpy_gb300 import ops
from qimpy_gb300 import sphere as sp
from qimpy_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _problem(name, dtype):
    p = wl.get(name)
    b = wl.make_basis(p.Gbasis, p.k, p.ke_cutoff, p.grid_shape)
    t = sp.build_tables(b.fft_index, b.n, p.grid_shape)
    ds = sp.DeviceSphere(t, b.ke, DEV, dtype)
    ds.set_potential(torch.from_numpy(p.V_r))
    C = torch.from_numpy(wl.make_wavefunctions(p, b, 8)).to(DEV, dtype)
    beta = torch.from_numpy(wl.make_projectors(p, b)).to(DEV, dtype)
    D = torch.from_numpy(p.D_atom).to(DEV, dtype)
    split = ops.beta_split(beta) if dtype == torch.complex64 else None
    return ds, C, beta, D, split


def _apply(prob, dtype):
    ds, C, beta, D, split = prob
    if dtype == torch.complex64:
        return ops.hamiltonian_mixed(ds, C, split, D)[0]
    return ops.hamiltonian(ds, C, beta, D)[0]


@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_threads_on_own_streams_match_single_thread(dtype):
    probs = [_problem(name, dtype) for name in ("tiny_fcc", "tiny_ortho", "si2")]
    want = [_apply(pr, dtype) for pr in probs]
    torch.cuda.synchronize()

    def work(i):
        s = torch.cuda.Stream(device=DEV)
        s.wait_stream(torch.cuda.default_stream(DEV))
        outs = []
        with torch.cuda.stream(s):
            for rep in range(6):
                outs.append(_apply(probs[(i + rep) % len(probs)], dtype))
        s.synchronize()
        return [(i + rep) % len(probs) for rep in range(6)], outs

    with ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(work, range(8)))
    for idx, outs in results:
        for j, out in zip(idx, outs):
            assert torch.equal(out, want[j])
