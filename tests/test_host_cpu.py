"""Host-side logic on CPU: the batched-instance and serving-stream generators,
the grid rule, the serving memory estimate, and that the product path fails
loudly (no CPU fallback) when its library is missing."""
import math
import os
import subprocess
import sys
import types

import numpy as np
import torch

from qimpy_gb300 import batch as bt
from qimpy_gb300 import serve as sv
from qimpy_gb300 import sphere as sp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_grid_rule():
    # qimpy/grid/_grid.py:114-127: 4 * ceil(L sqrt(2 * 4 Ecut) / pi / 4), then the
    # next size that factors into two codelet sizes.
    for L, E in [(10.0, 15.0), (14.0, 20.0), (18.0, 22.0), (22.0, 25.0), (20.52, 20.0)]:
        n_min = 4 * math.ceil(L * math.sqrt(8.0 * E) / math.pi / 4)
        n = bt.reference_grid(L, E)
        assert n >= n_min and n % 4 == 0 and n - n_min < 16
        sp.factor_axis(n)  # factorable


def test_batch_specs_deterministic_and_in_range():
    a = bt.make_batch_specs(count=40, seed=31)
    b = bt.make_batch_specs(count=40, seed=31)
    for x, y in zip(a, b):
        assert x.side == y.side and x.grid == y.grid and x.n_bands == y.n_bands
        assert np.array_equal(x.positions, y.positions) and np.array_equal(x.k, y.k)
    assert {s.side for s in a} <= set(bt.CUBIC_SIDES)
    assert all(2 <= s.n_atoms <= 16 and 8 <= s.n_bands <= 64 and 1 <= len(s.k) <= 8 for s in a)
    assert all(15.0 <= s.ke_cutoff <= 25.0 for s in a)
    assert len({s.grid for s in a}) > 3  # uneven grids


def test_poisson_stream_arrivals_and_band_caps():
    specs = bt.make_batch_specs(count=200, seed=41)
    reqs = sv.poisson_stream(specs, rate_hz=200.0, seed=41)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate(([0.0], t)))
    assert abs(gaps.mean() - 1 / 200.0) < 0.3 / 200.0  # mean inter-arrival 1/rate
    for r in reqs:
        n_est = (2.0 * r.spec.ke_cutoff) ** 1.5 * r.spec.side ** 3 / (6 * math.pi ** 2)
        assert 4 <= r.n_bands <= max(160, 4) and r.n_bands <= max(4, 0.3 * n_est)
    again = sv.poisson_stream(specs, rate_hz=200.0, seed=41)
    assert [(r.arrival, r.n_bands) for r in again] == [(r.arrival, r.n_bands) for r in reqs]


def _fake_server(dtype, residual_threshold=None):
    fake = types.SimpleNamespace(dtype=dtype, residual_threshold=residual_threshold)
    fake.bands_extra = lambda nb, n_min: sv.EigenServer.bands_extra(fake, nb, n_min)
    return fake


def test_serving_extra_bands():
    """The reference's default without a residual target; with one, at least 4
    and a quarter of the bands, within Davidson's limit 2 (n_bands + extra) < n_min."""
    plain, target = _fake_server(torch.complex64), _fake_server(torch.complex64, 1e-6)
    assert [plain.bands_extra(nb, 10000) for nb in (6, 10, 11, 160)] == [1, 1, 2, 16]
    assert [target.bands_extra(nb, 10000) for nb in (6, 10, 40, 160)] == [4, 4, 10, 40]
    assert target.bands_extra(6, 21) == 4 and target.bands_extra(6, 19) == 3  # capped: 2 (6 + 3) < 19
    assert target.bands_extra(8, 17) == 1  # never below the reference's default


def test_serving_memory_estimate_grows_with_work():
    spec = bt.make_batch_specs(count=1, seed=3)[0]
    fake = _fake_server(torch.complex64)
    fake64 = _fake_server(torch.complex128)
    small = sv.EigenServer.estimate_bytes(fake, spec, 8)
    large = sv.EigenServer.estimate_bytes(fake, spec, 64)
    assert 0 < small < large
    assert sv.EigenServer.estimate_bytes(fake64, spec, 8) > small


def test_product_path_fails_loudly_without_library(tmp_path):
    """With the library absent, the first use raises instead of falling back."""
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "from qimpy_gb300 import _lib\n"
        "_lib.LIB_PATH = %r\n"
        "try:\n"
        "    _lib.lib()\n"
        "except Exception as e:\n"
        "    print('raised', type(e).__name__)\n"
        "else:\n"
        "    print('loaded')\n" % (ROOT, str(tmp_path / "missing.so")))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert "raised" in out.stdout, out.stdout + out.stderr


def test_randomize_selected_matches_oracle():
    """The GPU Davidson's null-band re-randomisation reproduces the reference's
    seeded xorshift generator (restated in the oracle), run here on CPU tensors."""
    from oracle import davidson as od
    from qimpy_gb300 import davidson as dv
    from qimpy_gb300.electrons import Wavefunction

    rng = np.random.default_rng(3)
    nk, nb, n_tot = 2, 5, 40
    n = np.array([37, 40])
    ke = rng.uniform(0.0, 3.0, (nk, n_tot))
    mask = np.arange(n_tot)[None, :] < n[:, None]
    basis = types.SimpleNamespace(n_max=int(n.max()), ke=torch.from_numpy(ke), mask=torch.from_numpy(mask))
    C = Wavefunction(basis, coeff=torch.zeros((nk, nb, n_tot), dtype=torch.complex128))
    i_k, i_b = np.array([0, 1, 1]), np.array([3, 0, 4])
    dv.randomize_selected(C, torch.from_numpy(i_k), torch.from_numpy(i_b), seed=7)
    want = np.zeros((nk, nb, n_tot), dtype=np.complex128)
    od.randomize_selected(want, i_k, i_b, 7, n, int(n.max()), nk, ke)
    assert np.allclose(C.coeff.numpy(), want, rtol=1e-13, atol=0)
