"""Continuous-batching eigensolve server: a request gives the same eigenvalues
alone and in a mix with other requests that arrive while it is on the GPU;
failures stay isolated to their request."""
import numpy as np
import pytest

from qimpy_gb300 import batch as bt
from qimpy_gb300 import serve as sv

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _specs():
    return bt.make_batch_specs(count=5, seed=9, bands_range=(4, 8), k_range=(1, 2), ke_range=(5.0, 9.0),
                               atoms_range=(2, 3), sides=(10.0, 12.0))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-12)])
def test_same_result_alone_and_in_mix(precision, tol):
    specs = _specs()
    alone = sv.EigenServer(DEV, precision=precision, eig_threshold=1e-7, residual_threshold=None)
    r0 = sv.EigenRequest(0, specs[0], 6, arrival=0.0)
    alone.run([r0], realtime=False)
    assert r0.status == "done", r0.error
    mix = sv.EigenServer(DEV, precision=precision, eig_threshold=1e-7, residual_threshold=None)
    reqs = [sv.EigenRequest(0, specs[0], 6, arrival=0.0)] + [
        sv.EigenRequest(i, specs[i], 5, arrival=0.01 * i) for i in range(1, 5)]
    rep = mix.run(reqs, realtime=True)
    assert rep["done"] == 5, [(r.rid, r.status, r.error) for r in mix.finished]
    assert mix.ticks < sum(r.iterations for r in reqs)  # requests shared ticks (batched H.psi)
    assert max(mix.tick_band_apps) > max(r.spec.n_bands for r in reqs)
    np.testing.assert_allclose(reqs[0].eig, r0.eig, rtol=0, atol=tol)


def test_failed_request_does_not_disturb_others():
    specs = _specs()
    srv = sv.EigenServer(DEV, precision="mixed", eig_threshold=1e-7, residual_threshold=None)
    good = sv.EigenRequest(0, specs[0], 6, arrival=0.0)
    too_many = sv.EigenRequest(1, specs[1], 100000, arrival=0.0)  # n_bands >= basis size
    ref = sv.EigenServer(DEV, precision="mixed", eig_threshold=1e-7, residual_threshold=None)
    solo = sv.EigenRequest(0, specs[0], 6, arrival=0.0)
    ref.run([solo], realtime=False)
    srv.run([good, too_many], realtime=False)
    assert too_many.status == "rejected" and "exceeds" in too_many.error
    assert good.status == "done"
    np.testing.assert_allclose(good.eig, solo.eig, rtol=0, atol=1e-12)


def test_admission_by_memory_budget():
    specs = _specs()
    srv = sv.EigenServer(DEV, precision="mixed", eig_threshold=1e-6, residual_threshold=None)
    need = srv.estimate_bytes(specs[0], 6)
    srv.budget = int(need * 1.5)  # room for one request at a time
    reqs = [sv.EigenRequest(i, specs[0], 6, arrival=0.0) for i in range(3)]
    rep = srv.run(reqs, realtime=False)
    assert rep["done"] == 3
    admits = sorted(r.t_admit for r in reqs)
    dones = sorted(r.t_done for r in reqs)
    assert admits[1] >= dones[0] - 1e-9 and admits[2] >= dones[1] - 1e-9  # one at a time
