"""CPU oracle for the plane-wave H.psi / Davidson path -- TEST INFRASTRUCTURE ONLY.

A numpy/scipy restatement of the reference's FP64 algorithm (nohm-devices/qimpy),
each function citing the reference file:line it follows.  The CUDA path's
results are compared with it: only the tests, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline and reference legs import it.  The product (``qimpy_gb300``) never imports it and
has no CPU fallback.

Parity pin: the oracle is checked against golden fixtures produced by running
the reference package itself (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.
"""
