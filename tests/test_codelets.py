"""The generated DFT codelets, executed as Python, against numpy's FFT (CPU)."""
import importlib.util
import os
import re

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GEN = os.path.join(HERE, "..", "qimpy_gb300", "csrc", "gen_codelets.py")


def _load_gen():
    spec = importlib.util.spec_from_file_location("gen_codelets", GEN)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _run_as_python(gen, R, s, x):
    e = gen.Emitter()
    xs = [(f"re[{j}]", f"im[{j}]") for j in range(R)]
    X = gen.dft(e, xs, s)
    env = {"re": list(x.real), "im": list(x.imag), "T": float}
    for line in e.lines:
        m = re.match(r"\s*const T (\w+) = (.*);", line)
        env[m.group(1)] = eval(m.group(2), env)
    return np.array([eval(a, env) + 1j * eval(b, env) for a, b in X])


@pytest.mark.parametrize("R", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16])
@pytest.mark.parametrize("s", [-1, 1])
def test_codelet_matches_dft(R, s):
    gen = _load_gen()
    rng = np.random.default_rng(R * 10 + (s > 0))
    x = rng.standard_normal(R) + 1j * rng.standard_normal(R)
    got = _run_as_python(gen, R, s, x)
    want = np.fft.fft(x) if s < 0 else np.fft.ifft(x) * R
    assert np.abs(got - want).max() <= 1e-14 * max(1.0, np.abs(want).max())


def test_header_is_current():
    """The committed header equals what the generator prints."""
    import io
    import contextlib

    gen = _load_gen()
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        gen.main()
    with open(os.path.join(HERE, "..", "qimpy_gb300", "csrc", "codelets.cuh")) as f:
        assert f.read() == buf.getvalue()
