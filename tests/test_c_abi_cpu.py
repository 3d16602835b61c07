"""The C ABI from plain C (no GPU needed): tests/c_abi/abi_check.c compiles as
C99 against include/qimpy_gb300.h, links the built library and checks version,
workspace sizing and argument validation."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "qimpy_gb300")


def test_c_client_compiles_links_and_validates(tmp_path):
    lib = os.path.join(PKG, "libqimpy_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "abi_check")
    build = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                            os.path.join(ROOT, "tests", "c_abi", "abi_check.c"), "-L", PKG, "-lqimpy_gb300",
                            "-Wl,-rpath," + PKG, "-o", exe], capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "FAIL" not in run.stdout
