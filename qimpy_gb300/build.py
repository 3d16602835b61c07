"""Build ``libqimpy_gb300.so`` in-tree for sm_103a (GB300).

Each ``csrc/*.cu`` is compiled by nvcc in parallel into ``_build/``, then
linked with cuSOLVER into ``qimpy_gb300/libqimpy_gb300.so``.  The measurement
and test aids (``csrc/aux/*.cu``, include/qimpy_gb300_aux.h) go into
``libqimpy_gb300_aux.so``, linked against the main library.  The DFT codelet
header is regenerated when its generator is newer.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libqimpy_gb300.so")
AUX_LIB = os.path.join(PKG, "libqimpy_gb300_aux.so")
AUX_SRC = os.path.join(CSRC, "aux")
#: Range-checked variant (-DQGB_DEBUG_CHECKS), loaded when QGB_DEBUG_CHECKS=1.
DEBUG_LIB = os.path.join(PKG, "libqimpy_gb300_debug.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build qimpy_gb300")
    return path


def _mtime(p: str) -> float:
    return os.path.getmtime(p) if os.path.exists(p) else -1.0


def _regen_codelets() -> None:
    gen = os.path.join(CSRC, "gen_codelets.py")
    hdr = os.path.join(CSRC, "codelets.cuh")
    if _mtime(hdr) < _mtime(gen):
        out = subprocess.run([sys.executable, gen], check=True, capture_output=True, text=True).stdout
        with open(hdr, "w") as f:
            f.write(out)


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def aux_sources() -> list[str]:
    return sorted(os.path.join(AUX_SRC, f) for f in os.listdir(AUX_SRC) if f.endswith(".cu"))


def _compile(src: str, extra: list[str], build_dir: str = BUILD) -> str:
    prefix = "aux_" if os.path.dirname(src) == AUX_SRC else ""
    obj = os.path.join(build_dir, prefix + os.path.basename(src)[:-3] + ".o")
    newest_dep = max([_mtime(src)] + [_mtime(h) for h in headers()])
    if _mtime(obj) >= newest_dep:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-I", INCLUDE, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> str:
    """Compile and link the library (or its range-checked debug variant); returns its path."""
    build_dir = BUILD + ("_debug" if debug else "")
    lib = DEBUG_LIB if debug else LIB
    extra = ["-DQGB_DEBUG_CHECKS"] if debug else []
    os.makedirs(build_dir, exist_ok=True)
    _regen_codelets()
    if force:
        for f in os.listdir(build_dir):
            if f.endswith(".o"):
                os.remove(os.path.join(build_dir, f))
    srcs = sources()
    asrcs = [] if debug else aux_sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs) + len(asrcs), os.cpu_count() or 4)) as ex:
        all_objs = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs + asrcs))
    objs, aux_objs = all_objs[: len(srcs)], all_objs[len(srcs):]
    relinked = False
    if force or _mtime(lib) < max(_mtime(o) for o in objs):
        soname = os.path.basename(lib)
        cmd = [nvcc()] + ARCH + ["-shared", "-Xlinker", f"-soname,{soname}", "-o", lib + ".tmp"] + objs + ["-lcusolver"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(lib + ".tmp", lib)
        relinked = True
        if verbose:
            print(f"built {lib}")
    if aux_objs and (force or relinked or _mtime(AUX_LIB) < max(_mtime(o) for o in aux_objs)):
        cmd = ([nvcc()] + ARCH + ["-shared", "-o", AUX_LIB + ".tmp"] + aux_objs +
               ["-L", PKG, "-lqimpy_gb300", "-Xlinker", "-rpath,$ORIGIN"])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of the aux library failed:\n{r.stdout}\n{r.stderr}")
        os.replace(AUX_LIB + ".tmp", AUX_LIB)
        if verbose:
            print(f"built {AUX_LIB}")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, debug="--debug" in sys.argv)
