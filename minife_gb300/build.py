"""Build the CUDA library libminife_gb300.so in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library next to this file.  mfe_assemble.cu is compiled with
-fmad=false: the Hex8 element math must round every multiply and add
separately to match the reference bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libminife_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
SOURCES = {
    "mfe_api.cu": [],
    "mfe_assemble.cu": ["-fmad=false"],
    "mfe_spmv.cu": [],
    "mfe_spmv_box.cu": [],
    "mfe_noalloc.cu": [],
    "mfe_mixed.cu": [],
    "mfe_multi.cu": [],
    "mfe_batch.cu": [],
    "mfe_dump.cu": [],
    "mfe_pcg.cu": [],
    "mfe_ell.cu": [],
    "mfe_adjoint.cu": [],
    "mfe_stencil.cu": [],
    "mfe_stencil64.cu": [],
    "mfe_cg.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
    if verbose:
        sys.stderr.write(res.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(os.path.join(HERE, "miniFE.x")):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(os.path.join(HERE, "miniFE.x")))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(HERE, "host", f) for f in os.listdir(os.path.join(HERE, "host"))]
    deps.append(os.path.join(ROOT, "include", "minife_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if sources changed) and return the path of the library."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), SOURCES.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    build_driver()
    return LIB


DRIVER = os.path.join(HERE, "miniFE.x")


def build_driver() -> str:
    """The miniFE.x command-line driver (host C++ over the C ABI)."""
    src = os.path.join(HERE, "host", "main.cpp")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-L", HERE,
           "-lminife_gb300", "-Wl,-rpath,$ORIGIN", "-o", DRIVER + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (res.stdout, res.stderr))
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
