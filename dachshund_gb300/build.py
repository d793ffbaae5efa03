"""In-tree build of the CUDA library for sm_103a (no CMake, no setuptools).

``build()`` compiles every ``csrc/*.cu`` translation unit in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` into ``_build/`` and links
``dachshund_gb300/libdsgb300.so``; the C++ API layer in ``lib/`` (the
reference's class interface over the C ABI) is linked into
``dachshund_gb300/libdachshund_gb300.so``.  Rebuilds only what changed.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBSRC = os.path.join(PKG, "lib")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libdsgb300.so")
CXXLIB = os.path.join(PKG, "libdachshund_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run_parallel(jobs, verbose):
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append((cmd, text))
        elif verbose and text.strip():
            print(text)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + t for c, t in failed)
        raise RuntimeError("build failed:\n" + msg)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link; returns the path of the CUDA library."""
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
               + glob.glob(os.path.join(INCLUDE, "*.h")))
    objs, jobs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + headers):
            cmd = [nv] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    _run_parallel(jobs, verbose)
    if jobs or not _newer(LIB, objs):
        _run_parallel([[nv] + ARCH + ["-shared", "-o", LIB] + objs], verbose)

    # C++ API layer (reference class interface) over the C ABI.
    cxx_srcs = sorted(glob.glob(os.path.join(LIBSRC, "*.cc")))
    if cxx_srcs:
        cxx_hdrs = glob.glob(os.path.join(LIBSRC, "*.h"))
        if not _newer(CXXLIB, cxx_srcs + cxx_hdrs + headers + [LIB]):
            cmd = ["g++", "-std=c++11", "-O2", "-fPIC", "-shared", "-I" + LIBSRC, "-I" + INCLUDE,
                   "-o", CXXLIB] + cxx_srcs + ["-L" + PKG, "-ldsgb300",
                                               "-Wl,-rpath,$ORIGIN"]
            _run_parallel([cmd], verbose)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
