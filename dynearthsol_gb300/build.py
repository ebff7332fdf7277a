"""In-tree build of libdesgpu.so for sm_103a (nvcc, no cmake).

The translation units compile in parallel; the library lands next to this
file, where ``capi.load_library`` finds it.  The kernels are compiled
without FMA contraction (``--fmad=false``) so that FP64 arithmetic follows
the reference's expression order operation by operation.  The reverse-mode
kernels (des_adjoint.cu) are the exception: their results are derivatives,
checked against finite differences rather than against the reference's
bits, and on GB300 every FP64 instruction saved counts, so they are compiled
with contraction.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdesgpu.so")

SOURCES = ["des_kernels.cu", "des_mixed.cu", "des_capi.cu", "des_noalloc.cu", "des_adjoint.cu",
           "des_adjoint_host.cu", "des_output.cu", "des_phase.cu", "des_topology.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off"]
CONTRACTED = {"des_adjoint.cu"}   # compiled with --fmad=true (see the module docstring)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    m = 0.0
    for f in os.listdir(CSRC):
        m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    hdr = os.path.join(os.path.dirname(HERE), "include", "desgpu.h")
    return max(m, os.path.getmtime(hdr))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libdesgpu.so (skipped when it is newer than every source)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        flags = [("--fmad=true" if f == "--fmad=false" and src in CONTRACTED else f) for f in NVCC_FLAGS]
        cmd = [nv, *ARCH, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
