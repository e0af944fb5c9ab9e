"""Compile the sm_103a CUDA library ``libuppasd_gb300.so`` in-tree.

Each translation unit is compiled by nvcc in parallel with one ``-gencode``
(compute_103a -> sm_103a); the FP64 parity kernels are compiled with
``--fmad=false`` so products and sums round separately, as in the reference's
Fortran.  Objects go to ``uppasd_gb300/_build``; the shared library is written
next to this file.
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
LIB = os.path.join(HERE, "libuppasd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
# (source, extra flags)
UNITS = [
    ("abi.cu", []),
    ("llg_generic.cu", ["--fmad=false"]),
    ("observables.cu", ["--fmad=false"]),
    ("mc.cu", ["--fmad=false"]),
    ("llg_stencil.cu", []),
    ("llg_mixed.cu", []),
    ("noalloc.cu", []),
    ("mc_batch.cu", []),
    ("tc_host.cu", []),
    ("learned.cu", []),
    ("mc_square.cu", []),
    ("dipole.cu", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libuppasd_gb300.so")


def _compile(src: str, extra: list, verbose: bool, ptxas_info: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if ptxas_info:
        cmd.insert(1, "-Xptxas=-v")
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if ptxas_info or verbose:
        sys.stdout.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "uppasd_gpu.h")
    return os.path.getmtime(hdr) > t


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(UNITS))) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose, ptxas_info), UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
