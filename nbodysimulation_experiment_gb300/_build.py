"""Build of the in-tree CUDA library ``libsph_gb300.so`` (sm_103a only).

The library is compiled with ``--fmad=false`` and ``-ffp-contract=off`` so
that neither nvcc nor the host compiler fuses ``a*b+c``: the reference's FP32
arithmetic rounds after every multiply and add.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from typing import List

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_NAME = "libsph_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)
BUILD_DIR = os.path.join(PKG_DIR, "_build")

SOURCES = [
    "sph_kernels.cu", "sph_springs.cu", "sph_learned.cu", "sph_render.cu", "sph_api.cu", "sph_noalloc.cu", "mpnn_gemm.cu",
    "mpnn_kernels.cu", "mpnn.cu", "sph_scenarios.cpp",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off"]
# The learned frame's kernels are checked against an FP64 reference within a
# tolerance, not bit for bit: fused multiply-adds are allowed there.
FMA_SOURCES = {"mpnn_gemm.cu", "mpnn.cu", "mpnn_kernels.cu"}


def _flags(src: str) -> List[str]:
    if src in FMA_SOURCES:
        return [f for f in NVCC_FLAGS if f != "--fmad=false"]
    return NVCC_FLAGS


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 SPH library needs the CUDA toolkit to build")


def _deps() -> List[str]:
    out = []
    for name in os.listdir(CSRC):
        if name.endswith((".cu", ".cuh", ".h", ".cpp")):
            out.append(os.path.join(CSRC, name))
    for h in ("sph_gb300.h", "sph_mpnn.h"):
        out.append(os.path.join(os.path.dirname(PKG_DIR), "include", h))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(d) <= t for d in _deps() if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library in place (parallel per translation unit)."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [cc] + ARCH + _flags(src) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    tmp = LIB_PATH + ".tmp"
    link = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s" % r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
