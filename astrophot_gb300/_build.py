"""Build recipe for the CUDA library (``libastrophot_gb300.so``), sm_103a only.

``python -m astrophot_gb300._build`` compiles the translation units in
parallel and links them into the package directory.  No cmake, no torch
extension machinery: plain ``nvcc`` with ``-gencode arch=compute_103a,code=sm_103a``.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libastrophot_gb300.so")
SOURCES = ("ap_kernels.cu", "ap_lm.cu", "ap_capi.cu", "ap_noalloc.cu", "ap_cnn.cu", "ap_scene.cu", "ap_refinit.cu",
           "ap_fft.cu", "ap_segmap.cu", "ap_tcgemm.cu", "ap_solve.cu")
# per-file flags: the initial-value heuristics round like numpy (no FMA contraction)
EXTRA = {"ap_refinit.cu": ("-fmad=false",)}
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")
FLAGS = ("-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2")


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build astrophot_gb300")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library if any source is newer than it; returns its path."""
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "astrophot_gb300.h"))
    if not force and _newer(LIB, deps):
        return LIB
    build_dir = os.path.join(HERE, "_build")
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(build_dir, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *EXTRA.get(src, ()), "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
