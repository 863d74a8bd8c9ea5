"""Builds liboxgb.so (the CUDA kernels and the C ABI) in-tree with nvcc for sm_103a.

Translation units compile in parallel; the library links the CUDA runtime statically, so the
only run-time dependency is the driver.  Output: oxdna_gb300/_build/liboxgb.so.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboxgb.so")
TOOLS = os.path.join(OUT, "liboxgb_tools.so")
SOURCES = ["forces.cu", "lists.cu", "integrate.cu", "api.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall,-Wno-unused-function",
         "-Xptxas", "-warn-spills"]


# The force kernels divide in FP32 with the fast (2-ulp) division: -2.7 us per force launch at
# 40k, with the force error against FP64 unchanged within its spread (normwise 1.3e-6 -> 1.5e-6,
# per-nucleotide maximum 3.5e-5 -> 3.6e-5); square roots stay IEEE (the fast ones raised the
# per-nucleotide maximum to 1.3e-4).  The list build keeps IEEE division (its geometry must
# match the reference's bit for bit) and spells it out with __fdiv_rn in any case.
FILE_FLAGS = {"forces.cu": ["-prec-div=false"]}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liboxgb.so")
    return exe


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "oxgb.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        cmd = [exe, *ARCH, *FLAGS, *FILE_FLAGS.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as pool:
        objs = list(pool.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([exe, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_tools()
    return LIB


def build_tools() -> str:
    """Host-only helpers (the force kernel's FLOP counter), g++."""
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", CSRC, "-x", "c++",
           os.path.join(CSRC, "flopcount.cpp"), "-o", TOOLS]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"tools build failed:\n{r.stderr}")
    return TOOLS


if __name__ == "__main__":
    print(build(force=True, verbose=True))
