"""Builds the in-tree shared library libi2gb300.so (CUDA, sm_103a) with plain nvcc.

The translation units are compiled in parallel and linked with `nvcc -shared`; the result sits
next to this file, where integrator2_gb300._lib loads it.  No torch extension machinery, no
cmake.  Needs only the CUDA toolkit (nvcc cross-compiles without a GPU).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libi2gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["i2_capi.cu", "i2_kernels_fp64.cu", "i2_kernels_mixed.cu", "i2_kernels_df.cu", "i2_calibrate.cu", "i2_noalloc.cu", "i2_adjoint.cu",
           "i2_pairs.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without floating-point contraction (GCC fuses a*b+c on Arm by default),
# so the host arithmetic the pair builders share rounds the same on every host
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off",
         "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "integrator2_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and not _stale():
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = OUT + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


CLI_SRC = os.path.join(HERE, "cli", "integrator2test3D.cpp")
CLI_OUT = os.path.join(HERE, "integrator2test3D")


def build_cli() -> str:
    """the command-line driver (host C++ over the C-ABI), linked to libi2gb300.so next to it"""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"), CLI_SRC,
                        "-o", CLI_OUT, "-L", HERE, "-li2gb300", "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stderr}")
    return CLI_OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
