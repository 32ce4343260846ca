"""Build libstab_gb300.so in-tree for sm_103a (no CMake, parallel nvcc)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libstab_gb300.so")
BIN = os.path.join(HERE, "bin")
# command-line drop-ins over the C ABI: `stab < input.dat` (with the sweep
# drivers), `getevec` and the sweep post-processors getab, getax, getalpha
TOOLS = {"stab_gpu": "stab_main.cpp", "getevec_gpu": "getevec_main.cpp", "getab_gpu": "post_main.cpp",
         "getax_gpu": "post_main.cpp", "getalpha_gpu": "post_main.cpp"}

CU_SOURCES = ["prep.cu", "assemble.cu", "lu.cu", "lu_tc.cu", "hqr.cu", "polish.cu", "post.cu", "probe.cu", "mlp.cu", "capi.cu", "fileio.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "stab_gb300.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *NVFLAGS, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(CU_SOURCES))) as ex:
        objs = list(ex.map(_compile, CU_SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    os.makedirs(BIN, exist_ok=True)
    inc = os.path.join(HERE, "..", "include")
    for exe, src in TOOLS.items():
        out = os.path.join(BIN, exe)
        path = os.path.join(CSRC, src)
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(path), os.path.getmtime(LIB)):
            continue
        cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-I", inc, path, "-o", out,
               "-L", HERE, "-lstab_gb300", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
