"""Builds libcmdg.so in-tree (``climatemachine.jl_gb300/_build/libcmdg.so``).

Every translation unit is compiled by nvcc for sm_103a only, in parallel,
then linked into one shared library with a plain C ABI (``include/cmdg.h``).
No cmake, no torch extension machinery: the library is loaded with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcmdg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-Xptxas",
              "-warn-spills"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libcmdg.so")
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _needs_build(objs) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "cmdg.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    objs = [os.path.join(OUT, os.path.basename(s) + ".o") for s in srcs]
    if not force and not _needs_build(objs):
        return LIB
    exe = nvcc()

    def compile_one(pair):
        src, obj = pair
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-x", "cu" if src.endswith(".cu") else "c++", "-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [exe, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose:
        for lg in logs:
            if lg.strip():
                print(lg, file=sys.stderr)
    tmp = LIB + ".tmp"
    r = subprocess.run([exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
