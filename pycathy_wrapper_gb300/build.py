"""Build libcathy_gb300.so in-tree (pycathy_wrapper_gb300/_build/).

Compiles the CUDA engine for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``) with nvcc; host code with portable flags
so the same recipe works on x86_64 and aarch64 hosts.  Translation units are
compiled in parallel.
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
LIB = os.path.join(OUT, "libcathy_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "capi.cu", "mesh.cpp", "noalloc.cu", "learned.cu"]
HEADERS = ["engine.h", "kernels.cuh", "mesh.h", "learned.h"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build")
    return p


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "cathy_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo",
              "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [nv] + ARCH + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nv] + common + ["-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
