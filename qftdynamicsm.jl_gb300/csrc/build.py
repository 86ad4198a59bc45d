"""Build libkb2pi.so for sm_103a with nvcc (in-tree, no cmake).

Each translation unit compiles in parallel, then nvcc links the shared
library next to the Python binding. Used by ``__graft_entry__.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
OUT_DIR = os.path.join(PKG, "kb2pi")
BUILD_DIR = os.path.join(PKG, "_build")
SOURCES = ["kb_api.cu", "kb_sunset.cu", "kb_sunset_tc.cu", "kb_memint.cu", "kb_adjoint.cu"]
HEADERS = ["kb_internal.cuh", os.path.join("..", "..", "include", "kb2pi.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC,-O2",
         "-Xptxas", "-warn-spills"]
LIB_NAME = "libkb2pi.so"
DEBUG_LIB_NAME = "libkb2pi_debug.so"


def nvcc() -> str:
    cand = os.environ.get("NVCC") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False, debug: bool = False) -> str:
    """Compile the library; debug=True builds libkb2pi_debug.so with the device-side
    bounds checks of ring, tile and Sigma indices (-DKB_DEBUG) next to it."""
    bdir = os.path.join(BUILD_DIR, "debug") if debug else BUILD_DIR
    os.makedirs(bdir, exist_ok=True)
    hdrs = [os.path.join(HERE, h) for h in HEADERS]
    objs = []
    jobs = []
    for s in SOURCES:
        src = os.path.join(HERE, s)
        obj = os.path.join(bdir, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs + [__file__]):
            cmd = [nvcc()] + ARCH + FLAGS + (["-DKB_DEBUG"] if debug else []) + ["-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for log in ex.map(run, jobs):
            if verbose and log:
                print(log, file=sys.stderr)
    lib = os.path.join(OUT_DIR, DEBUG_LIB_NAME if debug else LIB_NAME)
    if force or _newer(lib, objs):
        run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib


def build_all(verbose: bool = False, force: bool = False) -> list:
    """The release and the KB_DEBUG library, compiled side by side."""
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        return list(ex.map(lambda d: build(verbose, force, d), (False, True)))


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, debug="--debug" in sys.argv))
