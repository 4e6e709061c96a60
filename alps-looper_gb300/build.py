"""Build the engine library lib/liblooper_gb300.so (sm_103a only) and lib/loop_gpu.

    python alps-looper_gb300/build.py [--force] [--verbose]

Translation units are compiled in parallel with nvcc and linked into one shared library that
exports the C ABI of include/looper_gpu.h.  Host code is compiled with -ffp-contract=off so that
host-side float formulas are never fused.  loop_gpu (csrc/loop_gpu.cpp) is looper's standalone
loop program on the engine: a plain C++ program linked against the library.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "liblooper_gb300.so")
EXE = os.path.join(LIBDIR, "loop_gpu")
SOURCES = ["lg_engine.cu", "lg_host.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "looper_gpu.h"))
    return max(os.path.getmtime(f) for f in files)


def build_driver(nv: str) -> str:
    """lib/loop_gpu, found next to the library at run time (rpath $ORIGIN)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for loop_gpu")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nv))), "lib64")
    tmp = EXE + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(os.path.dirname(HERE), "include"),
           os.path.join(CSRC, "loop_gpu.cpp"), "-o", tmp, "-L" + LIBDIR, "-llooper_gb300",
           "-Wl,-rpath,$ORIGIN:" + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("loop_gpu build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, EXE)
    return EXE


def build(force: bool = False, verbose: bool = False) -> str:
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps()
            and os.path.exists(EXE) and os.path.getmtime(EXE) >= os.path.getmtime(LIB)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + CSRC, "-I" + os.path.join(os.path.dirname(HERE), "include")]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nv] + ARCH + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < _deps():
        with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
            objs = list(ex.map(compile_one, SOURCES))
        tmp = LIB + ".tmp"
        cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    build_driver(nv)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
