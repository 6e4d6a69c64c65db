"""Build libose3d.so (and the ose_3d host driver) in-tree with nvcc for sm_103a.

    python 3d-ose_gb300/build.py [--force]

Objects go to 3d-ose_gb300/_build/, the library to 3d-ose_gb300/lib/.  Each
translation unit compiles in its own process, in parallel.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libose3d.so")
DRIVER = os.path.join(LIBDIR, "ose_3d")
INCLUDE = os.path.abspath(os.path.join(HERE, "..", "include"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr", "-I" + INCLUDE]
SOURCES = ["ose_kernels.cu", "ose_plane.cu", "ose_capi.cu", "ose_host.cpp", "ose_noalloc.cu", "ose_io.cpp",
           "ose_batch.cu", "ose_tensor.cu", "ose_learn.cu", "ose_learn_tc.cu", "ose_cols.cu", "ose_bluestein.cu"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "ose3d.h")]


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if force or _stale(obj, [src] + _headers()):
        cmd = [nvcc()] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc()] + ["-x", "cu"] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        subprocess.run(cmd, check=True)
    drv_src = os.path.join(HERE, "driver", "ose_3d.cpp")
    if os.path.exists(drv_src) and (force or _stale(DRIVER, [drv_src, LIB])):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, drv_src, "-o", DRIVER,
               "-L" + LIBDIR, "-lose3d", "-Wl,-rpath,$ORIGIN"]
        subprocess.run(cmd, check=True)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    build(force=a.force, verbose=True)
    sys.exit(0)
