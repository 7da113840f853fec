"""Builds the CUDA library (lib/librsvdt.so) and the C host driver
(bin/rsvdt_main) in-tree with nvcc / gcc for sm_103a.

The translation units compile in parallel; the whole build takes well under
a minute. Nothing here is needed at run time once the files exist.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
HOST = os.path.join(PKG_ROOT, "host")
INCLUDE = os.path.join(REPO_ROOT, "include")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
BIN_DIR = os.path.join(PKG_ROOT, "bin")
LIB_PATH = os.path.join(LIB_DIR, "librsvdt.so")
# The bounds-checked debug build (RSVDT_DEBUG), used by the tests only.
DEBUG_LIB_PATH = os.path.join(LIB_DIR, "librsvdt_debug.so")
MAIN_PATH = os.path.join(BIN_DIR, "rsvdt_main")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
CU_SOURCES = ["api.cu", "step.cu", "dense.cu", "batch.cu", "mlp.cu", "trans.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed: " + " ".join(cmd) + "\n" + res.stdout)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, debug: bool = False) -> str:
    """Compiles csrc/*.cu into lib/librsvdt.so (static CUDA runtime); with
    debug=True, into lib/librsvdt_debug.so with the stage kernels' index
    checks (-DRSVDT_DEBUG)."""
    os.makedirs(LIB_DIR, exist_ok=True)
    obj_dir = os.path.join(LIB_DIR, "obj_debug" if debug else "obj")
    os.makedirs(obj_dir, exist_ok=True)
    out_path = DEBUG_LIB_PATH if debug else LIB_PATH
    flags = NVCC_FLAGS + (["-DRSVDT_DEBUG"] if debug else [])
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, "common.cuh"), os.path.join(INCLUDE, "rsvdt.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(obj_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *flags, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(out_path, objs):
        _run([nvcc, *ARCH, "-shared", "-o", out_path, *objs, "-cudart", "static"])
    if verbose:
        print("built", out_path)
    return out_path


def build_host(force: bool = False) -> str | None:
    """Compiles the C drop-in driver for main.c (bin/rsvdt_main) against
    lib/librsvdt.so. Returns None when there are no host sources."""
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".c")) if os.path.isdir(HOST) else []
    if not srcs:
        return None
    os.makedirs(BIN_DIR, exist_ok=True)
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [LIB_PATH]
    if force or _stale(MAIN_PATH, deps):
        _run(["gcc", "-O2", "-std=c11", "-fopenmp", "-Wall", "-I", INCLUDE, "-I", HOST, *srcs, "-o", MAIN_PATH,
              "-L", LIB_DIR, "-lrsvdt", "-Wl,-rpath,$ORIGIN/../lib", "-lm"])
    return MAIN_PATH


def build_all(force: bool = False) -> None:
    build_library(force=force)
    build_host(force=force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("ok")
