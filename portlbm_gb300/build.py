"""Builds libplbm.so in-tree: hand-written sm_103a kernels + the C++ host library.

Every translation unit is compiled in parallel with nvcc for ``-gencode
arch=compute_103a,code=sm_103a`` only, then linked into ``portlbm_gb300/libplbm.so``
with the CUDA runtime linked statically (the library has no run-time dependency on a
particular libcudart path).  Run ``python -m portlbm_gb300.build``.

``build(checked=True)`` (``python -m portlbm_gb300.build --checked``) compiles the same sources
with -DPLBM_CHECKED into ``libplbm_checked.so``: every index of the step kernels is compared with
its buffer's extent and an out-of-range access is skipped and reported as an error.  The package
loads it instead of libplbm.so when PLBM_CHECKED=1 is set in the environment.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libplbm.so")
LIB_CHECKED = os.path.join(PKG, "libplbm_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["k_nptl.cu", "k_lptl.cu", "k_npol.cu", "k_nsol.cu", "k_debug.cu", "plbm_util.cu", "plbm_noalloc.cu", "plbm_batch.cu", "plbm_nn.cu", "plbm_nn_tc.cu"]
CPP_SOURCES = ["plbm_host.cpp", "plbm_benchmark.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime() -> float:
    newest = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(PKG), "include")):
        for f in os.listdir(d):
            newest = max(newest, os.path.getmtime(os.path.join(d, f)))
    return max(newest, os.path.getmtime(__file__))


def up_to_date(checked: bool = False) -> bool:
    lib = LIB_CHECKED if checked else LIB
    return os.path.exists(lib) and os.path.getmtime(lib) >= _sources_mtime()


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    lib = LIB_CHECKED if checked else LIB
    if not force and up_to_date(checked):
        return lib
    build_dir = BUILD + ("_checked" if checked else "")
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()
    defs = ["-DPLBM_CHECKED"] if checked else []
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", *defs, "-I", CSRC,
              "-I", os.path.join(os.path.dirname(PKG), "include")]
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(build_dir, src + ".o")
        jobs.append([cc, *ARCH, *common, "-c", os.path.join(CSRC, src), "-o", obj])
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(cc)), "include")
    for src in CPP_SOURCES:
        obj = os.path.join(build_dir, src + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unknown-pragmas", *defs, "-I", cuda_inc,
                     "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = lib + ".tmp"
    link = [cc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
