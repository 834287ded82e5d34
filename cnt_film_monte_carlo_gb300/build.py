"""Build the engine's native code in-tree: libcntkmc.so (CUDA, sm_103a), its bounds-checked
twin libcntkmc_check.so and the drop-in driver.

nvcc cross-compiles sm_103a on a machine without a GPU.  Objects go to ``_build/`` next to
this file; the shared libraries and the ``cntkmc_run`` driver land in this package directory.
libcntkmc_check.so is the same library with the hop, neighbour-build and contacts kernels
compiled with -DKMC_CHECK: device bounds checks on site, row-block and link indices, MSD and
slab bins and Philox counters, reported as KMC_ERR_CHECK (engine.Engine(checked=True)).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libcntkmc.so")
LIB_CHECK = os.path.join(HERE, "libcntkmc_check.so")
DRIVER = os.path.join(HERE, "cntkmc_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-Wall", f"-I{INCLUDE}",
             f"-I{CSRC}"]

CU_SOURCES = ["kmc_kernels.cu", "kmc_mixed_small.cu", "kmc_mixed_large.cu", "cntkmc_api.cu", "kmc_noalloc.cu", "kmc_contacts.cu",
              "kmc_mlp.cu", "kmc_exciton.cu"]
CXX_SOURCES = ["kmc_host.cpp"]
CHECK_SOURCES = ["kmc_kernels.cu", "kmc_mixed_small.cu", "kmc_mixed_large.cu", "kmc_contacts.cu"]  # -DKMC_CHECK twins
DRIVER_SOURCES = ["driver.cpp"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    """Compile (when sources changed) and return the path of libcntkmc.so."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    headers.append(os.path.join(INCLUDE, "cntkmc.h"))
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    check_objs = []
    for src in CU_SOURCES:
        if src not in CHECK_SOURCES:
            check_objs.append(os.path.join(BUILD, src + ".o"))
            continue
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, "check_" + src + ".o")
        check_objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + ["-DKMC_CHECK", "-c", s, "-o", o])
    check_objs += [os.path.join(BUILD, src + ".o") for src in CXX_SOURCES]
    out = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for text in ex.map(_run, jobs):
            out.append(text)
    if force or jobs or _stale(LIB, objs):
        out.append(_run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-ldl", "-lpthread"]))
    if force or jobs or _stale(LIB_CHECK, check_objs):
        out.append(_run([nvcc()] + ARCH + ["-shared", "-o", LIB_CHECK] + check_objs + ["-lcudart", "-ldl", "-lpthread"]))
    drv_src = [os.path.join(CSRC, s) for s in DRIVER_SOURCES]
    if all(os.path.exists(s) for s in drv_src) and (force or _stale(DRIVER, drv_src + headers + [LIB])):
        out.append(_run(["g++"] + CXX_FLAGS + ["-o", DRIVER] + drv_src + ["-L" + HERE, "-lcntkmc",
                                                                         "-Wl,-rpath,$ORIGIN"]))
    if verbose:
        print("\n".join(t for t in out if t.strip()))
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
