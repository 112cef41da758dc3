"""Build recipe of the GB300 PIC library (libminipic_gb300.so) and its driver.

Compiles every translation unit for sm_103a only, in parallel, in-tree under
_build/.  Used by __graft_entry__.build() and by the test fixtures; needs
nvcc and g++, no cmake.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libminipic_gb300.so")
DRIVER = os.path.join(BUILD, "minipic_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
              "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["kernels.cu", "solver.cu", "mg.cu", "api.cu", "batch.cu"]
CXX_SOURCES = ["mesh_host.cpp", "mg_host.cpp"]
HEADERS = ["mpg_internal.h", "mpg_kernels.h", "mpg_device.cuh", "mpg_walk.cuh", "mpg_mg.cuh"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def build(force=False, verbose=False, ptxas_info=False, out_dir=None, extra_nvcc=()):
    """Compile the library (and the driver) into out_dir (default _build/)."""
    out = out_dir or BUILD
    lib = os.path.join(out, "libminipic_gb300.so")
    driver = os.path.join(out, "minipic_gb300")
    os.makedirs(out, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "minipic_gb300.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            extra = (["-Xptxas", "-v"] if ptxas_info else []) + list(extra_nvcc)
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    outs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or not os.path.exists(lib):
        _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    drv_src = os.path.join(CSRC, "main.cpp")
    if os.path.exists(drv_src) and (force or _newer(driver, [drv_src, lib, os.path.join(INCLUDE, "minipic_gb300.hpp")])):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, drv_src, "-o", driver, "-L" + out, "-lminipic_gb300",
              "-Wl,-rpath," + out])
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
