"""In-tree build of the native parts (no pip install, no cmake).

* ``libgravidy_gb300.so``: the CUDA kernels and the C ABI of
  include/gravidy_gb300.h, compiled for sm_103a only
  (``-gencode arch=compute_103a,code=sm_103a``), one nvcc process per
  translation unit, in parallel, then linked with nvcc.
* ``gravidy-gb300``: the command-line program (C++ host code over the C ABI).
* ``bounds/libgravidy_gb300.so`` (``build_library(bounds_check=True)``, or
  ``python -m gravidy_gb300.build --bounds-check``): the same library with
  ``-DH4_BOUNDS_CHECK``, whose kernels check every index range they touch
  and report a violation instead of making the access.  Loaded in place of
  the normal library when GRAVIDY_GB300_LIB names it.

Outputs go to gravidy_gb300/_build/ (git-ignored).  ``python -m
gravidy_gb300.build`` runs it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOSTSRC = os.path.join(CSRC, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libgravidy_gb300.so")
CLI = os.path.join(BUILD, "gravidy-gb300")
BOUNDS_LIB = os.path.join(BUILD, "bounds", "libgravidy_gb300.so")

CUDA_SOURCES = ["h4_capi.cu", "h4_step_kernels.cu", "h4_force_fp64.cu", "h4_energy.cu", "h4_probe.cu",
                "h4_noalloc.cu", "h4_force_mixed.cu", "h4_ensemble.cu", "h4_diagnostics.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
# Extra nvcc flags (e.g. -D build knobs of the kernels), space separated.
NVCC_FLAGS += os.environ.get("GRAVIDY_GB300_NVCC_FLAGS", "").split()


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gravidy_gb300")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, bounds_check: bool = False) -> str:
    out_dir = os.path.dirname(BOUNDS_LIB) if bounds_check else BUILD
    lib = BOUNDS_LIB if bounds_check else LIB
    flags = NVCC_FLAGS + (["-DH4_BOUNDS_CHECK"] if bounds_check else [])
    os.makedirs(out_dir, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "gravidy_gb300.h"))
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv, *ARCH, *flags, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if force or jobs or _stale(lib, objs):
        _run([nv, *ARCH, "-shared", "-o", lib, *objs, "-lcudart"])
    return lib


def build_cli(force: bool = False) -> str | None:
    srcs = sorted(os.path.join(HOSTSRC, f) for f in os.listdir(HOSTSRC) if f.endswith(".cpp")) \
        if os.path.isdir(HOSTSRC) else []
    if not srcs:
        return None
    hdrs = [os.path.join(HOSTSRC, f) for f in os.listdir(HOSTSRC) if f.endswith(".hpp")]
    if force or _stale(CLI, srcs + hdrs + [LIB]):
        gxx = os.environ.get("CXX", "g++")
        _run([gxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", HOSTSRC,
              "-o", CLI, *srcs, "-L", BUILD, "-lgravidy_gb300", f"-Wl,-rpath,{BUILD}", "-fopenmp"])
    return CLI


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_library(force=force, verbose=verbose)
    build_cli(force=force)


if __name__ == "__main__":
    if "--bounds-check" in sys.argv:
        print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv, bounds_check=True))
    else:
        build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
        print(LIB)
