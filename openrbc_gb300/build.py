"""Build liborbc_gpu.so (sm_103a) in-tree with nvcc and g++.

Sources: csrc/*.cu (device kernels + host engine), csrc/*.cpp (host-only
workload generators) and driver/openrbc_gpu.cpp (the command-line host
driver).  Objects go to _build/, the library to openrbc_gb300/liborbc_gpu.so.
Translation units compile in parallel; an up-to-date library is not rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liborbc_gpu.so")
DRIVER = os.path.join(PKG, "openrbc_gpu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                 + glob.glob(os.path.join(INCLUDE, "*.h")))
    return cu, cpp, hdr


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    cu, cpp, hdr = _sources()
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdr):
            jobs.append([nv, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdr):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
                         "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if force or _stale(LIB, objs):
        _run([nv, "-shared", *ARCH, "-o", LIB, *objs])
    drv = os.path.join(PKG, "driver", "openrbc_gpu.cpp")
    if os.path.exists(drv) and (force or _stale(DRIVER, [drv, LIB] + hdr)):
        _run(["g++", "-std=c++17", "-O2", "-I", INCLUDE, drv, "-o", DRIVER, "-L", PKG, "-lorbc_gpu",
              f"-Wl,-rpath,{PKG}"])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
