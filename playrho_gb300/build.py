"""Builds libprgpu.so (the CUDA world step behind include/prgpu.h) in-tree.

nvcc compiles each translation unit for sm_103a in parallel and links a shared
library next to this file.  --fmad=false keeps a*b+c as two rounded operations
(the reference's own arithmetic); host code is built with -ffp-contract=off for
the same reason on both x86-64 and aarch64 hosts.
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
LIB = os.path.join(HERE, "libprgpu.so")
# C++ host layer over the C ABI (HostWorld), a second library linked to the first
HOST_SOURCES = [os.path.join(HERE, "host", "host_world.cpp")]
HOST_LIB = os.path.join(HERE, "libprgpu_host.so")
# longest compiles first; prgpu_solver_{full,lean,tape}.cu each compile one
# k_world_solve instance out of prgpu_solver.cu
SOURCES = ["prgpu_solver_full.cu", "prgpu_solver_lean.cu", "prgpu_solver_tape.cu", "prgpu_solver.cu",
           "prgpu_adjoint.cu", "prgpu_toi.cu", "prgpu_contacts.cu", "prgpu_world.cu", "prgpu_prims.cu", "prgpu_query.cu"]
# files that include another .cu
CU_DEPS = {f: ["prgpu_solver.cu"] for f in ("prgpu_solver_full.cu", "prgpu_solver_lean.cu", "prgpu_solver_tape.cu")}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(HERE, "..", "include", "prgpu.h"))
    flags = NVCC_FLAGS + list(extra_flags or [])
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        deps = [s, __file__] + headers + [os.path.join(CSRC, x) for x in CU_DEPS.get(src, [])]
        if _stale(o, deps):
            jobs.append([nvcc(), *ARCH, *flags, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or res.returncode:
                sys.stderr.write(res.stdout + res.stderr)
            if res.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed")
    host_deps = HOST_SOURCES + [os.path.join(HERE, "host", "host_world.hpp"), LIB, __file__] + headers
    if _stale(HOST_LIB, host_deps):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared",
               "-I" + os.path.join(HERE, "..", "include"), *HOST_SOURCES, "-L" + HERE, "-lprgpu",
               "-Wl,-rpath,$ORIGIN", "-o", HOST_LIB]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("host library build failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
