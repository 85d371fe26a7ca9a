"""In-tree build of libbsgpu.so (sm_103a) and the drop-in blackscholes and
swaptions CLIs.

Compiles each translation unit with nvcc in parallel, links the shared
library next to this file and the CLIs into ``p3arsec_gb300/bin/``.  No
torch, no cmake: ``python -m p3arsec_gb300.build`` or ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbsgpu.so")
CLI = os.path.join(PKG, "bin", "blackscholes_gpu")
SWAPTIONS_CLI = os.path.join(PKG, "bin", "swaptions_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-Wall", "-I" + os.path.join(ROOT, "include"),
                     "-I" + CSRC]
CU_SOURCES = ["bsg_kernels.cu", "bsg_api.cu", "bsg_serve.cu", "bsg_noalloc.cu", "bsg_swaptions.cu"]
CPP_SOURCES = ["bsg_io.cpp"]  # host code, compiled with g++
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-pthread",
             "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbsgpu.so")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(ROOT, "include", "bsg.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    """Build libbsgpu.so and the CLI if stale; returns the library path.

    Processes building at once (one per rank under torchrun) take turns on a
    lock file, and the library and CLI are linked to a temporary name and
    renamed into place, so a process that has the library loaded never sees
    it rewritten."""
    os.makedirs(BUILD, exist_ok=True)
    import fcntl
    with open(os.path.join(BUILD, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(verbose, force)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(verbose: bool, force: bool) -> str:
    nv = nvcc()
    heads = _headers()
    jobs = []
    objs = []
    sources = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    for src in sources:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + heads):
            jobs.append([nv] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(BUILD, src.replace(".cpp", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + heads):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    for exe, src in ((CLI, "blackscholes_gpu.cpp"), (SWAPTIONS_CLI, "swaptions_gpu.cpp")):
        cli_src = os.path.join(HOST, src)
        if os.path.exists(cli_src) and (force or _stale(exe, [cli_src, LIB] + heads)):
            os.makedirs(os.path.dirname(exe), exist_ok=True)
            tmp = exe + ".tmp"
            _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"),
                  cli_src, "-o", tmp, "-L" + PKG, "-lbsgpu", "-Wl,-rpath,$ORIGIN/..",
                  "-lpthread"])
            os.replace(tmp, exe)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
