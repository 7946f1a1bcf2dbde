"""Build the engine in-tree: libvegas_gpu.so (CUDA, sm_103a) and the C++ host tools.

Sources are compiled in parallel with nvcc / g++ into ``_build/`` and linked
into ``vegas_gb300/libvegas_gpu.so`` and ``_build/bin/``.  One -gencode only
(sm_103a); nothing here depends on PyTorch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
HOST = os.path.join(ROOT, "host")
BUILD = os.path.join(ROOT, "_build")
PKG = os.path.join(ROOT, "vegas_gb300")
INCLUDE = os.path.join(REPO, "include")
LIB = os.path.join(PKG, "libvegas_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["vg_api.cu", "vg_ising.cu", "vg_heis.cu", "vg_noalloc.cu", "vg_batch.cu", "vg_resident.cu", "vg_hbatch.cu", "vg_wolff.cu", "vg_energy.cu", "vg_tiled.cu"]
HOST_PROGRAMS = {  # binary name -> source under host/
    "vegas_gpu_cli": "vegas_gpu_cli.cpp",
    "host_selftest": "host_selftest.cpp",
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvegas_gpu.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, "vegas_gpu.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    heads = _headers()
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + heads):
            cmd = [nv, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if jobs or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    build_host()
    return LIB


def build_host() -> None:
    """C++ host mirror programs (link against libvegas_gpu.so)."""
    bindir = os.path.join(BUILD, "bin")
    os.makedirs(bindir, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    hdrs = [os.path.join(HOST, "vegas", f) for f in os.listdir(os.path.join(HOST, "vegas"))] if os.path.isdir(
        os.path.join(HOST, "vegas")) else []
    jobs = []
    for name, src in HOST_PROGRAMS.items():
        s = os.path.join(HOST, src)
        if not os.path.exists(s):
            continue
        out = os.path.join(bindir, name)
        if _stale(out, [s, LIB, os.path.join(INCLUDE, "vegas_gpu.h")] + hdrs):
            jobs.append([cxx, "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, "-I", HOST, s, "-o", out,
                         "-L", PKG, "-lvegas_gpu", f"-Wl,-rpath,{PKG}"])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="-v" in sys.argv))
