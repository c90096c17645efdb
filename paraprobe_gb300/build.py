"""Build recipe for the native library (no cmake; nvcc + g++ in parallel).

Produces, in-tree:
  paraprobe_gb300/_lib/libparaprobe_gb300.so   CUDA kernels + C ABI + host I/O
  paraprobe_gb300/_lib/paraprobe_gpu           drop-in CLI: <simid> <settings.xml>
Device code is compiled for sm_103a only, with --fmad=false so that no float
expression is contracted into a fused multiply-add.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libparaprobe_gb300.so")
CLI = os.path.join(OUT, "paraprobe_gpu")

NVCC = os.environ.get("NVCC", "nvcc")


def _cuda_home():
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return env
    for d in os.environ.get("PATH", "").split(os.pathsep):
        if os.path.exists(os.path.join(d, "nvcc")):
            return os.path.dirname(os.path.abspath(d))
    return "/usr/local/cuda"


CUDA_HOME = _cuda_home()
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
           "-I" + os.path.join(ROOT, "include")] + ARCH
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
            "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]

CU_SOURCES = ["pp_kernels.cu", "pp_capi.cu", "pp_noalloc.cu"]
CPP_SOURCES = [os.path.join(CSRC, "pp_shuffle.cpp")]


def _host_sources():
    if not os.path.isdir(HOST):
        return []
    return sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp") and f != "paraprobe_gpu.cpp")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _check_machine():
    """Objects built on another architecture (the tree is shared between an
    x86 development host and Arm GPU hosts) are discarded, never linked."""
    import platform
    import shutil
    stamp = os.path.join(OUT, "machine.txt")
    here = platform.machine()
    if os.path.exists(stamp) and open(stamp).read().strip() == here:
        return
    shutil.rmtree(OUT, ignore_errors=True)
    os.makedirs(OBJ, exist_ok=True)
    with open(stamp, "w") as f:
        f.write(here + "\n")


def build(verbose: bool = False) -> str:
    _check_machine()
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h") or f.endswith(".cuh")]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([NVCC] + NVFLAGS + ["-c", s, "-o", o])
    for s in CPP_SOURCES + _host_sources():
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++"] + CXXFLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    cli_src = os.path.join(HOST, "paraprobe_gpu.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + headers):
        _run(["g++"] + CXXFLAGS + [cli_src, "-o", CLI, "-L" + OUT, "-lparaprobe_gb300",
                                   "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
