"""Build libipfem.so in-tree for sm_103a (GB300).

nvcc compiles the CUDA translation units (one -gencode, --fmad=false so that
multiply-adds are fused only where the source writes fma()), g++ the host
C++ (with -ffp-contract=off), in parallel; the shared library lands next to
this file.  No CMake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libipfem.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU = ["k_constitutive.cu", "k_assembly.cu", "k_solver.cu", "k_mlp.cu", "k_net_tc.cu", "capi_mlp.cu"]
CPP = ["capi.cpp", "host_setup.cpp", "host_gmsh.cpp"]
HEADERS = ["ipfem_internal.h", "constitutive.cuh", "tma.cuh", "pdl.cuh", "ldhint.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    h = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if h and os.path.exists(os.path.join(h, "bin", "nvcc")):
        return h
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    return "/usr/local/cuda"


def _deps():
    return [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "ipfem.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    inc = os.path.join(home, "include")
    jobs = []
    objs = []
    for f in CU:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + _deps()):
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler",
                                   "-fPIC,-ffp-contract=off", "-I" + INCLUDE, "-c", src, "-o", obj]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for f in CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + _deps()):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-I" + inc,
                         "-I" + INCLUDE, "-c", src, "-o", obj])
    out = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            out = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        for o in out:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
