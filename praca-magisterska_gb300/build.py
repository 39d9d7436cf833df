"""Builds libwmom.so in-tree for sm_103a (GB300).

Host C++ translation units are compiled with g++ (no multiply-add contraction, so
the float -> double geometry arithmetic rounds like the reference's CPU code); CUDA
translation units with nvcc for compute_103a/sm_103a only.  Objects go to
_build/, the library to this directory.  CUDA's runtime is linked statically, so
the library loads on machines without a GPU (calls then fail with
WMOM_ERR_UNSUPPORTED / WMOM_ERR_CUDA).
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwmom.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CPP_SOURCES = ["topology.cpp", "plan.cpp", "dropin.cpp"]
CU_SOURCES = ["fill.cu", "lu.cu", "solve.cu", "api.cu", "lu_tc.cu", "lu_emul.cu", "stats.cu", "noalloc.cu", "condest.cu", "lu_dmma.cu"]
HEADERS = ["wmom_internal.h", "lu_common.cuh", "lu_internal.h", "solve_internal.h", "stats.h"]


def _deps():
    deps = [os.path.join(CSRC, h) for h in HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "wmom.h"))
    deps.append(os.path.join(HERE, "..", "include", "wmom_dropin.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _deps())


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _stale(obj, path):
        return obj
    inc = ["-I", CSRC, "-I", os.path.join(HERE, "..", "include"), "-I", os.path.join(CUDA_HOME, "include")]
    if src.endswith(".cpp"):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-c", path, "-o", obj] + inc
    else:
        cmd = [NVCC] + ARCH + ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-c", path, "-o", obj,
                               "-Xptxas", "-warn-spills"] + inc
        if os.environ.get("WMOM_PTXAS_VERBOSE"):
            cmd += ["-Xptxas", "-v"]
    subprocess.check_call(cmd)
    return obj


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "ARCH")
    machine = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != machine:
        force = True  # objects from another host architecture
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = CPP_SOURCES + CU_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        subprocess.check_call(cmd)
    with open(stamp, "w") as f:
        f.write(machine)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
