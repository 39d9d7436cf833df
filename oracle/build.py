"""Build recipe for the oracle libraries (test infrastructure only).

* oracle/liboracle.so  -- the C restatements in oracle/wmom_oracle.c (fill, unblocked
  LU) and oracle/topology_oracle.c (geoinp + configwire), and the double-double
  residual of oracle/refine_oracle.c (always built).
* oracle/_ref/libwmomref.so -- the reference's own Configuration.cpp, Zmatrix.cpp and
  Complex.cpp, compiled UNMODIFIED where they lie in the reference checkout, plus
  oracle/ref_harness.cpp.  Built only when that checkout is present (it is not on
  the GPU machine); outputs go to oracle/_ref/ only.

Both use -ffp-contract=off so no multiply-add is fused, which keeps x86-64 and
aarch64 builds bit-identical to each other.

The reference checkout is found through WMOM_REFERENCE_DIR (or --reference-dir):
the directory holding the reference's CPU variant ("wersja referencyjna").  Without
it an existing oracle/_ref build is kept and nothing new is compiled from the
reference.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("WMOM_REFERENCE_DIR") or None
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"

PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libwmomref.so")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _arch_ok(lib):
    stamp = lib + ".arch"
    return os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()


def _stamp(lib):
    with open(lib + ".arch", "w") as f:
        f.write(platform.machine())


PORT_SOURCES = ["wmom_oracle.c", "topology_oracle.c", "refine_oracle.c"]


def build_port(force=False):
    srcs = [os.path.join(HERE, f) for f in PORT_SOURCES]
    if not force and _newer(PORT_SO, srcs) and _arch_ok(PORT_SO):
        return PORT_SO
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", PORT_SO] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    _stamp(PORT_SO)
    return PORT_SO


def reference_available():
    return bool(REF_DIR) and all(os.path.exists(os.path.join(REF_DIR, f))
                                 for f in ("Zmatrix.cpp", "Configuration.cpp", "Complex.cpp"))


def build_ref(force=False):
    if not reference_available():
        return REF_SO if os.path.exists(REF_SO) and _arch_ok(REF_SO) else None
    srcs = [os.path.join(REF_DIR, f) for f in ("Configuration.cpp", "Zmatrix.cpp", "Complex.cpp")]
    srcs.append(os.path.join(HERE, "ref_harness.cpp"))
    if not force and _newer(REF_SO, srcs) and _arch_ok(REF_SO):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-fpermissive",
           "-I", REF_DIR, "-I", CUDA_INC, "-o", REF_SO] + srcs
    subprocess.check_call(cmd)
    _stamp(REF_SO)
    return REF_SO


DRIVER_OBJ = os.path.join(HERE, "_ref", "Wire_MoM.o")
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")


def build_ref_driver(force=False):
    """The reference's driver, "wersja referencyjna/Wire_MoM.cu" (its main() and GPU
    fill kernels), compiled UNMODIFIED into oracle/_ref/Wire_MoM.o with the stand-in
    mkl.h / mpi.h of oracle/shim, for the test that links it against libwmom
    instead of Configuration.cpp, Zmatrix.cpp and Complex.cpp."""
    if not reference_available() or not os.path.exists(os.path.join(REF_DIR, "Wire_MoM.cu")):
        return DRIVER_OBJ if os.path.exists(DRIVER_OBJ) and _arch_ok(DRIVER_OBJ) else None
    srcs = [os.path.join(REF_DIR, f) for f in ("Wire_MoM.cu", "Wire_MoM.h")] + \
        [os.path.join(HERE, "shim", f) for f in ("mkl.h", "mpi.h")]
    if not force and _newer(DRIVER_OBJ, srcs) and _arch_ok(DRIVER_OBJ):
        return DRIVER_OBJ
    os.makedirs(os.path.dirname(DRIVER_OBJ), exist_ok=True)
    cmd = [NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-w", "-Xcompiler", "-fpermissive",
           "-I", os.path.join(HERE, "shim"), "-I", REF_DIR, "-c", os.path.join(REF_DIR, "Wire_MoM.cu"), "-o",
           DRIVER_OBJ]
    subprocess.check_call(cmd)
    _stamp(DRIVER_OBJ)
    return DRIVER_OBJ


def main():
    global REF_DIR
    if "--reference-dir" in sys.argv:
        REF_DIR = sys.argv[sys.argv.index("--reference-dir") + 1]
    print(build_port(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_driver(force="--force" in sys.argv))


if __name__ == "__main__":
    main()
