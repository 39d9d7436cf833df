"""The reference's unmodified driver links against libwmom (CPU, link only).

oracle/build.py compiles "wersja referencyjna/Wire_MoM.cu" (the reference's main()
and its own GPU fill kernels) unmodified into oracle/_ref/Wire_MoM.o, with stand-in
mkl.h / mpi.h headers; that object exists only where the reference checkout was
available when the oracle was built.  This test links it against libwmom.so instead
of the reference's Configuration.cpp, Zmatrix.cpp and Complex.cpp (the LAPACKE pair
comes from the oracle's unblocked LU, so no MKL is needed) and checks that:
* the link succeeds;
* geoinp, config and zmatrix -- the calls of Wire_MoM.cu:90,162,342 -- are
  undefined in the program and defined by libwmom.so, which the program needs;
* the program defines none of the reference's fill or topology functions, i.e. no
  reference object besides the driver itself was linked.
Running it needs a GPU (its fill runs in libwmom); the GPU tests exercise the same
drop-in symbols through the C ABI and the mangled names (tests/test_cli_gpu.py).
"""
import os
import re
import subprocess

import pytest

from conftest import ROOT

OBJ = os.path.join(ROOT, "oracle", "_ref", "Wire_MoM.o")
PKG = os.path.join(ROOT, "praca-magisterska_gb300")
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")


def _symbols(path, dynamic=False, defined=None):
    """Demangled symbol names from nm (the text after the symbol type letter)."""
    cmd = ["nm", "-C"] + (["-D"] if dynamic else []) + (["--defined-only"] if defined else []) + \
        (["--undefined-only"] if defined is False else []) + [path]
    out = subprocess.run(cmd, capture_output=True, text=True, check=True).stdout
    names = []
    for line in out.splitlines():
        m = re.match(r"^\s*(?:[0-9a-fA-F]+\s+)?[A-Za-z?-]\s+(.*)$", line)
        if m:
            names.append(m.group(1))
    return names


def test_reference_driver_links_against_libwmom(tmp_path, wmom):
    from oracle import build as ob
    if not (os.path.exists(OBJ) and ob._arch_ok(OBJ)):
        pytest.skip("oracle/_ref/Wire_MoM.o is built only where the reference checkout is "
                    "(WMOM_REFERENCE_DIR)")
    exe = str(tmp_path / "wire_mom")
    cmd = [NVCC, "-o", exe, OBJ, os.path.join(ROOT, "oracle", "shim", "lapacke_oracle.c"),
           os.path.join(ROOT, "oracle", "wmom_oracle.c"), "-I", os.path.join(ROOT, "oracle", "shim"),
           "-L", PKG, "-lwmom", "-Xlinker", "-rpath," + PKG, "-Xcompiler", "-fopenmp"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]

    undefined = " ".join(_symbols(exe, defined=False))
    lib_defined = " ".join(_symbols(os.path.join(PKG, "libwmom.so"), dynamic=True, defined=True))
    for call in ("geoinp(int, int, int, int&,", "config(int&, int,", "zmatrix(double2*, float*,"):
        assert call in undefined, call
        assert call in lib_defined, call
    needed = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True, check=True).stdout
    assert "libwmom.so" in needed

    # nothing from the reference's Zmatrix.cpp, Configuration.cpp or Complex.cpp
    exe_defined = set(s.split("(")[0] for s in _symbols(exe, defined=True))
    for fn in ("wim", "cwire1_re", "cwire2_re", "ckmn", "cknn", "delick", "geoinp", "config", "configwire",
               "zmatrix", "clCmul", "clCdiv", "clCabs"):
        assert fn not in exe_defined, fn
    # the driver's own GPU fill entry point stays the reference's (it is in Wire_MoM.cu)
    assert "zmatrix_gpu" in exe_defined
